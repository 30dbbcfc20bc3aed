"""CPU tests of the C ABI boundary: the library builds, loads and exports exactly what
include/qkgw.h declares (no compute calls: there may be no GPU here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "include", "qkgw.h")


def declared_symbols():
    txt = open(HDR).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char\*|long long|void)\s+(qk_\w+)\s*\(", txt,
                                 flags=re.M)))


@pytest.fixture(scope="module")
def libpath():
    from quack_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("qk_init", "qk_RG0W0", "qk_evRGW", "qk_phRLR", "qk_RGW_excitation_density",
              "qk_RGW_self_energy_diag", "qk_RGW_QP_graph", "qk_AOtoMO_ERI_RHF",
              "qk_DIIS_extrapolation", "qk_dsyev_dev"):
        assert s in syms


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_api_binds_every_symbol(libpath):
    from quack_gb300 import api
    L = api.lib()
    for s in declared_symbols():
        getattr(L, s)


def test_fortran_module_binds_declared_symbols_with_their_arity(libpath):
    """Every bind(C, name=...) interface of include/qk_gw_module.f90 names a symbol that the C
    header declares and the library exports, with the same number of arguments."""
    f90 = open(os.path.join(ROOT, "include", "qk_gw_module.f90")).read()
    hdr = re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)
    lib = ctypes.CDLL(libpath)
    found = re.findall(r"function\s+(\w+)\s*\(([^)]*)\)\s*(?:&\s*)?bind\(C,\s*name=\"(\w+)\"\)",
                       f90.replace("&\n", " "))
    assert len(found) >= 10
    for fname, args, cname in found:
        assert fname == cname
        assert hasattr(lib, cname), cname
        m = re.search(r"\b" + cname + r"\s*\(([^;]*)\);", hdr)
        assert m, cname
        n_c = len([x for x in m.group(1).split(",") if x.strip()])
        n_f = len([x for x in args.split(",") if x.strip()])
        assert n_c == n_f, (cname, n_c, n_f)


def test_init_without_gpu_reports_no_device(libpath):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    lib = ctypes.CDLL(libpath)
    h = ctypes.c_void_p()
    rc = lib.qk_init(0, ctypes.byref(h))
    assert rc == 8  # QK_ERR_NO_DEVICE, and no exit()/abort


def test_gauss_legendre_nodes_match_numpy(libpath):
    """Host code of the frequency quadrature: the Gauss-Legendre rule against numpy."""
    import numpy as np
    from quack_gb300 import api
    for n in (1, 2, 5, 24, 32, 48, 64):
        x, w = api.gauss_legendre(n)
        xr, wr = np.polynomial.legendre.leggauss(n)
        assert np.allclose(x, xr, rtol=0, atol=1e-14), n
        assert np.allclose(w, wr, rtol=1e-11, atol=1e-15), n  # end weights: P_n' cancellation
