"""GPU test of the allocation-free self-energy entry point.

Hosts that own all device memory (a single preallocated pool, a hard memory budget, or an
allocation-free hot loop) cannot let the library call cudaMalloc; they use
qk_RGW_self_energy_diag_noalloc_dev, whose only scratch is a static device array.  This test
calls it through the C ABI on device buffers and checks it against the existing entry point
qk_RGW_self_energy_diag, at the tolerance of the other self-energy tests, on two calls in a row
with different systems (the second, smaller one must not see the first call's leftovers).
The file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from oracle import qkgw_oracle as O
from quack_gb300 import api, synth

pytestmark = pytest.mark.gpu


def _case(N, nO, seed, eta):
    s = synth.small_system(N, nO, 3 * N, seed)
    E = synth.eri_phys_numpy(s["L"])
    nS = nO * (N - nO)
    A = O.phRLR_A(1, True, N, 0, nO, N - nO, 0, nS, 1.0, s["eHF"], E)
    B = O.phRLR_B(1, True, N, 0, nO, N - nO, 0, nS, 1.0, E)
    _, Om, XpY, _ = O.phRLR(False, nS, A, B)
    rho = O.RGW_excitation_density(N, 0, nO, 0, nS, E, XpY)
    return dict(N=N, nC=0, nO=nO, nR=0, nS=nS, e=s["eHF"], Om=Om, rho=rho, eta=eta)


def _rand_case(N, nC, nO, nR, seed, eta):
    """Random energies, excitation energies and densities: only the two entry points are compared."""
    rng = np.random.default_rng(seed)
    nS = (nO - nC) * (N - nO - nR)
    e = np.sort(np.concatenate([rng.uniform(-20.0, -0.3, nO), rng.uniform(0.05, 5.0, N - nO)]))
    Om = np.sort(rng.uniform(0.3, 30.0, nS))
    rho = rng.standard_normal((N, N, nS)) * 0.05
    return dict(N=N, nC=nC, nO=nO, nR=nR, nS=nS, e=e, Om=Om, rho=rho, eta=eta)


def _run_noalloc(lib, case):
    import torch
    N, nC, nO, nR, nS = case["N"], case["nC"], case["nO"], case["nR"], case["nS"]
    de = torch.from_numpy(case["e"]).cuda()
    dOm = torch.from_numpy(case["Om"]).cuda()
    drho = torch.from_numpy(np.asfortranarray(case["rho"]).ravel(order="F")).cuda()
    dSig = torch.full((N,), np.nan, dtype=torch.float64, device="cuda")
    dZ = torch.full((N,), np.nan, dtype=torch.float64, device="cuda")
    dgm = torch.full((1,), np.nan, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.qk_RGW_self_energy_diag_noalloc_dev(
        ctypes.c_double(case["eta"]), N, N, nC, nO, N - nO, nR, nS,
        ctypes.c_void_p(de.data_ptr()), ctypes.c_void_p(dOm.data_ptr()),
        ctypes.c_void_p(drho.data_ptr()), ctypes.c_void_p(dgm.data_ptr()),
        ctypes.c_void_p(dSig.data_ptr()), ctypes.c_void_p(dZ.data_ptr()), ctypes.c_void_p(0))
    return rc, dSig.cpu().numpy(), dZ.cpu().numpy(), float(dgm.cpu()[0])


def _check_against_existing(ctx, lib, case):
    N, nC, nO, nR, nS = case["N"], case["nC"], case["nO"], case["nR"], case["nS"]
    # existing entry point (host pointers, context workspace)
    gm_ref, Sig_ref, Z_ref = api.RGW_self_energy_diag(case["eta"], N, N, nC, nO, N - nO, nR, nS,
                                                      case["e"], case["Om"], case["rho"], ctx=ctx)
    # allocation-free entry point on caller-owned device buffers
    rc, Sig, Z, gm = _run_noalloc(lib, case)
    assert rc == api.QK_OK
    assert np.allclose(Sig, Sig_ref, rtol=1e-11, atol=1e-13)
    assert np.allclose(Z, Z_ref, rtol=1e-11, atol=1e-13)
    assert abs(gm - gm_ref) < 1e-11 * max(1.0, abs(gm_ref))


def test_self_energy_noalloc_matches_existing_entry_point(ctx):
    lib = api.lib()
    assert hasattr(lib, "qk_RGW_self_energy_diag_noalloc_dev")
    # two calls in a row; the second, smaller one must not see the first call's leftovers
    for case in (_case(40, 5, 31, 0.0), _case(24, 3, 32, 0.05)):
        _check_against_existing(ctx, lib, case)


def test_self_energy_noalloc_frozen_and_limits(ctx):
    lib = api.lib()
    # frozen core and frozen virtuals: the p offset (nC) and the p < nBas - nR bound
    _check_against_existing(ctx, lib, _rand_case(40, 2, 8, 3, 41, 0.0))
    # 3 orbital tiles and nS = 1024: 128 chunks of 8 excitations, the chunk cap
    _check_against_existing(ctx, lib, _rand_case(80, 0, 16, 0, 42, 0.01))
    # nBas at the 1024-orbital maximum (one occupied, two active virtuals, the rest frozen)
    _check_against_existing(ctx, lib, _rand_case(1024, 0, 1, 1021, 43, 0.0))


def test_self_energy_noalloc_rejects_bad_counts(ctx):
    lib = api.lib()
    case = _rand_case(24, 0, 3, 0, 44, 0.0)
    N, nO, nS = case["N"], case["nO"], case["nS"]
    p = ctypes.c_void_p(8)
    # nV must be nBas - nO; nOrb must lie in [nO, nBas]
    for nOrb, nV in ((N, N - nO - 1), (N + 1, N - nO), (nO - 1, N - nO)):
        rc = lib.qk_RGW_self_energy_diag_noalloc_dev(ctypes.c_double(0.0), N, nOrb, 0, nO, nV, 0,
                                                     nS, p, p, p, p, p, p, ctypes.c_void_p(0))
        assert rc == api.QK_ERR_ARG


def test_self_energy_noalloc_rejects_oversized(ctx):
    lib = api.lib()
    N, nO = 1100, 10
    rc = lib.qk_RGW_self_energy_diag_noalloc_dev(
        ctypes.c_double(0.0), N, N, 0, nO, N - nO, 0, nO * (N - nO), ctypes.c_void_p(8),
        ctypes.c_void_p(8), ctypes.c_void_p(8), ctypes.c_void_p(8), ctypes.c_void_p(8),
        ctypes.c_void_p(8), ctypes.c_void_p(0))
    assert rc == api.QK_ERR_ARG
