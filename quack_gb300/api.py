"""Python mirror of QuAcK's restricted G0W0/evGW call chain on top of libqkgw.so.

Each function has the name, argument order and meaning of the Fortran subroutine it replaces
(the C ABI in include/qkgw.h cites the reference file:line of each).  Arrays are numpy arrays
indexed like the Fortran ones with 0-based indices (ERI[p,q,r,s] = ERI(p+1,q+1,r+1,s+1)); they
are handed to the library in Fortran (column-major) memory order.  Every call runs on the GPU;
there is no CPU fallback -- if the CUDA library is missing or no GB300 is visible the calls
raise :class:`QkError`.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBPATH = os.path.join(_HERE, "libqkgw.so")
_lib = None

QK_OK, QK_ERR_ARG, QK_ERR_CUDA, QK_ERR_NOMEM, QK_ERR_NOT_PD, QK_ERR_NO_CONV = 0, 1, 2, 3, 4, 5
QK_ERR_UNSUPPORTED, QK_ERR_DEVICE, QK_ERR_NO_DEVICE = 6, 7, 8
# device-side status bits of the last call (qk_last_device_status)
QKD_BARRIER_TIMEOUT, QKD_BAD_INDEX, QKD_NEG_AMB, QKD_NEG_OMEGA, QKD_QP_NOCONV, QKD_MBAR_TIMEOUT = \
    1, 2, 4, 8, 16, 32
QK_PREC_FP64, QK_PREC_BF16X3 = 0, 1

_dp = C.POINTER(C.c_double)


class QkError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("qkgw error %d: %s" % (code, msg))
        self.code = code


class qk_gw_params(C.Structure):
    _fields_ = [("eta", C.c_double), ("linearize", C.c_int), ("doSRG", C.c_int),
                ("TDA_W", C.c_int), ("maxSCF", C.c_int), ("thresh", C.c_double),
                ("max_diis", C.c_int), ("precision", C.c_int), ("qp_guess", C.c_int)]


def lib():
    """Load libqkgw.so (built in-tree by quack_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIBPATH):
            raise QkError(QK_ERR_NO_DEVICE, "libqkgw.so not built (run quack_gb300.build.build())")
        _lib = C.CDLL(_LIBPATH)
        _lib.qk_last_error_string.restype = C.c_char_p
        _lib.qk_timing_name.restype = C.c_char_p
        _lib.qk_launch_count.restype = C.c_longlong
        for name in ("qk_RGW_self_energy_diag", "qk_RGW_SRG_self_energy_diag", "qk_RGW_QP_graph",
                     "qk_phRLR_A", "qk_phRLR_B"):
            getattr(_lib, name).restype = C.c_int
    return _lib


def _ptr(a):
    return a.ctypes.data_as(_dp)


def _f(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


class qk_bse_params(C.Structure):
    _fields_ = [("TDA_W", C.c_int), ("TDA", C.c_int), ("singlet", C.c_int), ("triplet", C.c_int),
                ("exchange_kernel", C.c_int), ("eta", C.c_double)]


class qk_sys_desc(C.Structure):
    _fields_ = [("nOrb", C.c_int), ("nC", C.c_int), ("nO", C.c_int), ("nR", C.c_int),
                ("naux", C.c_int), ("offset_L", C.c_longlong), ("offset_e", C.c_longlong)]


class Context:
    """A qk_ctx: one CUDA stream plus cached device workspace on one GPU."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        rc = lib().qk_init(C.c_int(device), C.byref(self._h))
        if rc != QK_OK:
            raise QkError(rc, "qk_init failed (no usable sm_103a device?)")

    @property
    def handle(self):
        return self._h

    def check(self, rc, allow=()):
        if rc != QK_OK and rc not in allow:
            raise QkError(rc, lib().qk_last_error_string(self._h).decode())
        return rc

    def timings(self):
        L = lib()
        n = L.qk_num_timings()
        buf = (C.c_double * n)()
        L.qk_get_timings(self._h, buf, n)
        return {L.qk_timing_name(i).decode(): buf[i] for i in range(n)}

    def batch_group_stats(self):
        """(grouped tridiagonalisation launches, matrices) of the last batched call."""
        a, b = C.c_longlong(), C.c_longlong()
        self.check(lib().qk_batch_group_stats(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def last_device_status(self) -> int:
        """QKD_* bits recorded on the device during the last call."""
        return int(lib().qk_last_device_status(self._h))

    def launches(self) -> int:
        return int(lib().qk_launch_count(self._h))

    def qp_evals(self) -> int:
        """Sigma evaluations (orbital x Newton step) of the last graphical QP solve."""
        lib().qk_qp_evals.restype = C.c_longlong
        return int(lib().qk_qp_evals(self._h))

    def autotune(self, nOrb, nS):
        """Time the tunable launch parameters on problems of these sizes; keep the fastest."""
        self.check(lib().qk_autotune(self._h, nOrb, nS, 0))

    def tune_query(self, name, size):
        lib().qk_tune_query.argtypes = [C.c_void_p, C.c_char_p, C.c_longlong]
        return int(lib().qk_tune_query(self._h, name.encode(), size))

    def tune_set(self, name, size, value):
        lib().qk_tune_set.argtypes = [C.c_void_p, C.c_char_p, C.c_longlong, C.c_int]
        self.check(lib().qk_tune_set(self._h, name.encode(), size, value))

    def tune_save(self, path):
        self.check(lib().qk_tune_save(self._h, str(path).encode()))

    def tune_load(self, path):
        self.check(lib().qk_tune_load(self._h, str(path).encode()))

    def set_graph_mode(self, on=True):
        """evGW cycles 2.. replayed from one CUDA graph with a device-side WHILE loop."""
        self.check(lib().qk_set_graph_mode(self._h, int(bool(on))))

    def set_stage_precision(self, precision):
        """Tier of the stage-level drop-ins (excitation density, self-energy, QP graph)."""
        self.check(lib().qk_set_stage_precision(self._h, int(precision)))

    def set_feature_capture(self, on=True):
        self.check(lib().qk_set_feature_capture(self._h, int(bool(on))))

    def features(self, N):
        """Raw per-orbital features (N x 16) captured by the last G0W0 driver call."""
        buf = (C.c_float * (N * 16))()
        lib().qk_get_features(self._h, buf, N * 16)
        return np.array(buf[:], dtype=np.float32).reshape(N, 16)

    def set_qp_model(self, model):
        self.check(lib().qk_set_qp_model(self._h, model.handle if model is not None else None))

    def qp_iters(self, n):
        """Newton steps per orbital of the last graphical QP solve (64 = not converged)."""
        buf = (C.c_int * n)()
        lib().qk_get_qp_iters(self._h, buf, n)
        return np.array(buf[:], dtype=np.int64)

    def close(self):
        if self._h:
            lib().qk_finalize(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default = None


def default_context() -> Context:
    global _default
    if _default is None:
        _default = Context(0)
    return _default


def _ctx(ctx):
    return ctx if ctx is not None else default_context()


# ------------------------------------------------------------------------------------------
# stage-level drop-ins (same names/arguments as the Fortran subroutines)
# ------------------------------------------------------------------------------------------
def phRLR_A(ispin, dRPA, nBas, nC, nO, nV, nR, nS, lam, e, ERI, ctx=None):
    """LR/phRLR_A.f90.  Returns Aph (nS, nS)."""
    c = _ctx(ctx)
    e, ERI = _f(e), _f(ERI)
    out = np.empty((nS, nS), order="F")
    c.check(lib().qk_phRLR_A(c.handle, ispin, int(bool(dRPA)), nBas, nC, nO, nV, nR, nS,
                             C.c_double(lam), _ptr(e), _ptr(ERI), _ptr(out)))
    return out


def phRLR_B(ispin, dRPA, nBas, nC, nO, nV, nR, nS, lam, ERI, ctx=None):
    """LR/phRLR_B.f90.  Returns Bph (nS, nS)."""
    c = _ctx(ctx)
    ERI = _f(ERI)
    out = np.empty((nS, nS), order="F")
    c.check(lib().qk_phRLR_B(c.handle, ispin, int(bool(dRPA)), nBas, nC, nO, nV, nR, nS,
                             C.c_double(lam), _ptr(ERI), _ptr(out)))
    return out


def phRLR(TDA, nS, Aph, Bph, ctx=None):
    """LR/phRLR.f90.  Returns (EcRPA, Om, XpY, XmY) with XpY[m, ia]."""
    c = _ctx(ctx)
    Aph, Bph = _f(Aph), _f(Bph)
    Om = np.empty(nS)
    XpY = np.empty((nS, nS), order="F")
    XmY = np.empty((nS, nS), order="F")
    Ec = C.c_double()
    c.check(lib().qk_phRLR(c.handle, int(bool(TDA)), nS, _ptr(Aph), _ptr(Bph), C.byref(Ec),
                           _ptr(Om), _ptr(XpY), _ptr(XmY)))
    return Ec.value, Om, XpY, XmY


def RGW_excitation_density(nOrb, nC, nO, nR, nS, ERI, XpY, ctx=None):
    """GW/RGW_excitation_density.f90.  Returns rho (nOrb, nOrb, nS)."""
    c = _ctx(ctx)
    ERI, XpY = _f(ERI), _f(XpY)
    rho = np.empty((nOrb, nOrb, nS), order="F")
    c.check(lib().qk_RGW_excitation_density(c.handle, nOrb, nC, nO, nR, nS, _ptr(ERI), _ptr(XpY),
                                            _ptr(rho)))
    return rho


def RGW_self_energy_diag(eta, nBas, nOrb, nC, nO, nV, nR, nS, e, Om, rho, ctx=None):
    """GW/RGW_self_energy_diag.f90.  Returns (EcGM, Sig, Z)."""
    c = _ctx(ctx)
    e, Om, rho = _f(e), _f(Om), _f(rho)
    Sig = np.empty(nBas)
    Z = np.empty(nBas)
    gm = C.c_double()
    c.check(lib().qk_RGW_self_energy_diag(c.handle, C.c_double(eta), nBas, nOrb, nC, nO, nV, nR,
                                          nS, _ptr(e), _ptr(Om), _ptr(rho), C.byref(gm),
                                          _ptr(Sig), _ptr(Z)))
    return gm.value, Sig, Z


def RGW_self_energy(eta, nBas, nOrb, nC, nO, nV, nR, nS, e, Om, rho, ctx=None, srg_flow=None):
    """GW/RGW_self_energy.f90 (or, with srg_flow, GW/RGW_SRG_self_energy.f90): the full
    unsymmetrised SigC(nOrb, nOrb).  Returns (EcGM, SigC, Z)."""
    c = _ctx(ctx)
    e, Om, rho = _f(e), _f(Om), _f(rho)
    Sig = np.empty((nOrb, nOrb), order="F")
    Z = np.empty(nOrb)
    gm = C.c_double()
    if srg_flow is None:
        fn, x = lib().qk_RGW_self_energy, eta
    else:
        fn, x = lib().qk_RGW_SRG_self_energy, srg_flow
    c.check(fn(c.handle, C.c_double(x), nBas, nOrb, nC, nO, nV, nR, nS, _ptr(e), _ptr(Om),
               _ptr(rho), C.byref(gm), _ptr(Sig), _ptr(Z)))
    return gm.value, Sig, Z


def Hartree_matrix_AO_basis(nBas, P, ERI, ctx=None):
    """AOtoMO/Hartree_matrix_AO_basis.f90.  Returns H(nBas, nBas)."""
    c = _ctx(ctx)
    P, ERI = _f(P), _f(ERI)
    H = np.empty((nBas, nBas), order="F")
    c.check(lib().qk_Hartree_matrix_AO_basis(c.handle, nBas, _ptr(P), _ptr(ERI), _ptr(H)))
    return H


def exchange_matrix_AO_basis(nBas, P, ERI, ctx=None):
    """AOtoMO/exchange_matrix_AO_basis.f90.  Returns K(nBas, nBas)."""
    c = _ctx(ctx)
    P, ERI = _f(P), _f(ERI)
    K = np.empty((nBas, nBas), order="F")
    c.check(lib().qk_exchange_matrix_AO_basis(c.handle, nBas, _ptr(P), _ptr(ERI), _ptr(K)))
    return K


def RGW_SRG_self_energy_diag(flow, nBas, nOrb, nC, nO, nV, nR, nS, e, Om, rho, ctx=None):
    """GW/RGW_SRG_self_energy_diag.f90.  Returns (EcGM, SigC, Z)."""
    c = _ctx(ctx)
    e, Om, rho = _f(e), _f(Om), _f(rho)
    Sig = np.empty(nOrb)
    Z = np.empty(nOrb)
    gm = C.c_double()
    c.check(lib().qk_RGW_SRG_self_energy_diag(c.handle, C.c_double(flow), nBas, nOrb, nC, nO, nV,
                                              nR, nS, _ptr(e), _ptr(Om), _ptr(rho), C.byref(gm),
                                              _ptr(Sig), _ptr(Z)))
    return gm.value, Sig, Z


def RGW_QP_graph(doSRG, eta, flow, nBas, nC, nO, nV, nR, nS, eHF, Om, rho, eGWlin, eOld, Z,
                 ctx=None):
    """GW/RGW_QP_graph.f90.  ``Z`` is the entry renormalisation factor (kept for orbitals whose
    Newton search fails).  Returns (eGW, Z)."""
    c = _ctx(ctx)
    eHF, Om, rho, eGWlin, eOld = _f(eHF), _f(Om), _f(rho), _f(eGWlin), _f(eOld)
    Zio = np.array(Z, dtype=np.float64, copy=True)
    eGW = np.empty(nBas)
    c.check(lib().qk_RGW_QP_graph(c.handle, int(bool(doSRG)), C.c_double(eta), C.c_double(flow),
                                  nBas, nC, nO, nV, nR, nS, _ptr(eHF), _ptr(Om), _ptr(rho),
                                  _ptr(eGWlin), _ptr(eOld), _ptr(eGW), _ptr(Zio)))
    return eGW, Zio


def AOtoMO_ERI_RHF(nBas, nOrb, c_mo, ERI_AO, ctx=None):
    """AOtoMO/AOtoMO_ERI_RHF.f90.  Returns ERI_MO (nOrb,)*4."""
    c = _ctx(ctx)
    cm, E = _f(c_mo), _f(ERI_AO)
    out = np.empty((nOrb,) * 4, order="F")
    c.check(lib().qk_AOtoMO_ERI_RHF(c.handle, nBas, nOrb, _ptr(cm), _ptr(E), _ptr(out)))
    return out


def DIIS_extrapolation(n_err, n_e, n_diis, error, e, error_in, e_inout, ctx=None):
    """utils/DIIS_extrapolation.f90.  ``error``/``e`` hold at least n_diis columns; they are
    updated in place (prepend).  Returns (rcond, e_out)."""
    c = _ctx(ctx)
    assert error.flags.f_contiguous and e.flags.f_contiguous
    err_in = _f(error_in)
    eio = np.array(e_inout, dtype=np.float64, copy=True)
    rc = C.c_double()
    c.check(lib().qk_DIIS_extrapolation(c.handle, C.byref(rc), n_err, n_e, n_diis, _ptr(error),
                                        _ptr(e), _ptr(err_in), _ptr(eio)))
    return rc.value, eio


# ------------------------------------------------------------------------------------------
# drivers
# ------------------------------------------------------------------------------------------
@dataclass
class GWOptions:
    """GW line of QuAcK's options file (QuAcK/read_options.f90:242-267)."""
    maxSCF: int = 64
    thresh: float = 1e-5
    max_diis: int = 1
    linearize: bool = False
    eta: float = 0.0
    TDA_W: bool = False
    reg: bool = False
    precision: int = QK_PREC_FP64
    qp_guess: int = 0  # 0 reference start, 1 learned guess, 2 HF start (comparison)

    def c(self):
        return qk_gw_params(self.eta, int(self.linearize), int(self.reg), int(self.TDA_W),
                            self.maxSCF, self.thresh, self.max_diis, self.precision,
                            int(self.qp_guess))


@dataclass
class BSEOptions:
    """BSE line of QuAcK's options (phBSE with TDA / singlet / triplet / exchange kernel)."""
    TDA_W: bool = False
    TDA: bool = False
    singlet: bool = True
    triplet: bool = True
    exchange_kernel: bool = False
    eta: float = 0.0

    def c(self):
        return qk_bse_params(int(self.TDA_W), int(self.TDA), int(self.singlet), int(self.triplet),
                             int(self.exchange_kernel), self.eta)


def RGW_phACFDT(opts: BSEOptions, doXBS, nBas, nOrb, nC, nO, nV, nR, nS, ERI, eW, eGW, ctx=None):
    """GW/RGW_phACFDT.f90: adiabatic-connection correlation energy of phBSE@GW.
    Returns [EcAC singlet, EcAC triplet]."""
    c = _ctx(ctx)
    ERI, eW, eGW = _f(ERI), _f(eW), _f(eGW)
    ec = (C.c_double * 2)()
    prm = opts.c()
    c.check(lib().qk_RGW_phACFDT(c.handle, C.byref(prm), int(bool(doXBS)), nBas, nOrb, nC, nO, nV,
                                 nR, nS, _ptr(ERI), _ptr(eW), _ptr(eGW), ec))
    return [ec[0], ec[1]]


def RGW_phBSE(opts: BSEOptions, nBas, nOrb, nC, nO, nV, nR, nS, ERI, eW, eGW, ctx=None):
    """GW/RGW_phBSE.f90 (static kernel).  Returns dict(EcBSE=[singlet, triplet], Om_singlet,
    Om_triplet) -- the excitation energies of the manifolds asked for (else None)."""
    c = _ctx(ctx)
    ERI, eW, eGW = _f(ERI), _f(eW), _f(eGW)
    ec = (C.c_double * 2)()
    oms = np.empty(nS) if opts.singlet else None
    omt = np.empty(nS) if opts.triplet else None
    prm = opts.c()
    c.check(lib().qk_RGW_phBSE(c.handle, C.byref(prm), nBas, nOrb, nC, nO, nV, nR, nS, _ptr(ERI),
                               _ptr(eW), _ptr(eGW), ec, _ptr(oms) if oms is not None else None,
                               _ptr(omt) if omt is not None else None))
    return dict(EcBSE=[ec[0], ec[1]], Om_singlet=oms, Om_triplet=omt)


def RGW_phBSE_dev(opts: BSEOptions, nOrb, nC, nO, nR, d_ERI, d_eW, d_eGW, d_OmS=None, d_OmT=None,
                  ctx=None):
    """Static phBSE@GW on device buffers (full ERI tensor).  Returns [EcBSE singlet, triplet]."""
    c = _ctx(ctx)
    ec = (C.c_double * 2)()
    prm = opts.c()
    c.check(lib().qk_RGW_phBSE_dev(c.handle, C.byref(prm), nOrb, nC, nO, nR, C.c_void_p(d_ERI),
                                   C.c_void_p(d_eW), C.c_void_p(d_eGW), ec,
                                   C.c_void_p(d_OmS or None), C.c_void_p(d_OmT or None)))
    return [ec[0], ec[1]]


def RG0W0(opts: GWOptions, nBas, nOrb, nC, nO, nV, nR, nS, ERI, eHF, ctx=None):
    """GW/RG0W0.f90 (dRPA singlet W).  Returns dict(eGW, SigC, Z, Om, EcRPA, EcGM)."""
    c = _ctx(ctx)
    ERI, eHF = _f(ERI), _f(eHF)
    eGW, SigC, Z, Om = np.empty(nOrb), np.empty(nOrb), np.empty(nOrb), np.empty(nS)
    Ec, gm = C.c_double(), C.c_double()
    prm = opts.c()
    c.check(lib().qk_RG0W0(c.handle, C.byref(prm), nBas, nOrb, nC, nO, nV, nR, nS, _ptr(eHF),
                           _ptr(ERI), _ptr(eGW), _ptr(SigC), _ptr(Z), _ptr(Om), C.byref(Ec),
                           C.byref(gm)))
    return dict(eGW=eGW, SigC=SigC, Z=Z, Om=Om, EcRPA=Ec.value, EcGM=gm.value)


def evRGW(opts: GWOptions, nBas, nOrb, nC, nO, nV, nR, nS, ERI, eHF, ctx=None, raise_on_fail=True):
    """GW/evRGW.f90.  Returns dict(eGW, SigC, Z, EcRPA, EcGM, nSCF, Conv, failed)."""
    c = _ctx(ctx)
    ERI, eHF = _f(ERI), _f(eHF)
    eGW, SigC, Z = np.empty(nOrb), np.empty(nOrb), np.empty(nOrb)
    Ec, gm, conv = C.c_double(), C.c_double(), C.c_double()
    nscf = C.c_int()
    prm = opts.c()
    rc = c.check(lib().qk_evRGW(c.handle, C.byref(prm), nBas, nOrb, nC, nO, nV, nR, nS, _ptr(eHF),
                                _ptr(ERI), _ptr(eGW), _ptr(SigC), _ptr(Z), C.byref(Ec),
                                C.byref(gm), C.byref(nscf), C.byref(conv)),
                 allow=() if raise_on_fail else (QK_ERR_NO_CONV,))
    return dict(eGW=eGW, SigC=SigC, Z=Z, EcRPA=Ec.value, EcGM=gm.value, nSCF=nscf.value,
                Conv=conv.value, failed=(rc == QK_ERR_NO_CONV))


def qsRGW(opts: GWOptions, nBas, nOrb, nC, nO, nV, nR, nS, eHF, cHF, PHF, S, T, V, Hc, X, ERI_AO,
          ctx=None, raise_on_fail=True):
    """GW/qsRGW.f90 (nBas >= nOrb; opts.reg selects the SRG self-energy).  ERI_AO[mu,nu,la,si] =
    <mu nu|la si>.  Returns dict(eGW, c, P, SigC (MO basis), Z, EqsGW (electronic), EcRPA, EcGM,
    nSCF, Conv, failed)."""
    c = _ctx(ctx)
    ins = [_f(a) for a in (eHF, cHF, PHF, S, T, V, Hc, X, ERI_AO)]
    eGW, Z = np.empty(nOrb), np.empty(nOrb)
    cq, P, SigC = (np.empty((nBas, nOrb), order="F"), np.empty((nBas, nBas), order="F"),
                   np.empty((nOrb, nOrb), order="F"))
    E, Ec, gm, conv = C.c_double(), C.c_double(), C.c_double(), C.c_double()
    nscf = C.c_int()
    prm = opts.c()
    rc = c.check(lib().qk_qsRGW(c.handle, C.byref(prm), nBas, nOrb, nC, nO, nV, nR, nS,
                                *[_ptr(a) for a in ins], _ptr(eGW), _ptr(cq), _ptr(P), _ptr(SigC),
                                _ptr(Z), C.byref(E), C.byref(Ec), C.byref(gm), C.byref(nscf),
                                C.byref(conv)),
                 allow=() if raise_on_fail else (QK_ERR_NO_CONV,))
    return dict(eGW=eGW, c=cq, P=P, SigC=SigC, Z=Z, EqsGW=E.value, EcRPA=Ec.value, EcGM=gm.value,
                nSCF=nscf.value, Conv=conv.value, failed=(rc == QK_ERR_NO_CONV))


def qsRGW_dev(opts: GWOptions, nOrb, nC, nO, nR, d_eHF, d_cHF, d_PHF, d_S, d_T, d_V, d_Hc, d_X,
              d_ERI_AO, d_eGW, d_c, d_P, d_Z, d_SigC=None, ctx=None, raise_on_fail=True,
              nBas=None):
    """Device-pointer qsGW (integer device addresses; nBas defaults to nOrb).  Returns
    dict(EqsGW, EcRPA, EcGM, nSCF, Conv, failed)."""
    nBas = nOrb if nBas is None else nBas
    c = _ctx(ctx)
    nS = (nO - nC) * (nOrb - nO - nR)
    E, Ec, gm, conv = C.c_double(), C.c_double(), C.c_double(), C.c_double()
    nscf = C.c_int()
    prm = opts.c()
    ptrs = [C.c_void_p(a) for a in (d_eHF, d_cHF, d_PHF, d_S, d_T, d_V, d_Hc, d_X, d_ERI_AO, d_eGW,
                                    d_c, d_P, d_SigC, d_Z)]
    rc = c.check(lib().qk_qsRGW_dev(c.handle, C.byref(prm), nBas, nOrb, nC, nO, nOrb - nO, nR, nS,
                                    *ptrs, C.byref(E), C.byref(Ec), C.byref(gm), C.byref(nscf),
                                    C.byref(conv)),
                 allow=() if raise_on_fail else (QK_ERR_NO_CONV,))
    return dict(EqsGW=E.value, EcRPA=Ec.value, EcGM=gm.value, nSCF=nscf.value, Conv=conv.value,
                failed=(rc == QK_ERR_NO_CONV))


def RG0W0_dev(opts: GWOptions, nOrb, nC, nO, nR, d_ERI, d_eHF, d_eGW, d_SigC, d_Z, d_Om,
              ctx=None):
    """Device-pointer driver: arguments are integer device addresses (e.g. tensor.data_ptr()).
    Returns (EcRPA, EcGM)."""
    c = _ctx(ctx)
    nS = (nO - nC) * (nOrb - nO - nR)
    Ec, gm = C.c_double(), C.c_double()
    prm = opts.c()
    c.check(lib().qk_RG0W0_dev(c.handle, C.byref(prm), nOrb, nOrb, nC, nO, nOrb - nO, nR, nS,
                               C.c_void_p(d_eHF), C.c_void_p(d_ERI), C.c_void_p(d_eGW),
                               C.c_void_p(d_SigC), C.c_void_p(d_Z), C.c_void_p(d_Om),
                               C.byref(Ec), C.byref(gm)))
    return Ec.value, gm.value


def evRGW_dev(opts: GWOptions, nOrb, nC, nO, nR, d_ERI, d_eHF, d_eGW, d_SigC, d_Z, ctx=None,
              raise_on_fail=True):
    """Device-pointer evGW driver (integer device addresses).  Returns dict(EcRPA, EcGM, nSCF,
    Conv, failed)."""
    c = _ctx(ctx)
    nS = (nO - nC) * (nOrb - nO - nR)
    Ec, gm, conv = C.c_double(), C.c_double(), C.c_double()
    nscf = C.c_int()
    prm = opts.c()
    rc = c.check(lib().qk_evRGW_dev(c.handle, C.byref(prm), nOrb, nOrb, nC, nO, nOrb - nO, nR, nS,
                                    C.c_void_p(d_eHF), C.c_void_p(d_ERI), C.c_void_p(d_eGW),
                                    C.c_void_p(d_SigC), C.c_void_p(d_Z), C.byref(Ec), C.byref(gm),
                                    C.byref(nscf), C.byref(conv)),
                 allow=() if raise_on_fail else (QK_ERR_NO_CONV,))
    return dict(EcRPA=Ec.value, EcGM=gm.value, nSCF=nscf.value, Conv=conv.value,
                failed=(rc == QK_ERR_NO_CONV))


def dsyev_dev(n, d_A, lda, d_w, d_Zt, want_vectors=True, ctx=None):
    """GPU dsyev on device buffers (A destroyed; Zt rows are eigenvectors)."""
    c = _ctx(ctx)
    c.check(lib().qk_dsyev_dev(c.handle, n, C.c_void_p(d_A), lda, C.c_void_p(d_w),
                               C.c_void_p(d_Zt), int(bool(want_vectors))))


def dgemm_dev(transa, transb, m, n, k, alpha, d_A, lda, d_B, ldb, beta, d_C, ldc, ctx=None):
    """FP64 GEMM on device buffers, column-major."""
    c = _ctx(ctx)
    c.check(lib().qk_dgemm_dev(c.handle, C.c_char(transa.encode()), C.c_char(transb.encode()), m,
                               n, k, C.c_double(alpha), C.c_void_p(d_A), lda, C.c_void_p(d_B), ldb,
                               C.c_double(beta), C.c_void_p(d_C), ldc))


def rpa_ecorr_quad_dev(nOrb, nC, nO, nR, d_e, d_ERI=None, d_L=None, naux=0, ctx=None):
    """dRPA correlation energy at orbital energies d_e by imaginary-frequency quadrature, from
    the device ERI tensor or the device factor L (one of the two).  Returns EcRPA, or None when
    the quadrature does not apply (the caller then uses the Casida eigenvalues)."""
    c = _ctx(ctx)
    ec = C.c_double(0.0)
    applied = C.c_int(0)
    c.check(lib().qk_RPA_ecorr_quad_dev(c.handle, nOrb, nC, nO, nR, naux, C.c_void_p(d_e),
                                        C.c_void_p(d_ERI or None), C.c_void_p(d_L or None),
                                        C.byref(ec), C.byref(applied)))
    return ec.value if applied.value else None


def gauss_legendre(n):
    """Nodes (ascending) and weights of the n-point Gauss-Legendre rule on [-1, 1] (host code
    of the library; no GPU needed)."""
    x = np.zeros(n)
    w = np.zeros(n)
    rc = lib().qk_gauss_legendre(n, _ptr(x), _ptr(w))
    if rc != 0:
        raise QkError(rc, "qk_gauss_legendre")
    return x, w


def read_eri_bin(path, nBas, d_ERI, ctx=None):
    """int/ERI.bin (nBas^4 doubles, <pq|rs> column-major) streamed into the device buffer."""
    c = _ctx(ctx)
    c.check(lib().qk_read_eri_bin(c.handle, str(path).encode(), nBas, C.c_void_p(d_ERI)))


def read_eri_chem_bin(path, nBas, d_ERI, ctx=None):
    """int/ERI_chem.bin (8-fold packed chemist integrals) streamed to the device and expanded
    into the full <pq|rs> tensor."""
    c = _ctx(ctx)
    c.check(lib().qk_read_eri_chem_bin(c.handle, str(path).encode(), nBas, C.c_void_p(d_ERI)))


def unpack_eri_s8_dev(nBas, d_packed, d_ERI, ctx=None):
    c = _ctx(ctx)
    c.check(lib().qk_unpack_eri_s8_dev(c.handle, nBas, C.c_void_p(d_packed), C.c_void_p(d_ERI)))


def AOtoMO_ERI_RHF_dev(nBas, nOrb, d_c, d_ERI_AO, d_ERI_MO, ctx=None):
    c = _ctx(ctx)
    c.check(lib().qk_AOtoMO_ERI_RHF_dev(c.handle, nBas, nOrb, C.c_void_p(d_c), C.c_void_p(d_ERI_AO),
                                        C.c_void_p(d_ERI_MO)))


def dgemm_f32p_dev(transa, transb, m, n, k, alpha, d_A, lda, d_B, ldb, beta, d_C, ldc, ctx=None):
    """The dgemm_dev contract with FP32 products (compensated FP32 sums, FP64 in/out)."""
    c = _ctx(ctx)
    c.check(lib().qk_dgemm_f32p_dev(c.handle, C.c_char(transa.encode()), C.c_char(transb.encode()),
                                    m, n, k, C.c_double(alpha), C.c_void_p(d_A), lda,
                                    C.c_void_p(d_B), ldb, C.c_double(beta), C.c_void_p(d_C), ldc))


def dgemm_df_dev(transa, transb, m, n, k, alpha, d_A, lda, d_B, ldb, beta, d_C, ldc, ctx=None):
    """The dgemm_dev contract in double-float (FP32 pairs, exact products, compensated sums)."""
    c = _ctx(ctx)
    c.check(lib().qk_dgemm_df_dev(c.handle, C.c_char(transa.encode()), C.c_char(transb.encode()),
                                  m, n, k, C.c_double(alpha), C.c_void_p(d_A), lda,
                                  C.c_void_p(d_B), ldb, C.c_double(beta), C.c_void_p(d_C), ldc))


def gemm_bf16x3_ex_dev(transa, transb, m, n, k, alpha, d_A, lda, d_B, ldb, beta, d_C, ldc,
                       ctx=None):
    """C = alpha op(A) op(B) + beta C with the BF16x3 split on the tensor cores (FP64 in/out)."""
    c = _ctx(ctx)
    c.check(lib().qk_gemm_bf16x3_ex_dev(c.handle, C.c_char(transa.encode()),
                                        C.c_char(transb.encode()), m, n, k, C.c_double(alpha),
                                        C.c_void_p(d_A), lda, C.c_void_p(d_B), ldb,
                                        C.c_double(beta), C.c_void_p(d_C), ldc))


def gemm_bf16x3_dev(m, n, k, d_A, lda, d_B, ldb, d_C, ldc, ctx=None):
    """C = A B^T with the BF16x3 split on the tensor cores (FP64 in/out, FP32 accumulate)."""
    c = _ctx(ctx)
    c.check(lib().qk_gemm_bf16x3_dev(c.handle, m, n, k, C.c_void_p(d_A), lda, C.c_void_p(d_B), ldb,
                                     C.c_void_p(d_C), ldc))


def stream_handle(ctx=None) -> int:
    """cudaStream_t of the context (for events on the stream the kernels run on)."""
    c = _ctx(ctx)
    lib().qk_stream.restype = C.c_void_p
    return int(lib().qk_stream(c.handle) or 0)


def probe_fp64_peak(ctx=None):
    """(DMMA TFLOP/s, DFMA TFLOP/s) measured on this GPU."""
    c = _ctx(ctx)
    a, b = C.c_double(), C.c_double()
    c.check(lib().qk_probe_fp64_peak(c.handle, C.byref(a), C.byref(b)))
    return a.value, b.value


def probe_fp32_peak(ctx=None):
    """FFMA TFLOP/s measured on this GPU."""
    c = _ctx(ctx)
    a = C.c_double()
    c.check(lib().qk_probe_fp32_peak(c.handle, C.byref(a)))
    return a.value


def RGW_self_energy_diag_noalloc_dev(eta, nBas, nOrb, nC, nO, nV, nR, nS, d_e, d_Om, d_rho,
                                     d_EcGM, d_Sig, d_Z, stream=0):
    """Allocation-free self-energy on caller-owned device buffers (integer device addresses).
    Returns the status code (QK_OK = 0); needs no Context."""
    L = lib()
    f = L.qk_RGW_self_energy_diag_noalloc_dev
    f.restype = C.c_int
    return f(C.c_double(eta), nBas, nOrb, nC, nO, nV, nR, nS, C.c_void_p(d_e), C.c_void_p(d_Om),
             C.c_void_p(d_rho), C.c_void_p(d_EcGM), C.c_void_p(d_Sig), C.c_void_p(d_Z),
             C.c_void_p(stream))


def RG0W0_L_dev(opts: GWOptions, nOrb, nC, nO, nR, naux, d_L, d_eHF, d_eGW, d_SigC, d_Z, d_Om,
                ctx=None):
    """Factorised-integral G0W0 on device buffers.  Returns (EcRPA, EcGM)."""
    c = _ctx(ctx)
    Ec, gm = C.c_double(), C.c_double()
    prm = opts.c()
    c.check(lib().qk_RG0W0_L_dev(c.handle, C.byref(prm), nOrb, nC, nO, nR, naux, C.c_void_p(d_L),
                                 C.c_void_p(d_eHF), C.c_void_p(d_eGW), C.c_void_p(d_SigC),
                                 C.c_void_p(d_Z), C.c_void_p(d_Om), C.byref(Ec), C.byref(gm)))
    return Ec.value, gm.value


def evRGW_L_dev(opts: GWOptions, nOrb, nC, nO, nR, naux, d_L, d_eHF, d_eGW, d_SigC, d_Z,
                ctx=None, raise_on_fail=True):
    """Factorised-integral evGW on device buffers.  Returns dict(EcRPA, EcGM, nSCF, Conv, failed)."""
    c = _ctx(ctx)
    Ec, gm, conv = C.c_double(), C.c_double(), C.c_double()
    nscf = C.c_int()
    prm = opts.c()
    rc = c.check(lib().qk_evRGW_L_dev(c.handle, C.byref(prm), nOrb, nC, nO, nR, naux,
                                      C.c_void_p(d_L), C.c_void_p(d_eHF), C.c_void_p(d_eGW),
                                      C.c_void_p(d_SigC), C.c_void_p(d_Z), C.byref(Ec),
                                      C.byref(gm), C.byref(nscf), C.byref(conv)),
                 allow=() if raise_on_fail else (QK_ERR_NO_CONV,))
    return dict(EcRPA=Ec.value, EcGM=gm.value, nSCF=nscf.value, Conv=conv.value,
                failed=(rc == QK_ERR_NO_CONV))


def L_fortran_flat(L):
    """Factor L[P,p,q] (numpy) as the flat Fortran-order L(p,q,P) the *_L entry points take."""
    L = np.asarray(L, dtype=np.float64)
    return np.ascontiguousarray(L.reshape(L.shape[0], -1)).ravel()


def pack_systems(systems):
    """Pack synthetic systems (dicts with L[P,p,q], eHF, nO) for the batched driver.
    Returns (desc array, flat L, flat eHF)."""
    nsys = len(systems)
    desc = (qk_sys_desc * nsys)()
    offL = offE = 0
    Ls, Es = [], []
    for i, s in enumerate(systems):
        naux, N, _ = s["L"].shape
        desc[i] = qk_sys_desc(N, 0, int(s["nO"]), 0, naux, offL, offE)
        Ls.append(L_fortran_flat(s["L"]))
        Es.append(np.asarray(s["eHF"], dtype=np.float64))
        offL += naux * N * N
        offE += N
    return desc, np.concatenate(Ls), np.concatenate(Es)


def gw_batch_L_dev(opts: GWOptions, method, desc, d_L, d_eHF, d_eGW, n_workers=8, ctx=None):
    """Batched G0W0 (method 0) / evGW (method 1) over packed device arrays.
    Returns dict(status, EcRPA, nSCF, rc) with per-system host arrays."""
    c = _ctx(ctx)
    n = len(desc)
    st = (C.c_int * n)()
    ns = (C.c_int * n)()
    ec = (C.c_double * n)()
    prm = opts.c()
    rc = lib().qk_gw_batch_L_dev(c.handle, C.byref(prm), int(method), n, desc, C.c_void_p(d_L),
                                 C.c_void_p(d_eHF), C.c_void_p(d_eGW), ec, st, ns, int(n_workers))
    err = lib().qk_last_error_string(c.handle).decode() if rc != QK_OK else ""
    return dict(status=np.array(st[:]), EcRPA=np.array(ec[:]), nSCF=np.array(ns[:]), rc=rc,
                error=err)
