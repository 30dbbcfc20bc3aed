"""CPU oracle for the restricted G0W0 / evGW call chain of QuAcK.

TEST INFRASTRUCTURE ONLY.  This module is the checker that the CUDA library
is compared against; it is imported only by ``tests/``, by
``__graft_entry__.smoke()`` and by the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py``.  Nothing in ``quack_gb300`` imports it and no product
path routes through it.

It restates QuAcK's Fortran (pfloos/QuAcK, ``src/``) in NumPy/SciPy, one
function per reference routine, with the same loop bounds, index maps and
product order (LAPACK ``dsyev('V','U')`` and ``dsysvx('N','U')`` through
``scipy.linalg.lapack``).  Arrays follow the Fortran meaning of the reference
arguments with 0-based indices: ``ERI[p,q,r,s]`` is ``ERI(p+1,q+1,r+1,s+1)``
= <pq|rs> = (pr|qs) (physicist layout, PyDuck.py:342 + read_2e_integrals.f90:61),
``rho[p,q,m]`` is ``rho(p+1,q+1,m+1)``, ``XpY[m,ia]`` is ``XpY(m+1,ia+1)``.

Parity status: pinned end to end by the He/6-31G FeatherBench goldens
(tests/feather_bench.py:86-91 of the reference) through ``oracle/he631g.py``.
Eigenvectors are compared only up to sign / degenerate rotation.
"""
from __future__ import annotations

import numpy as np
from scipy.linalg import lapack

HaToeV = 27.211386245988          # include/parameters.h:16


# ---------------------------------------------------------------------------
# LAPACK wrappers (src/utils/wrap_lapack.f90)
# ---------------------------------------------------------------------------
def diagonalize_matrix(A):
    """dsyev('V','U') -- wrap_lapack.f90:99-136.  Returns (eigvecs, eigvals)."""
    w, v, info = lapack.dsyev(np.asfortranarray(A), compute_v=1, lower=0)
    if info != 0:
        # the reference prints and carries on (wrap_lapack.f90:131-133)
        import warnings
        warnings.warn("Problem in diagonalize_matrix (dsyev)!! info=%d" % info)
    return v, w


def linear_solve(A, b):
    """dsysvx('N','U') -- wrap_lapack.f90:560-598.  Returns (x, rcond)."""
    out = lapack.dsysvx(np.asfortranarray(A), np.asfortranarray(b.reshape(-1, 1)), lower=0)
    # scipy returns (a_s, udut, ipiv, b_s, x, rcond, ferr, berr, info)
    x, rcond = out[4], out[5]
    return np.asarray(x).reshape(-1), float(rcond)


# ---------------------------------------------------------------------------
# small matrix helpers (src/utils/utils.f90)
# ---------------------------------------------------------------------------
def ADAt(A, D):
    """B = A.diag(D).A^T -- utils.f90:634-678 (tmp(i,j)=D(i)*A(j,i); dgemm(A,tmp))."""
    tmp = D[:, None] * A.T
    return A @ tmp


def DA(D, A):
    """A <- diag(D).A (row scaling) -- utils.f90:680-699."""
    return D[:, None] * A


def trace_matrix(A):
    """utils.f90:328-352."""
    return float(np.sum(np.diag(A)))


def prepend(A, b):
    """Shift columns right by one and put b in column 1 -- utils.f90:506-536."""
    out = np.empty_like(A)
    out[:, 1:] = A[:, :-1]
    out[:, 0] = b
    return out


# ---------------------------------------------------------------------------
# index helpers
# ---------------------------------------------------------------------------
def _ov(nBas, nC, nO, nR):
    occ = np.arange(nC, nO)
    vir = np.arange(nO, nBas - nR)
    return occ, vir


# ---------------------------------------------------------------------------
# Linear response (src/LR)
# ---------------------------------------------------------------------------
def phRLR_A(ispin, dRPA, nBas, nC, nO, nV, nR, nS, lam, e, ERI):
    """Resonant ph block -- LR/phRLR_A.f90:43-72 (singlet), :92-118 (triplet).

    A(ia,jb) = ct1*ERI(b,i,j,a) + ct2*ERI(b,j,a,i) + delta_ij delta_ab (e_a - e_i),
    ia = a - nO + (i-nC-1)*nn  (0-based: ia = (i-nC)*nn + (a-nO)).
    """
    occ, vir = _ov(nBas, nC, nO, nR)
    no, nv = len(occ), len(vir)
    assert no * nv == nS
    delta = 1.0 if dRPA else 0.0
    ct2 = -(1.0 - delta) * lam
    if ispin == 1:
        ct1 = 2.0 * lam
        T1 = ERI[np.ix_(vir, occ, occ, vir)]          # [b,i,j,a]
        A4 = ct1 * T1.transpose(1, 3, 2, 0)           # [i,a,j,b]
    elif ispin == 2:
        A4 = np.zeros((no, nv, no, nv))
    else:
        raise ValueError("ispin must be 1 or 2")
    if ct2 != 0.0:
        T2 = ERI[np.ix_(vir, occ, vir, occ)]          # [b,j,a,i]
        A4 = A4 + ct2 * T2.transpose(3, 2, 1, 0)      # [i,a,j,b]
    A = A4.reshape(nS, nS).copy()
    ea = np.broadcast_to(e[vir][None, :], (no, nv)).reshape(nS)
    ei = np.broadcast_to(e[occ][:, None], (no, nv)).reshape(nS)
    di = np.diag_indices(nS)
    A[di] = (A[di] + ea) - ei           # Aph(ia,jb) + e(a) - e(i), evaluated left to right
    return A


def phRLR_B(ispin, dRPA, nBas, nC, nO, nV, nR, nS, lam, ERI):
    """Coupling ph block -- LR/phRLR_B.f90:34-59 (singlet), :78-98 (triplet).

    B(ia,jb) = ct1*ERI(b,i,j,a) + ct2*ERI(b,j,i,a).
    """
    occ, vir = _ov(nBas, nC, nO, nR)
    no, nv = len(occ), len(vir)
    assert no * nv == nS
    delta = 1.0 if dRPA else 0.0
    ct2 = -(1.0 - delta) * lam
    if ispin == 1:
        T1 = ERI[np.ix_(vir, occ, occ, vir)]          # [b,i,j,a]
        B4 = 2.0 * lam * T1.transpose(1, 3, 2, 0)
    elif ispin == 2:
        B4 = np.zeros((no, nv, no, nv))
    else:
        raise ValueError("ispin must be 1 or 2")
    if ct2 != 0.0:
        T2 = ERI[np.ix_(vir, occ, occ, vir)]          # [b,j,i,a]
        B4 = B4 + ct2 * T2.transpose(2, 3, 1, 0)      # [i,a,j,b]
    return B4.reshape(nS, nS).copy()


def phRLR(TDA, nS, Aph, Bph):
    """Casida solve -- LR/phRLR.f90:45-95.

    Returns (EcRPA, Om, XpY, XmY) with XpY[m, ia] (row m = excitation).
    """
    if TDA:
        Zv, Om = diagonalize_matrix(Aph)
        XpY = Zv.T.copy()
        XmY = XpY.copy()
    else:
        ApB = Aph + Bph
        AmB = Aph - Bph
        U, lam = diagonalize_matrix(AmB)                      # phRLR.f90:54
        AmBSq = ADAt(U, 1.0 * np.sqrt(lam))                   # :59
        AmBIv = ADAt(U, 1.0 / np.sqrt(lam))                   # :60
        tmp = ApB @ AmBSq                                     # :62
        Zm = AmBSq @ tmp                                      # :63
        Zv, Om = diagonalize_matrix(Zm)                       # :67
        Om = np.sqrt(np.abs(Om))                              # :76
        XpY = DA(1.0 / np.sqrt(Om), Zv.T @ AmBSq)             # :77-78
        XmY = DA(1.0 * np.sqrt(Om), Zv.T @ AmBIv)             # :80-81
    EcRPA = 0.5 * (float(np.sum(Om)) - trace_matrix(Aph))     # :95
    return EcRPA, Om, XpY, XmY


# ---------------------------------------------------------------------------
# GW kernels (src/GW)
# ---------------------------------------------------------------------------
def RGW_excitation_density(nOrb, nC, nO, nR, nS, ERI, XpY):
    """rho(p,q,m) = sum_jb ERI(p,j,q,b) XpY(m,jb) -- GW/RGW_excitation_density.f90:30-50.

    jb runs j = nC+1..nO (outer), b = nO+1..nOrb-nR (inner).  The reference
    gathers tmp(p,q,jb) over all p,q and multiplies by XpY^T (dgemm 'N','T').
    """
    occ, vir = _ov(nOrb, nC, nO, nR)
    tmp = ERI[:, occ][:, :, :, vir]                          # [p,j,q,b]
    tmp = tmp.transpose(0, 2, 1, 3).reshape(nOrb, nOrb, nS)  # [p,q,jb]
    rho = (tmp.reshape(nOrb * nOrb, nS) @ XpY.T).reshape(nOrb, nOrb, nS)
    return rho


def RGW_self_energy_diag(eta, nBas, nOrb, nC, nO, nV, nR, nS, e, Om, rho):
    """Diagonal Sigma_c, Z and EcGM -- GW/RGW_self_energy_diag.f90:35-111.

    Returns (EcGM, Sig, Z).
    """
    occ, vir = _ov(nBas, nC, nO, nR)
    act = np.arange(nC, nBas - nR)
    Sig = np.zeros(nBas)
    dZ = np.zeros(nBas)
    eta2 = eta * eta
    for p in act:
        # occupied part (:44-62): eps = e(p) - e(i) + Om(m)
        eps = e[p] - e[occ][:, None] + Om[None, :]           # [i,m]
        num = 2.0 * rho[p, occ, :] ** 2
        Sig[p] += np.sum(num * eps / (eps ** 2 + eta2))
        dZ[p] -= np.sum(num * (eps ** 2 - eta2) / (eps ** 2 + eta2) ** 2)
        # virtual part (:66-84): eps = e(p) - e(a) - Om(m)
        eps = e[p] - e[vir][:, None] - Om[None, :]
        num = 2.0 * rho[p, vir, :] ** 2
        Sig[p] += np.sum(num * eps / (eps ** 2 + eta2))
        dZ[p] -= np.sum(num * (eps ** 2 - eta2) / (eps ** 2 + eta2) ** 2)
    # Galitskii-Migdal (:88-107): eps = e(a) - e(i) + Om(m)
    eps = e[vir][:, None, None] - e[occ][None, :, None] + Om[None, None, :]
    num = 4.0 * rho[np.ix_(vir, occ, np.arange(nS))] ** 2
    EcGM = -float(np.sum(num * eps / (eps ** 2 + eta2)))
    Z = 1.0 / (1.0 - dZ)                                      # :111
    return EcGM, Sig, Z


def RGW_SRG_self_energy_diag(flow, nBas, nOrb, nC, nO, nV, nR, nS, e, Om, rho):
    """SRG-regularised diagonal Sigma_c, Z, EcGM -- GW/RGW_SRG_self_energy_diag.f90:55-158."""
    occ, vir = _ov(nOrb, nC, nO, nR)
    act = np.arange(nC, nOrb - nR)
    s = flow
    SigC = np.zeros(nOrb)
    dZ = np.zeros(nOrb)
    for p in act:
        D = e[p] - e[occ][:, None] + Om[None, :]
        r2 = 2.0 * rho[p, occ, :] ** 2
        reg = 1.0 - np.exp(-2.0 * s * D * D)
        SigC[p] += np.sum(r2 * reg / D)
        dZ[p] -= np.sum(r2 * reg / D ** 2)
        D = e[p] - e[vir][:, None] - Om[None, :]
        r2 = 2.0 * rho[p, vir, :] ** 2
        reg = 1.0 - np.exp(-2.0 * s * D * D)
        SigC[p] += np.sum(r2 * reg / D)
        dZ[p] -= np.sum(r2 * reg / D ** 2)
    Z = 1.0 / (1.0 - dZ)
    D = e[vir][:, None, None] - e[occ][None, :, None] + Om[None, None, :]
    r = rho[np.ix_(vir, occ, np.arange(nS))]
    EcGM = -float(np.sum(4.0 * r * r * (1.0 - np.exp(-2.0 * s * D * D)) / D))
    return EcGM, SigC, Z


def RGW_Re_SigC(p, w, eta, nBas, nC, nO, nV, nR, nS, e, Om, rho):
    """GW/RGW_Re_SigC.f90:30-50."""
    occ, vir = _ov(nBas, nC, nO, nR)
    eta2 = eta * eta
    eps = w - e[occ][:, None] + Om[None, :]
    num = 2.0 * rho[p, occ, :] ** 2
    s = np.sum(num * eps / (eps ** 2 + eta2))
    eps = w - e[vir][:, None] - Om[None, :]
    num = 2.0 * rho[p, vir, :] ** 2
    return float(s + np.sum(num * eps / (eps ** 2 + eta2)))


def RGW_Re_dSigC(p, w, eta, nBas, nC, nO, nV, nR, nS, e, Om, rho):
    """GW/RGW_Re_dSigC.f90:30-50."""
    occ, vir = _ov(nBas, nC, nO, nR)
    eta2 = eta * eta
    eps = w - e[occ][:, None] + Om[None, :]
    num = 2.0 * rho[p, occ, :] ** 2
    s = -np.sum(num * (eps ** 2 - eta2) / (eps ** 2 + eta2) ** 2)
    eps = w - e[vir][:, None] - Om[None, :]
    num = 2.0 * rho[p, vir, :] ** 2
    return float(s - np.sum(num * (eps ** 2 - eta2) / (eps ** 2 + eta2) ** 2))


def RGW_SRG_Re_SigC(p, w, flow, nBas, nC, nO, nV, nR, nS, e, Om, rho):
    """GW/RGW_SRG_Re_SigC.f90."""
    occ, vir = _ov(nBas, nC, nO, nR)
    s = flow
    D = w - e[occ][:, None] + Om[None, :]
    v = np.sum(2.0 * rho[p, occ, :] ** 2 * (1.0 - np.exp(-2.0 * s * D * D)) / D)
    D = w - e[vir][:, None] - Om[None, :]
    return float(v + np.sum(2.0 * rho[p, vir, :] ** 2 * (1.0 - np.exp(-2.0 * s * D * D)) / D))


def RGW_SRG_Re_dSigC(p, w, flow, nBas, nC, nO, nV, nR, nS, e, Om, rho):
    """GW/RGW_SRG_Re_dSigC.f90."""
    occ, vir = _ov(nBas, nC, nO, nR)
    s = flow
    D = w - e[occ][:, None] + Om[None, :]
    v = -np.sum(2.0 * rho[p, occ, :] ** 2 * (1.0 - np.exp(-2.0 * s * D * D)) / D ** 2)
    D = w - e[vir][:, None] - Om[None, :]
    return float(v - np.sum(2.0 * rho[p, vir, :] ** 2 * (1.0 - np.exp(-2.0 * s * D * D)) / D ** 2))


QP_MAXIT = 64        # RGW_QP_graph.f90:38
QP_THRESH = 1e-6     # RGW_QP_graph.f90:39


def RGW_QP_graph(doSRG, eta, flow, nBas, nC, nO, nV, nR, nS, eHF, Om, rho, eGWlin, eOld, Z_in,
                 return_iters=False, maxit=QP_MAXIT):
    """Newton root search of w - eHF(p) - SigC(w) = 0 -- GW/RGW_QP_graph.f90:50-92.

    ``Z_in`` is the renormalisation factor on entry: the reference leaves Z(p)
    untouched for orbitals whose Newton search fails (:78-81).  Returns
    (eGW, Z) and, if asked, the per-orbital iteration counts.  ``maxit`` is the reference's
    maxIt parameter (:38), exposed for the failure-path tests.
    """
    eGW = np.array(eGWlin, dtype=np.float64, copy=True)
    Z = np.array(Z_in, dtype=np.float64, copy=True)
    iters = np.zeros(nBas, dtype=np.int64)
    for p in range(nC, nBas - nR):
        w = eGWlin[p]
        nIt = 0
        f = 1.0
        df = 1.0
        while abs(f) > QP_THRESH and nIt < maxit:
            nIt += 1
            if doSRG:
                SigC = RGW_SRG_Re_SigC(p, w, flow, nBas, nC, nO, nV, nR, nS, eOld, Om, rho)
                dSigC = RGW_SRG_Re_dSigC(p, w, flow, nBas, nC, nO, nV, nR, nS, eOld, Om, rho)
            else:
                SigC = RGW_Re_SigC(p, w, eta, nBas, nC, nO, nV, nR, nS, eOld, Om, rho)
                dSigC = RGW_Re_dSigC(p, w, eta, nBas, nC, nO, nV, nR, nS, eOld, Om, rho)
            f = w - eHF[p] - SigC
            df = 1.0 / (1.0 - dSigC)
            w = w - df * f
        iters[p] = nIt
        if nIt == maxit:
            eGW[p] = eGWlin[p]
        else:
            eGW[p] = w
            Z[p] = df
    if return_iters:
        return eGW, Z, iters
    return eGW, Z


# ---------------------------------------------------------------------------
# DIIS (src/utils/DIIS_extrapolation.f90:1-61)
# ---------------------------------------------------------------------------
def DIIS_extrapolation(n_diis, error, e, error_in, e_inout):
    """Returns (rcond, error, e, e_out).  ``error``/``e`` hold the history in
    columns 0..n_diis-1 (column 0 = newest after prepend)."""
    error = error.copy()
    e = e.copy()
    error[:, :n_diis] = prepend(error[:, :n_diis], error_in)        # :30
    e[:, :n_diis] = prepend(e[:, :n_diis], e_inout)                 # :31
    A = np.zeros((n_diis + 1, n_diis + 1))
    A[:n_diis, :n_diis] = error[:, :n_diis].T @ error[:, :n_diis]   # :36
    A[:n_diis, n_diis] = -1.0
    A[n_diis, :n_diis] = -1.0
    A[n_diis, n_diis] = 0.0
    b = np.zeros(n_diis + 1)
    b[n_diis] = -1.0
    w, rcond = linear_solve(A, b)                                   # :50
    e_out = np.array(e_inout, copy=True)
    if rcond > 10e-14:                                              # :54
        e_out = e[:, :n_diis] @ w[:n_diis]
    return rcond, error, e, e_out


# ---------------------------------------------------------------------------
# AO -> MO (src/AOtoMO/AOtoMO_ERI_RHF.f90:26-53)
# ---------------------------------------------------------------------------
def AOtoMO_ERI_RHF(nBas, nOrb, c, ERI_AO):
    """Four successive dgemm('T','N') quarter transforms.

    In Fortran order each step contracts the first index and appends the new
    MO index last; after four steps ERI_MO(p,q,r,s) = sum c(mu,p)...ERI_AO.
    """
    X = np.asfortranarray(ERI_AO)
    for _ in range(4):
        n0 = X.shape[0]
        rest = X.shape[1:]
        M = X.reshape(n0, -1, order="F")           # (nBas, prod(rest))
        Y = M.T @ c                                # (prod(rest), nOrb)
        X = Y.reshape(rest + (c.shape[1],), order="F")
    return np.ascontiguousarray(X)


# ---------------------------------------------------------------------------
# Bethe-Salpeter equation on top of GW (src/GW/RGW_phBSE*.f90)
# ---------------------------------------------------------------------------
def RGW_phBSE_static_kernel_A(eta, nBas, nC, nO, nV, nR, nS, lam, Om, rho):
    """Static BSE kernel, resonant block -- GW/RGW_phBSE_static_kernel_A.f90:32-52.

    KA(ia,jb) = 4 lam^2 sum_kc rho(i,j,kc) rho(a,b,kc) Om(kc) / (Om(kc)^2 + eta^2).
    """
    occ, vir = _ov(nBas, nC, nO, nR)
    f = Om / (Om ** 2 + eta ** 2)
    roo = rho[np.ix_(occ, occ)]                       # [i,j,kc]
    rvv = rho[np.ix_(vir, vir)]                       # [a,b,kc]
    K = np.einsum("ijk,abk,k->iajb", roo, rvv, f, optimize=True)
    return 4.0 * lam ** 2 * K.reshape(nS, nS)


def RGW_phBSE_static_kernel_B(eta, nBas, nC, nO, nV, nR, nS, lam, Om, rho):
    """Static BSE kernel, coupling block -- GW/RGW_phBSE_static_kernel_B.f90:32-52.

    KB(ia,jb) = 4 lam^2 sum_kc rho(i,b,kc) rho(a,j,kc) Om(kc) / (Om(kc)^2 + eta^2).
    """
    occ, vir = _ov(nBas, nC, nO, nR)
    f = Om / (Om ** 2 + eta ** 2)
    rov = rho[np.ix_(occ, vir)]                       # [i,b,kc]
    rvo = rho[np.ix_(vir, occ)]                       # [a,j,kc]
    K = np.einsum("ibk,ajk,k->iajb", rov, rvo, f, optimize=True)
    return 4.0 * lam ** 2 * K.reshape(nS, nS)


def RGW_phBSE(TDA_W, TDA, singlet, triplet, exchange_kernel, eta, nOrb, nC, nO, nV, nR, nS, ERI,
              eW, eGW):
    """Static phBSE@GW excitation energies -- GW/RGW_phBSE.f90:83-190 (no second-order kernel,
    no dynamical correction).  Screening: dRPA singlet at eW (:89-95); kernels from its Om, rho
    (:97-98); per spin A = phRLR_A(ispin, dRPA=False, eGW) + KA, B = phRLR_B + KB (:110-133,
    :146-154).  Returns dict(EcBSE=[singlet, triplet], Om_singlet, Om_triplet, Om_RPA)."""
    Aw = phRLR_A(1, True, nOrb, nC, nO, nV, nR, nS, 1.0, eW, ERI)
    Bw = np.zeros((nS, nS)) if TDA_W else phRLR_B(1, True, nOrb, nC, nO, nV, nR, nS, 1.0, ERI)
    _, OmRPA, XpY, _ = phRLR(TDA_W, nS, Aw, Bw)
    rho = RGW_excitation_density(nOrb, nC, nO, nR, nS, ERI, XpY)
    KA = RGW_phBSE_static_kernel_A(eta, nOrb, nC, nO, nV, nR, nS, 1.0, OmRPA, rho)
    KB = np.zeros((nS, nS)) if TDA else RGW_phBSE_static_kernel_B(eta, nOrb, nC, nO, nV, nR, nS,
                                                                    1.0, OmRPA, rho)
    EcBSE = [0.0, 0.0]
    out = dict(Om_RPA=OmRPA, Om_singlet=None, Om_triplet=None)
    for ispin, on, key in ((1, singlet, "Om_singlet"), (2, triplet, "Om_triplet")):
        if not on:
            continue
        A = phRLR_A(ispin, False, nOrb, nC, nO, nV, nR, nS, 1.0, eGW, ERI) + KA
        B = np.zeros((nS, nS)) if TDA else phRLR_B(ispin, False, nOrb, nC, nO, nV, nR, nS, 1.0,
                                                   ERI) + KB
        EcBSE[ispin - 1], Om, _, _ = phRLR(TDA, nS, A, B)
        out[key] = Om
    EcBSE[1] = 3.0 * EcBSE[1]                                          # :184
    if exchange_kernel:
        EcBSE = [0.5 * x for x in EcBSE]                               # :186-187
    out["EcBSE"] = EcBSE
    return out


def phACFDT_correlation_energy(ispin, exchange_kernel, nBas, nC, nO, nV, nR, nS, ERI, XpY, XmY):
    """RPA/phACFDT_correlation_energy.f90:56-80: Ec = tr(X Bp Y^T + Y Bp X^T)
    + tr(X Ap X^T + Y Ap Y^T) - tr(Ap), Ap(ia,jb) = (1+ds) ERI(i,b,a,j) - dK ERI(i,b,j,a),
    Bp(ia,jb) = (1+ds) ERI(i,j,a,b) - dK ERI(i,j,b,a), X = (XpY+XmY)/2, Y = (XpY-XmY)/2."""
    o, v = _ov(nBas, nC, nO, nR)
    ds = 1.0 if ispin == 1 else -1.0
    dK = 1.0 if exchange_kernel else 0.0
    E_ibaj = ERI[np.ix_(o, v, v, o)]                      # [i,b,a,j]
    E_ibja = ERI[np.ix_(o, v, o, v)]                      # [i,b,j,a]
    E_ijab = ERI[np.ix_(o, o, v, v)]                      # [i,j,a,b] (also [i,j,b,a] swapped)
    Ap = ((1.0 + ds) * E_ibaj.transpose(0, 2, 3, 1) - dK * E_ibja.transpose(0, 3, 2, 1)).reshape(nS, nS)
    Bp = ((1.0 + ds) * E_ijab.transpose(0, 2, 1, 3) - dK * E_ijab.transpose(0, 3, 1, 2)).reshape(nS, nS)
    X = 0.5 * (XpY + XmY)
    Y = 0.5 * (XpY - XmY)
    return (trace_matrix(X @ Bp @ Y.T + Y @ Bp @ X.T) + trace_matrix(X @ Ap @ X.T + Y @ Ap @ Y.T)
            - trace_matrix(Ap))


def RGW_phACFDT(exchange_kernel, doXBS, TDA_W, TDA, singlet, triplet, eta, nBas, nC, nO, nV, nR,
                nS, ERI, eW, eGW):
    """Adiabatic-connection correlation energy of phBSE@GW -- GW/RGW_phACFDT.f90:94-210.
    The 21 Gauss-Legendre nodes/weights on [0, 1] of include/quadrature.h, computed here
    (r = (1+x)/2, w/2).  Returns [EcAC singlet, EcAC triplet]."""
    x, wq = np.polynomial.legendre.leggauss(21)
    rAC, wAC = 0.5 * (1.0 + x), 0.5 * wq

    def kernels(lam):
        Aw = phRLR_A(1, True, nBas, nC, nO, nV, nR, nS, lam, eW, ERI)
        Bw = np.zeros((nS, nS)) if TDA_W else phRLR_B(1, True, nBas, nC, nO, nV, nR, nS, lam, ERI)
        _, OmRPA, XpY, _ = phRLR(TDA_W, nS, Aw, Bw)
        rho = RGW_excitation_density(nBas, nC, nO, nR, nS, ERI, XpY)
        KA = RGW_phBSE_static_kernel_A(eta, nBas, nC, nO, nV, nR, nS, lam, OmRPA, rho)
        KB = np.zeros((nS, nS)) if TDA else RGW_phBSE_static_kernel_B(eta, nBas, nC, nO, nV, nR,
                                                                        nS, lam, OmRPA, rho)
        return KA, KB

    KA, KB = kernels(1.0)                                              # :96-103
    EcAC = [0.0, 0.0]
    for ispin, on in ((1, singlet), (2, triplet)):
        if not on:
            continue
        Ec = np.zeros(21)
        for k, lam in enumerate(rAC):                                  # :120, :177
            if doXBS:
                KA, KB = kernels(lam)
            A = phRLR_A(ispin, False, nBas, nC, nO, nV, nR, nS, lam, eGW, ERI) + KA
            B = (np.zeros((nS, nS)) if TDA
                 else phRLR_B(ispin, False, nBas, nC, nO, nV, nR, nS, lam, ERI) + KB)
            _, _, XpY, XmY = phRLR(TDA, nS, A, B)
            Ec[k] = phACFDT_correlation_energy(ispin, exchange_kernel, nBas, nC, nO, nV, nR, nS,
                                               ERI, XpY, XmY)
        e = 0.5 * float(np.dot(wAC, Ec))                               # :151, :208
        if exchange_kernel:
            e *= 0.5 if ispin == 1 else 1.5                            # :153, :210
        EcAC[ispin - 1] = e
    return EcAC


# ---------------------------------------------------------------------------
# Drivers (src/GW/RG0W0.f90, src/GW/evRGW.f90)
# ---------------------------------------------------------------------------
def RG0W0(linearize, eta, doSRG, nBas, nOrb, nC, nO, nV, nR, nS, ERI, eHF, TDA_W=False):
    """G0W0@RHF -- GW/RG0W0.f90:109-233 (dRPA singlet screening).

    Returns a dict with eGW, SigC, Z, Om, XpY, rho, EcRPA (second Casida at
    eGW, :222-225), EcGM, eGWlin and the first-Casida EcRPA.
    """
    flow = 500.0                                                     # :98
    isp_W, dRPA_W = 1, True
    Aph = phRLR_A(isp_W, dRPA_W, nOrb, nC, nO, nV, nR, nS, 1.0, eHF, ERI)
    Bph = np.zeros((nS, nS)) if TDA_W else phRLR_B(isp_W, dRPA_W, nOrb, nC, nO, nV, nR, nS, 1.0,
                                                   ERI)                # :116-117
    EcRPA0, Om, XpY, XmY = phRLR(TDA_W, nS, Aph, Bph)                 # :119
    rho = RGW_excitation_density(nOrb, nC, nO, nR, nS, ERI, XpY)
    if doSRG:
        EcGM, SigC, Z = RGW_SRG_self_energy_diag(flow, nBas, nOrb, nC, nO, nV, nR, nS, eHF, Om, rho)
    else:
        EcGM, SigC, Z = RGW_self_energy_diag(eta, nBas, nOrb, nC, nO, nV, nR, nS, eHF, Om, rho)
    eGWlin = eHF + Z * SigC                                          # :188
    iters = None
    if linearize:
        eGW = eGWlin.copy()
    else:
        eGW, Z, iters = RGW_QP_graph(doSRG, eta, flow, nOrb, nC, nO, nV, nR, nS, eHF, Om, rho,
                                     eGWlin, eHF, Z, return_iters=True)
    Aph2 = phRLR_A(isp_W, dRPA_W, nOrb, nC, nO, nV, nR, nS, 1.0, eGW, ERI)
    Bph2 = np.zeros((nS, nS)) if TDA_W else phRLR_B(isp_W, dRPA_W, nOrb, nC, nO, nV, nR, nS, 1.0,
                                                    ERI)               # :222-223
    EcRPA, Om2, _, _ = phRLR(TDA_W, nS, Aph2, Bph2)                   # :225
    return dict(eGW=eGW, SigC=SigC, Z=Z, Om=Om, XpY=XpY, XmY=XmY, rho=rho, EcRPA=EcRPA,
                EcRPA_HF=EcRPA0, EcGM=EcGM, eGWlin=eGWlin, Om_GW=Om2, qp_iters=iters)


def evRGW(maxSCF, thresh, max_diis, linearize, eta, doSRG, nBas, nOrb, nC, nO, nV, nR, nS,
          ERI, eHF, TDA_W=False, raise_on_fail=True):
    """evGW@RHF -- GW/evRGW.f90:110-198.

    Returns a dict with eGW (after the last DIIS step), EcRPA (Casida of the
    last cycle), SigC, Z, Conv, nSCF and the per-cycle Conv history.
    """
    flow = 500.0
    ispin, dRPA = 1, True
    nSCF = 0
    n_diis = 0
    Conv = 1.0
    e_diis = np.zeros((nOrb, max(max_diis, 1)))
    error_diis = np.zeros((nOrb, max(max_diis, 1)))
    eGW = eHF.copy()
    eOld = eGW.copy()
    Z = np.ones(nOrb)
    hist = []
    EcRPA = EcGM = 0.0
    SigC = np.zeros(nOrb)
    while Conv > thresh and nSCF <= maxSCF:                          # :119
        Aph = phRLR_A(ispin, dRPA, nOrb, nC, nO, nV, nR, nS, 1.0, eGW, ERI)
        Bph = np.zeros((nS, nS)) if TDA_W else phRLR_B(ispin, dRPA, nOrb, nC, nO, nV, nR, nS, 1.0,
                                                       ERI)            # :123-124
        EcRPA, Om, XpY, XmY = phRLR(TDA_W, nS, Aph, Bph)               # :126
        rho = RGW_excitation_density(nOrb, nC, nO, nR, nS, ERI, XpY)
        if doSRG:
            EcGM, SigC, Z = RGW_SRG_self_energy_diag(flow, nBas, nOrb, nC, nO, nV, nR, nS, eGW, Om, rho)
        else:
            EcGM, SigC, Z = RGW_self_energy_diag(eta, nBas, nOrb, nC, nO, nV, nR, nS, eGW, Om, rho)
        if linearize:
            eGW = eHF + SigC                                         # :147
        else:
            eGW, Z = RGW_QP_graph(doSRG, eta, flow, nOrb, nC, nO, nV, nR, nS, eHF, Om, rho,
                                  eOld, eOld, Z)                     # :154
        Conv = float(np.max(np.abs(eGW - eOld)))                     # :160
        hist.append(Conv)
        if max_diis > 1:                                             # :166-171
            n_diis = min(n_diis + 1, max_diis)
            _, error_diis, e_diis, eGW = DIIS_extrapolation(n_diis, error_diis, e_diis, eGW - eOld, eGW)
        eOld = eGW.copy()                                            # :177
        nSCF += 1
    failed = (nSCF == maxSCF + 1)
    if failed and raise_on_fail:
        raise RuntimeError("evGW convergence failed")               # :190-198
    return dict(eGW=eGW, EcRPA=EcRPA, EcGM=EcGM, SigC=SigC, Z=Z, Conv=Conv, nSCF=nSCF,
                conv_hist=hist, failed=failed)


# ---------------------------------------------------------------------------
# Quasiparticle self-consistent GW (src/GW/qsRGW.f90)
# ---------------------------------------------------------------------------
def Hartree_matrix_AO_basis(nBas, P, ERI):
    """J(mu,nu) = sum_{la,si} P(la,si) ERI(mu,la,nu,si) -- AOtoMO/Hartree_matrix_AO_basis.f90:23-31."""
    return np.einsum("ls,mlns->mn", P, ERI, optimize=True)


def exchange_matrix_AO_basis(nBas, P, ERI):
    """K(mu,nu) = -sum_{la,si} P(la,si) ERI(mu,la,si,nu) -- AOtoMO/exchange_matrix_AO_basis.f90:22-31."""
    return -np.einsum("ls,mlsn->mn", P, ERI, optimize=True)


def AOtoMO(nBas, nOrb, c, M):
    """c^T M c -- AOtoMO/AOtoMO.f90:21-29."""
    return c.T @ (M @ c)


def MOtoAO(nBas, nOrb, S, c, M):
    """(S c) M (S c)^T -- AOtoMO/MOtoAO.f90:26-36."""
    SC = S @ c
    return SC @ (M @ SC.T)


def RGW_self_energy(eta, nBas, nOrb, nC, nO, nV, nR, nS, e, Om, rho):
    """Full correlation self-energy matrix, Z and EcGM -- GW/RGW_self_energy.f90:40-156:
    Sig(p,q) = sum_m [sum_i 2 rho(p,i,m) rho(q,i,m) eps/(eps^2+eta^2), eps = e(p)-e(i)+Om(m)]
             + sum_m [sum_a 2 rho(p,a,m) rho(q,a,m) eps/(eps^2+eta^2), eps = e(p)-e(a)-Om(m)].
    Returns (EcGM, Sig, Z)."""
    occ, vir = _ov(nOrb, nC, nO, nR)
    act = np.arange(nC, nOrb - nR)
    eta2 = eta * eta
    Sig = np.zeros((nOrb, nOrb))
    dZ = np.zeros(nOrb)
    for x, sgn in ((occ, 1.0), (vir, -1.0)):
        eps = e[act][:, None, None] - e[x][None, :, None] + sgn * Om[None, None, :]   # [p,x,m]
        w = eps / (eps ** 2 + eta2)
        rp = rho[np.ix_(act, x)]                                                     # [p,x,m]
        Sig[np.ix_(act, act)] += 2.0 * np.einsum("pxm,pxm,qxm->pq", w, rp, rp, optimize=True)
        dZ[act] -= np.einsum("pxm,pxm->p", 2.0 * rp ** 2, (eps ** 2 - eta2) / (eps ** 2 + eta2) ** 2)
    Z = 1.0 / (1.0 - dZ)
    EcGM, _, _ = RGW_self_energy_diag(eta, nOrb, nOrb, nC, nO, nV, nR, nS, e, Om, rho)
    return EcGM, Sig, Z


def RGW_SRG_self_energy(flow, nBas, nOrb, nC, nO, nV, nR, nS, e, Om, rho):
    """SRG-regularised full self-energy -- GW/RGW_SRG_self_energy.f90:40-80:
    Sig(p,q) = sum_(x,m) 2 rho(p,x,m) rho(q,x,m) (1 - exp(-s Dp^2) exp(-s Dq^2)) (Dp+Dq)/(Dp^2+Dq^2),
    D = e - e_x + Om (x occupied) or e - e_x - Om (x virtual).  Z and EcGM are those of
    RGW_SRG_self_energy_diag (RGW_SRG_self_energy.f90:86-130 has the same formulas)."""
    occ, vir = _ov(nOrb, nC, nO, nR)
    act = np.arange(nC, nOrb - nR)
    s = flow
    Sig = np.zeros((nOrb, nOrb))
    for x, sgn in ((occ, 1.0), (vir, -1.0)):
        D = e[act][:, None, None] - e[x][None, :, None] + sgn * Om[None, None, :]   # [p,x,m]
        g = np.exp(-s * D * D)
        r = rho[np.ix_(act, x)]
        for ip, p in enumerate(act):
            Dp, Dq = D[ip][None], D
            f = (1.0 - g[ip][None] * g) * (Dp + Dq) / (Dp * Dp + Dq * Dq)
            Sig[p, act] += np.einsum("xm,qxm->q", 2.0 * r[ip], r * f)
    EcGM, _, Z = RGW_SRG_self_energy_diag(flow, nOrb, nOrb, nC, nO, nV, nR, nS, e, Om, rho)
    return EcGM, Sig, Z


def qsRGW(maxSCF, thresh, max_diis, eta, TDA_W, nBas, nOrb, nC, nO, nV, nR, nS, eHF, cHF, PHF, S,
          T, V, Hc, X, ERI_AO, raise_on_fail=True, doSRG=False):
    """Quasiparticle self-consistent GW@RHF -- GW/qsRGW.f90:193-359 (without the linearised
    density-matrix correction, dipoles and the post-processing BSE).  nOrb < nBas follows the
    reference's projected branch (:281-284, :329-333).
    Returns dict(eGW, c, P, EqsGW (electronic), EcRPA, EcGM, SigC (MO), Z, nSCF, Conv, failed)."""
    assert nOrb <= nBas
    nSCF = -1
    n_diis = 0
    Conv = 1.0
    P = PHF.copy()
    eGW = eHF.copy()
    c = cHF.copy()
    nsq = nBas * nBas
    F_diis = np.zeros((nsq, max(max_diis, 1)))
    err_diis = np.zeros((nsq, max(max_diis, 1)))
    EcRPA = EcGM = EqsGW = 0.0
    SigC = Z = None
    while Conv > thresh and nSCF < maxSCF:                                     # :193
        nSCF += 1
        J = Hartree_matrix_AO_basis(nBas, P, ERI_AO)                           # :201
        K = exchange_matrix_AO_basis(nBas, P, ERI_AO)                          # :202
        ERI_MO = AOtoMO_ERI_RHF(nBas, nOrb, c, ERI_AO)                         # :210
        Aph = phRLR_A(1, True, nOrb, nC, nO, nV, nR, nS, 1.0, eGW, ERI_MO)      # :214
        Bph = np.zeros((nS, nS)) if TDA_W else phRLR_B(1, True, nOrb, nC, nO, nV, nR, nS, 1.0,
                                                       ERI_MO)                  # :215
        EcRPA, Om, XpY, XmY = phRLR(TDA_W, nS, Aph, Bph)                       # :217
        rho = RGW_excitation_density(nOrb, nC, nO, nR, nS, ERI_MO, XpY)       # :220
        if doSRG:                                                              # :257-264
            EcGM, SigC, Z = RGW_SRG_self_energy(500.0, nBas, nOrb, nC, nO, nV, nR, nS, eGW, Om,
                                                rho)
        else:
            EcGM, SigC, Z = RGW_self_energy(eta, nBas, nOrb, nC, nO, nV, nR, nS, eGW, Om, rho)
        SigC = 0.5 * (SigC + SigC.T)                                           # :269
        SigCp = MOtoAO(nBas, nOrb, S, c, SigC)                                 # :276
        F = Hc + J + 0.5 * K + SigCp                                           # :280
        if nBas != nOrb:                                                       # :281-284
            F = MOtoAO(nBas, nOrb, S, c, AOtoMO(nBas, nOrb, c, F))
        err = F @ (P @ S) - (S @ P) @ F                                        # :288
        if nSCF > 1:
            Conv = float(np.max(np.abs(err)))                                  # :290
        ET = trace_matrix(P @ T)                                               # :294
        EV = trace_matrix(P @ V)                                               # :298
        EJ = 0.5 * trace_matrix(P @ J)                                         # :302
        EK = 0.25 * trace_matrix(P @ K)                                        # :306
        EqsGW = ET + EV + EJ + EK                                              # :310
        if max_diis > 1:                                                       # :314-319
            n_diis = min(n_diis + 1, max_diis)
            _, err_diis, F_diis, Fv = DIIS_extrapolation(n_diis, err_diis, F_diis,
                                                         err.reshape(-1, order="F"),
                                                         F.reshape(-1, order="F"))
            F = Fv.reshape((nBas, nBas), order="F")
        if nBas == nOrb:
            Fp = X.T @ (F @ X)                                                 # :324
            cp, eGW = diagonalize_matrix(Fp)                                   # :326
            c = X @ cp                                                         # :327
        else:
            Fp = c.T @ (F @ c)                                                 # :329
            cp, eGW = diagonalize_matrix(Fp)                                   # :331
            c = c @ cp                                                         # :332
        SigC = AOtoMO(nBas, nOrb, c, SigCp)                                    # :335
        P = 2.0 * c[:, :nO] @ c[:, :nO].T                                      # :339
    failed = (nSCF == maxSCF)                                                  # :354
    if failed and raise_on_fail:
        raise RuntimeError("qsGW convergence failed")
    return dict(eGW=eGW, c=c, P=P, EqsGW=EqsGW, EcRPA=EcRPA, EcGM=EcGM, SigC=SigC, Z=Z,
                nSCF=nSCF, Conv=Conv, failed=failed)


def homo_lumo(eGW, nO):
    """print_RG0W0.f90:27-29."""
    return float(np.max(eGW[:nO])), float(np.min(eGW[nO:]))


# ---------------------------------------------------------------------------
# Checks at the benchmark sizes (nS in the thousands)
# ---------------------------------------------------------------------------
def drpa_casida_factored(nO, e, L):
    """The dRPA singlet Casida of LR/phRLR.f90:45-95 (with phRLR_A/B.f90, dRPA, ispin = 1, no
    frozen orbitals) for integrals given as the factor L[P,p,q], (pq|rs) = sum_P L_Ppq L_Prs.

    Same mathematics as ``phRLR(False, nS, phRLR_A(...), phRLR_B(...))``: A - B = diag(e_a - e_i)
    exactly, so AmBSq = diag(sqrt(e_a - e_i)) and M = AmBSq (A + B) AmBSq with
    (A + B)(ia,jb) = delta (e_a - e_i) + 4 (ia|jb).  The eigensolver is LAPACK dsyevr instead of
    dsyev (10x faster at nS = 3600): the eigenvalues agree to rounding, the eigenvectors up to
    sign and rotation inside degenerate subspaces, to which every GW quantity is invariant.
    Returns (EcRPA, Om, XpY) with XpY[m, ia]."""
    from scipy.linalg import eigh
    N = len(e)
    Lov = L[:, :nO, nO:].reshape(L.shape[0], -1)                 # [P, ia], ia = i*nv + a
    d = (e[None, nO:] - e[:nO, None]).reshape(-1)                 # e_a - e_i
    K = Lov.T @ Lov                                               # (ia|jb)
    s = np.sqrt(d)
    M = (4.0 * K) * s[:, None] * s[None, :]
    M[np.diag_indices_from(M)] += d * d
    lam, Zv = eigh(M, driver="evr")
    Om = np.sqrt(np.abs(lam))
    XpY = (Zv.T * s[None, :]) / np.sqrt(Om)[:, None]
    EcRPA = 0.5 * (float(np.sum(Om)) - float(np.sum(d + 2.0 * np.diag(K))))
    assert N == L.shape[1]
    return EcRPA, Om, XpY


def rho_row_factored(p, nO, L, XpY):
    """Row p of RGW_excitation_density.f90:30-50, rho(p,q,m) = sum_jb (pq|jb) XpY(m,jb), from
    the factor: sum_P L_Ppq (sum_jb L_Pjb XpY(m,jb)).  Returns rho_p[q, m]."""
    Lov = L[:, :nO, nO:].reshape(L.shape[0], -1)
    T = Lov @ XpY.T                                               # [P, m]
    return L[:, p, :].T @ T


def qp_residual(p, w, eHF, Om, rho_p, nO, eta=0.0):
    """f(w) = w - eHF(p) - SigC_p(w) of RGW_QP_graph.f90:56-76 (Sigma from RGW_Re_SigC.f90:30-50
    with e = eHF, as in G0W0), given row p of rho."""
    N = len(eHF)
    nS = len(Om)
    sig = RGW_Re_SigC(0, w, eta, N, 0, nO, N - nO, 0, nS, eHF, Om, rho_p[None])
    return float(w - eHF[p] - sig)


def qp_root_certificate(p, r, w0, nBas, nC, nO, nR, e, Om, rho):
    """The library's root certificate for a guess-started Newton search, restated (eta = 0, no
    SRG): True if no pole e_q -+ Om_m lies between w0 (the reference start eGWlin) and r (the
    root reached from the guess) and f''(r) = 2 (A - B) has the sign of w0 - r, where
    A = sum_{poles above r} R/(pole - r)^3 and B = sum_{poles below r} R/(r - pole)^3.  Then the
    Newton search of RGW_QP_graph.f90:56-76 started at w0 converges monotonically to r."""
    occ, vir = _ov(nBas, nC, nO, nR)
    R = np.concatenate([2.0 * rho[p, occ, :] ** 2, 2.0 * rho[p, vir, :] ** 2]).ravel()
    poles = np.concatenate([(e[occ][:, None] - Om[None, :]), (e[vir][:, None] + Om[None, :])]).ravel()
    eps, eps0 = r - poles, w0 - poles
    if np.any(~(eps * eps0 > 0.0)):
        return False
    t = R / eps ** 3
    a, b = -np.sum(t[eps < 0]), np.sum(t[eps > 0])
    margin = 1e-9 * (a + b)
    return bool((w0 > r and a - b > margin) or (w0 < r and b - a > margin) or w0 == r)
