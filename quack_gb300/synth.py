"""Seeded synthetic GW systems with the shapes and value distributions of the benchmark configs.

Every system is an RI-factorised closed-shell problem:
  L[P,p,q] = L[P,q,p] ~ N(0,1) * 0.5/sqrt(naux)   (upper triangle drawn, then mirrored)
  (pq|rs)  = sum_P L[P,p,q] L[P,r,s]               (8-fold symmetric and PSD, so A+B and A-B
                                                    of the dRPA Casida stay positive definite)
  occupied e ~ U[-20, -0.3] Ha sorted, virtual e ~ U[0.05, 5] Ha sorted.
Draw order for one system with generator ``rng``: (1) the naux * N(N+1)/2 normals of the upper
triangles, row-major over (P, p<=q); (2) nO occupied energies; (3) N-nO virtual energies.

The batched configurations draw their sizes first: N ~ U{Nmin..Nmax} (``rng.integers``) for
every system, then the systems in order with the same generator.  nO = floor(N/8 + 1/2)
(round half up; Python's round() would round half to even).

The physicist-layout MO ERIs used by the reference (ERI(p,q,r,s) = <pq|rs> = (pr|qs)) are
built from L on the host (numpy, small N) or on the GPU (torch, large N).
"""
from __future__ import annotations

import math

import numpy as np

SYSTEMS = {
    # name: (N, nO, naux, seed)
    "g0w0_n200_o20_aux600": (200, 20, 600, 0),
    "g0w0_n400_o40_aux1200": (400, 40, 1200, 2),
}


def n_occ(N: int) -> int:
    """nO = floor(N/8 + 1/2)."""
    return int(math.floor(N / 8.0 + 0.5))


def gen_system(N: int, nO: int, naux: int, rng: np.random.Generator) -> dict:
    iu = np.triu_indices(N)
    ntri = iu[0].size
    up = rng.standard_normal((naux, ntri)) * (0.5 / math.sqrt(naux))
    L = np.zeros((naux, N, N))
    L[:, iu[0], iu[1]] = up
    L[:, iu[1], iu[0]] = up
    e_occ = np.sort(rng.uniform(-20.0, -0.3, size=nO))
    e_vir = np.sort(rng.uniform(0.05, 5.0, size=N - nO))
    eHF = np.concatenate([e_occ, e_vir])
    return dict(N=N, nO=nO, naux=naux, L=L, eHF=eHF)


def named_system(name: str) -> dict:
    N, nO, naux, seed = SYSTEMS[name]
    return gen_system(N, nO, naux, np.random.default_rng(seed))


def small_system(N: int, nO: int, naux: int, seed: int) -> dict:
    return gen_system(N, nO, naux, np.random.default_rng(seed))


def batch_systems(nsys: int, Nmin: int, Nmax: int, seed: int, naux_per_N: int = 3) -> list:
    rng = np.random.default_rng(seed)
    Ns = rng.integers(Nmin, Nmax + 1, size=nsys)
    out = []
    for N in Ns:
        N = int(N)
        out.append(gen_system(N, n_occ(N), naux_per_N * N, rng))
    return out


def eri_phys_numpy(L: np.ndarray) -> np.ndarray:
    """ERI[p,q,r,s] = (pr|qs) as a numpy array indexed like the Fortran ERI(p,q,r,s).  Built a
    few p at a time, so that no second N^4 copy and no single huge GEMM is needed."""
    naux, N, _ = L.shape
    out = np.empty((N, N, N, N))
    Lf = L.reshape(naux, N * N)
    pb = max(1, min(N, (1 << 27) // (N * N * N)))  # ~1 GB blocks of (pr|..)
    for p0 in range(0, N, pb):
        p1 = min(N, p0 + pb)
        blk = (L[:, p0:p1, :].reshape(naux, (p1 - p0) * N).T @ Lf).reshape(p1 - p0, N, N, N)
        out[p0:p1] = blk.transpose(0, 2, 1, 3)
    return out


def eri_fortran_flat_torch(L: np.ndarray, device="cuda"):
    """The same ERI as a flat float64 torch tensor in Fortran (column-major) memory order:
    element ERI(p,q,r,s) at p + N*(q + N*(r + N*s)).  Built on the device."""
    import torch

    naux, N, _ = L.shape
    Lt = torch.from_numpy(np.ascontiguousarray(L.reshape(naux, N * N))).to(device)
    chem = (Lt.T @ Lt).reshape(N, N, N, N)          # chem[p,q,r,s] = (pq|rs)
    # T[s,r,q,p] = (pr|qs) = chem[p,r,q,s]  ->  C-order T has Fortran order of ERI(p,q,r,s)
    T = chem.permute(3, 1, 2, 0).contiguous()
    del chem, Lt
    return T.reshape(-1)


# ------------------------------------------------------------------------------------------
# AO-basis input for quasiparticle self-consistent GW: linear hydrogen chains in uncontracted
# s-type Gaussian bases.  All one- and two-electron integrals of s primitives have closed forms
# (Boys function F0), so the chain is a real molecular problem -- non-orthogonal basis, 8-fold
# symmetric positive-definite ERIs -- without an integral library.
# ------------------------------------------------------------------------------------------
HCHAIN_EXPONENTS = (3.42525091, 0.62391373, 0.16885540)   # the STO-3G hydrogen exponents


def _boys0(t):
    from scipy.special import erf
    t = np.asarray(t, dtype=np.float64)
    small = t < 1e-12
    ts = np.where(small, 1.0, t)
    return np.where(small, 1.0 - t / 3.0, 0.5 * np.sqrt(np.pi / ts) * erf(np.sqrt(ts)))


def hchain_integrals(n_atoms: int, spacing: float = 1.6, exponents=HCHAIN_EXPONENTS):
    """Integrals of a linear H chain (z axis, ``spacing`` bohr) in normalised s primitives.
    Returns (S, T, V, ERI, ENuc) with ERI[p,q,r,s] = <pq|rs> = (pr|qs), the physicist layout of
    the reference's ERI_AO."""
    zc = np.arange(n_atoms, dtype=np.float64) * spacing
    a = np.array([x for _ in range(n_atoms) for x in exponents])
    z = np.array([zc[i] for i in range(n_atoms) for _ in exponents])
    nrm = (2.0 * a / np.pi) ** 0.75
    p = a[:, None] + a[None, :]
    mu = a[:, None] * a[None, :] / p
    R2 = (z[:, None] - z[None, :]) ** 2
    K = np.exp(-mu * R2) * nrm[:, None] * nrm[None, :]
    S = K * (np.pi / p) ** 1.5
    T = mu * (3.0 - 2.0 * mu * R2) * S
    P = (a[:, None] * z[:, None] + a[None, :] * z[None, :]) / p
    V = np.zeros_like(S)
    for C in zc:
        V -= 2.0 * np.pi / p * K * _boys0(p * (P - C) ** 2)
    n = a.size
    iu = np.triu_indices(n)
    pp, kk, PP = p[iu], K[iu], P[iu]           # unique pairs
    chem_pairs = np.empty((pp.size, pp.size))
    for i0 in range(0, pp.size, 512):
        sl = slice(i0, i0 + 512)
        q1, k1, P1 = pp[sl, None], kk[sl, None], PP[sl, None]
        al = q1 * pp[None, :] / (q1 + pp[None, :])
        chem_pairs[sl] = (2.0 * np.pi ** 2.5 / (q1 * pp[None, :] * np.sqrt(q1 + pp[None, :]))
                          * k1 * kk[None, :] * _boys0(al * (P1 - PP[None, :]) ** 2))
    pidx = np.zeros((n, n), dtype=np.int64)
    pidx[iu] = np.arange(pp.size)
    pidx[iu[1], iu[0]] = np.arange(pp.size)
    chem = chem_pairs[pidx[:, :, None, None], pidx[None, None, :, :]]   # (pq|rs)
    ERI = np.ascontiguousarray(chem.transpose(0, 2, 1, 3))              # <pr|qs> -> <pq|rs>
    ENuc = sum(1.0 / abs(zc[i] - zc[j]) for i in range(n_atoms) for j in range(i))
    return S, T, V, ERI, float(ENuc)


def rhf_start(S, Hc, ERI, nO, maxit=500, tol=1e-10, n_drop=0):
    """Closed-shell RHF with DIIS on F (commutator error), the qsGW starting point.
    Returns (E_elec, eps, C, P, X) with X = S^-1/2 (symmetric orthogonalisation), or, with
    n_drop > 0, the canonical orthogonalisation X = U s^-1/2 without the n_drop eigenvectors of
    the smallest overlap eigenvalues (nOrb = nBas - n_drop)."""
    s, U = np.linalg.eigh(S)
    if n_drop > 0:
        X = U[:, n_drop:] * s[n_drop:] ** -0.5
    else:
        X = (U * s ** -0.5) @ U.T
    F = Hc.copy()
    P = np.zeros_like(S)
    hist_F, hist_e = [], []
    for _ in range(maxit):
        eps, Cp = np.linalg.eigh(X.T @ F @ X)
        C = X @ Cp
        P = 2.0 * C[:, :nO] @ C[:, :nO].T
        J = np.einsum("ls,mlns->mn", P, ERI, optimize=True)
        Kx = np.einsum("ls,mlsn->mn", P, ERI, optimize=True)
        F = Hc + J - 0.5 * Kx
        err = F @ P @ S - S @ P @ F
        if np.max(np.abs(err)) < tol:
            break
        hist_F.append(F.copy())
        hist_e.append(err.ravel())
        hist_F, hist_e = hist_F[-8:], hist_e[-8:]
        m = len(hist_F)
        B = -np.ones((m + 1, m + 1))
        B[m, m] = 0.0
        B[:m, :m] = np.array([[ei @ ej for ej in hist_e] for ei in hist_e])
        rhs = np.zeros(m + 1)
        rhs[m] = -1.0
        try:
            w = np.linalg.solve(B, rhs)[:m]
            F = sum(wi * Fi for wi, Fi in zip(w, hist_F))
        except np.linalg.LinAlgError:
            pass
    eps, Cp = np.linalg.eigh(X.T @ F @ X)
    C = X @ Cp
    P = 2.0 * C[:, :nO] @ C[:, :nO].T
    E = 0.5 * float(np.sum(P * (Hc + F)))
    return E, eps, C, P, X


def hchain_system(n_atoms: int, spacing: float = 1.6, exponents=HCHAIN_EXPONENTS,
                  n_drop: int = 0) -> dict:
    """Everything qsRGW reads for an H chain: dict(nBas, nOrb, nO, S, T, V, Hc, X, ERI_AO, ENuc,
    ERHF, eHF, cHF, PHF).  n_atoms must be even (closed shell); n_drop > 0 removes that many
    near-linearly-dependent combinations (nOrb = nBas - n_drop)."""
    assert n_atoms % 2 == 0
    S, T, V, ERI, ENuc = hchain_integrals(n_atoms, spacing, exponents)
    Hc = T + V
    nO = n_atoms // 2
    E, eps, C, P, X = rhf_start(S, Hc, ERI, nO, n_drop=n_drop)
    return dict(nBas=S.shape[0], nOrb=X.shape[1], nO=nO, S=S, T=T, V=V, Hc=Hc, X=X, ERI_AO=ERI,
                ENuc=ENuc, ERHF=E, eHF=eps, cHF=C, PHF=P)
