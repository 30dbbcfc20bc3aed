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

CONFIGS = {
    # name: (N, nO, naux, seed)
    "c2_g0w0_n200": (200, 20, 600, 0),
    "c4_large_n400": (400, 40, 1200, 2),
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


def config_system(name: str) -> dict:
    N, nO, naux, seed = CONFIGS[name]
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
