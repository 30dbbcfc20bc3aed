"""He / 6-31G integrals and RHF, for the known-answer test of the oracle.

TEST INFRASTRUCTURE ONLY (imported by tests/ and the golden-fixture script).

He/6-31G has one centre and two contracted s functions (basis/6-31g:22-27 of
the reference), so every integral has a closed form (the Boys function at
argument zero is 1).  The contraction is normalised the way PySCF does it
(primitive norms folded into the coefficients, then the contracted function
normalised), because the reference's integrals come from PySCF
(PyDuck.py:156-159,342).  The AO ERIs are returned in QuAcK's physicist layout
ERI(mu,nu,la,si) = <mu nu|la si> = (mu la|nu si).

The RHF is a plain closed-shell Roothaan SCF (the reference's RHF.f90 reaches
the same fixed point); it is converged to 1e-13 in the density.
"""
from __future__ import annotations

import numpy as np

# basis/6-31g:22-27 (exponent, contraction coefficient)
HE_631G = [
    [(0.3842163400e02, 0.4013973935e-01),
     (0.5778030000e01, 0.2612460970e00),
     (0.1241774000e01, 0.7931846246e00)],
    [(0.2979640000e00, 1.0)],
]
Z_HE = 2.0

# Golden values, tests/feather_bench.py:62-91 of the reference (He, 6-31g)
GOLDEN = {
    "RHF energy": -2.855160426154444,
    "RHF HOMO energy": -0.914126628640145,
    "RHF LUMO energy": 1.399859335255765,
    "phRPA correlation energy": -0.018845374128748,
    "G0W0 correlation energy": -0.019314094399372,
    "G0W0 HOMO energy": -0.87053388021722,
    "G0W0 LUMO energy": 1.377171287041735,
    "evGW correlation energy": -0.019335511771337,
    "evGW HOMO energy": -0.868460640984803,
    "evGW LUMO energy": 1.376287581502582,
}


def _contracted(shells):
    out = []
    for sh in shells:
        a = np.array([p[0] for p in sh])
        c = np.array([p[1] for p in sh]) * (2.0 * a / np.pi) ** 0.75
        s = np.sum(c[:, None] * c[None, :] * (np.pi / (a[:, None] + a[None, :])) ** 1.5)
        out.append((a, c / np.sqrt(s)))
    return out


def integrals():
    """Return (S, T, V, ERI_AO_phys) for He/6-31G."""
    bf = _contracted(HE_631G)
    n = len(bf)
    S = np.zeros((n, n))
    T = np.zeros((n, n))
    V = np.zeros((n, n))
    for m, (am, cm) in enumerate(bf):
        for v, (av, cv) in enumerate(bf):
            p = am[:, None] + av[None, :]
            cc = cm[:, None] * cv[None, :]
            S[m, v] = np.sum(cc * (np.pi / p) ** 1.5)
            T[m, v] = np.sum(cc * 3.0 * am[:, None] * av[None, :] / p * (np.pi / p) ** 1.5)
            V[m, v] = np.sum(cc * (-Z_HE) * 2.0 * np.pi / p)
    chem = np.zeros((n, n, n, n))
    for i in range(n):
        for j in range(n):
            for k in range(n):
                for l in range(n):
                    ai, ci = bf[i]
                    aj, cj = bf[j]
                    ak, ck = bf[k]
                    al, cl = bf[l]
                    p = ai[:, None, None, None] + aj[None, :, None, None]
                    q = ak[None, None, :, None] + al[None, None, None, :]
                    cc = (ci[:, None, None, None] * cj[None, :, None, None]
                          * ck[None, None, :, None] * cl[None, None, None, :])
                    chem[i, j, k, l] = np.sum(cc * 2.0 * np.pi ** 2.5 / (p * q * np.sqrt(p + q)))
    eri_phys = chem.transpose(0, 2, 1, 3).copy()      # PyDuck.py:342
    return S, T, V, eri_phys


def rhf(S, Hc, eri_phys, nO, maxit=200, tol=1e-13):
    """Closed-shell RHF.  Returns (E_elec, eps, C)."""
    chem = eri_phys.transpose(0, 2, 1, 3)             # back to (mu nu|la si)
    s, U = np.linalg.eigh(S)
    X = U @ np.diag(s ** -0.5) @ U.T
    F = Hc.copy()
    P = np.zeros_like(S)
    E = 0.0
    for _ in range(maxit):
        Fp = X.T @ F @ X
        eps, Cp = np.linalg.eigh(Fp)
        C = X @ Cp
        Pn = 2.0 * C[:, :nO] @ C[:, :nO].T
        J = np.einsum("mnls,ls->mn", chem, Pn)
        K = np.einsum("mlns,ls->mn", chem, Pn)
        F = Hc + J - 0.5 * K
        E = 0.5 * np.sum(Pn * (Hc + F))
        if np.max(np.abs(Pn - P)) < tol:
            P = Pn
            break
        P = Pn
    Fp = X.T @ F @ X
    eps, Cp = np.linalg.eigh(Fp)
    C = X @ Cp
    return float(E), eps, C


def he_system():
    """Full He/6-31G input to the GW chain: dict(nBas, nO, eHF, ERI_MO, ERI_AO, c, ERHF)."""
    from oracle.qkgw_oracle import AOtoMO_ERI_RHF
    S, T, V, eri = integrals()
    nO = 1
    E, eps, C = rhf(S, T + V, eri, nO)
    eri_mo = AOtoMO_ERI_RHF(2, 2, C, eri)
    return dict(nBas=2, nO=nO, eHF=eps, ERI_MO=eri_mo, ERI_AO=eri, c=C, ERHF=E)
