"""Oracle fixtures at the sizes the benchmark times.

    python tests/golden/make_bench_golden.py [c2] [c3]

c2: the synthetic N=200 G0W0 (nO=20, naux=600, seed 0; Casida dimension nS=3600), the system
    of the headline benchmark line.
c3: the first 16 systems of the 256-system batch generator (seed 1, N ~ U{24..160},
    nO = floor(N/8 + 1/2), naux = 3N), the batched benchmark leg's systems.

Every system is run through the oracle's RG0W0 (GW/RG0W0.f90:109-233) on the physicist ERI
tensor built from L, Newton QP and linearised QP, eta = 0.  Stored per system: the Casida
energies at eHF (Om), EcRPA at eHF, the self-energy and Z at eHF, the linearised QP energies and
the EcRPA of the second Casida at them, the Newton roots with their iteration counts, and a
mask of the orbitals whose Newton root is reproducible (at most 10 steps, and no change above
1e-10 Ha under three random elementwise 1e-13 perturbations of rho): with eta = 0 the other
orbitals' roots move with perturbations at the rounding level, and the tests check those as
roots of the oracle's QP equation instead.  Likewise the spread of Sigma, Z and eGWlin under
1e-13 perturbations of Om and rho (near-resonant pole terms make a few orbitals' values
reproducible only to that spread).  Only energies and masks are stored; the tests
regenerate L from the seed (a checksum of L is stored to detect a generator mismatch).
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import qkgw_oracle as O  # noqa: E402
from quack_gb300 import synth  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def l_checksum(L):
    """Order-fixed checksum of the generated factor: sum and a strided sample."""
    flat = L.reshape(-1)
    sample = flat[:: max(1, flat.size // 61)][:61]
    return np.array([float(np.sum(flat)), float(np.sum(flat * flat))] + list(sample))


def stable_mask(N, nO, nS, eHF, Om, rho, eGWlin, Z, iters, seed=0):
    base = O.RGW_QP_graph(False, 0.0, 500.0, N, 0, nO, N - nO, 0, nS, eHF, Om, rho, eGWlin, eHF,
                          Z)[0]
    ok = np.asarray(iters) <= 10
    rng = np.random.default_rng(seed)
    for _ in range(3):
        f = 1.0 + 1e-13 * rng.standard_normal(rho.shape)
        e = O.RGW_QP_graph(False, 0.0, 500.0, N, 0, nO, N - nO, 0, nS, eHF, Om, rho * f, eGWlin,
                           eHF, Z)[0]
        ok &= np.abs(e - base) < 1e-10
        del f
    return ok


def sensitivity(N, nO, nS, eHF, Om, rho, SigC, Z, eGWlin, seed=1):
    """Spread of Sigma, Z and eGWlin at eHF under three random elementwise 1e-13 relative
    perturbations of Om and rho: with eta = 0, terms 2 rho^2/(e_p - e_q +- Om_m) whose
    denominator is nearly zero amplify rounding-level changes of the screening, so these values
    of some orbitals are reproducible only to this spread (not to 1e-8)."""
    rng = np.random.default_rng(seed)
    out = {"SigC": np.zeros(N), "Z": np.zeros(N), "eGWlin": np.zeros(N)}
    for _ in range(3):
        Om_p = Om * (1.0 + 1e-13 * rng.standard_normal(Om.shape))
        rho_p = rho * (1.0 + 1e-13 * rng.standard_normal(rho.shape))
        _, S, Zp = O.RGW_self_energy_diag(0.0, N, N, 0, nO, N - nO, 0, nS, eHF, Om_p, rho_p)
        del rho_p
        for k, v in (("SigC", S - SigC), ("Z", Zp - Z), ("eGWlin", eHF + Zp * S - eGWlin)):
            out[k] = np.maximum(out[k], np.abs(v))
    return out


def run_system(s, log=""):
    N, nO = s["N"], s["nO"]
    nS = nO * (N - nO)
    eHF = s["eHF"]
    t0 = time.time()
    E = synth.eri_phys_numpy(s["L"])
    A = O.phRLR_A(1, True, N, 0, nO, N - nO, 0, nS, 1.0, eHF, E)
    B = O.phRLR_B(1, True, N, 0, nO, N - nO, 0, nS, 1.0, E)
    EcRPA_HF, Om, XpY, _ = O.phRLR(False, nS, A, B)                  # RG0W0.f90:116-119
    del A, B
    rho = O.RGW_excitation_density(N, 0, nO, 0, nS, E, XpY)
    del XpY
    EcGM, SigC, Z = O.RGW_self_energy_diag(0.0, N, N, 0, nO, N - nO, 0, nS, eHF, Om, rho)
    eGWlin = eHF + Z * SigC                                            # RG0W0.f90:188
    eGW, Znew, iters = O.RGW_QP_graph(False, 0.0, 500.0, N, 0, nO, N - nO, 0, nS, eHF, Om, rho,
                                      eGWlin, eHF, Z, return_iters=True)
    stable = stable_mask(N, nO, nS, eHF, Om, rho, eGWlin, Z, iters)
    sens = sensitivity(N, nO, nS, eHF, Om, rho, SigC, Z, eGWlin)
    del rho
    # second Casida at the linearised energies (RG0W0.f90:222-225 of a linearised run)
    A = O.phRLR_A(1, True, N, 0, nO, N - nO, 0, nS, 1.0, eGWlin, E)
    B = O.phRLR_B(1, True, N, 0, nO, N - nO, 0, nS, 1.0, E)
    gap_lin = float(eGWlin[nO:].min() - eGWlin[:nO].max())
    EcRPA_lin = O.phRLR(False, nS, A, B)[0] if gap_lin > 0 else float("nan")
    del A, B, E
    print("%s N=%d nS=%d: %.1f s, %d of %d orbitals stable, max iters %d" %
          (log, N, nS, time.time() - t0, int(stable.sum()), N, int(iters.max())), flush=True)
    return dict(N=N, nO=nO, naux=s["naux"], Om=Om, EcRPA_HF=EcRPA_HF, EcGM=EcGM, SigC=SigC, Z=Z,
                eGWlin=eGWlin, EcRPA_lin=EcRPA_lin, eGW=eGW, Z_newton=Znew, qp_iters=iters,
                stable=stable, sens_SigC=sens["SigC"], sens_Z=sens["Z"],
                sens_eGWlin=sens["eGWlin"], L_check=l_checksum(s["L"]))


def make_c2():
    N, nO, naux, seed = synth.SYSTEMS["g0w0_n200_o20_aux600"]
    s = synth.gen_system(N, nO, naux, np.random.default_rng(seed))
    r = run_system(s, "c2")
    np.savez(os.path.join(OUT, "bench_c2_n200.npz"), seed=seed, **r)


def make_c3(nsys=16):
    systems = synth.batch_systems(256, 24, 160, seed=1)[:nsys]
    out = {"seed": 1, "nsys": nsys}
    for i, s in enumerate(systems):
        r = run_system(s, "c3[%d]" % i)
        for k, v in r.items():
            if k != "Om":  # the batched driver returns no Casida energies: keep the file small
                out["s%02d_%s" % (i, k)] = v
    np.savez(os.path.join(OUT, "bench_c3_first16.npz"), **out)


if __name__ == "__main__":
    which = sys.argv[1:] or ["c2", "c3"]
    if "c2" in which:
        make_c2()
    if "c3" in which:
        make_c3()
