"""Generate the committed golden fixtures of tests/golden/ from the CPU oracle.

    python tests/golden/make_golden.py

He/6-31G: analytic integrals + RHF (oracle/he631g.py) and the oracle's G0W0/evGW on them.  The
oracle itself is pinned against the FeatherBench values of the reference
(tests/feather_bench.py:62-91) by tests/test_oracle_golden.py.
Synthetic systems: quack_gb300.synth generators (seeded); only L and the energies are stored,
the ERIs are rebuilt from L by the tests.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import qkgw_oracle as O  # noqa: E402
from oracle.he631g import GOLDEN, he_system  # noqa: E402
from quack_gb300 import synth  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# name: (N, nO, naux, seed, nC, nR)
SYNTH = {
    "synth_n24": (24, 5, 72, 11, 0, 0),
    "synth_n13_frozen": (13, 3, 39, 12, 1, 1),
}


def run_all(N, nO, nC, nR, ERI, eHF):
    nS = (nO - nC) * (N - nO - nR)
    nV = N - nO
    res = {}
    g = O.RG0W0(False, 0.0, False, N, N, nC, nO, nV, nR, nS, ERI, eHF)
    for k in ("eGW", "SigC", "Z", "Om", "EcRPA", "EcGM", "eGWlin", "EcRPA_HF"):
        res["g0w0_" + k] = np.asarray(g[k])
    res["g0w0_qp_iters"] = np.asarray(g["qp_iters"])
    g = O.RG0W0(True, 0.0, False, N, N, nC, nO, nV, nR, nS, ERI, eHF)
    for k in ("eGW", "SigC", "Z", "EcRPA", "EcGM"):
        res["g0w0lin_" + k] = np.asarray(g[k])
    g = O.RG0W0(False, 0.05, True, N, N, nC, nO, nV, nR, nS, ERI, eHF)
    for k in ("eGW", "SigC", "Z", "EcRPA", "EcGM"):
        res["g0w0srg_" + k] = np.asarray(g[k])
    for nd in (1, 5):
        v = O.evRGW(64, 1e-5, nd, False, 0.0, False, N, N, nC, nO, nV, nR, nS, ERI, eHF,
                    raise_on_fail=False)
        for k in ("eGW", "SigC", "Z", "EcRPA", "EcGM", "Conv", "nSCF"):
            res["evgw_d%d_%s" % (nd, k)] = np.asarray(v[k])
    v = O.evRGW(64, 1e-5, 5, True, 0.0, False, N, N, nC, nO, nV, nR, nS, ERI, eHF,
                raise_on_fail=False)
    for k in ("eGW", "EcRPA", "nSCF"):
        res["evgwlin_" + k] = np.asarray(v[k])
    return res


def main():
    he = he_system()
    res = run_all(2, 1, 0, 0, he["ERI_MO"], he["eHF"])
    np.savez_compressed(os.path.join(OUT, "he631g.npz"), ERI_MO=he["ERI_MO"], ERI_AO=he["ERI_AO"],
                        c=he["c"], eHF=he["eHF"], ERHF=he["ERHF"],
                        golden_keys=np.array(list(GOLDEN.keys())),
                        golden_vals=np.array(list(GOLDEN.values())), **res)
    for name, (N, nO, naux, seed, nC, nR) in SYNTH.items():
        s = synth.small_system(N, nO, naux, seed)
        ERI = synth.eri_phys_numpy(s["L"])
        res = run_all(N, nO, nC, nR, ERI, s["eHF"])
        np.savez_compressed(os.path.join(OUT, name + ".npz"), L=s["L"], eHF=s["eHF"], N=N, nO=nO,
                            nC=nC, nR=nR, naux=naux, seed=seed, **res)
        print(name, "G0W0 HOMO/LUMO", O.homo_lumo(res["g0w0_eGW"], nO),
              "iters", res["g0w0_qp_iters"].tolist())


if __name__ == "__main__":
    main()
