"""GPU tests of the static phBSE@GW excitation energies (GW/RGW_phBSE.f90) against the oracle:
singlet and triplet manifolds, full and Tamm-Dancoff BSE, full and TDA screening, a frozen core
and frozen virtual, and a finite broadening of the static kernels; plus the TDA Casida solve of
the stage-level drop-in (LR/phRLR.f90 with TDA)."""
import numpy as np
import pytest

from oracle import qkgw_oracle as O
from quack_gb300 import api, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,nO,nC,nR,naux,seed,TDA_W,TDA,eta",
                         [(24, 4, 0, 0, 48, 41, False, False, 0.0),
                          (24, 4, 0, 0, 48, 42, False, True, 0.0),
                          (30, 5, 1, 1, 60, 43, True, False, 0.05),
                          (28, 4, 0, 0, 56, 44, True, True, 0.0)])
def test_phbse_matches_oracle(ctx, N, nO, nC, nR, naux, seed, TDA_W, TDA, eta):
    s = synth.small_system(N, nO, naux, seed)
    E = synth.eri_phys_numpy(s["L"])
    nS = (nO - nC) * (N - nO - nR)
    rng = np.random.default_rng(seed)
    eGW = s["eHF"] + 0.02 * rng.standard_normal(N)
    ref = O.RGW_phBSE(TDA_W, TDA, True, True, False, eta, N, nC, nO, N - nO, nR, nS, E, s["eHF"],
                      eGW)
    r = api.RGW_phBSE(api.BSEOptions(TDA_W=TDA_W, TDA=TDA, eta=eta), N, N, nC, nO, N - nO, nR, nS,
                      E, s["eHF"], eGW, ctx=ctx)
    for key in ("Om_singlet", "Om_triplet"):
        assert np.max(np.abs(r[key] - ref[key])) < 1e-8, key
    for k in range(2):
        assert abs(r["EcBSE"][k] - ref["EcBSE"][k]) < 1e-8 * max(1.0, abs(ref["EcBSE"][k]))


def test_phbse_exchange_kernel_and_single_manifold(ctx):
    N, nO, naux, seed = 24, 4, 48, 45
    s = synth.small_system(N, nO, naux, seed)
    E = synth.eri_phys_numpy(s["L"])
    nS = nO * (N - nO)
    eGW = s["eHF"].copy()
    ref = O.RGW_phBSE(False, False, True, False, True, 0.0, N, 0, nO, N - nO, 0, nS, E, s["eHF"], eGW)
    r = api.RGW_phBSE(api.BSEOptions(triplet=False, exchange_kernel=True), N, N, 0, nO, N - nO, 0,
                      nS, E, s["eHF"], eGW, ctx=ctx)
    assert r["Om_triplet"] is None and r["EcBSE"][1] == 0.0
    assert np.max(np.abs(r["Om_singlet"] - ref["Om_singlet"])) < 1e-8
    assert abs(r["EcBSE"][0] - ref["EcBSE"][0]) < 1e-8 * max(1.0, abs(ref["EcBSE"][0]))


@pytest.mark.parametrize("ispin", [1, 2])
def test_phrlr_tda_matches_oracle(ctx, ispin):
    """CIS-like TDA solve of a non-dRPA A block through the stage-level drop-ins."""
    N, nO, naux, seed = 20, 3, 40, 46
    s = synth.small_system(N, nO, naux, seed)
    E = synth.eri_phys_numpy(s["L"])
    nS = nO * (N - nO)
    A = api.phRLR_A(ispin, False, N, 0, nO, N - nO, 0, nS, 1.0, s["eHF"], E, ctx=ctx)
    Aref = O.phRLR_A(ispin, False, N, 0, nO, N - nO, 0, nS, 1.0, s["eHF"], E)
    assert np.max(np.abs(A - Aref)) < 1e-13
    Ec, Om, XpY, XmY = api.phRLR(True, nS, A, np.zeros((nS, nS)), ctx=ctx)
    Ec0, Om0, XpY0, _ = O.phRLR(True, nS, Aref, np.zeros((nS, nS)))
    assert np.max(np.abs(Om - Om0)) < 1e-10
    assert abs(Ec - Ec0) < 1e-9
    # eigenvectors as rows, up to sign
    ov = np.abs(np.sum(XpY * XpY0, axis=1))
    assert np.all(np.abs(ov - 1.0) < 1e-8)
    assert np.array_equal(XpY, XmY)


@pytest.mark.parametrize("TDA_W,TDA,xk,doXBS,eta", [(False, False, False, False, 0.0),
                                                    (False, True, True, False, 0.0),
                                                    (True, False, True, False, 0.05),
                                                    (False, False, False, True, 0.0)])
def test_phacfdt_matches_oracle(ctx, TDA_W, TDA, xk, doXBS, eta):
    """Adiabatic-connection correlation energy of phBSE@GW (GW/RGW_phACFDT.f90): singlet and
    triplet, full and Tamm-Dancoff BSE, TDA screening, the exchange kernel and the scaled
    screening (doXBS), against the oracle's 21-node quadrature."""
    N, nO, nC, nR, naux, seed = 16, 3, 0, 0, 32, 47
    s = synth.small_system(N, nO, naux, seed)
    E = synth.eri_phys_numpy(s["L"])
    nS = (nO - nC) * (N - nO - nR)
    rng = np.random.default_rng(seed)
    eGW = s["eHF"] + 0.02 * rng.standard_normal(N)
    ref = O.RGW_phACFDT(xk, doXBS, TDA_W, TDA, True, True, eta, N, nC, nO, N - nO, nR, nS, E,
                        s["eHF"], eGW)
    got = api.RGW_phACFDT(api.BSEOptions(TDA_W=TDA_W, TDA=TDA, exchange_kernel=xk, eta=eta),
                          doXBS, N, N, nC, nO, N - nO, nR, nS, E, s["eHF"], eGW, ctx=ctx)
    for k in range(2):
        assert abs(got[k] - ref[k]) < 1e-8 * max(1.0, abs(ref[k])), (k, got, ref)
