"""GPU parity tests: every stage and driver of libqkgw.so (through the C ABI) against the CPU
oracle on the same seeded inputs, plus the committed golden fixtures.

Tolerances (FP64 plain form): quasiparticle energies and Casida excitation energies within
1e-8 Ha of the oracle (the bar of the FP64 path); stage outputs that involve no eigensolve are
compared at 1e-12 relative; eigenvectors are compared up to sign (rows of XpY), since LAPACK
and the GPU solver may pick either sign.
"""
import os

import numpy as np
import pytest

from oracle import qkgw_oracle as O
from oracle.he631g import GOLDEN, he_system
from quack_gb300 import api, synth

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
E_TOL = 1e-8


def _sys(N, nO, naux, seed):
    s = synth.small_system(N, nO, naux, seed)
    return s, synth.eri_phys_numpy(s["L"])


def _align_rows(X, R):
    sg = np.sign(np.sum(X * R, axis=1))
    sg[sg == 0] = 1.0
    return X * sg[:, None]


# --------------------------------------------------------------------------------------------
# eigensolver
# --------------------------------------------------------------------------------------------
@pytest.mark.parametrize("n", [1, 2, 3, 5, 17, 64, 130, 257, 700])
def test_dsyev_random(ctx, n):
    import torch
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    A = A + A.T
    w_ref, V_ref = np.linalg.eigh(A)
    dA = torch.from_numpy(np.asfortranarray(A).ravel(order="F")).cuda()
    dw = torch.empty(n, dtype=torch.float64, device="cuda")
    dZ = torch.empty(n * n, dtype=torch.float64, device="cuda")
    api.dsyev_dev(n, dA.data_ptr(), n, dw.data_ptr(), dZ.data_ptr(), True, ctx=ctx)
    torch.cuda.synchronize()
    w = dw.cpu().numpy()
    Zt = dZ.cpu().numpy().reshape((n, n), order="F")   # rows = eigenvectors
    nrm = np.abs(w_ref).max()
    assert np.max(np.abs(w - w_ref)) < 1e-12 * nrm * max(1, np.sqrt(n))
    res = A @ Zt.T - Zt.T * w[None, :]
    assert np.max(np.abs(res)) < 1e-11 * nrm
    assert np.max(np.abs(Zt @ Zt.T - np.eye(n))) < 1e-10


def test_dsyev_degenerate_clusters(ctx):
    """Exactly repeated eigenvalues (block copies) exercise the cluster Gram-Schmidt."""
    import torch
    rng = np.random.default_rng(7)
    k = 40
    B = rng.standard_normal((k, k))
    B = B + B.T
    Q, _ = np.linalg.qr(rng.standard_normal((3 * k, 3 * k)))
    A = Q @ np.kron(np.eye(3), B) @ Q.T
    A = 0.5 * (A + A.T)
    n = 3 * k
    w_ref = np.linalg.eigvalsh(A)
    dA = torch.from_numpy(np.asfortranarray(A).ravel(order="F")).cuda()
    dw = torch.empty(n, dtype=torch.float64, device="cuda")
    dZ = torch.empty(n * n, dtype=torch.float64, device="cuda")
    api.dsyev_dev(n, dA.data_ptr(), n, dw.data_ptr(), dZ.data_ptr(), True, ctx=ctx)
    w = dw.cpu().numpy()
    Zt = dZ.cpu().numpy().reshape((n, n), order="F")
    assert np.max(np.abs(w - w_ref)) < 1e-11
    assert np.max(np.abs(Zt @ Zt.T - np.eye(n))) < 1e-9
    assert np.max(np.abs(A @ Zt.T - Zt.T * w[None, :])) < 1e-10


def test_dsyev_values_only(ctx):
    import torch
    rng = np.random.default_rng(3)
    n = 333
    A = rng.standard_normal((n, n))
    A = A @ A.T
    dA = torch.from_numpy(np.asfortranarray(A).ravel(order="F")).cuda()
    dw = torch.empty(n, dtype=torch.float64, device="cuda")
    api.dsyev_dev(n, dA.data_ptr(), n, dw.data_ptr(), 0, False, ctx=ctx)
    w_ref = np.linalg.eigvalsh(A)
    assert np.max(np.abs(dw.cpu().numpy() - w_ref)) < 1e-12 * w_ref.max()


# --------------------------------------------------------------------------------------------
# stages
# --------------------------------------------------------------------------------------------
@pytest.mark.parametrize("ispin,dRPA", [(1, True), (1, False), (2, True), (2, False)])
def test_phRLR_A_B(ctx, ispin, dRPA):
    s, E = _sys(11, 3, 33, 1)
    N, nO, nC, nR = 11, 3, 0, 1
    nS = (nO - nC) * (N - nO - nR)
    A = api.phRLR_A(ispin, dRPA, N, nC, nO, N - nO, nR, nS, 0.7, s["eHF"], E, ctx=ctx)
    B = api.phRLR_B(ispin, dRPA, N, nC, nO, N - nO, nR, nS, 0.7, E, ctx=ctx)
    Ar = O.phRLR_A(ispin, dRPA, N, nC, nO, N - nO, nR, nS, 0.7, s["eHF"], E)
    Br = O.phRLR_B(ispin, dRPA, N, nC, nO, N - nO, nR, nS, 0.7, E)
    if dRPA:
        assert np.array_equal(A, Ar) and np.array_equal(B, Br)   # same arithmetic, bit-exact
    else:
        assert np.allclose(A, Ar, rtol=1e-14, atol=1e-15)
        assert np.allclose(B, Br, rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize("dRPA", [True, False])
def test_phRLR(ctx, dRPA):
    s, E = _sys(14, 4, 42, 2)
    N, nO = 14, 4
    nS = nO * (N - nO)
    Ar = O.phRLR_A(1, dRPA, N, 0, nO, N - nO, 0, nS, 1.0, s["eHF"], E)
    Br = O.phRLR_B(1, dRPA, N, 0, nO, N - nO, 0, nS, 1.0, E)
    Ec, Om, XpY, XmY = api.phRLR(False, nS, Ar, Br, ctx=ctx)
    Ecr, Omr, XpYr, XmYr = O.phRLR(False, nS, Ar, Br)
    assert abs(Ec - Ecr) < E_TOL
    assert np.max(np.abs(Om - Omr)) < 1e-10
    assert np.allclose(_align_rows(XpY, XpYr), XpYr, atol=1e-8)
    assert np.allclose(_align_rows(XmY, XmYr), XmYr, atol=1e-8)


def test_excitation_density(ctx):
    s, E = _sys(13, 3, 39, 3)
    N, nO, nC, nR = 13, 3, 1, 0
    nS = (nO - nC) * (N - nO - nR)
    X = np.random.default_rng(0).standard_normal((nS, nS))
    rho = api.RGW_excitation_density(N, nC, nO, nR, nS, E, X, ctx=ctx)
    ref = O.RGW_excitation_density(N, nC, nO, nR, nS, E, X)
    assert np.allclose(rho, ref, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("eta,srg", [(0.0, False), (0.1, False), (0.0, True)])
def test_self_energy_diag(ctx, eta, srg):
    s, E = _sys(12, 3, 36, 4)
    N, nO, nC, nR = 12, 3, 0, 1
    nS = (nO - nC) * (N - nO - nR)
    A = O.phRLR_A(1, True, N, nC, nO, N - nO, nR, nS, 1.0, s["eHF"], E)
    B = O.phRLR_B(1, True, N, nC, nO, N - nO, nR, nS, 1.0, E)
    _, Om, XpY, _ = O.phRLR(False, nS, A, B)
    rho = O.RGW_excitation_density(N, nC, nO, nR, nS, E, XpY)
    if srg:
        gm, Sig, Z = api.RGW_SRG_self_energy_diag(500.0, N, N, nC, nO, N - nO, nR, nS, s["eHF"], Om,
                                                  rho, ctx=ctx)
        gmr, Sigr, Zr = O.RGW_SRG_self_energy_diag(500.0, N, N, nC, nO, N - nO, nR, nS, s["eHF"], Om, rho)
    else:
        gm, Sig, Z = api.RGW_self_energy_diag(eta, N, N, nC, nO, N - nO, nR, nS, s["eHF"], Om, rho,
                                              ctx=ctx)
        gmr, Sigr, Zr = O.RGW_self_energy_diag(eta, N, N, nC, nO, N - nO, nR, nS, s["eHF"], Om, rho)
    assert np.allclose(Sig, Sigr, rtol=1e-11, atol=1e-13)
    assert np.allclose(Z, Zr, rtol=1e-11, atol=1e-13)
    assert abs(gm - gmr) < 1e-11


@pytest.mark.parametrize("srg", [False, True])
def test_qp_graph(ctx, srg):
    s, E = _sys(12, 3, 36, 5)
    N, nO, nC, nR = 12, 3, 0, 0
    nS = nO * (N - nO)
    A = O.phRLR_A(1, True, N, nC, nO, N - nO, nR, nS, 1.0, s["eHF"], E)
    B = O.phRLR_B(1, True, N, nC, nO, N - nO, nR, nS, 1.0, E)
    _, Om, XpY, _ = O.phRLR(False, nS, A, B)
    rho = O.RGW_excitation_density(N, nC, nO, nR, nS, E, XpY)
    if srg:
        _, Sig, Z = O.RGW_SRG_self_energy_diag(500.0, N, N, nC, nO, N - nO, nR, nS, s["eHF"], Om, rho)
    else:
        _, Sig, Z = O.RGW_self_energy_diag(0.0, N, N, nC, nO, N - nO, nR, nS, s["eHF"], Om, rho)
    lin = s["eHF"] + Z * Sig
    eGW, Zn = api.RGW_QP_graph(srg, 0.0, 500.0, N, nC, nO, N - nO, nR, nS, s["eHF"], Om, rho, lin,
                               s["eHF"], Z, ctx=ctx)
    eR, ZR = O.RGW_QP_graph(srg, 0.0, 500.0, N, nC, nO, N - nO, nR, nS, s["eHF"], Om, rho, lin,
                            s["eHF"], Z)
    assert np.max(np.abs(eGW - eR)) < 1e-10
    assert np.max(np.abs(Zn - ZR)) < 1e-9


def test_aotomo(ctx):
    rng = np.random.default_rng(9)
    nB, nOrb = 9, 7
    ERI = rng.standard_normal((nB,) * 4)
    c = rng.standard_normal((nB, nOrb))
    out = api.AOtoMO_ERI_RHF(nB, nOrb, c, ERI, ctx=ctx)
    ref = O.AOtoMO_ERI_RHF(nB, nOrb, c, ERI)
    assert np.allclose(out, ref, rtol=1e-12, atol=1e-11)


def test_aotomo_mixed_stage_precision(ctx):
    """The mixed tier's quarter transforms run in double-float (FP32 pairs, exact products):
    ~1e-13 of sum |a b| even with coefficients that cancel (x30 here)."""
    rng = np.random.default_rng(19)
    nB, nOrb = 24, 20
    ERI = rng.standard_normal((nB,) * 4)
    c = 30.0 * rng.standard_normal((nB, nOrb))
    ref = O.AOtoMO_ERI_RHF(nB, nOrb, c, ERI)
    bound = np.einsum("pqrs,pi,qj,rk,sl->ijkl", np.abs(ERI), np.abs(c), np.abs(c), np.abs(c),
                      np.abs(c), optimize=True)
    ctx.set_stage_precision(api.QK_PREC_BF16X3)
    try:
        out = api.AOtoMO_ERI_RHF(nB, nOrb, c, ERI, ctx=ctx)
    finally:
        ctx.set_stage_precision(api.QK_PREC_FP64)
    assert np.max(np.abs(out - ref) / bound) < 1e-12


def test_diis(ctx):
    rng = np.random.default_rng(4)
    n, md = 10, 4
    err = np.zeros((n, md), order="F")
    ee = np.zeros((n, md), order="F")
    err_r, ee_r = err.copy(), ee.copy()
    for nd in range(1, 6):
        r, e = rng.standard_normal(n), rng.standard_normal(n)
        k = min(nd, md)
        rc, out = api.DIIS_extrapolation(n, n, k, err, ee, r, e, ctx=ctx)
        rcr, err_r, ee_r, outr = O.DIIS_extrapolation(k, err_r, ee_r, r, e)
        assert np.allclose(out, outr, rtol=1e-10, atol=1e-12)
        assert np.allclose(err, err_r) and np.allclose(ee, ee_r)


# --------------------------------------------------------------------------------------------
# drivers
# --------------------------------------------------------------------------------------------
def test_he_g0w0_featherbench(ctx):
    he = he_system()
    r = api.RG0W0(api.GWOptions(), 2, 2, 0, 1, 1, 0, 1, he["ERI_MO"], he["eHF"], ctx=ctx)
    assert abs(r["EcRPA"] - GOLDEN["G0W0 correlation energy"]) < 1e-9
    assert abs(r["eGW"][0] - GOLDEN["G0W0 HOMO energy"]) < 1e-9
    assert abs(r["eGW"][1] - GOLDEN["G0W0 LUMO energy"]) < 1e-9


def test_he_evgw_featherbench(ctx):
    he = he_system()
    opt = api.GWOptions(maxSCF=256, thresh=1e-5, max_diis=1)
    r = api.evRGW(opt, 2, 2, 0, 1, 1, 0, 1, he["ERI_MO"], he["eHF"], ctx=ctx)
    assert abs(r["EcRPA"] - GOLDEN["evGW correlation energy"]) < 1e-9
    assert abs(r["eGW"][0] - GOLDEN["evGW HOMO energy"]) < 1e-9
    assert abs(r["eGW"][1] - GOLDEN["evGW LUMO energy"]) < 1e-9


@pytest.mark.parametrize("name", ["synth_n24", "synth_n13_frozen"])
def test_g0w0_fixtures(ctx, name):
    f = np.load(os.path.join(GOLD, name + ".npz"))
    N, nO, nC, nR = int(f["N"]), int(f["nO"]), int(f["nC"]), int(f["nR"])
    E = synth.eri_phys_numpy(f["L"])
    nS = (nO - nC) * (N - nO - nR)
    for tag, opt in (("g0w0", api.GWOptions()), ("g0w0lin", api.GWOptions(linearize=True)),
                     ("g0w0srg", api.GWOptions(reg=True, eta=0.05))):
        r = api.RG0W0(opt, N, N, nC, nO, N - nO, nR, nS, E, f["eHF"], ctx=ctx)
        act = slice(nC, N - nR)
        assert np.max(np.abs(r["eGW"][act] - f[tag + "_eGW"][act])) < E_TOL, tag
        assert np.max(np.abs(r["SigC"] - f[tag + "_SigC"])) < E_TOL, tag
        assert np.max(np.abs(r["Z"][act] - f[tag + "_Z"][act])) < 1e-7, tag
        assert abs(r["EcRPA"] - float(f[tag + "_EcRPA"])) < E_TOL, tag
        assert abs(r["EcGM"] - float(f[tag + "_EcGM"])) < E_TOL, tag
        if tag == "g0w0":
            assert np.max(np.abs(r["Om"] - f["g0w0_Om"])) < E_TOL


@pytest.mark.parametrize("name", ["synth_n24", "synth_n13_frozen"])
def test_evgw_fixtures(ctx, name):
    f = np.load(os.path.join(GOLD, name + ".npz"))
    N, nO, nC, nR = int(f["N"]), int(f["nO"]), int(f["nC"]), int(f["nR"])
    E = synth.eri_phys_numpy(f["L"])
    nS = (nO - nC) * (N - nO - nR)
    act = slice(nC, N - nR)
    for nd in (1, 5):
        r = api.evRGW(api.GWOptions(maxSCF=64, thresh=1e-5, max_diis=nd), N, N, nC, nO, N - nO, nR,
                      nS, E, f["eHF"], ctx=ctx)
        assert r["nSCF"] == int(f["evgw_d%d_nSCF" % nd])
        assert np.max(np.abs(r["eGW"][act] - f["evgw_d%d_eGW" % nd][act])) < E_TOL
        assert abs(r["EcRPA"] - float(f["evgw_d%d_EcRPA" % nd])) < E_TOL
    r = api.evRGW(api.GWOptions(maxSCF=64, thresh=1e-5, max_diis=5, linearize=True), N, N, nC, nO,
                  N - nO, nR, nS, E, f["eHF"], ctx=ctx)
    assert r["nSCF"] == int(f["evgwlin_nSCF"])
    assert np.max(np.abs(r["eGW"][act] - f["evgwlin_eGW"][act])) < E_TOL


def test_evgw_maxscf_failure_reported(ctx):
    """maxSCF exhausted -> QK_ERR_NO_CONV (the reference stops, evRGW.f90:190-198)."""
    f = np.load(os.path.join(GOLD, "synth_n24.npz"))
    E = synth.eri_phys_numpy(f["L"])
    with pytest.raises(api.QkError) as ei:
        api.evRGW(api.GWOptions(maxSCF=0, thresh=1e-12, max_diis=1), 24, 24, 0, 5, 19, 0, 95, E,
                  f["eHF"], ctx=ctx)
    assert ei.value.code == api.QK_ERR_NO_CONV


def test_bad_arguments_rejected(ctx):
    f = np.load(os.path.join(GOLD, "synth_n24.npz"))
    E = synth.eri_phys_numpy(f["L"])
    with pytest.raises(api.QkError) as ei:
        api.RG0W0(api.GWOptions(), 24, 24, 0, 5, 19, 0, 96, E, f["eHF"], ctx=ctx)
    assert ei.value.code == api.QK_ERR_ARG


@pytest.mark.parametrize("lin", [True, False])
def test_g0w0_tda_screening_matches_oracle(ctx, lin):
    """TDA_W: the screening Casida in the Tamm-Dancoff form (Om = eig(A), XpY = eigenvectors),
    RG0W0.f90:116-119,222-225; ERI driver and factorised driver."""
    import torch
    f = np.load(os.path.join(GOLD, "synth_n24.npz"))
    N, nO = 24, 5
    nS = nO * (N - nO)
    E = synth.eri_phys_numpy(f["L"])
    ref = O.RG0W0(lin, 0.0, False, N, N, 0, nO, N - nO, 0, nS, E, f["eHF"], TDA_W=True)
    r = api.RG0W0(api.GWOptions(TDA_W=True, linearize=lin), N, N, 0, nO, N - nO, 0, nS, E,
                  f["eHF"], ctx=ctx)
    assert np.max(np.abs(r["Om"] - ref["Om"])) < 1e-10
    assert abs(r["EcRPA"] - ref["EcRPA"]) < 1e-9
    assert abs(r["EcGM"] - ref["EcGM"]) < 1e-9 * max(1.0, abs(ref["EcGM"]))
    ok = np.ones(N, bool) if lin else (ref["qp_iters"] <= 10)
    assert np.max(np.abs(r["eGW"][ok] - ref["eGW"][ok])) < 1e-8
    naux = f["L"].shape[0]
    dL = torch.from_numpy(api.L_fortran_flat(f["L"])).cuda()
    de = torch.from_numpy(f["eHF"]).cuda()
    out = [torch.empty(N, dtype=torch.float64, device="cuda") for _ in range(3)]
    dOm = torch.empty(nS, dtype=torch.float64, device="cuda")
    ec, gm = api.RG0W0_L_dev(api.GWOptions(TDA_W=True, linearize=lin), N, 0, nO, 0, naux,
                             dL.data_ptr(), de.data_ptr(), out[0].data_ptr(), out[1].data_ptr(),
                             out[2].data_ptr(), dOm.data_ptr(), ctx=ctx)
    assert np.max(np.abs(dOm.cpu().numpy() - ref["Om"])) < 1e-10
    assert np.max(np.abs(out[0].cpu().numpy()[ok] - ref["eGW"][ok])) < 1e-8


def test_evgw_tda_screening_matches_oracle_and_graph(ctx):
    f = np.load(os.path.join(GOLD, "synth_n24.npz"))
    N, nO = 24, 5
    nS = nO * (N - nO)
    E = synth.eri_phys_numpy(f["L"])
    ref = O.evRGW(5, 1e-5, 5, True, 0.0, False, N, N, 0, nO, N - nO, 0, nS, E, f["eHF"],
                  TDA_W=True, raise_on_fail=False)
    opts = api.GWOptions(TDA_W=True, linearize=True, maxSCF=5, thresh=1e-5, max_diis=5)
    r = api.evRGW(opts, N, N, 0, nO, N - nO, 0, nS, E, f["eHF"], ctx=ctx, raise_on_fail=False)
    assert r["nSCF"] == ref["nSCF"]
    assert np.max(np.abs(r["eGW"] - ref["eGW"])) < 1e-8
    assert abs(r["EcRPA"] - ref["EcRPA"]) < 1e-9
    ctx.set_graph_mode(True)
    try:
        g = api.evRGW(opts, N, N, 0, nO, N - nO, 0, nS, E, f["eHF"], ctx=ctx, raise_on_fail=False)
    finally:
        ctx.set_graph_mode(False)
    assert g["nSCF"] == r["nSCF"]
    assert np.max(np.abs(g["eGW"] - r["eGW"])) < 1e-12


def newton_stable_mask(N, nO, nS, eHF, Om, rho, eGWlin, Z, iters):
    """Orbitals whose oracle Newton root is reproducible: at most 10 Newton steps and no change
    above 1e-10 Ha under three random elementwise 1e-13 perturbations of rho.

    With eta = 0 the QP equation has a pole at every e_q +/- Om_m; on strongly coupled synthetic
    systems Newton can wander for tens of steps and then land on a root that moves with
    perturbations at the 1e-14 level (the reference's own result is not reproducible across BLAS
    builds there).  Such orbitals are checked as roots of the QP equation instead."""
    base = O.RGW_QP_graph(False, 0.0, 500.0, N, 0, nO, N - nO, 0, nS, eHF, Om, rho, eGWlin, eHF, Z)[0]
    ok = np.asarray(iters) <= 10
    rng = np.random.default_rng(0)
    for _ in range(3):
        f = 1.0 + 1e-13 * rng.standard_normal(rho.shape)
        e = O.RGW_QP_graph(False, 0.0, 500.0, N, 0, nO, N - nO, 0, nS, eHF, Om, rho * f, eGWlin,
                           eHF, Z)[0]
        ok &= np.abs(e - base) < 1e-10
    return ok


@pytest.mark.parametrize("N,nO,seed", [(40, 5, 21), (57, 7, 22), (96, 12, 23)])
def test_g0w0_vs_live_oracle(ctx, N, nO, seed):
    """Strongly coupled synthetic systems: |Sigma| reaches several Ha, so Sigma-dependent
    quantities are compared at 1e-8 relative to max(1, |value|); Casida energies at 1e-8 Ha."""
    s, E = _sys(N, nO, 3 * N, seed)
    nS = nO * (N - nO)
    r = api.RG0W0(api.GWOptions(), N, N, 0, nO, N - nO, 0, nS, E, s["eHF"], ctx=ctx)
    ref = O.RG0W0(False, 0.0, False, N, N, 0, nO, N - nO, 0, nS, E, s["eHF"])
    scale = np.maximum(1.0, np.abs(ref["SigC"]))
    assert np.max(np.abs(r["Om"] - ref["Om"])) < E_TOL
    assert np.max(np.abs(r["SigC"] - ref["SigC"]) / scale) < E_TOL
    assert abs(r["EcGM"] - ref["EcGM"]) < E_TOL * max(1.0, abs(ref["EcGM"]))
    Z0 = O.RGW_self_energy_diag(0.0, N, N, 0, nO, N - nO, 0, nS, s["eHF"], ref["Om"], ref["rho"])[2]
    stable = newton_stable_mask(N, nO, nS, s["eHF"], ref["Om"], ref["rho"], ref["eGWlin"], Z0,
                                ref["qp_iters"])
    assert stable.sum() >= N // 3
    assert np.max(np.abs(r["eGW"][stable] - ref["eGW"][stable]) / scale[stable]) < E_TOL
    # other orbitals: the GPU answer is a root of the oracle's QP equation (or the linearised
    # fallback after 64 steps, as in the reference)
    for p in np.where(~stable)[0]:
        w = r["eGW"][p]
        f = w - s["eHF"][p] - O.RGW_Re_SigC(p, w, 0.0, N, 0, nO, N - nO, 0, nS, s["eHF"], ref["Om"],
                                            ref["rho"])
        assert abs(f) < 1e-5 or abs(w - ref["eGWlin"][p]) < E_TOL * scale[p], (p, f)


@pytest.mark.parametrize("N,nO,seed", [(40, 5, 21), (64, 8, 24)])
def test_g0w0_linearized_vs_live_oracle(ctx, N, nO, seed):
    s, E = _sys(N, nO, 3 * N, seed)
    nS = nO * (N - nO)
    r = api.RG0W0(api.GWOptions(linearize=True), N, N, 0, nO, N - nO, 0, nS, E, s["eHF"], ctx=ctx)
    ref = O.RG0W0(True, 0.0, False, N, N, 0, nO, N - nO, 0, nS, E, s["eHF"])
    assert np.max(np.abs(r["eGW"] - ref["eGW"])) < E_TOL
    assert np.max(np.abs(r["Z"] - ref["Z"])) < 1e-7
    if np.isfinite(ref["EcRPA"]):
        assert abs(r["EcRPA"] - ref["EcRPA"]) < E_TOL


# --------------------------------------------------------------------------------------------
# factorised-integral drivers (slab and Casida coupling built on the device from L)
# --------------------------------------------------------------------------------------------
def _dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


@pytest.mark.parametrize("N,nO,seed,lin", [(24, 5, 11, False), (40, 5, 21, True), (33, 4, 25, False)])
def test_g0w0_L_path_vs_oracle(ctx, N, nO, seed, lin):
    import torch
    s = synth.small_system(N, nO, 3 * N, seed)
    E = synth.eri_phys_numpy(s["L"])
    nS = nO * (N - nO)
    ref = O.RG0W0(lin, 0.0, False, N, N, 0, nO, N - nO, 0, nS, E, s["eHF"])
    dL = _dev(api.L_fortran_flat(s["L"]))
    de = _dev(s["eHF"])
    out = [torch.empty(N, dtype=torch.float64, device="cuda") for _ in range(3)]
    dOm = torch.empty(nS, dtype=torch.float64, device="cuda")
    Ec, gm = api.RG0W0_L_dev(api.GWOptions(linearize=lin), N, 0, nO, 0, 3 * N, dL.data_ptr(),
                             de.data_ptr(), out[0].data_ptr(), out[1].data_ptr(),
                             out[2].data_ptr(), dOm.data_ptr(), ctx=ctx)
    eGW = out[0].cpu().numpy()
    scale = np.maximum(1.0, np.abs(ref["SigC"]))
    assert np.max(np.abs(dOm.cpu().numpy() - ref["Om"])) < E_TOL
    assert np.max(np.abs(out[1].cpu().numpy() - ref["SigC"]) / scale) < E_TOL
    if lin:
        assert np.max(np.abs(eGW - ref["eGW"]) / scale) < E_TOL
    else:
        stable = np.asarray(ref["qp_iters"]) <= 4
        assert np.max(np.abs(eGW[stable] - ref["eGW"][stable]) / scale[stable]) < E_TOL
    if np.isfinite(ref["EcRPA"]):
        assert abs(Ec - ref["EcRPA"]) < E_TOL * max(1.0, abs(ref["EcRPA"]))


def test_evgw_L_path_vs_fixture(ctx):
    import torch
    f = np.load(os.path.join(GOLD, "synth_n24.npz"))
    N, nO = int(f["N"]), int(f["nO"])
    dL = _dev(api.L_fortran_flat(f["L"]))
    de = _dev(f["eHF"])
    out = [torch.empty(N, dtype=torch.float64, device="cuda") for _ in range(3)]
    r = api.evRGW_L_dev(api.GWOptions(maxSCF=64, thresh=1e-5, max_diis=5), N, 0, nO, 0, 3 * N,
                        dL.data_ptr(), de.data_ptr(), out[0].data_ptr(), out[1].data_ptr(),
                        out[2].data_ptr(), ctx=ctx)
    assert r["nSCF"] == int(f["evgw_d5_nSCF"])
    assert np.max(np.abs(out[0].cpu().numpy() - f["evgw_d5_eGW"])) < E_TOL
    assert abs(r["EcRPA"] - float(f["evgw_d5_EcRPA"])) < E_TOL


def test_qp_iteration_counts_match_oracle(ctx):
    f = np.load(os.path.join(GOLD, "synth_n24.npz"))
    N, nO = int(f["N"]), int(f["nO"])
    E = synth.eri_phys_numpy(f["L"])
    api.RG0W0(api.GWOptions(), N, N, 0, nO, N - nO, 0, nO * (N - nO), E, f["eHF"], ctx=ctx)
    assert np.array_equal(ctx.qp_iters(N), f["g0w0_qp_iters"])


# --------------------------------------------------------------------------------------------
# batched driver: uneven systems on several streams, each checked against the oracle
# --------------------------------------------------------------------------------------------
def _batch_systems():
    rng = np.random.default_rng(99)
    out = []
    for N in (13, 40, 24, 31, 18, 36, 27):
        nO = synth.n_occ(N)
        out.append(synth.gen_system(N, nO, 3 * N, rng))
    return out


@pytest.mark.parametrize("method", [0, 1])
def test_batched_driver_vs_oracle(ctx, method):
    import torch
    systems = _batch_systems()
    desc, Lf, Ef = api.pack_systems(systems)
    dL, dE = _dev(Lf), _dev(Ef)
    dG = torch.zeros_like(dE)
    opt = api.GWOptions(linearize=(method == 0), maxSCF=64, thresh=1e-5, max_diis=5)
    r = api.gw_batch_L_dev(opt, method, desc, dL.data_ptr(), dE.data_ptr(), dG.data_ptr(),
                           n_workers=3, ctx=ctx)
    assert r["rc"] == api.QK_OK, (r["error"], r["status"])
    eG = dG.cpu().numpy()
    for i, s in enumerate(systems):
        N, nO = s["N"], s["nO"]
        nS = nO * (N - nO)
        E = synth.eri_phys_numpy(s["L"])
        if method == 0:
            ref = O.RG0W0(True, 0.0, False, N, N, 0, nO, N - nO, 0, nS, E, s["eHF"])
        else:
            ref = O.evRGW(64, 1e-5, 5, False, 0.0, False, N, N, 0, nO, N - nO, 0, nS, E, s["eHF"],
                          raise_on_fail=False)
        got = eG[desc[i].offset_e:desc[i].offset_e + N]
        assert r["status"][i] == (api.QK_ERR_NO_CONV if ref.get("failed") else api.QK_OK)
        scale = np.maximum(1.0, np.abs(ref["SigC"]))
        assert np.max(np.abs(got - ref["eGW"]) / scale) < 1e-7, i
        if method == 1:
            assert r["nSCF"][i] == ref["nSCF"]
    # the tridiagonalisations ran as grouped launches, several matrices per launch
    launches, matrices = ctx.batch_group_stats()
    assert launches > 0 and matrices > launches


def test_batched_driver_isolates_bad_system(ctx):
    import torch
    systems = _batch_systems()[:3]
    desc, Lf, Ef = api.pack_systems(systems)
    desc[1].nO = desc[1].nOrb  # no virtual orbitals: invalid
    dL, dE = _dev(Lf), _dev(Ef)
    dG = torch.zeros_like(dE)
    r = api.gw_batch_L_dev(api.GWOptions(linearize=True), 0, desc, dL.data_ptr(), dE.data_ptr(),
                           dG.data_ptr(), n_workers=2, ctx=ctx)
    assert r["status"][1] == api.QK_ERR_ARG
    assert r["status"][0] == api.QK_OK and r["status"][2] == api.QK_OK


# --------------------------------------------------------------------------------------------
# evGW cycles replayed from a CUDA graph (device-side WHILE loop) == eager cycles
# --------------------------------------------------------------------------------------------
@pytest.mark.parametrize("lin,nd", [(False, 5), (True, 5), (False, 1)])
def test_evgw_graph_mode_matches_fixture(ctx, lin, nd):
    import torch
    f = np.load(os.path.join(GOLD, "synth_n24.npz"))
    N, nO = int(f["N"]), int(f["nO"])
    E = synth.eri_phys_numpy(f["L"])
    opt = api.GWOptions(maxSCF=64, thresh=1e-5, max_diis=nd, linearize=lin)
    key = "evgwlin" if lin else "evgw_d%d" % nd
    ctx.set_graph_mode(True)
    try:
        for _ in range(2):  # second call reuses the cached graph
            r = api.evRGW(opt, N, N, 0, nO, N - nO, 0, nO * (N - nO), E, f["eHF"], ctx=ctx)
            assert r["nSCF"] == int(f[key + "_nSCF"])
            assert np.max(np.abs(r["eGW"] - f[key + "_eGW"])) < E_TOL
        dL = _dev(api.L_fortran_flat(f["L"]))
        de = _dev(f["eHF"])
        out = [torch.empty(N, dtype=torch.float64, device="cuda") for _ in range(3)]
        r = api.evRGW_L_dev(opt, N, 0, nO, 0, 3 * N, dL.data_ptr(), de.data_ptr(),
                            out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), ctx=ctx)
        assert r["nSCF"] == int(f[key + "_nSCF"])
        assert np.max(np.abs(out[0].cpu().numpy() - f[key + "_eGW"])) < E_TOL
    finally:
        ctx.set_graph_mode(False)


# --------------------------------------------------------------------------------------------
# autotuner: picks from its candidate sets, persists as JSON, and does not change results
# --------------------------------------------------------------------------------------------
def test_autotuner_roundtrip_and_parity(ctx, tmp_path):
    f = np.load(os.path.join(GOLD, "synth_n24.npz"))
    N, nO = int(f["N"]), int(f["nO"])
    nS = nO * (N - nO)
    E = synth.eri_phys_numpy(f["L"])
    ctx.autotune(N, nS)
    assert ctx.tune_query("bf16x3_chunk", (nS + 63) // 64 * 64) in (1, 2, 4)
    assert ctx.tune_query("splitk_mult", nS) in (1, 2, 4)
    assert ctx.tune_query("sytrd_grid", nS) in (2, 3, 4)
    assert ctx.tune_query("dgemm_path", nS * nS) in (1, 2)
    assert ctx.tune_query("stebz_k", nS) in (2, 4, 8)
    path = tmp_path / "tune.json"
    ctx.tune_save(path)
    c2 = api.Context(0)
    c2.tune_load(path)
    for name, size in (("bf16x3_chunk", (nS + 63) // 64 * 64), ("splitk_mult", nS),
                       ("sytrd_grid", nS), ("dgemm_path", nS * nS)):
        assert c2.tune_query(name, size) == ctx.tune_query(name, size)
    c2.close()
    r = api.RG0W0(api.GWOptions(), N, N, 0, nO, N - nO, 0, nS, E, f["eHF"], ctx=ctx)
    assert np.max(np.abs(r["eGW"] - f["g0w0_eGW"])) < E_TOL
