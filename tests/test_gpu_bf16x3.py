"""GPU tests of the BF16x3 tensor-core tier (tcgen05): the GEMM against an FP64 reference and the
mixed-precision G0W0 against the FP64 oracle at the 1 meV (3.67e-5 Ha) bar."""
import numpy as np
import pytest

from oracle import qkgw_oracle as O
from quack_gb300 import api, synth

pytestmark = pytest.mark.gpu
MEV = 1e-3 / O.HaToeV


@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (300, 200, 130), (1000, 257, 1000),
                                   (4096, 384, 3600), (1, 1, 1), (129, 1, 65)])
def test_gemm_bf16x3_accuracy(ctx, m, n, k):
    import torch
    rng = np.random.default_rng(m + n + k)
    A = rng.standard_normal((m, k)) * np.exp(rng.uniform(-3, 3, size=(m, 1)))
    B = rng.standard_normal((n, k))
    dA = torch.from_numpy(np.asfortranarray(A).ravel(order="F")).cuda()
    dB = torch.from_numpy(np.asfortranarray(B).ravel(order="F")).cuda()
    dC = torch.zeros(m * n, dtype=torch.float64, device="cuda")
    api.gemm_bf16x3_dev(m, n, k, dA.data_ptr(), m, dB.data_ptr(), n, dC.data_ptr(), m, ctx=ctx)
    C = dC.cpu().numpy().reshape((m, n), order="F")
    ref = A @ B.T
    scale = np.abs(A) @ np.abs(B).T
    ratio = np.max(np.abs(C - ref) / scale)
    # six-term BF16x3 product (2^-24 per term) accumulated in FP32 tensor memory; the tensor
    # core's accumulation error grows with the number of k steps
    assert ratio < 4e-6 * max(1.0, np.sqrt(k / 64.0)), ratio


@pytest.mark.parametrize("path", [1, 2])
def test_dgemm_dev_matches_numpy(ctx, path):
    """Both FP64 GEMM paths (1 = DFMA, 2 = DMMA tensor path), all transposes, ragged sizes and a
    split-K shape (few output tiles, long k)."""
    import torch
    rng = np.random.default_rng(1)
    shapes = (("N", "N", (70, 33, 45)), ("T", "N", (64, 65, 66)), ("N", "T", (129, 17, 3)),
              ("T", "T", (5, 200, 77)), ("N", "N", (300, 128, 2000)))
    old = {m * n: ctx.tune_query("dgemm_path", m * n) for _, _, (m, n, _) in shapes}
    for _, _, (m, n, _) in shapes:
        ctx.tune_set("dgemm_path", m * n, path)
    for ta, tb, (m, n, k) in shapes:
        A = rng.standard_normal((k, m) if ta == "T" else (m, k))
        B = rng.standard_normal((n, k) if tb == "T" else (k, n))
        C0 = rng.standard_normal((m, n))
        dA = torch.from_numpy(np.asfortranarray(A).ravel(order="F")).cuda()
        dB = torch.from_numpy(np.asfortranarray(B).ravel(order="F")).cuda()
        dC = torch.from_numpy(np.asfortranarray(C0).ravel(order="F")).cuda()
        api.dgemm_dev(ta, tb, m, n, k, 0.5, dA.data_ptr(), A.shape[0], dB.data_ptr(), B.shape[0],
                      -1.5, dC.data_ptr(), m, ctx=ctx)
        opA = A.T if ta == "T" else A
        opB = B.T if tb == "T" else B
        ref = 0.5 * opA @ opB - 1.5 * C0
        C = dC.cpu().numpy().reshape((m, n), order="F")
        assert np.allclose(C, ref, rtol=1e-13, atol=1e-12 * max(1.0, np.sqrt(k / 64.0)))
    for key, v in old.items():
        ctx.tune_set("dgemm_path", key, max(v, 0))


@pytest.mark.parametrize("ta,tb,m,n,k", [("T", "N", 4000, 20, 150), ("N", "N", 1000, 25, 77),
                                         ("N", "T", 513, 7, 33), ("T", "T", 1000, 150, 40),
                                         ("N", "N", 200, 20, 5000), ("T", "N", 300, 31, 4097)])
def test_dgemm_tall_tiles(ctx, ta, tb, m, n, k):
    """The DFMA path's 128 x 32 tiles (chosen for outputs with few columns, like the quarter
    transforms of qsGW): every transpose, ragged sizes, split-K (few tiles, long k)."""
    import torch
    rng = np.random.default_rng(m + 5 * n + 11 * k)
    A = rng.standard_normal((k, m) if ta == "T" else (m, k))
    B = rng.standard_normal((n, k) if tb == "T" else (k, n))
    C0 = rng.standard_normal((m, n))
    old = ctx.tune_query("dgemm_path", m * n)
    ctx.tune_set("dgemm_path", m * n, 1)
    dA = torch.from_numpy(np.asfortranarray(A).ravel(order="F")).cuda()
    dB = torch.from_numpy(np.asfortranarray(B).ravel(order="F")).cuda()
    dC = torch.from_numpy(np.asfortranarray(C0).ravel(order="F")).cuda()
    api.dgemm_dev(ta, tb, m, n, k, 0.5, dA.data_ptr(), A.shape[0], dB.data_ptr(), B.shape[0],
                  -1.5, dC.data_ptr(), m, ctx=ctx)
    ctx.tune_set("dgemm_path", m * n, max(old, 0))
    opA = A.T if ta == "T" else A
    opB = B.T if tb == "T" else B
    ref = 0.5 * opA @ opB - 1.5 * C0
    C = dC.cpu().numpy().reshape((m, n), order="F")
    assert np.allclose(C, ref, rtol=1e-13, atol=1e-12 * max(1.0, np.sqrt(k / 64.0)))


@pytest.mark.parametrize("ta,tb,m,n,k", [("N", "N", 70, 33, 45), ("T", "N", 64, 65, 66),
                                         ("N", "T", 129, 17, 3), ("T", "T", 5, 200, 77),
                                         ("N", "N", 300, 128, 3000), ("T", "N", 128, 600, 3600),
                                         ("N", "T", 257, 300, 128)])
def test_gemm_bf16x3_ex_transposes_alpha_beta_splitk(ctx, ta, tb, m, n, k):
    """General BF16x3 GEMM: every transpose, alpha and beta, ragged sizes, and the split-K shapes
    of the back-transformation (few output tiles, long k)."""
    import torch
    rng = np.random.default_rng(m + 3 * n + 7 * k)
    A = rng.standard_normal((k, m) if ta == "T" else (m, k))
    B = rng.standard_normal((n, k) if tb == "T" else (k, n))
    C0 = rng.standard_normal((m, n))
    dA = torch.from_numpy(np.asfortranarray(A).ravel(order="F")).cuda()
    dB = torch.from_numpy(np.asfortranarray(B).ravel(order="F")).cuda()
    dC = torch.from_numpy(np.asfortranarray(C0).ravel(order="F")).cuda()
    api.gemm_bf16x3_ex_dev(ta, tb, m, n, k, -0.75, dA.data_ptr(), A.shape[0], dB.data_ptr(),
                           B.shape[0], 1.25, dC.data_ptr(), m, ctx=ctx)
    opA = A.T if ta == "T" else A
    opB = B.T if tb == "T" else B
    ref = -0.75 * opA @ opB + 1.25 * C0
    scale = 0.75 * np.abs(opA) @ np.abs(opB)
    C = dC.cpu().numpy().reshape((m, n), order="F")
    assert np.all(np.abs(C - ref) <= 4e-6 * max(1.0, np.sqrt(k / 64.0)) * scale
                  + 1e-13 * np.abs(ref)), (ta, tb)


def test_dgemm_f32p_dev_error_bound(ctx):
    """FP32-product GEMM (the mixed tier's back-transformation): every transpose, ragged sizes
    and the split-K shape; the error stays within a few FP32 roundings of sum |a_ik b_kj|."""
    import torch
    rng = np.random.default_rng(2)
    shapes = (("N", "N", (70, 33, 45)), ("T", "N", (64, 65, 66)), ("N", "T", (129, 17, 3)),
              ("T", "T", (5, 200, 77)), ("N", "N", (300, 128, 2000)), ("N", "T", (257, 300, 128)))
    for ta, tb, (m, n, k) in shapes:
        A = rng.standard_normal((k, m) if ta == "T" else (m, k))
        B = rng.standard_normal((n, k) if tb == "T" else (k, n))
        C0 = rng.standard_normal((m, n))
        dA = torch.from_numpy(np.asfortranarray(A).ravel(order="F")).cuda()
        dB = torch.from_numpy(np.asfortranarray(B).ravel(order="F")).cuda()
        dC = torch.from_numpy(np.asfortranarray(C0).ravel(order="F")).cuda()
        api.dgemm_f32p_dev(ta, tb, m, n, k, 0.5, dA.data_ptr(), A.shape[0], dB.data_ptr(),
                           B.shape[0], -1.5, dC.data_ptr(), m, ctx=ctx)
        opA = A.T if ta == "T" else A
        opB = B.T if tb == "T" else B
        ref = 0.5 * opA @ opB - 1.5 * C0
        scale = 0.5 * np.abs(opA) @ np.abs(opB)
        C = dC.cpu().numpy().reshape((m, n), order="F")
        # FP32 rounding of both operands (2^-23 per product) plus the 16-term FP32 tile sums
        assert np.all(np.abs(C - ref) <= 1e-6 * scale + 1e-13 * np.abs(ref)), (ta, tb)


@pytest.mark.parametrize("N,nO,seed", [(40, 5, 21), (64, 8, 24)])
def test_mixed_g0w0_within_1mev(ctx, N, nO, seed):
    s = synth.small_system(N, nO, 3 * N, seed)
    E = synth.eri_phys_numpy(s["L"])
    nS = nO * (N - nO)
    ref = O.RG0W0(True, 0.0, False, N, N, 0, nO, N - nO, 0, nS, E, s["eHF"])
    r = api.RG0W0(api.GWOptions(linearize=True, precision=api.QK_PREC_BF16X3), N, N, 0, nO,
                  N - nO, 0, nS, E, s["eHF"], ctx=ctx)
    err = np.max(np.abs(r["eGW"] - ref["eGW"]))
    assert err < MEV, err
    assert np.max(np.abs(r["Om"] - ref["Om"])) < 1e-8     # the Casida stays FP64


def _stage_inputs(N, nO, seed):
    s = synth.small_system(N, nO, 3 * N, seed)
    E = synth.eri_phys_numpy(s["L"])
    nS = nO * (N - nO)
    A = O.phRLR_A(1, True, N, 0, nO, N - nO, 0, nS, 1.0, s["eHF"], E)
    B = O.phRLR_B(1, True, N, 0, nO, N - nO, 0, nS, 1.0, E)
    _, Om, XpY, _ = O.phRLR(False, nS, A, B)
    rho = O.RGW_excitation_density(N, 0, nO, 0, nS, E, XpY)
    return s, nS, Om, rho


class _StagePrecision:
    def __init__(self, ctx, prec):
        self.ctx, self.prec = ctx, prec

    def __enter__(self):
        self.ctx.set_stage_precision(self.prec)

    def __exit__(self, *exc):
        self.ctx.set_stage_precision(api.QK_PREC_FP64)


@pytest.mark.parametrize("N,nO,seed", [(40, 5, 21), (64, 8, 24)])
def test_mixed_pole_sums_vs_fp64(ctx, N, nO, seed):
    """FP32 far-pole / FP64 near-pole evaluation of Sigma, Z and EcGM with the exact FP64 rho:
    the only error left is the FP32 rounding of the far terms (a few 1e-7 relative per term)."""
    s, nS, Om, rho = _stage_inputs(N, nO, seed)
    gmr, Sigr, Zr = O.RGW_self_energy_diag(0.0, N, N, 0, nO, N - nO, 0, nS, s["eHF"], Om, rho)
    with _StagePrecision(ctx, api.QK_PREC_BF16X3):
        gm, Sig, Z = api.RGW_self_energy_diag(0.0, N, N, 0, nO, N - nO, 0, nS, s["eHF"], Om, rho,
                                              ctx=ctx)
    assert np.max(np.abs(Sig - Sigr) / np.maximum(1.0, np.abs(Sigr))) < 1e-7
    assert np.max(np.abs(Z - Zr) / np.maximum(1.0, np.abs(Zr))) < 1e-6
    assert abs(gm - gmr) < 1e-7 * max(1.0, abs(gmr))


def test_mixed_pole_sums_unsorted_screening_goes_fp64(ctx):
    """Om out of order (here: permuted together with rho's m index, which leaves Sigma unchanged)
    cannot be windowed; every term then takes the FP64 branch and the FP64 bar holds."""
    N, nO = 24, 3
    s, nS, Om, rho = _stage_inputs(N, nO, 31)
    perm = np.random.default_rng(3).permutation(nS)
    gmr, Sigr, Zr = O.RGW_self_energy_diag(0.0, N, N, 0, nO, N - nO, 0, nS, s["eHF"], Om, rho)
    with _StagePrecision(ctx, api.QK_PREC_BF16X3):
        gm, Sig, Z = api.RGW_self_energy_diag(0.0, N, N, 0, nO, N - nO, 0, nS, s["eHF"], Om[perm],
                                              np.ascontiguousarray(rho[:, :, perm]), ctx=ctx)
    assert np.allclose(Sig, Sigr, rtol=1e-11, atol=1e-13)
    assert np.allclose(Z, Zr, rtol=1e-11, atol=1e-13)
    assert abs(gm - gmr) < 1e-11 * max(1.0, abs(gmr))


def test_mixed_qp_graph_vs_fp64(ctx):
    """Newton with the mixed pole sums: on orbitals whose FP64 search is regular (at most 6
    steps) the root agrees with the FP64 oracle far inside 1 meV; every other orbital ends on a
    root of the FP64 QP equation or on the linearised fallback."""
    N, nO = 40, 5
    s, nS, Om, rho = _stage_inputs(N, nO, 21)
    _, Sig, Z = O.RGW_self_energy_diag(0.0, N, N, 0, nO, N - nO, 0, nS, s["eHF"], Om, rho)
    lin = s["eHF"] + Z * Sig
    eR, _, iters = O.RGW_QP_graph(False, 0.0, 500.0, N, 0, nO, N - nO, 0, nS, s["eHF"], Om, rho,
                                  lin, s["eHF"], Z, return_iters=True)
    with _StagePrecision(ctx, api.QK_PREC_BF16X3):
        eGW, _ = api.RGW_QP_graph(False, 0.0, 500.0, N, 0, nO, N - nO, 0, nS, s["eHF"], Om, rho, lin,
                                  s["eHF"], Z, ctx=ctx)
    regular = np.asarray(iters) <= 6
    assert regular.sum() >= N // 2
    assert np.max(np.abs(eGW[regular] - eR[regular])) < 1e-7
    for p in np.where(~regular)[0]:
        w = eGW[p]
        f = w - s["eHF"][p] - O.RGW_Re_SigC(p, w, 0.0, N, 0, nO, N - nO, 0, nS, s["eHF"], Om, rho)
        assert abs(f) < 1e-5 or abs(w - lin[p]) < 1e-12, (p, f)


@pytest.mark.parametrize("N,nO,seed", [(40, 5, 21)])
def test_mixed_g0w0_newton_regular_orbitals(ctx, N, nO, seed):
    """Mixed driver (BF16x3 rho + mixed pole sums) with the Newton QP: regular orbitals within
    1 meV of the FP64 oracle."""
    s = synth.small_system(N, nO, 3 * N, seed)
    E = synth.eri_phys_numpy(s["L"])
    nS = nO * (N - nO)
    ref = O.RG0W0(False, 0.0, False, N, N, 0, nO, N - nO, 0, nS, E, s["eHF"])
    r = api.RG0W0(api.GWOptions(precision=api.QK_PREC_BF16X3), N, N, 0, nO, N - nO, 0, nS, E,
                  s["eHF"], ctx=ctx)
    regular = np.asarray(ref["qp_iters"]) <= 6
    assert regular.sum() >= N // 2
    assert np.max(np.abs(r["eGW"][regular] - ref["eGW"][regular])) < MEV
    assert abs(r["EcGM"] - ref["EcGM"]) < 1e-5 * max(1.0, abs(ref["EcGM"]))


def test_persistent_newton_matches_per_step_sweeps(ctx):
    """The mixed tier's persistent Newton kernel (one CTA per orbital, on-chip iterations) and
    the per-step sweeps (qp_persist = 2) follow the same search: regular orbitals agree to the
    roundoff of the FP32 partial sums, step counts within one, and within 1 meV of the FP64
    oracle."""
    N, nO, seed = 48, 6, 23
    s = synth.small_system(N, nO, 3 * N, seed)
    E = synth.eri_phys_numpy(s["L"])
    nS = nO * (N - nO)
    opts = api.GWOptions(precision=api.QK_PREC_BF16X3)
    old = ctx.tune_query("qp_persist", nS)
    res = {}
    try:
        for mode in (1, 2):
            ctx.tune_set("qp_persist", nS, mode)
            r = api.RG0W0(opts, N, N, 0, nO, N - nO, 0, nS, E, s["eHF"], ctx=ctx)
            res[mode] = (r["eGW"], np.array(ctx.qp_iters(N)))
    finally:
        ctx.tune_set("qp_persist", nS, max(old, 0))
    ref = O.RG0W0(False, 0.0, False, N, N, 0, nO, N - nO, 0, nS, E, s["eHF"])
    regular = (np.asarray(ref["qp_iters"]) <= 6) & (res[1][1] <= 6) & (res[2][1] <= 6)
    assert regular.sum() >= N // 2
    # the FP32 far-pole partial sums are added in another order: roundoff of ~1e-8 Ha
    assert np.max(np.abs(res[1][0][regular] - res[2][0][regular])) < 1e-6
    assert np.max(np.abs(res[1][1][regular] - res[2][1][regular])) <= 1
    assert np.max(np.abs(res[1][0][regular] - ref["eGW"][regular])) < MEV


@pytest.mark.parametrize("ta,tb,m,n,k", [("T", "N", 4000, 20, 150), ("N", "N", 70, 33, 45),
                                         ("N", "T", 129, 17, 3), ("T", "T", 300, 150, 40),
                                         ("N", "N", 200, 20, 5000), ("N", "T", 257, 300, 128)])
def test_dgemm_df_dev_accuracy_under_cancellation(ctx, ta, tb, m, n, k):
    """Double-float GEMM: every transpose, both tile shapes, split-K; operands with large
    entries whose products cancel (the qsGW quarter transforms in a near-linearly-dependent
    basis), where FP32 products fail: the error stays at ~1e-13 of sum |a_ik b_kj|."""
    import torch
    rng = np.random.default_rng(m + 7 * n + 13 * k)
    A = rng.standard_normal((k, m) if ta == "T" else (m, k)) * 30.0
    B = rng.standard_normal((n, k) if tb == "T" else (k, n))
    C0 = rng.standard_normal((m, n))
    opA = A.T if ta == "T" else A
    opB = B.T if tb == "T" else B
    dA = torch.from_numpy(np.asfortranarray(A).ravel(order="F")).cuda()
    dB = torch.from_numpy(np.asfortranarray(B).ravel(order="F")).cuda()
    dC = torch.from_numpy(np.asfortranarray(C0).ravel(order="F")).cuda()
    api.dgemm_df_dev(ta, tb, m, n, k, 0.5, dA.data_ptr(), A.shape[0], dB.data_ptr(), B.shape[0],
                     -1.5, dC.data_ptr(), m, ctx=ctx)
    ref = 0.5 * opA @ opB - 1.5 * C0
    scale = 0.5 * np.abs(opA) @ np.abs(opB) + 1.5 * np.abs(C0)
    C = dC.cpu().numpy().reshape((m, n), order="F")
    ratio = np.max(np.abs(C - ref) / scale)
    assert ratio < 1e-12 * max(1.0, k / 64.0), ratio
