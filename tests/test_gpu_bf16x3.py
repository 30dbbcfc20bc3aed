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


def test_dgemm_dev_matches_numpy(ctx):
    import torch
    rng = np.random.default_rng(1)
    for ta, tb, (m, n, k) in (("N", "N", (70, 33, 45)), ("T", "N", (64, 65, 66)),
                              ("N", "T", (129, 17, 3)), ("T", "T", (5, 200, 77))):
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
        assert np.allclose(C, ref, rtol=1e-13, atol=1e-12)


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
