"""The double-float tridiagonalisation of the mixed tier (k_sytrd_df).

The mixed tier's Casida solve runs the Householder tridiagonalisation in double-float arithmetic
on the FP32 pipe (about 47 significant bits per value); the tridiagonal eigenproblem and the
back-transformation keep their FP64 arithmetic.  These tests call it through qk_dsyev_dev with
the context setting "dsyev_df" = 1 and hold it to:

- eigenvalues within 1e-11 ||A||_2 of LAPACK's (numpy.linalg.eigvalsh), residuals
  ||A z - lambda z|| and orthogonality of the eigenvectors within 1e-10 (FP64 Householder reaches
  about 1e-13 here; the double-float unit roundoff is 2^-46 instead of 2^-53);
- bitwise repetition (the same exact mat-vec accumulators as the FP64 kernel);
- any magnitude: the matrix is scaled by a power of two before it goes to double-float;
- the grouped launch of the batched driver in the mixed tier: its results repeat bitwise for any
  grouping;
- a size whose per-CTA vectors live in global memory (n = 6900), for both kernels.
"""
import numpy as np
import pytest

from quack_gb300 import api, synth

pytestmark = pytest.mark.gpu


def _dsyev(ctx, A, df, want_vectors=True):
    import torch
    n = A.shape[0]
    ctx.tune_set("dsyev_df", 0, 1 if df else 0)
    try:
        dA = torch.from_numpy(np.asfortranarray(A).ravel(order="F")).cuda()
        dw = torch.empty(n, dtype=torch.float64, device="cuda")
        dZ = torch.empty(n * n, dtype=torch.float64, device="cuda")
        api.dsyev_dev(n, dA.data_ptr(), n, dw.data_ptr(), dZ.data_ptr(), want_vectors, ctx=ctx)
        torch.cuda.synchronize()
        return dw.cpu().numpy(), dZ.cpu().numpy().reshape((n, n), order="F")  # rows = vectors
    finally:
        ctx.tune_set("dsyev_df", 0, 0)


def _casida_like(n, seed):
    """A positive definite matrix shaped like the Casida matrix D^2 + 2 D^1/2 K D^1/2 (diagonal
    energy differences plus a low-rank coupling), the matrix the mixed tier hands this kernel."""
    rng = np.random.default_rng(seed)
    dia = np.sort(rng.uniform(0.3, 4.0, n))
    L = rng.standard_normal((n, n // 4)) * 0.05
    sd = np.sqrt(dia)
    return np.diag(dia**2) + 2.0 * (sd[:, None] * (L @ L.T) * sd[None, :])


@pytest.mark.parametrize("n,kind", [(300, "random"), (301, "random"), (1500, "random"),
                                    (2000, "casida")])
def test_df_eigenpairs_match_lapack(ctx, n, kind):
    if kind == "random":
        rng = np.random.default_rng(11 + n)
        A = rng.standard_normal((n, n))
        A = A + A.T
    else:
        A = _casida_like(n, 5)
    w_ref = np.linalg.eigvalsh(A)
    w, Zt = _dsyev(ctx, A, True)
    scale = np.abs(w_ref).max()
    assert np.max(np.abs(w - w_ref)) < 1e-11 * scale
    R = A @ Zt.T - Zt.T * w[None, :]
    assert np.max(np.linalg.norm(R, axis=0)) < 1e-10 * scale
    G = Zt @ Zt.T
    assert np.max(np.abs(G - np.eye(n))) < 1e-10
    # and close to the FP64 kernel's eigenvalues
    w64, _ = _dsyev(ctx, A, False)
    assert np.max(np.abs(w - w64)) < 1e-11 * scale


def test_df_bitwise_repeatable(ctx):
    A = _casida_like(1200, 9)
    outs = [_dsyev(ctx, A, True) for _ in range(3)]
    for w, Z in outs[1:]:
        assert np.array_equal(w, outs[0][0])
        assert np.array_equal(Z, outs[0][1])


@pytest.mark.parametrize("scale", [1e12, 1e-9, 2.0**-300])
def test_df_any_magnitude(ctx, scale):
    """The kernel scales the matrix by the power of two that brings ||A||_F into [1/2, 1) before
    it goes to double-float: magnitudes far outside float's range keep the relative accuracy."""
    rng = np.random.default_rng(3)
    A = rng.standard_normal((400, 400))
    A = A + A.T
    w1, _ = _dsyev(ctx, A, True)
    w, _ = _dsyev(ctx, A * scale, True)
    w_ref = np.linalg.eigvalsh(A * scale)
    assert np.max(np.abs(w - w_ref)) < 1e-11 * np.abs(w_ref).max()
    assert np.max(np.abs(w / scale - w1)) < 1e-12 * np.abs(w1).max()


def test_mixed_batched_grouped_df_repeatable(ctx):
    """Mixed-tier batch: the workers' double-float tridiagonalisations share grouped launches
    whose composition depends on timing; results repeat bitwise."""
    import torch
    rng = np.random.default_rng(78)
    systems = [synth.gen_system(N, synth.n_occ(N), 3 * N, rng) for N in (40, 57, 24, 66, 31, 48)]
    desc, Lf, Ef = api.pack_systems(systems)
    dL = torch.from_numpy(Lf).cuda()
    dE = torch.from_numpy(Ef).cuda()
    opts = api.GWOptions(precision=api.QK_PREC_BF16X3)
    outs = []
    for nw in (3, 3, 2):
        dG = torch.zeros_like(dE)
        r = api.gw_batch_L_dev(opts, 0, desc, dL.data_ptr(), dE.data_ptr(), dG.data_ptr(),
                               n_workers=nw, ctx=ctx)
        assert r["rc"] == api.QK_OK, (r["error"], r["status"])
        outs.append(dG.cpu().numpy())
    for o in outs[1:]:
        assert np.array_equal(o, outs[0], equal_nan=True)


def test_df_vectors_in_global_memory(ctx):
    """n = 6900: the three vectors of every CTA no longer fit in shared memory beside the tiles,
    so both kernels keep them in global memory (the FP64 kernel from n ~ 3800 on); eigenvalues
    against LAPACK's."""
    n = 6900
    rng = np.random.default_rng(17)
    A = rng.standard_normal((n, n))
    A = A + A.T
    w_ref = np.linalg.eigvalsh(A)
    scale = np.abs(w_ref).max()
    w_df, _ = _dsyev(ctx, A, True, want_vectors=False)
    assert np.max(np.abs(w_df - w_ref)) < 1e-11 * scale
    w_64, _ = _dsyev(ctx, A, False, want_vectors=False)
    assert np.max(np.abs(w_64 - w_ref)) < 1e-11 * scale
