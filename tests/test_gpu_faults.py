"""Failure paths, made on purpose without faulting the GPU.

- A bounded grid-barrier wait runs out: the "spin_limit" hook shortens every barrier wait to two
  polls, the cooperative tridiagonalisation's CTAs give up at their first barrier, leave the
  kernel, and the call reports QK_ERR_DEVICE; with the limit restored the same context returns
  the right eigenvalues (the context stays usable).
- Newton gives up: with maxIt = 1 or 2 (the "newton_maxit" hook; the reference's parameter at
  RGW_QP_graph.f90:38) every search of the N=24 fixture ends at step maxIt and keeps eGWlin
  (:78-81) -- at maxIt = 2 also the searches whose second step met the threshold, since the
  reference tests nIt == maxIt after the loop; at maxIt = 3 they all converge.
- A workspace allocation fails (the "fail_alloc" hook makes the n-th growing allocation fail as
  cudaMalloc would): the call returns QK_ERR_NOMEM before anything uses the buffer, and the next
  call on the same context succeeds.
- Non-finite and inconsistent inputs: a NaN orbital energy and an orbital ordering with a
  negative e_a - e_i (A - B not positive) complete and propagate NaN, as the reference's dsqrt of
  a negative number does (LR/phRLR.f90:56-58), with the A - B warning bit set.
"""
import os

import numpy as np
import pytest

from oracle import qkgw_oracle as O
from quack_gb300 import api, synth

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _fixture():
    f = np.load(os.path.join(GOLD, "synth_n24.npz"))
    N, nO = int(f["N"]), int(f["nO"])
    return f, N, nO, synth.eri_phys_numpy(f["L"])


def test_barrier_wait_runs_out_and_context_recovers():
    import torch
    c = api.Context(0)
    try:
        n = 600  # the cooperative tridiagonalisation runs on many CTAs at this size
        rng = np.random.default_rng(5)
        A = rng.standard_normal((n, n))
        A = A + A.T
        w_ref = np.linalg.eigvalsh(A)

        def run():
            dA = torch.from_numpy(np.asfortranarray(A).ravel(order="F")).cuda()
            dw = torch.empty(n, dtype=torch.float64, device="cuda")
            dZ = torch.empty(n * n, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            api.dsyev_dev(n, dA.data_ptr(), n, dw.data_ptr(), dZ.data_ptr(), True, ctx=c)
            return dw.cpu().numpy()

        c.tune_set("spin_limit", 0, 1)
        with pytest.raises(api.QkError) as ei:
            run()
        assert ei.value.code == api.QK_ERR_DEVICE
        c.tune_set("spin_limit", 0, 0)
        w = run()
        assert np.max(np.abs(w - w_ref)) < 1e-11 * np.abs(w_ref).max()
    finally:
        c.close()


@pytest.mark.parametrize("maxit", [1, 2, 3])
def test_newton_maxit_fallback_matches_oracle(maxit):
    f, N, nO, E = _fixture()
    nS = nO * (N - nO)
    c = api.Context(0)
    try:
        c.tune_set("newton_maxit", 0, maxit)
        assert c.tune_query("newton_maxit", 0) == maxit
        r = api.RG0W0(api.GWOptions(), N, N, 0, nO, N - nO, 0, nS, E, f["eHF"], ctx=c)
        iters = c.qp_iters(N)
    finally:
        c.close()
    ref = O.RG0W0(True, 0.0, False, N, N, 0, nO, N - nO, 0, nS, E, f["eHF"])
    Z0 = O.RGW_self_energy_diag(0.0, N, N, 0, nO, N - nO, 0, nS, f["eHF"], ref["Om"],
                                ref["rho"])[2]
    eGW, Z, it = O.RGW_QP_graph(False, 0.0, 500.0, N, 0, nO, N - nO, 0, nS, f["eHF"], ref["Om"],
                                ref["rho"], ref["eGWlin"], f["eHF"], Z0, return_iters=True,
                                maxit=maxit)
    assert np.array_equal(iters, it)
    assert np.max(np.abs(r["eGW"] - eGW)) < 1e-8
    assert np.max(np.abs(r["Z"] - Z)) < 1e-8
    if maxit < 3:
        assert np.all(it == maxit)
        assert np.max(np.abs(r["eGW"] - ref["eGWlin"])) < 1e-8
    else:
        assert np.all(it < maxit)
        assert np.max(np.abs(r["eGW"] - f["g0w0_eGW"])) < 1e-8


@pytest.mark.parametrize("nth", [1, 4])
def test_allocation_failure_is_reported_and_recovers(nth):
    f, N, nO, E = _fixture()
    nS = nO * (N - nO)
    c = api.Context(0)
    try:
        c.tune_set("fail_alloc", 0, nth)
        with pytest.raises(api.QkError) as ei:
            api.RG0W0(api.GWOptions(), N, N, 0, nO, N - nO, 0, nS, E, f["eHF"], ctx=c)
        assert ei.value.code == api.QK_ERR_NOMEM
        r = api.RG0W0(api.GWOptions(), N, N, 0, nO, N - nO, 0, nS, E, f["eHF"], ctx=c)
    finally:
        c.close()
    assert np.max(np.abs(r["eGW"] - f["g0w0_eGW"])) < 1e-8


def test_nan_energy_propagates(ctx):
    f, N, nO, E = _fixture()
    nS = nO * (N - nO)
    e = f["eHF"].copy()
    e[nO + 2] = np.nan
    r = api.RG0W0(api.GWOptions(linearize=True), N, N, 0, nO, N - nO, 0, nS, E, e, ctx=ctx)
    assert np.isnan(r["eGW"]).any()
    # the context is still usable
    r = api.RG0W0(api.GWOptions(), N, N, 0, nO, N - nO, 0, nS, E, f["eHF"], ctx=ctx)
    assert np.max(np.abs(r["eGW"] - f["g0w0_eGW"])) < 1e-8


def test_negative_gap_gives_nan_and_warning(ctx):
    f, N, nO, E = _fixture()
    nS = nO * (N - nO)
    e = f["eHF"].copy()
    e[nO] = e[nO - 1] - 0.5  # lowest virtual below the highest occupied: A - B not positive
    A = api.phRLR_A(1, True, N, 0, nO, N - nO, 0, nS, 1.0, e, E, ctx=ctx)
    B = api.phRLR_B(1, True, N, 0, nO, N - nO, 0, nS, 1.0, E, ctx=ctx)
    assert np.min(np.diag(A - B)) < 0
    Ec, Om, XpY, XmY = api.phRLR(False, nS, A, B, ctx=ctx)
    assert np.isnan(Ec)
    assert ctx.last_device_status() & api.QKD_NEG_AMB
    with np.errstate(invalid="ignore"):
        Ec_ref = O.phRLR(False, nS, A, B)[0]
    assert np.isnan(Ec_ref)
