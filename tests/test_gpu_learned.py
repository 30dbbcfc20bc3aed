"""GPU tests of the learned QP guess: the perceptron's forward/backward/Adam kernels against the
NumPy oracle, BF16 inference against FP32, and the guess-seeded Newton search returning the
reference roots."""
import numpy as np
import pytest

from oracle import mlp_oracle as M
from quack_gb300 import api, learned, synth

pytestmark = pytest.mark.gpu


def _t(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).cuda()


def test_mlp_gradient_matches_oracle(ctx):
    import torch
    m = learned.QPModel(ctx, seed=7)
    rng = np.random.default_rng(1)
    p = (rng.standard_normal(M.NPARAM) * 0.3).astype(np.float32)
    m.set_params(p)
    X = rng.standard_normal((300, 16)).astype(np.float32)
    T = rng.standard_normal(300).astype(np.float32)
    dX, dT = _t(X), _t(T)
    dG = torch.zeros(M.NPARAM, dtype=torch.float32, device="cuda")
    loss = m.grad_dev(300, dX.data_ptr(), dT.data_ptr(), dG.data_ptr())
    ref_loss, ref_g = M.loss_and_grad(p.astype(np.float64), X.astype(np.float64), T.astype(np.float64))
    g = dG.cpu().numpy()
    assert abs(loss - ref_loss) < 1e-4 * max(1.0, ref_loss)
    scale = np.abs(ref_g).max()
    assert np.max(np.abs(g - ref_g)) < 2e-4 * scale


def test_mlp_training_and_bf16_inference(ctx):
    import torch
    m = learned.QPModel(ctx, seed=3)
    rng = np.random.default_rng(2)
    X = rng.standard_normal((4096, 16)).astype(np.float32)
    T = (np.sin(X[:, 0]) + 0.5 * X[:, 1] * X[:, 2] - 0.3 * X[:, 3]).astype(np.float32)
    dX, dT = _t(X), _t(T)
    Y0 = torch.zeros(4096, dtype=torch.float32, device="cuda")
    m.predict_dev(4096, dX.data_ptr(), Y0.data_ptr(), bf16=False)
    loss0 = float(np.mean((Y0.cpu().numpy() - T) ** 2))
    loss = m.train_dev(4096, dX.data_ptr(), dT.data_ptr(), epochs=60, batch=256, lr=3e-3)
    assert loss < 0.1 * loss0
    # forward kernel against the oracle with the trained parameters
    Y = torch.zeros(4096, dtype=torch.float32, device="cuda")
    m.predict_dev(4096, dX.data_ptr(), Y.data_ptr(), bf16=False)
    Yref, _ = M.forward(m.get_params().astype(np.float64), X.astype(np.float64))
    assert np.max(np.abs(Y.cpu().numpy() - Yref)) < 1e-3 * max(1.0, np.abs(Yref).max())
    # BF16 inference stays close to FP32
    Yb = torch.zeros(4096, dtype=torch.float32, device="cuda")
    m.predict_dev(4096, dX.data_ptr(), Yb.data_ptr(), bf16=True)
    assert np.sqrt(np.mean((Yb.cpu().numpy() - Yref) ** 2)) < 0.05 * np.std(Yref)


def test_learned_guess_keeps_reference_roots(ctx):
    rng = np.random.default_rng(11)
    train_sys = [synth.gen_system(N, synth.n_occ(N), 3 * N, rng) for N in (24, 28, 32, 36, 30, 26)]
    test_sys = [synth.gen_system(N, synth.n_occ(N), 3 * N, rng) for N in (25, 34)]
    X, T = learned.collect(ctx, train_sys)
    assert len(T) > 50
    m = learned.QPModel(ctx, seed=5)
    learned.train(m, X, T, epochs=150, batch=128, lr=3e-3)
    rows = learned.evaluate(ctx, m, test_sys)
    n_conv = sum(r["n_conv"] for r in rows)
    n_same = sum(r["n_same"] for r in rows)
    # the guess path reproduces the reference root for every converged orbital: orbitals the
    # gate sends to the reference start follow the reference trajectory exactly, and a
    # guess-started root is kept only when the root certificate proves that the reference
    # search from eGWlin converges to it (otherwise the orbital restarts from eGWlin)
    assert n_same == n_conv, rows


def test_learned_guess_saves_newton_evaluations(ctx):
    """What the trained network gains: Newton Sigma evaluations with the guess vs the reference
    search from eGWlin on held-out systems (same generator family, N = 24..60)."""
    systems = synth.batch_systems(60, 24, 60, seed=7)
    X, T = learned.collect(ctx, systems[:48])
    m = learned.QPModel(ctx, seed=2)
    learned.train(m, X, T, epochs=200, batch=256, lr=2e-3)
    rows = learned.evaluate(ctx, m, systems[48:])
    ev_ref = sum(r["evals_ref"] for r in rows)
    ev_g = sum(r["evals_guess"] for r in rows)
    n_conv = sum(r["n_conv"] for r in rows)
    n_same = sum(r["n_same"] for r in rows)
    ev_hf = sum(r["evals_hf_start"] for r in rows)
    print("newton evals: reference %d, learned guess %d (%.1f%% fewer), HF start %d; same root %d/%d"
          % (ev_ref, ev_g, 100.0 * (1.0 - ev_g / ev_ref), ev_hf, n_same, n_conv))
    assert ev_g < ev_hf
    assert ev_g < ev_ref
    assert n_same == n_conv


def test_batched_driver_uses_the_attached_model(ctx):
    """The batched driver's worker contexts take the caller's learned model: a batched G0W0 with
    qp_guess = 1 succeeds for every system and gives the per-system guess-path energies."""
    import torch
    from quack_gb300 import api
    rng = np.random.default_rng(31)
    train_sys = [synth.gen_system(N, synth.n_occ(N), 3 * N, rng) for N in (24, 28, 32, 30)]
    test_sys = [synth.gen_system(N, synth.n_occ(N), 3 * N, rng) for N in (26, 34, 29)]
    X, T = learned.collect(ctx, train_sys)
    m = learned.QPModel(ctx, seed=9)
    learned.train(m, X, T, epochs=60, batch=128, lr=3e-3)
    ctx.set_qp_model(m)
    try:
        desc, Lf, Ef = api.pack_systems(test_sys)
        dL = torch.from_numpy(np.ascontiguousarray(Lf)).cuda()
        dE = torch.from_numpy(np.ascontiguousarray(Ef)).cuda()
        dG = torch.zeros_like(dE)
        opts = api.GWOptions(qp_guess=1)
        r = api.gw_batch_L_dev(opts, 0, desc, dL.data_ptr(), dE.data_ptr(), dG.data_ptr(),
                               n_workers=2, ctx=ctx)
        assert r["rc"] == api.QK_OK, (r["error"], r["status"])
        eG = dG.cpu().numpy()
        for i, s in enumerate(test_sys):
            one = learned.run_g0w0_L(ctx, s, opts)
            got = eG[desc[i].offset_e:desc[i].offset_e + s["N"]]
            conv = np.asarray(one["iters"]) < 16
            assert np.max(np.abs(got[conv] - one["eGW"][conv])) < 1e-8, i
    finally:
        ctx.set_qp_model(None)


@pytest.mark.parametrize("N,nO,seed", [(57, 7, 22), (96, 12, 23), (150, 19, 24)])
def test_started_elsewhere_keeps_reference_roots(ctx, N, nO, seed):
    """The restart protocol alone (qp_guess = 2: searches started at eHF, kept only where the
    root certificate proves the reference search ends there, the others restarted from eGWlin)
    gives the reference-start roots for every orbital whose reference search converged -- also
    the chaotic ones, which need each orbital's Sigma(w) to be independent of which other
    orbitals are still searching."""
    s = synth.small_system(N, nO, 3 * N, seed)
    a = learned.run_g0w0_L(ctx, s, api.GWOptions())
    b = learned.run_g0w0_L(ctx, s, api.GWOptions(qp_guess=2))
    ok = (a["iters"] < 64) & np.isfinite(a["eGW"])
    d = np.abs(a["eGW"] - b["eGW"])
    assert ok.sum() > N // 2
    # same root: within the Newton threshold (the two searches stop at different iterates)
    assert np.all(d[ok] < 1e-6 * np.maximum(1.0, np.abs(a["SigC"][ok]))), np.where(ok & (d > 1e-6))
