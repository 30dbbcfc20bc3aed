"""Learned quasiparticle guess: data collection, training and evaluation on the GPU.

The model (16 -> 64 -> 64 -> 1 SiLU) and its forward/backward/Adam kernels live in libqkgw.so
(k_mlp.cu).  Features are the 16 per-orbital quantities of the linearised G0W0 stage that the
driver captures: orbital energy and its distance to the frontier orbitals, Sigma_c(e_p), Z_p,
the linearised shift Z*Sigma (= eGWlin - eHF), dSigma/dw, then from one pole sweep at eGWlin the
Newton and Halley steps of the QP equation, its residual and slope there, the distance to the
nearest pole and that pole's strength, and finally the lowest screening energy and log N.  The
target is the nonlinear part of the converged QP shift, eGW_p - eGWlin_p, of the plain FP64
Newton search on the orbitals whose search from eGWlin is regular (few steps, small correction);
the guess is eGWlin_p plus the prediction.  Trained weights are saved as a flat float32 binary
plus a JSON file with the normalisation.
"""
from __future__ import annotations

import ctypes as C
import json
import time

import numpy as np

from . import api

NPARAM = 64 * 16 + 64 + 64 * 64 + 64 + 64 + 1


class QPModel:
    def __init__(self, ctx: api.Context, seed: int = 1234):
        self.ctx = ctx
        self._h = C.c_void_p()
        L = api.lib()
        L.qk_mlp_create.argtypes = [C.c_void_p, C.c_ulonglong, C.POINTER(C.c_void_p)]
        ctx.check(L.qk_mlp_create(ctx.handle, C.c_ulonglong(seed), C.byref(self._h)))
        self.xmean = np.zeros(16, np.float32)
        self.xstd = np.ones(16, np.float32)
        self.ymean, self.ystd = 0.0, 1.0

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            api.lib().qk_mlp_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- parameters --------------------------------------------------------------------------
    def get_params(self) -> np.ndarray:
        buf = np.zeros(NPARAM, np.float32)
        self.ctx.check(api.lib().qk_mlp_params(self.ctx.handle, self._h,
                                               buf.ctypes.data_as(C.POINTER(C.c_float)), 0))
        return buf

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == NPARAM
        self.ctx.check(api.lib().qk_mlp_params(self.ctx.handle, self._h,
                                               p.ctypes.data_as(C.POINTER(C.c_float)), 1))

    def set_scaling(self, xmean, xstd, ymean, ystd):
        self.xmean = np.ascontiguousarray(xmean, np.float32)
        self.xstd = np.ascontiguousarray(np.where(np.asarray(xstd) > 0, xstd, 1.0), np.float32)
        self.ymean, self.ystd = float(ymean), float(ystd if ystd > 0 else 1.0)
        fp = C.POINTER(C.c_float)
        api.lib().qk_mlp_set_scaling(self._h, self.xmean.ctypes.data_as(fp),
                                     self.xstd.ctypes.data_as(fp), C.c_float(self.ymean),
                                     C.c_float(self.ystd))

    def save(self, prefix):
        self.get_params().tofile(prefix + ".bin")
        with open(prefix + ".json", "w") as f:
            json.dump({"layers": [16, 64, 64, 1], "activation": "silu", "nparam": NPARAM,
                       "xmean": self.xmean.tolist(), "xstd": self.xstd.tolist(),
                       "ymean": self.ymean, "ystd": self.ystd}, f)

    def load(self, prefix):
        self.set_params(np.fromfile(prefix + ".bin", dtype=np.float32))
        with open(prefix + ".json") as f:
            meta = json.load(f)
        self.set_scaling(meta["xmean"], meta["xstd"], meta["ymean"], meta["ystd"])

    # -- kernels -----------------------------------------------------------------------------
    def grad_dev(self, n, d_X, d_T, d_G):
        loss = C.c_float()
        self.ctx.check(api.lib().qk_mlp_grad_dev(self.ctx.handle, self._h, n, C.c_void_p(d_X),
                                                 C.c_void_p(d_T), C.c_void_p(d_G), C.byref(loss)))
        return loss.value

    def train_dev(self, n, d_X, d_T, epochs, batch, lr):
        loss = C.c_float()
        self.ctx.check(api.lib().qk_mlp_train_dev(self.ctx.handle, self._h, n, C.c_void_p(d_X),
                                                  C.c_void_p(d_T), epochs, batch, C.c_float(lr),
                                                  C.byref(loss)))
        return loss.value

    def predict_dev(self, n, d_X, d_Y, bf16=True):
        self.ctx.check(api.lib().qk_mlp_predict_dev(self.ctx.handle, self._h, n, C.c_void_p(d_X),
                                                    C.c_void_p(d_Y), int(bool(bf16))))


def run_g0w0_L(ctx, system, opts, capture=False):
    """One G0W0 from the factorised integrals of a synthetic system (device arrays).
    Returns dict(eGW, SigC, Z, iters, evals, features, qp_ms)."""
    import torch
    N, nO = system["N"], system["nO"]
    naux = system["L"].shape[0]
    dL = torch.from_numpy(api.L_fortran_flat(system["L"])).cuda()
    de = torch.from_numpy(np.asarray(system["eHF"], dtype=np.float64)).cuda()
    out = [torch.empty(N, dtype=torch.float64, device="cuda") for _ in range(3)]
    dOm = torch.empty(nO * (N - nO), dtype=torch.float64, device="cuda")
    ctx.set_feature_capture(capture)
    api.RG0W0_L_dev(opts, N, 0, nO, 0, naux, dL.data_ptr(), de.data_ptr(), out[0].data_ptr(),
                    out[1].data_ptr(), out[2].data_ptr(), dOm.data_ptr(), ctx=ctx)
    res = dict(eGW=out[0].cpu().numpy(), SigC=out[1].cpu().numpy(), Z=out[2].cpu().numpy(),
               iters=ctx.qp_iters(N), evals=ctx.qp_evals(), qp_ms=ctx.timings()["qp"])
    if capture:
        res["features"] = ctx.features(N)
    ctx.set_feature_capture(False)
    return res


def collect(ctx, systems, maxit_ok=16, max_corr=0.25):
    """Features and targets eGW - eGWlin from plain FP64 Newton G0W0 runs.  Feature 6 is the
    linearised shift Z*Sigma = eGWlin - eHF.  Orbitals whose search wandered (more than maxit_ok
    steps) or jumped far from the linearised root carry no learnable signal and are left out."""
    X, T = [], []
    for s in systems:
        r = run_g0w0_L(ctx, s, api.GWOptions(), capture=True)
        F = r["features"]
        corr = r["eGW"] - s["eHF"] - F[:, 6].astype(np.float64)
        ok = ((r["iters"] <= maxit_ok) & np.isfinite(r["eGW"]) & np.all(np.isfinite(F), 1)
              & (np.abs(corr) <= max_corr))
        X.append(F[ok])
        T.append(corr[ok])
    return np.concatenate(X).astype(np.float32), np.concatenate(T).astype(np.float32)


def train(model: QPModel, X, T, epochs=200, batch=256, lr=2e-3):
    """Normalise, upload and train with the library's Adam kernels.  Returns the final MSE
    (normalised units)."""
    import torch
    xm, xs = X.mean(0), X.std(0) + 1e-6
    ym, ys = float(T.mean()), float(T.std() + 1e-6)
    model.set_scaling(xm, xs, ym, ys)
    Xn = ((X - xm) / xs).astype(np.float32)
    Tn = ((T - ym) / ys).astype(np.float32)
    dX = torch.from_numpy(np.ascontiguousarray(Xn)).cuda()
    dT = torch.from_numpy(np.ascontiguousarray(Tn)).cuda()
    return model.train_dev(len(T), dX.data_ptr(), dT.data_ptr(), epochs, min(batch, len(T)), lr)


def evaluate(ctx, model, systems, tol=1e-6):
    """Newton from the reference start vs from the learned guess on held-out systems.  A QP
    energy counts as the same root when the two agree within tol * max(1, |Sigma|): the Newton
    threshold |f| <= 1e-6 of RGW_QP_graph.f90:59 (two searches that end on one root stop at
    different iterates)."""
    ctx.set_qp_model(model)
    rows = []
    for s in systems:
        t0 = time.time()
        a = run_g0w0_L(ctx, s, api.GWOptions())
        t1 = time.time()
        b = run_g0w0_L(ctx, s, api.GWOptions(qp_guess=1))
        t2 = time.time()
        h = run_g0w0_L(ctx, s, api.GWOptions(qp_guess=2))
        both = (a["iters"] < 64) & np.isfinite(a["eGW"])
        d = np.abs(a["eGW"] - b["eGW"])
        rows.append(dict(N=s["N"], evals_ref=a["evals"], evals_guess=b["evals"],
                         evals_hf_start=h["evals"],
                         qp_ms_ref=a["qp_ms"], qp_ms_guess=b["qp_ms"], wall_ref=t1 - t0,
                         wall_guess=t2 - t1, n_conv=int(both.sum()),
                         max_diff_conv=float(d[both].max()) if both.any() else 0.0,
                         n_same=int((d[both] < tol * np.maximum(1.0, np.abs(a["SigC"][both]))).sum())))
    ctx.set_qp_model(None)
    return rows
