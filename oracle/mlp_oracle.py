"""NumPy float64 restatement of the learned-guess perceptron (16 -> 64 -> 64 -> 1, SiLU) and its
mean-squared-error gradient.  TEST INFRASTRUCTURE ONLY: it checks the GPU forward/backward
kernels of libqkgw.so (k_mlp.cu); no product path imports it.  Parameter layout: flat vector
[W1 (64x16) | b1 | W2 (64x64) | b2 | W3 (1x64) | b3], row-major weights."""
import numpy as np

NIN, NH = 16, 64
SIZES = [("W1", (NH, NIN)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (1, NH)),
         ("b3", (1,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    out, o = {}, 0
    for name, shp in SIZES:
        n = int(np.prod(shp))
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(shp)
        o += n
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, X):
    w = unpack(p)
    Z1 = X @ w["W1"].T + w["b1"]
    A1 = silu(Z1)
    Z2 = A1 @ w["W2"].T + w["b2"]
    A2 = silu(Z2)
    Y = (A2 @ w["W3"].T + w["b3"])[:, 0]
    return Y, (Z1, A1, Z2, A2)


def loss_and_grad(p, X, T):
    w = unpack(p)
    B = X.shape[0]
    Y, (Z1, A1, Z2, A2) = forward(p, X)
    dY = 2.0 * (Y - T) / B
    gW3 = dY[None, :] @ A2
    gb3 = np.array([dY.sum()])
    D2 = (dY[:, None] * w["W3"]) * dsilu(Z2)
    gW2 = D2.T @ A1
    gb2 = D2.sum(0)
    D1 = (D2 @ w["W2"]) * dsilu(Z1)
    gW1 = D1.T @ X
    gb1 = D1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return float(np.mean((Y - T) ** 2)), g
