"""CPU: the perceptron oracle's analytic gradient agrees with central finite differences."""
import numpy as np

from oracle import mlp_oracle as M


def test_oracle_gradient_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.standard_normal(M.NPARAM) * 0.2
    X = rng.standard_normal((12, 16))
    T = rng.standard_normal(12)
    _, g = M.loss_and_grad(p, X, T)
    h = 1e-6
    for i in rng.choice(M.NPARAM, 40, replace=False):
        e = np.zeros(M.NPARAM)
        e[i] = h
        fd = (M.loss_and_grad(p + e, X, T)[0] - M.loss_and_grad(p - e, X, T)[0]) / (2 * h)
        assert abs(fd - g[i]) < 1e-7 * max(1.0, abs(g[i]))


def test_parameter_count():
    assert M.NPARAM == 64 * 16 + 64 + 64 * 64 + 64 + 64 + 1 == 5313
