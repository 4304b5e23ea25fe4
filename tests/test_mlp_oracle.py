"""CPU self-check of the FP64 MLP restatement used as the gradient oracle: its backward
pass agrees with central finite differences."""
import numpy as np

from oracle import mlp


def test_param_count_matches_spec():
    assert mlp.param_count() == 492800


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    theta = mlp.glorot(1)
    X = rng.standard_normal((3, 896))
    dY = rng.standard_normal((3, 512))
    g = mlp.backward(theta, X, dY)
    idx = rng.choice(theta.size, 40, replace=False)
    h = 1e-6
    for i in idx:
        tp, tm = theta.copy(), theta.copy()
        tp[i] += h
        tm[i] -= h
        fd = (np.sum(mlp.forward(tp, X)[0] * dY) - np.sum(mlp.forward(tm, X)[0] * dY)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])
