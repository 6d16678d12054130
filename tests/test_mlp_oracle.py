"""The FP64 restatement of the engine-switch MLP (oracle/mlp.py) against central finite
differences, so that the GPU gradient check rests on a verified oracle."""
import numpy as np

from oracle import mlp as M


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    p = rng.normal(0, 0.4, M.NP)
    X = rng.uniform(0, 1, (64, M.F))
    Y = (rng.random(64) < 0.5).astype(np.float64)
    W = rng.uniform(0.5, 1.5, 64)
    _, g = M.loss_and_grad(p, X, Y, W)
    idx = rng.choice(M.NP, 120, replace=False)
    idx = np.union1d(idx, [M.OFF_B3, M.OFF_W3, M.OFF_B2, M.OFF_W2, M.OFF_B1, M.OFF_W1])
    h = 1e-6
    for i in idx:
        e = np.zeros(M.NP)
        e[i] = h
        fd = (M.loss_and_grad(p + e, X, Y, W)[0] - M.loss_and_grad(p - e, X, Y, W)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), i


def test_loss_is_weighted_cross_entropy():
    rng = np.random.default_rng(6)
    p = rng.normal(0, 0.3, M.NP)
    X = rng.uniform(0, 1, (10, M.F))
    Y = (rng.random(10) < 0.5).astype(np.float64)
    W = rng.uniform(0.5, 1.5, 10)
    z, _ = M.forward(p, X)
    s = 1 / (1 + np.exp(-z))
    ce = -(Y * np.log(s) + (1 - Y) * np.log(1 - s))
    loss, _ = M.loss_and_grad(p, X, Y, W)
    assert abs(loss - np.mean(W * ce)) < 1e-12
