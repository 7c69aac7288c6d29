"""The corrector network's CPU oracle: back-propagated gradient against
central finite differences, and the Adam step against its definition."""
import numpy as np

from oracle import mlp


def _problem(seed=3, n=40, F=9):
    rng = np.random.default_rng(seed)
    p = rng.normal(scale=0.3, size=mlp.nparams(F))
    X = rng.normal(size=(n, F))
    T = rng.normal(size=n)
    W = rng.uniform(0.1, 2.0, size=n)
    return p, X, T, W


def test_gradient_matches_finite_differences():
    p, X, T, W = _problem()
    loss, g = mlp.loss_grad(p, X, T, W)
    assert loss == mlp.loss(p, X, T, W)
    rng = np.random.default_rng(0)
    idx = rng.choice(len(p), 80, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (mlp.loss(p + e, X, T, W) - mlp.loss(p - e, X, T, W)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_unit_weights_default():
    p, X, T, _ = _problem(seed=4)
    l1, g1 = mlp.loss_grad(p, X, T)
    l2, g2 = mlp.loss_grad(p, X, T, np.full(len(T), 3.0))
    assert abs(l1 - l2) <= 1e-14 * l1
    np.testing.assert_allclose(g1, g2, rtol=1e-12)


def test_adam_first_step_is_signed_lr():
    # with zero moments, the bias-corrected first step is lr * g / (|g| + eps)
    g = np.array([0.5, -2.0, 1e-3])
    p, m, v = mlp.adam_step(np.zeros(3), g, np.zeros(3), np.zeros(3), 1, lr=0.01)
    np.testing.assert_allclose(p, -0.01 * g / (np.abs(g) + 1e-8), rtol=1e-12)
