"""CPU: the surrogate-network oracle's parameter gradient (reverse mode through
both the forward and the input-gradient pass) against central finite
differences, on a narrow network so the check is quick."""
import numpy as np

from oracle import mlp_oracle as M


def _params(h, rng):
    n = 3 * h + h + 3 * (h * h + h) + h + 1
    return rng.normal(0, 0.5, n)


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    h = 8
    p = _params(h, rng)
    X = rng.uniform(-1, 1, (5, 3))
    ys = rng.normal(size=5)
    Gs = rng.normal(size=(5, 3))
    L, g = M.loss_and_grad(p, X, ys, Gs, alpha=0.7, beta=1.3, h=h)
    eps = 1e-6
    idx = rng.choice(p.size, 60, replace=False)
    for i in idx:
        d = np.zeros_like(p)
        d[i] = eps
        Lp, _ = M.loss_and_grad(p + d, X, ys, Gs, alpha=0.7, beta=1.3, h=h)
        Lm, _ = M.loss_and_grad(p - d, X, ys, Gs, alpha=0.7, beta=1.3, h=h)
        fd = (Lp - Lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_input_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    h = 8
    p = _params(h, rng)
    X = rng.uniform(-1, 1, (4, 3))
    y, G, _ = M.forward(p, X, h)
    eps = 1e-6
    for j in range(3):
        d = np.zeros_like(X)
        d[:, j] = eps
        fd = (M.forward(p, X + d, h)[0] - M.forward(p, X - d, h)[0]) / (2 * eps)
        np.testing.assert_allclose(G[:, j], fd, rtol=1e-6, atol=1e-9)
