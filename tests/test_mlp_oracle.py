"""The cost model's CPU oracle pinned on the CPU: its backward pass against
central finite differences of its own forward pass, and its Adam step against
the update written out for one scalar."""
import numpy as np

from oracle import mlp_oracle as mo


def _params(rng, n_in, width, n_out):
    n = width * n_in + width + width * width + width + n_out * width + n_out
    return rng.standard_normal(n) * 0.5


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    n_in, width, n_out = 5, 7, 3
    p = _params(rng, n_in, width, n_out)
    X = rng.standard_normal((9, n_in))
    T = rng.standard_normal((9, n_out))
    mask = (rng.random((9, n_out)) < 0.7).astype(float)
    loss, g = mo.loss_and_grad(p, X, T, n_in, width, n_out, mask)
    h = 1e-6
    for i in rng.choice(p.size, 40, replace=False):
        e = np.zeros_like(p)
        e[i] = h
        lp, _ = mo.loss_and_grad(p + e, X, T, n_in, width, n_out, mask)
        lm, _ = mo.loss_and_grad(p - e, X, T, n_in, width, n_out, mask)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_adam_first_step():
    p, m, v = mo.adam_step(np.array([1.0]), np.array([0.5]), np.zeros(1), np.zeros(1), 1, 0.1)
    # bias-corrected first step moves by lr * sign(g) (up to eps)
    assert abs(p[0] - (1.0 - 0.1 * 0.5 / (0.5 + 1e-8))) < 1e-12
    assert abs(m[0] - 0.05) < 1e-15 and abs(v[0] - 0.00025) < 1e-15
