"""CPU restatement of the cost model's network, forward and backward.

TEST INFRASTRUCTURE ONLY: the oracle the library's MLP kernels (tq_mlp_*) are
checked against; only ``tests/`` import it.  The reference (Walter-Feng/Torque)
has no learned component, so this oracle restates the textbook algorithm, in
float64: a 3-layer perceptron n_in -> width -> width -> n_out with ReLU after
the two hidden layers, loss = mean over samples and outputs of
mask * (y - t)^2, gradients by reverse-mode differentiation, and one Adam
step (Kingma-Ba 2015, bias-corrected, eps added to the square root).

Parameter layout (the library's): W1[width][n_in] b1 W2[width][width] b2
W3[n_out][width] b3, row-major, back to back.
"""
from __future__ import annotations

import numpy as np


def unpack(p, n_in, width, n_out):
    p = np.asarray(p, np.float64)
    o = 0
    out = []
    for shape in ((width, n_in), (width,), (width, width), (width,), (n_out, width), (n_out,)):
        n = int(np.prod(shape))
        out.append(p[o:o + n].reshape(shape))
        o += n
    assert o == p.size
    return out


def forward(p, X, n_in, width, n_out):
    W1, b1, W2, b2, W3, b3 = unpack(p, n_in, width, n_out)
    X = np.asarray(X, np.float64)
    z1 = X @ W1.T + b1
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0.0)
    y = h2 @ W3.T + b3
    return y, (X, h1, h2)


def loss_and_grad(p, X, T, n_in, width, n_out, mask=None):
    W1, b1, W2, b2, W3, b3 = unpack(p, n_in, width, n_out)
    y, (X, h1, h2) = forward(p, X, n_in, width, n_out)
    T = np.asarray(T, np.float64)
    w = np.ones_like(T) if mask is None else np.asarray(mask, np.float64)
    scale = 1.0 / T.size
    d = y - T
    loss = float(np.sum(w * d * d) * scale)
    dy = 2.0 * w * d * scale
    gW3 = dy.T @ h2
    gb3 = dy.sum(0)
    d2 = (dy @ W3) * (h2 > 0)
    gW2 = d2.T @ h1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * (h1 > 0)
    gW1 = d1.T @ X
    gb1 = d1.sum(0)
    g = np.concatenate([a.ravel() for a in (gW1, gb1, gW2, gb2, gW3, gb3)])
    return loss, g


def adam_step(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update; step counts from 1.  Returns (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = p - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v
