"""CPU oracle of the learned initial-guess corrector's network (test
infrastructure: only tests and the smoke check use it).

The corrector has no counterpart in the reference; this module restates, in
float64 numpy, the network the library trains on the GPU so that its forward
pass, loss gradient and Adam step can be checked:

    h1 = tanh(W1 x + b1)          W1: 64 x F
    h2 = tanh(W2 h1 + b2)         W2: 64 x 64 (out, in)
    y  = W3 . h2 + b3             W3: 64
    loss = sum_s w_s (y_s - t_s)^2 / sum_s w_s

Parameters are one flat vector in the library's order: W1 (row-major), b1,
W2 (row-major), b2, W3, b3.  The analytic gradient is itself pinned against
central finite differences in the tests.
"""
import numpy as np

H = 64


def nparams(F):
    return H * F + H + H * H + H + H + 1


def unpack(p, F):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + H * F].reshape(H, F); o += H * F
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def forward(p, X):
    X = np.asarray(X, dtype=np.float64)
    W1, b1, W2, b2, W3, b3 = unpack(p, X.shape[1])
    h1 = np.tanh(X @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    return h2 @ W3 + b3, (h1, h2)


def loss(p, X, T, W=None):
    y, _ = forward(p, X)
    W = np.ones(len(y)) if W is None else np.asarray(W, dtype=np.float64)
    return float(np.sum(W * (y - T) ** 2) / np.sum(W))


def loss_grad(p, X, T, W=None):
    """(loss, gradient) by back-propagation."""
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    F = X.shape[1]
    W = np.ones(len(X)) if W is None else np.asarray(W, dtype=np.float64)
    W1, b1, W2, b2, W3, b3 = unpack(p, F)
    y, (h1, h2) = forward(p, X)
    r = y - T
    ws = np.sum(W)
    dy = 2.0 * W * r / ws                       # d loss / d y_s
    gW3 = dy @ h2
    gb3 = np.sum(dy)
    dz2 = np.outer(dy, W3) * (1.0 - h2 ** 2)    # samples x 64
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(axis=0)
    dz1 = (dz2 @ W2) * (1.0 - h1 ** 2)
    gW1 = dz1.T @ X
    gb1 = dz1.sum(axis=0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return float(np.sum(W * r ** 2) / ws), g


def adam_step(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba); t counts from 1.  Returns (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
