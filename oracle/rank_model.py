"""NumPy (float64) restatement of the learned skeleton-rank model.

Test infrastructure only: the checker of the rank model's CUDA inference,
gradient and Adam kernels (ie-solver_gb300/csrc/rank_model.cu).  The model
has no counterpart in the reference; it predicts the rank fraction k/n that
the reference's ID rule (ie_solver/ie_mat.cpp:548-588, first |R_ii| <
tol |R_00|) gives a box, and this restatement is pinned by central finite
differences of its own loss (tests/test_rank_model.py), not by reference
outputs.

Model: y = sigmoid(w3 . relu(W2 relu(W1 x + b1) + b2) + b3), loss = mean
(y - t)^2; weights packed as W1 (64 x 16, row major), b1, W2 (64 x 64), b2,
w3, b3.
"""
from __future__ import annotations

import numpy as np

FEATURES, HIDDEN = 16, 64
SHAPES = ((HIDDEN, FEATURES), (HIDDEN,), (HIDDEN, HIDDEN), (HIDDEN,), (HIDDEN,), (1,))
WEIGHTS = sum(int(np.prod(s)) for s in SHAPES)


def unpack(w):
    out, o = [], 0
    for s in SHAPES:
        n = int(np.prod(s))
        out.append(np.asarray(w[o:o + n], dtype=np.float64).reshape(s))
        o += n
    return out


def pack(parts):
    return np.concatenate([np.asarray(p, dtype=np.float64).ravel() for p in parts])


def forward(w, X):
    """Predicted rank fractions of the feature rows X (count x 16)."""
    W1, b1, W2, b2, w3, b3 = unpack(w)
    h1 = np.maximum(X @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    return 1.0 / (1.0 + np.exp(-(h2 @ w3 + b3[0])))


def loss_and_gradient(w, X, t):
    """Mean squared error of the fractions and its gradient (packed)."""
    W1, b1, W2, b2, w3, b3 = unpack(w)
    X = np.asarray(X, dtype=np.float64)
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0.0)
    y = 1.0 / (1.0 + np.exp(-(h2 @ w3 + b3[0])))
    n = len(t)
    loss = float(np.mean((y - t) ** 2))
    dz = 2.0 * (y - t) * y * (1.0 - y) / n
    g_w3 = h2.T @ dz
    g_b3 = np.array([dz.sum()])
    d2 = np.outer(dz, w3) * (a2 > 0)
    g_W2 = d2.T @ h1
    g_b2 = d2.sum(axis=0)
    d1 = (d2 @ W2) * (a1 > 0)
    g_W1 = d1.T @ X
    g_b1 = d1.sum(axis=0)
    return loss, pack((g_W1, g_b1, g_W2, g_b2, g_w3, g_b3))


def adam_step(w, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (Kingma & Ba 2015) with bias correction; returns (w, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return w - lr * mh / (np.sqrt(vh) + eps), m, v


def sketch_rows(y, n, headroom=1.15, extra=10):
    """Sketch rows of a box of n DOFs for the predicted fraction y."""
    k = np.ceil(np.asarray(y) * n)
    ell = np.maximum(np.ceil(headroom * k) + extra, 12)
    return np.minimum(ell, np.asarray(n) + 16).astype(int)
