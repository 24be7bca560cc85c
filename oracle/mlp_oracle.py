"""CPU oracle of the learned cost model's perceptron (TEST INFRASTRUCTURE
ONLY; the product trains and infers with the kernels of
qflex_gb300/csrc/mlp.cu). Same parameter packing: W1[h][d], b1[h],
W2[h][h], b2[h], W3[h], b3; loss = mean((y - target)^2). Float64."""
from __future__ import annotations

import numpy as np


def unpack(p: np.ndarray, d: int, h: int):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + h * d].reshape(h, d); o += h * d
    b1 = p[o:o + h]; o += h
    W2 = p[o:o + h * h].reshape(h, h); o += h * h
    b2 = p[o:o + h]; o += h
    W3 = p[o:o + h]; o += h
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def forward(p, X, d, h):
    W1, b1, W2, b2, W3, b3 = unpack(p, d, h)
    X = np.asarray(X, dtype=np.float64)
    H1 = np.maximum(X @ W1.T + b1, 0)
    H2 = np.maximum(H1 @ W2.T + b2, 0)
    return H2 @ W3 + b3, H1, H2


def loss_grad(p, X, t, d, h):
    W1, b1, W2, b2, W3, b3 = unpack(p, d, h)
    X = np.asarray(X, dtype=np.float64)
    y, H1, H2 = forward(p, X, d, h)
    n = len(y)
    e = y - np.asarray(t, dtype=np.float64)
    loss = float(np.mean(e ** 2))
    dy = 2 * e / n
    gW3 = H2.T @ dy
    gb3 = dy.sum()
    dH2 = np.outer(dy, W3) * (H2 > 0)
    gW2 = dH2.T @ H1
    gb2 = dH2.sum(axis=0)
    dH1 = (dH2 @ W2) * (H1 > 0)
    gW1 = dH1.T @ X
    gb1 = dH1.sum(axis=0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, g
