"""FP64 restatement of the proposal MLP (4 -> 64 -> 64 -> 1, ReLU) and of the
gradient of its centred squared-error loss.

TEST INFRASTRUCTURE ONLY: the checker for the library's BF16-weight /
FP32-accumulate forward and backward kernels.  The network has no counterpart
in LightGraphs.jl; this file restates the mathematics the kernels implement:

    x' = (x - mean) / stdev
    h1 = relu(W1 x' + b1),  a2 = W2 h1 + b2,  h2 = relu(a2),  y = W3 . h2 + b3
    loss = (1/B) sum_r (e_r - mean(e))^2,   e_r = y_r - target_r

Parameters are laid out as W1[64][4], b1[64], W2[64][64], b2[64], W3[64], b3.
"""
from __future__ import annotations

import numpy as np

H = 64
W1, B1 = 0, 256
W2 = B1 + H
B2 = W2 + H * H
W3 = B2 + H
B3 = W3 + H
NPARAMS = B3 + 1


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[W1:B1].reshape(H, 4), p[B1:W2], p[W2:B2].reshape(H, H), p[B2:W3], p[W3:B3],
            p[B3])


def forward(p, mean, stdev, x, return_cache=False):
    w1, b1, w2, b2, w3, b3 = unpack(p)
    xs = (np.asarray(x, np.float64) - np.asarray(mean, np.float64)) / np.asarray(stdev, np.float64)
    a1 = xs @ w1.T + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ w2.T + b2
    h2 = np.maximum(a2, 0.0)
    y = h2 @ w3 + b3
    if return_cache:
        return y, (xs, a1, h1, a2, h2)
    return y


def loss_and_grad(p, mean, stdev, x, target):
    """(loss, gradient in the parameter layout, pre-activations a1, a2)."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    y, (xs, a1, h1, a2, h2) = forward(p, mean, stdev, x, return_cache=True)
    e = y - np.asarray(target, np.float64)
    B = len(e)
    c = e - e.mean()
    loss = float((c * c).mean())
    gy = 2.0 * c / B
    g = np.zeros(NPARAMS)
    g[W3:B3] = gy @ h2
    g[B3] = gy.sum()
    d2 = np.outer(gy, w3) * (a2 > 0)
    g[W2:B2] = (d2.T @ h1).ravel()
    g[B2:W3] = d2.sum(0)
    d1 = (d2 @ w2) * (a1 > 0)
    g[W1:B1] = (d1.T @ xs).ravel()
    g[B1:W2] = d1.sum(0)
    return loss, g, a1, a2
