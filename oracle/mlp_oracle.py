"""TEST INFRASTRUCTURE ONLY: FP64 restatement of the cost-model network.

The learned fusion planner's perceptron (qsim_gb300/csrc/mlp.cu) has no
counterpart in the reference; this file restates its mathematics in numpy
float64 so that the device forward pass, the device gradients and the host
inference can be checked: 16 inputs, two hidden layers of 64 ReLU units,
one linear output, mean-squared-error loss.  Parameter layout: W1 [16][64],
b1 [64], W2 [64][64], b2 [64], W3 [64], b3 [1] (row i holds the weights out
of unit i).  Used by tests/ only.
"""
from __future__ import annotations

import numpy as np

N_IN, N_H = 16, 64
N_PARAMS = N_IN * N_H + N_H + N_H * N_H + N_H + N_H + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + N_IN * N_H].reshape(N_IN, N_H); o += N_IN * N_H
    b1 = p[o:o + N_H]; o += N_H
    W2 = p[o:o + N_H * N_H].reshape(N_H, N_H); o += N_H * N_H
    b2 = p[o:o + N_H]; o += N_H
    W3 = p[o:o + N_H]; o += N_H
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def forward(p, x):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    z1 = x @ W1 + b1
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ W2 + b2
    h2 = np.maximum(z2, 0.0)
    return h2 @ W3 + b3


def loss_and_grad(p, x, y):
    """Mean squared error over the samples and its gradient (flat, in the
    parameter layout)."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = len(y)
    z1 = x @ W1 + b1
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ W2 + b2
    h2 = np.maximum(z2, 0.0)
    pred = h2 @ W3 + b3
    err = pred - y
    loss = float(np.mean(err ** 2))
    d3 = 2.0 * err / n                       # dL/dpred
    gW3 = h2.T @ d3
    gb3 = d3.sum()
    d2 = np.outer(d3, W3) * (z2 > 0)
    gW2 = h1.T @ d2
    gb2 = d2.sum(axis=0)
    d1 = (d2 @ W2.T) * (z1 > 0)
    gW1 = x.T @ d1
    gb1 = d1.sum(axis=0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, g


def finite_difference_grad(p, x, y, idx, h=1e-6):
    """Central differences of the loss for the parameters in `idx`."""
    p = np.asarray(p, dtype=np.float64).copy()
    out = []
    for i in idx:
        old = p[i]
        p[i] = old + h
        lp, _ = loss_and_grad(p, x, y)
        p[i] = old - h
        lm, _ = loss_and_grad(p, x, y)
        p[i] = old
        out.append((lp - lm) / (2 * h))
    return np.array(out)
