"""numpy restatement of the selector MLP — TEST INFRASTRUCTURE ONLY.

Same parameter layout, forward pass and loss as the device kernels
(16 -> 64 -> 64 -> one output per arm, ReLU; loss = sum of 0.5*(y - t)^2 / (rows*arms)),
with the backward pass derived by hand; tests compare the device gradients
against these.
"""
from __future__ import annotations

import numpy as np

F, H, K = 16, 64, 10
P = F * H + H + H * H + H + H * K + K


def unpack(w: np.ndarray):
    w = np.asarray(w, np.float64)
    o = 0
    W1 = w[o:o + F * H].reshape(F, H); o += F * H
    b1 = w[o:o + H]; o += H
    W2 = w[o:o + H * H].reshape(H, H); o += H * H
    b2 = w[o:o + H]; o += H
    W3 = w[o:o + H * K].reshape(H, K); o += H * K
    b3 = w[o:o + K]
    return W1, b1, W2, b2, W3, b3


def forward(w, X):
    W1, b1, W2, b2, W3, b3 = unpack(w)
    z1 = X @ W1 + b1
    a1 = np.maximum(z1, 0)
    z2 = a1 @ W2 + b2
    a2 = np.maximum(z2, 0)
    return a2 @ W3 + b3, (z1, a1, z2, a2)


def loss_and_grad(w, X, T):
    X = np.asarray(X, np.float64)
    T = np.asarray(T, np.float64)
    W1, b1, W2, b2, W3, b3 = unpack(w)
    y, (z1, a1, z2, a2) = forward(w, X)
    norm = 1.0 / (X.shape[0] * K)
    d = y - T
    loss = 0.5 * np.sum(d * d) * norm
    dy = d * norm
    gW3 = a2.T @ dy
    gb3 = dy.sum(0)
    dz2 = (dy @ W3.T) * (z2 > 0)
    gW2 = a1.T @ dz2
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2.T) * (z1 > 0)
    gW1 = X.T @ dz1
    gb1 = dz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g


def targets(costs):
    """log2(1 + cost) centred per row, as the trainer builds them."""
    y = np.log2(1.0 + np.maximum(np.asarray(costs, np.float64), 0))
    return y - y.mean(axis=1, keepdims=True)
