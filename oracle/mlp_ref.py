"""ORACLE -- test infrastructure only (never imported by the product).

FP64 numpy forward/backward of the learned preconditioner's network and loss
(the network of adc_ottawa_gb300/csrc/mlp.cu), used to check the GPU
training kernels' gradients.  BF16 rounding is applied at the points where
the device rounds (inputs, weights, hidden activations, back-propagated
pre-activation gradients); everything else is FP64.

  Z1 = X W1^T + b1, H1 = silu(Z1), Z2 = H1 W2^T + b2, H2 = silu(Z2),
  m = H2 w3 + b3, t = m t0, per group: L = 1 - <t,e>^2 / (|t|^2 |e|^2).
"""
from __future__ import annotations

import numpy as np

NIN, H = 16, 256


def bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.asarray(x, np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + H * NIN].reshape(H, NIN); o += H * NIN
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    return W1, b1, W2, b2, w3, p[o]


def loss_and_grad(p, F, t0, e, G, S):
    """Returns (mean loss, gradient summed over groups) like the device."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    X = bf16(F)
    W1b, W2b = bf16(W1), bf16(W2)
    Z1 = X @ W1b.T + b1
    H1 = bf16(silu(Z1))
    Z2 = H1 @ W2b.T + b2
    H2 = bf16(silu(Z2))
    m = H2 @ w3 + b3
    t0 = np.asarray(t0, np.float64).reshape(G, S)
    e = np.asarray(e, np.float64).reshape(G, S)
    t = m.reshape(G, S) * t0
    a = (t * e).sum(1, keepdims=True)
    b = np.maximum((t * t).sum(1, keepdims=True), 1e-30)
    c = np.maximum((e * e).sum(1, keepdims=True), 1e-30)
    L = 1.0 - a * a / (b * c)
    dLdt = -2 * a / (b * c) * e + 2 * a * a / (b * b * c) * t
    dm = (dLdt * t0).reshape(-1)
    gw3 = H2.T @ dm
    gb3 = dm.sum()
    dZ2 = bf16(dm[:, None] * w3[None, :] * dsilu(Z2))
    gb2 = dZ2.sum(0)
    gW2 = dZ2.T @ H1
    dH1 = dZ2 @ W2b
    dZ1 = bf16(dH1 * dsilu(Z1))
    gb1 = dZ1.sum(0)
    gW1 = dZ1.T @ X
    grad = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gw3, [gb3]])
    return float(L.mean()), grad


def forward_m(p, F):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    X = bf16(F)
    H1 = bf16(silu(X @ bf16(W1).T + b1))
    H2 = silu(H1 @ bf16(W2).T + b2)
    return H2 @ w3 + b3
