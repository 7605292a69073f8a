"""FP64 CPU oracle of the learned preconditioner's network (test infrastructure).

The reference has no learned component (it solves with plain CG,
CG_CUDA.cuh:256-324); this restates the network the library runs on the tensor
cores (csrc/learned.cu, csrc/mlp.cuh) so that its forward pass and gradients can
be checked:

  y = w3 . relu(W2 relu(W1 x + b1) + b2) + b3,   loss = mean (y - t)^2

Parameters are one float vector (8385): W1 [64 out][64 in], b1 [64], W2 [64][64],
b2 [64], w3 [64], b3.  With ``emulate=True`` the values are rounded to bfloat16
where the library feeds the tensor cores -- W1, W2, h1, and in the backward pass
dz2 and dz1 -- so that the library's results can be compared tightly; with
``emulate=False`` everything is FP64, the reference for finite differences.
"""
from __future__ import annotations

import numpy as np

P_W1, P_B1, P_W2, P_B2, P_W3, P_B3, P_COUNT = 0, 4096, 4160, 8256, 8320, 8384, 8385


def bf16(a):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[P_W1:P_B1].reshape(64, 64), p[P_B1:P_W2], p[P_W2:P_B2].reshape(64, 64), p[P_B2:P_W3],
            p[P_W3:P_B3], p[P_B3])


def forward(p, x, emulate=True):
    """x: [n, 64] (the features, already bfloat16 values)."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    if emulate:
        W1, W2 = bf16(W1), bf16(W2)
    z1 = x @ W1.T + b1
    h1 = np.maximum(z1, 0.0)
    h1m = bf16(h1) if emulate else h1
    z2 = h1m @ W2.T + b2
    h2 = np.maximum(z2, 0.0)
    y = h2 @ w3 + b3
    return y, (x, z1, h1m, z2, h2)


def loss_and_grad(p, x, t, emulate=True):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    if emulate:
        W2 = bf16(W2)
    y, (xx, z1, h1m, z2, h2) = forward(p, x, emulate)
    t = np.asarray(t, dtype=np.float64)
    n = len(t)
    d = y - t
    loss = float(np.mean(d * d))
    dy = 2.0 * d / n
    g = np.zeros(P_COUNT)
    g[P_W3:P_B3] = h2.T @ dy
    g[P_B3] = dy.sum()
    dz2 = np.where(z2 > 0, dy[:, None] * w3[None, :], 0.0)
    g[P_B2:P_W3] = dz2.sum(0)
    dz2m = bf16(dz2) if emulate else dz2
    g[P_W2:P_B2] = (dz2m.T @ h1m).ravel()
    dh1 = dz2m @ W2
    dz1 = np.where(z1 > 0, dh1, 0.0)
    g[P_B1:P_W2] = dz1.sum(0)
    dz1m = bf16(dz1) if emulate else dz1
    g[P_W1:P_B1] = (dz1m.T @ xx).ravel()
    return loss, g


def finite_difference(p, x, t, idx, eps=1e-4):
    """Central differences of the FP64 loss for the parameters in idx."""
    p = np.asarray(p, dtype=np.float64)
    out = np.zeros(len(idx))
    for k, i in enumerate(idx):
        a, b = p.copy(), p.copy()
        a[i] += eps
        b[i] -= eps
        la = np.mean((forward(a, x, False)[0] - t) ** 2)
        lb = np.mean((forward(b, x, False)[0] - t) ** 2)
        out[k] = (la - lb) / (2 * eps)
    return out
