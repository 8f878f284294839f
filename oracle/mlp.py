"""FP64 CPU restatement of the acceptance network (TEST INFRASTRUCTURE ONLY).

8 -> 64 -> 64 -> 1 with ReLU; the weights and every layer input are rounded
to bfloat16 (round to nearest even) exactly as the GPU kernels do, the rest
is FP64.  Loss: mean squared error.  Gradients are with respect to the FP32
master weights, with the BF16 rounding treated as the identity (the
straight-through convention of the GPU trainer).  Used to check the GPU's
forward/backward kernels (bh_mlp_gradient) and the traversal's fused
inference.  The network has no counterpart in the reference.
"""
from __future__ import annotations

import numpy as np

FEAT, HID = 8, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + HID * FEAT
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID
NPARAMS = OFF_B3 + 1


def bf16(x) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    finite = (u & 0x7F800000) != 0x7F800000
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) & 0xFFFF0000).astype(np.uint32)
    r = np.where(finite, r, a.view(np.uint32))
    return r.view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float32)
    return (p[OFF_W1:OFF_B1].reshape(HID, FEAT), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(HID, HID),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3], p[OFF_B3])


def forward(p, X):
    """Returns (y, cache) for inputs X (n, 8)."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    xb = bf16(X)
    a1 = b1.astype(np.float64) + xb @ bf16(W1).T
    h1 = bf16(np.maximum(a1, 0.0))
    a2 = b2.astype(np.float64) + h1 @ bf16(W2).T
    h2 = bf16(np.maximum(a2, 0.0))
    y = float(b3) + h2 @ bf16(W3)
    return y, (xb, h1, h2)


def loss_and_grad(p, X, T):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    y, (xb, h1, h2) = forward(p, X)
    n = len(T)
    diff = y - np.asarray(T, np.float64)
    loss = float(np.mean(diff * diff))
    dy = 2.0 * diff / n
    dh2 = np.where(h2 > 0, dy[:, None] * bf16(W3)[None, :], 0.0)
    dh1 = np.where(h1 > 0, dh2 @ bf16(W2), 0.0)
    g = np.zeros(NPARAMS)
    g[OFF_W1:OFF_B1] = (dh1.T @ xb).ravel()
    g[OFF_B1:OFF_W2] = dh1.sum(0)
    g[OFF_W2:OFF_B2] = (dh2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = dh2.sum(0)
    g[OFF_W3:OFF_B3] = dy @ h2
    g[OFF_B3] = dy.sum()
    return loss, g
