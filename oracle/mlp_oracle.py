"""CPU oracle of the warm-start network (TEST INFRASTRUCTURE ONLY).

Only tests/ and the bench's checks import this module.  It restates the device MLP of
itensorcpd.jl_gb300/csrc/k_mlp.cu in numpy so that the device forward pass and gradients
can be checked:

    h1 = relu(bf16(x) bf16(W1)^T + b1), h2 = relu(bf16(h1) bf16(W2)^T + b2),
    y = bf16(h2) bf16(W3)^T + b3,  loss = mean((y - t)^2)

with every GEMM operand rounded to BF16 (round to nearest even) as the device stores it
and the products accumulated in FP64 here (FP32 on the device).  The backward pass rounds
the output gradient and the masked hidden gradients to BF16 before their GEMMs, as the
device does.  There is no counterpart in the reference (the warm start is new to this
build), so this restatement follows the equations above and Adam (Kingma and Ba 2015).
"""
from __future__ import annotations

import numpy as np


def bf16(x) -> np.ndarray:
    """Round FP32 values to BF16 (nearest, ties to even), returned as FP32."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32)).view(np.uint32)
    r = ((a >> 16) & 1) + np.uint32(0x7FFF)
    return ((a + r) & np.uint32(0xFFFF0000)).view(np.float32)


def split_params(p, widths):
    """W1 [h1][in], b1, W2 [h2][h1], b2, W3 [out][h2], b3 from the flat FP32 vector."""
    out, o = [], 0
    for l in range(3):
        n_in, n_out = widths[l], widths[l + 1]
        W = p[o:o + n_out * n_in].reshape(n_out, n_in)
        o += n_out * n_in
        b = p[o:o + n_out]
        o += n_out
        out += [W, b]
    return out


def init_params(widths, rng) -> np.ndarray:
    """He-uniform weights, zero biases (FP32 flat vector)."""
    parts = []
    for l in range(3):
        n_in, n_out = widths[l], widths[l + 1]
        lim = np.sqrt(6.0 / n_in)
        parts.append(rng.uniform(-lim, lim, size=n_out * n_in).astype(np.float32))
        parts.append(np.zeros(n_out, dtype=np.float32))
    return np.concatenate(parts)


def forward(p, widths, x):
    W1, b1, W2, b2, W3, b3 = split_params(np.asarray(p, np.float32), widths)
    xb = bf16(x).astype(np.float64)
    h1 = np.maximum(xb @ bf16(W1).astype(np.float64).T + b1, 0.0).astype(np.float32)
    h2 = np.maximum(bf16(h1).astype(np.float64) @ bf16(W2).astype(np.float64).T + b2, 0.0).astype(np.float32)
    y = (bf16(h2).astype(np.float64) @ bf16(W3).astype(np.float64).T + b3).astype(np.float32)
    return y, (xb, h1, h2)


def loss_and_gradients(p, widths, x, t):
    W1, b1, W2, b2, W3, b3 = split_params(np.asarray(p, np.float32), widths)
    y, (xb, h1, h2) = forward(p, widths, x)
    n = y.size
    d = y.astype(np.float64) - np.asarray(t, np.float64)
    loss = float(np.sum(d * d) / n)
    dy = (2.0 * d / n).astype(np.float32)
    dyb = bf16(dy).astype(np.float64)
    h1b, h2b = bf16(h1).astype(np.float64), bf16(h2).astype(np.float64)
    gW3 = dyb.T @ h2b
    gb3 = dy.astype(np.float64).sum(axis=0)
    dh2 = (dyb @ bf16(W3).astype(np.float64)).astype(np.float32) * (bf16(h2) > 0)
    dh2b = bf16(dh2).astype(np.float64)
    gW2 = dh2b.T @ h1b
    gb2 = dh2.astype(np.float64).sum(axis=0)
    dh1 = (dh2b @ bf16(W2).astype(np.float64)).astype(np.float32) * (bf16(h1) > 0)
    dh1b = bf16(dh1).astype(np.float64)
    gW1 = dh1b.T @ xb
    gb1 = dh1.astype(np.float64).sum(axis=0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g
