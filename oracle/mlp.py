"""FP64 NumPy restatement of the scan-surrogate MLP -- TEST INFRASTRUCTURE ONLY.

The network (no counterpart in the reference; the learned part of the scan
path): inputs H0 (bf16), hidden layers H_l = ReLU(H_{l-1} W_l^T + b_l) stored
as bf16 for the next layer, output Y = H_L W_o^T + b_o (float), MSE loss
mean((Y - T)^2). The GPU computes in FP32 on bf16 operands; this oracle does
the same products in float64 and rounds to bf16 at exactly the points where
the GPU does (GEMM operands), so the two agree up to float32 accumulation
order and the rare bf16 rounding flip it causes.
"""
from __future__ import annotations

import numpy as np


def bf16(x):
    """Round to bfloat16 (round to nearest even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) >> 16 << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(H0, Ws, bs):
    """H0 (B, K0) bf16-valued; Ws[l] (N_l, K_l) bf16-valued; bs[l] (N_l,).
    Returns (post-activations per hidden layer (float64), output Y)."""
    H = [np.asarray(H0, dtype=np.float64)]
    posts = []
    for l in range(len(Ws) - 1):
        pre = H[-1] @ np.asarray(Ws[l], np.float64).T + np.asarray(bs[l], np.float64)
        post = np.maximum(pre, 0.0).astype(np.float32).astype(np.float64)
        posts.append(post)
        H.append(bf16(post))
    Y = (H[-1] @ np.asarray(Ws[-1], np.float64).T + np.asarray(bs[-1], np.float64))
    return H, posts, Y.astype(np.float32).astype(np.float64)


def backward(H, posts, Y, T, Ws, col_w=None):
    """Gradients of mean(w (Y - T)^2) (w per output column, 1 without
    ``col_w``) w.r.t. every W and b, with the GPU's rounding points: bf16
    gradient operands, float bias sums."""
    n = Y.size
    w = np.ones(Y.shape[1]) if col_w is None else np.asarray(col_w, np.float64)
    g = (2.0 * w * (Y - T) / n).astype(np.float32).astype(np.float64)
    dWs, dbs = [None] * len(Ws), [None] * len(Ws)
    for l in range(len(Ws) - 1, -1, -1):
        gb = bf16(g)
        dWs[l] = gb.T @ H[l]
        dbs[l] = g.sum(axis=0)
        if l == 0:
            break
        dH = (gb @ np.asarray(Ws[l], np.float64)).astype(np.float32).astype(np.float64)
        g = np.where(posts[l - 1] > 0.0, dH, 0.0)
    loss = float(np.mean(w * (Y - T) ** 2))
    return dWs, dbs, loss
