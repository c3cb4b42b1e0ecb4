"""ORACLE (test infrastructure only): numpy restatement of the warm-start
message-passing network, forward and backward, used to check the CUDA
kernels' gradients.  Only ``tests/`` import it; the product never does.

The network (no counterpart in the reference) maps per-cell features x [N,6]
to y [N,3]:

    z0 = x W0^T + b0,                 h0 = relu(z0)
    for l = 1..L:  m_l = A h_{l-1},   z_l = [h_{l-1} | m_l] W_l^T + b_l,
                                      h_l = h_{l-1} + relu(z_l)
    y  = h_L W_out^T + b_out
    loss = sum((y - t)^2) / (3 N)

A_l is layer l's aggregation matrix (the mean over the neighbours through
interior faces, or a bin mean on a coarse grid); ``A`` may be one matrix for
every layer or a list with one per layer.  Weights are the bfloat16 values
the kernels use; the arithmetic here is float64.
"""
from __future__ import annotations

import numpy as np


def bf16_round(a):
    """float32 -> nearest-even bfloat16 value (as float32)."""
    u = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def adjacency(n, row_ptr, col, wt):
    A = np.zeros((n, n))
    for i in range(n):
        for e in range(row_ptr[i], row_ptr[i + 1]):
            A[i, col[e]] += wt[e]
    return A


def forward(params, x, A):
    """params: list of (W, b) float arrays (encoder, L layers, decoder)."""
    x = np.asarray(x, np.float64)
    (W0, b0), *mid, (Wo, bo) = [(np.asarray(W, np.float64), np.asarray(b, np.float64)) for W, b in params]
    cache = {"x": x, "h": [], "z": [], "m": []}
    z = x @ W0.T + b0
    h = np.maximum(z, 0.0)
    cache["z"].append(z)
    cache["h"].append(h)
    As = A if isinstance(A, (list, tuple)) else [A] * len(mid)
    for (W, b), Al in zip(mid, As):
        m = Al @ h
        z = np.concatenate([h, m], 1) @ W.T + b
        h = h + np.maximum(z, 0.0)
        cache["m"].append(m)
        cache["z"].append(z)
        cache["h"].append(h)
    y = h @ Wo.T + bo
    return y, cache


def loss_and_grads(params, x, A, t):
    y, cache = forward(params, x, A)
    t = np.asarray(t, np.float64)
    n = y.size
    loss = float(np.sum((y - t) ** 2) / n)
    dy = 2.0 * (y - t) / n
    P = [(np.asarray(W, np.float64), np.asarray(b, np.float64)) for W, b in params]
    grads = [None] * len(P)
    Wo, _ = P[-1]
    hL = cache["h"][-1]
    grads[-1] = (dy.T @ hL, dy.sum(0))
    dh = dy @ Wo
    As = A if isinstance(A, (list, tuple)) else [A] * (len(P) - 2)
    for l in range(len(P) - 2, 0, -1):
        W, _ = P[l]
        z, hp, m = cache["z"][l], cache["h"][l - 1], cache["m"][l - 1]
        dz = dh * (z > 0)
        grads[l] = (dz.T @ np.concatenate([hp, m], 1), dz.sum(0))
        dx = dz @ W
        d = hp.shape[1]
        dh = dh + dx[:, :d] + As[l - 1].T @ dx[:, d:]
    dz = dh * (cache["z"][0] > 0)
    grads[0] = (dz.T @ cache["x"], dz.sum(0))
    return loss, y, grads
