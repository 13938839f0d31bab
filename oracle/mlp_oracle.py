"""CPU ORACLE of the planner network (test infrastructure only).

Float64 restatement of the 24 -> 64 -> 64 -> 2 ReLU network the planner trains on the GPU: the FP32
master weights are rounded to BF16 (round to nearest even) exactly as the device does before use,
the forward pass and the gradient of mean_n sum_k (y_k - t_k)^2 are computed in float64 with
respect to those BF16 weights. Only tests import this module; it checks the device's forward and
backward kernels, and is itself pinned by finite differences.
"""
from __future__ import annotations

import numpy as np

N_IN, N_H, N_OUT = 24, 64, 2
W1 = 0
B1 = W1 + N_H * N_IN
W2 = B1 + N_H
B2 = W2 + N_H * N_H
W3 = B2 + N_H
B3 = W3 + N_OUT * N_H
NPARAM = B3 + N_OUT


def to_bf16(w: np.ndarray) -> np.ndarray:
    """FP32 -> BF16 (round to nearest, ties to even), returned widened to float32."""
    u = np.ascontiguousarray(w, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(w: np.ndarray):
    w = np.asarray(w, np.float64)
    return (w[W1:B1].reshape(N_H, N_IN), w[B1:W2], w[W2:B2].reshape(N_H, N_H), w[B2:W3],
            w[W3:B3].reshape(N_OUT, N_H), w[B3:NPARAM])


def forward(w_master: np.ndarray, x: np.ndarray):
    a1w, a1b, a2w, a2b, a3w, a3b = unpack(to_bf16(w_master))
    x = np.asarray(x, np.float64)
    h1 = np.maximum(x @ a1w.T + a1b, 0.0)
    h2 = np.maximum(h1 @ a2w.T + a2b, 0.0)
    y = h2 @ a3w.T + a3b
    return y, (x, h1, h2)


def loss_and_grad(w_master: np.ndarray, x: np.ndarray, t: np.ndarray):
    """Mean squared error over the samples and its gradient with respect to the BF16 weights."""
    a1w, a1b, a2w, a2b, a3w, a3b = unpack(to_bf16(w_master))
    y, (x, h1, h2) = forward(w_master, x)
    n = x.shape[0]
    r = y - np.asarray(t, np.float64)
    loss = float((r * r).sum() / n)
    d3 = 2.0 * r / n
    g3w = d3.T @ h2
    g3b = d3.sum(0)
    d2 = (d3 @ a3w) * (h2 > 0)
    g2w = d2.T @ h1
    g2b = d2.sum(0)
    d1 = (d2 @ a2w) * (h1 > 0)
    g1w = d1.T @ x
    g1b = d1.sum(0)
    g = np.concatenate([g1w.ravel(), g1b, g2w.ravel(), g2b, g3w.ravel(), g3b])
    return loss, g, y


def loss_of_bf16_weights(w_bf16: np.ndarray, x: np.ndarray, t: np.ndarray) -> float:
    """The same loss as a function of the (already rounded) weights, in float64, for finite
    differences."""
    a1w, a1b, a2w, a2b, a3w, a3b = unpack(w_bf16)
    x = np.asarray(x, np.float64)
    h1 = np.maximum(x @ a1w.T + a1b, 0.0)
    h2 = np.maximum(h1 @ a2w.T + a2b, 0.0)
    y = h2 @ a3w.T + a3b
    r = y - np.asarray(t, np.float64)
    return float((r * r).sum() / x.shape[0])
