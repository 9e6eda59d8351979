"""Oracle of the learned preconditioner network (numpy, CPU) - test infrastructure only.

The network of pyprop_gb300's preconditioner (no counterpart in the reference): bias-free
3-layer ReLU MLP y = W3^T relu(W2^T relu(W1^T x)) with loss mean_rows ||y - t||^2. The
device computes its products from BF16 operands with FP32 accumulation; ``bf16`` rounds a
float array the same way (round to nearest even on the upper 16 bits), so the oracle can
feed the products the values the device sees and keep everything else in float64.
"""
from __future__ import annotations

import numpy as np


def bf16(a):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float64."""
    x = np.ascontiguousarray(a, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    rounded = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    out = rounded.astype(np.uint32).view(np.float32).astype(np.float64)
    nan = np.isnan(x)
    out[nan] = np.nan
    return out


def forward(W, X, round_bf16=True):
    """Activations (h1, h2, y) of the network on rows X; W = (W1, W2, W3) fan-in rows."""
    r = bf16 if round_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    W1, W2, W3 = (r(w) for w in W)
    x = r(X)
    h1 = np.maximum(x @ W1, 0.0)
    h1b = r(h1)
    h2 = np.maximum(h1b @ W2, 0.0)
    h2b = r(h2)
    y = h2b @ W3
    return h1b, h2b, y


def loss_and_gradients(W, X, T, round_bf16=True):
    """Mean-over-rows squared error and its gradients with respect to W1, W2, W3."""
    r = bf16 if round_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    W1, W2, W3 = (r(w) for w in W)
    x = r(X)
    h1, h2, y = forward(W, X, round_bf16)
    B = X.shape[0]
    d = y - T
    loss = float(np.sum(d * d) / B)
    dY = r(2.0 * d / B)
    g3 = h2.T @ dY
    dh2 = r((dY @ W3.T) * (h2 > 0))
    g2 = h1.T @ dh2
    dh1 = r((dh2 @ W2.T) * (h1 > 0))
    g1 = x.T @ dh1
    return loss, (g1, g2, g3)
