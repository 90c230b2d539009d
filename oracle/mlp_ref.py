"""ORACLE -- CPU restatement of the learned-entry MLP step (test infrastructure).

The MLP has no counterpart in the reference; this restates the GPU code in
rt_entry_gb300/csrc/learned.cpp (fwd_bwd) in FP64 numpy, rounding to BF16
exactly where the GPU stores BF16 tensors (inputs, weights, hidden
activations, dlogits, hidden gradients), so that the GPU gradients can be
checked against it.  `grads(..., bf16=False)` is the plain FP64 math, which
tests/test_mlp_oracle.py pins against central finite differences.
"""
from __future__ import annotations

import numpy as np


def bf16(x):
    """Round to BF16 (nearest even), returned as float64."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16 << 16).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def _id(x):
    return np.asarray(x, np.float64)


def forward(X, W1, b1, W2, b2, W3, b3, bf=True):
    r = bf16 if bf else _id
    Xb, W1b, W2b, W3b = r(X), r(W1), r(W2), r(W3)
    A1 = Xb @ W1b.T + b1
    H1 = r(np.maximum(A1, 0))
    A2 = H1 @ W2b.T + b2
    H2 = r(np.maximum(A2, 0))
    Z = H2 @ W3b.T + b3
    return Xb, W1b, W2b, W3b, H1, H2, Z


def loss_and_grads(X, y, W1, b1, W2, b2, W3, b3, bf=True):
    """Mean softmax cross-entropy over the batch and its gradients."""
    r = bf16 if bf else _id
    M = X.shape[0]
    Xb, W1b, W2b, W3b, H1, H2, Z = forward(X, W1, b1, W2, b2, W3, b3, bf)
    Zs = Z - Z.max(1, keepdims=True)
    P = np.exp(Zs)
    P /= P.sum(1, keepdims=True)
    loss_rows = -np.log(P[np.arange(M), y])
    G = P.copy()
    G[np.arange(M), y] -= 1.0
    dZ = r(G / M)
    g = {}
    g["W3"] = dZ.T @ H2
    g["b3"] = dZ.sum(0)
    dH2 = r((dZ @ W3b) * (H2 > 0))
    g["W2"] = dH2.T @ H1
    g["b2"] = dH2.sum(0)
    dH1 = r((dH2 @ W2b) * (H1 > 0))
    g["W1"] = dH1.T @ Xb
    g["b1"] = dH1.sum(0)
    return loss_rows, g
