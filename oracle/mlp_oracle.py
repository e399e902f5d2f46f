"""ORACLE — test infrastructure only.

numpy (float64) restatement of the pressure-guess MLP's forward pass, loss
and gradient, to check the library's hand-written GPU training kernels. The
network has no counterpart in the reference: it is defined by
mara3p_gb300/csrc/srhd_mlp.cuh (4-64-64-1, tanh, y = log(p E / q)).
"""
from __future__ import annotations

import numpy as np


def invariants(cons: np.ndarray):
    """E = tau + D, q = E^2 - S^2 - D^2 and S^2 in float64, as the kernels do."""
    D, S1, S2, S3, tau = (cons[k] for k in range(5))
    E = tau + D
    SS = S1 * S1 + S2 * S2 + S3 * S3
    q = (E - D) * (E + D) - SS
    return E, q, SS


def raw_features(cons: np.ndarray) -> np.ndarray:
    """cons (5, n) -> features (n, 4): log(q/E^2), S/E, D/E, log((E - S)/E)."""
    E, q, SS = invariants(cons)
    D = cons[0]
    Ef = E.astype(np.float32)
    S = np.sqrt(SS.astype(np.float32))
    f = np.stack([np.log((q / (E * E)).astype(np.float32)), S / Ef, D.astype(np.float32) / Ef,
                  np.log((q + D * D).astype(np.float32) / ((Ef + S) * Ef))], axis=1)
    return f.astype(np.float32)


def target(cons: np.ndarray, p: np.ndarray) -> np.ndarray:
    """y = log(p E / q)."""
    E, q, _ = invariants(cons)
    return np.log(p * E / q).astype(np.float32)


def forward(p: dict, feat: np.ndarray):
    x = (feat.astype(np.float64) - p["norm_shift"]) * p["norm_scale"]
    a1 = x @ p["w1"].astype(np.float64).T + p["b1"]
    h1 = np.tanh(a1)
    a2 = h1 @ p["w2"].astype(np.float64).T + p["b2"]
    h2 = np.tanh(a2)
    y = h2 @ p["w3"].astype(np.float64) + float(p["b3"])
    out = float(p["out_shift"]) + float(p["out_scale"]) * y
    return x, h1, h2, out


def loss_and_gradient(p: dict, feat: np.ndarray, target: np.ndarray):
    """Mean squared error of `out` and its gradient, flattened in the kernels'
    parameter order (w1, b1, w2, b2, w3, b3)."""
    n = feat.shape[0]
    x, h1, h2, out = forward(p, feat)
    err = out - target.astype(np.float64)
    loss = float(np.mean(err * err))
    dy = 2.0 * err / n * float(p["out_scale"])
    g_w3 = h2.T @ dy
    g_b3 = dy.sum()
    da2 = (dy[:, None] * p["w3"][None, :]) * (1.0 - h2 * h2)
    g_w2 = da2.T @ h1
    g_b2 = da2.sum(0)
    da1 = (da2 @ p["w2"].astype(np.float64)) * (1.0 - h1 * h1)
    g_w1 = da1.T @ x
    g_b1 = da1.sum(0)
    flat = np.concatenate([g_w1.ravel(), g_b1, g_w2.ravel(), g_b2, g_w3, [g_b3]])
    return loss, flat
