"""FP64 CPU restatement of the learned step-size proposer's network
(16 -> 64 -> 64 -> 1, SiLU) -- test infrastructure only: the oracle for the
GPU training kernels' forward pass and gradients.  The reference has no
learned component; this module restates the standard MLP algebra
(h = SiLU(W x + b)), nothing else.
"""
from __future__ import annotations

import numpy as np

IN, HID = 16, 64


def unpack(m) -> dict:
    """Fields of a gb_mlp ctypes structure as float64 arrays."""
    g = lambda name: np.ctypeslib.as_array(getattr(m, name)).astype(np.float64)
    return {"w1": g("w1"), "b1": g("b1"), "w2": g("w2"), "b2": g("b2"), "w3": g("w3"),
            "b3": float(m.b3), "in_mean": g("in_mean"), "in_scale": g("in_scale"),
            "out_scale": float(m.out_scale), "out_bias": float(m.out_bias)}


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p: dict, x: np.ndarray):
    xn = (x - p["in_mean"]) * p["in_scale"]
    z1 = xn @ p["w1"].T + p["b1"]
    h1 = silu(z1)
    z2 = h1 @ p["w2"].T + p["b2"]
    h2 = silu(z2)
    y = h2 @ p["w3"] + p["b3"]
    return p["out_scale"] * y + p["out_bias"], (xn, z1, h1, z2, h2)


def backward(p: dict, x: np.ndarray, dy: np.ndarray) -> dict:
    """Gradients of sum_b dy_b * out_b with respect to the trainable weights."""
    _, (xn, z1, h1, z2, h2) = forward(p, x)
    g = dy * p["out_scale"]
    gw3 = h2.T @ g
    gb3 = g.sum()
    dz2 = (g[:, None] * p["w3"][None, :]) * dsilu(z2)
    gw2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ p["w2"]) * dsilu(z1)
    gw1 = dz1.T @ xn
    gb1 = dz1.sum(0)
    return {"w1": gw1, "b1": gb1, "w2": gw2, "b2": gb2, "w3": gw3, "b3": gb3}


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round-to-nearest-even to bfloat16, returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    r = ((u + rounding) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)
