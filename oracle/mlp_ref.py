"""TEST INFRASTRUCTURE ONLY: CPU reference of the presize MLP.

The learned presize has no counterpart in the reference, so this is a plain
float64 restatement of the network the library trains and runs: layers
32 -> 128 -> 128 -> 1 with ReLU, parameters flat in the order w1[128][32],
b1[128], w2[128][128], b2[128], w3[128], b3 (include/gls.h), and the Huber
loss on y - target averaged over rows.  The GPU training kernels' gradients
and the two inference kernels' outputs are checked against it; it is pinned
itself by central finite differences in the CPU test suite.
"""
from __future__ import annotations

import numpy as np

IN, HID = 32, 128
SIZES = [("w1", (HID, IN)), ("b1", (HID,)), ("w2", (HID, HID)), ("b2", (HID,)), ("w3", (HID,)), ("b3", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p: np.ndarray) -> dict:
    out, k = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[k:k + n], np.float64).reshape(shape)
        k += n
    return out


def pack(d: dict) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in SIZES])


def forward(p: np.ndarray, X: np.ndarray):
    w = unpack(p)
    X = np.asarray(X, np.float64)
    z1 = X @ w["w1"].T + w["b1"]
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ w["w2"].T + w["b2"]
    h2 = np.maximum(z2, 0.0)
    y = h2 @ w["w3"] + w["b3"][0]
    return y, (X, z1, h1, z2, h2)


def loss_grad(p: np.ndarray, X: np.ndarray, t: np.ndarray, huber: float = 1.0):
    """Mean Huber loss and its gradient with respect to the flat parameters."""
    w = unpack(p)
    y, (X, z1, h1, z2, h2) = forward(p, X)
    n = len(y)
    r = y - np.asarray(t, np.float64)
    a = np.abs(r)
    inside = a <= huber
    loss = np.where(inside, 0.5 * r * r, huber * (a - 0.5 * huber)).mean()
    dy = np.where(inside, r, huber * np.sign(r)) / n
    g = {"w3": h2.T @ dy, "b3": np.array([dy.sum()])}
    dz2 = np.outer(dy, w["w3"]) * (z2 > 0)
    g["w2"] = dz2.T @ h1
    g["b2"] = dz2.sum(0)
    dz1 = (dz2 @ w["w2"]) * (z1 > 0)
    g["w1"] = dz1.T @ X
    g["b1"] = dz1.sum(0)
    return float(loss), pack(g)


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), as float32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def forward_bf16(p: np.ndarray, X: np.ndarray) -> np.ndarray:
    """The tensor-core kernel's arithmetic: BF16 inputs, weights and hidden
    layer 1, exact products, float accumulation, FP32 biases and output layer."""
    w = unpack(np.asarray(p, np.float32))
    xb = bf16(np.asarray(X, np.float32)).astype(np.float64)
    z1 = xb @ bf16(w["w1"].astype(np.float32)).astype(np.float64).T + w["b1"]
    h1 = bf16(np.maximum(z1, 0.0).astype(np.float32)).astype(np.float64)
    z2 = h1 @ bf16(w["w2"].astype(np.float32)).astype(np.float64).T + w["b2"]
    return np.maximum(z2, 0.0) @ w["w3"] + w["b3"][0]
