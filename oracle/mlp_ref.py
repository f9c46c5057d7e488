"""CPU restatement of the warm-start network — TEST INFRASTRUCTURE ONLY.

Forward and backward of the 16 -> 64 -> 64 -> 64 -> 1 SiLU MLP exactly as
the library's tensor-core kernels define them: bf16 (round-to-nearest-even)
weights and layer inputs, f32 biases, f32 output layer on the f32 SiLU of
the last pre-activation, mean squared error over the rows. Used to check the
GPU forward values and gradients.
"""
from __future__ import annotations

import numpy as np

IN, HID = 16, 64
SIZES = [("W1", (HID, IN)), ("b1", (HID,)), ("W2", (HID, HID)), ("b2", (HID,)), ("W3", (HID, HID)),
         ("b3", (HID,)), ("w4", (HID,)), ("b4", (1,))]
COUNT = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n], np.float64).reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float32).reshape(-1) for name, _ in SIZES])


def bf16(x):
    """Round f32 values to bf16 (nearest even) and widen back."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def init(seed=0):
    """He-style initialisation used for training from scratch."""
    rng = np.random.default_rng(seed)
    d = {"W1": rng.standard_normal((HID, IN)) * np.sqrt(2.0 / IN), "b1": np.zeros(HID),
         "W2": rng.standard_normal((HID, HID)) * np.sqrt(2.0 / HID), "b2": np.zeros(HID),
         "W3": rng.standard_normal((HID, HID)) * np.sqrt(2.0 / HID), "b3": np.zeros(HID),
         "w4": rng.standard_normal(HID) * np.sqrt(1.0 / HID), "b4": np.zeros(1)}
    return pack(d)


def forward(X, p):
    P = unpack(p)
    a0 = bf16(X)
    z1 = a0 @ bf16(P["W1"]).T + P["b1"]
    a1 = bf16(silu(z1))
    z2 = a1 @ bf16(P["W2"]).T + P["b2"]
    a2 = bf16(silu(z2))
    z3 = a2 @ bf16(P["W3"]).T + P["b3"]
    h3 = silu(z3)
    y = h3 @ bf16(P["w4"]) + P["b4"][0]
    return y, (a0, z1, a1, z2, a2, z3, h3)


def grad(X, T, p):
    """(gradient vector, mean squared error)."""
    P = unpack(p)
    y, (a0, z1, a1, z2, a2, z3, h3) = forward(X, p)
    n = len(X)
    e = y - np.asarray(T, np.float64)
    dy = 2.0 * e / n
    g = {"w4": h3.T @ dy, "b4": np.array([dy.sum()])}
    dz3 = np.outer(dy, bf16(P["w4"])) * dsilu(z3)
    g["W3"] = dz3.T @ a2
    g["b3"] = dz3.sum(0)
    da2 = bf16(dz3) @ bf16(P["W3"])
    dz2 = da2 * dsilu(z2)
    g["W2"] = dz2.T @ a1
    g["b2"] = dz2.sum(0)
    da1 = bf16(dz2) @ bf16(P["W2"])
    dz1 = da1 * dsilu(z1)
    g["W1"] = dz1.T @ a0
    g["b1"] = dz1.sum(0)
    return pack(g).astype(np.float64), float((e * e).mean())
