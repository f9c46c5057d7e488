"""The warm-start network through the C ABI (tensor-core kernels).

Parameters are one f32 vector of ``param_count()`` entries:
W1[64][16] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] w4[64] b4.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._abi import check, lib


def _f(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def param_count() -> int:
    return int(lib().xpbi_mlp_param_count())


def forward(X, params):
    X = np.ascontiguousarray(X, np.float32).reshape(-1, 16)
    p = np.ascontiguousarray(params, np.float32)
    y = np.empty(len(X), np.float32)
    check(lib().xpbi_mlp_forward(_f(X), len(X), _f(p), _f(y)))
    return y


def grad(X, T, params):
    X = np.ascontiguousarray(X, np.float32).reshape(-1, 16)
    T = np.ascontiguousarray(T, np.float32)
    p = np.ascontiguousarray(params, np.float32)
    g = np.empty(param_count(), np.float32)
    loss = np.zeros(1, np.float32)
    check(lib().xpbi_mlp_grad(_f(X), _f(T), len(X), _f(p), _f(g), _f(loss)))
    return g, float(loss[0])


def train(X, T, params, steps: int, batch: int, lr: float):
    """Adam on the GPU; returns (trained params, per-step loss)."""
    X = np.ascontiguousarray(X, np.float32).reshape(-1, 16)
    T = np.ascontiguousarray(T, np.float32)
    p = np.ascontiguousarray(params, np.float32).copy()
    hist = np.zeros(max(steps, 1), np.float32)
    check(lib().xpbi_mlp_train(_f(X), _f(T), len(X), _f(p), steps, batch, lr, _f(hist)))
    return p, hist[:steps]
