"""ctypes front end of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Only tests, the smoke check and the benchmark's CPU-baseline leg use this
module; the library never imports it. See xpbi_oracle.cpp for what it
restates and its parity status.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        u32p = C.POINTER(C.c_uint32)
        for name, real in (("xo_substep_f32", C.c_float), ("xo_substep_f64", C.c_double)):
            f = getattr(L, name)
            rp = C.POINTER(real)
            f.restype = C.c_int
            f.argtypes = [u32p, u32p, C.c_uint32, rp, rp, rp, rp, rp, u32p, u32p,
                          C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.xo_svd3_f32.argtypes = [C.POINTER(C.c_float)] * 4
        L.xo_return_map_f64.argtypes = [u32p, C.c_double, C.c_uint32, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.xo_return_map_f32.argtypes = [u32p, C.c_float, C.c_uint32, C.POINTER(C.c_float),
                                        C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.xo_stvk_f64.argtypes = [C.c_double, C.c_double, C.c_uint32] + [C.POINTER(C.c_double)] * 3
        L.xo_kernel_f64.argtypes = [C.c_double, C.c_uint32] + [C.POINTER(C.c_double)] * 3
        L.xo_pbf_kernels_f64.argtypes = [C.c_double, C.c_uint32] + [C.POINTER(C.c_double)] * 3
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def substep(params_words, material_words, state: dict, iterations: int, has_water: bool,
            pbf_iterations: int = -1, substeps: int = 1, threads: int = 0, f64: bool = False) -> dict:
    """Run `substeps` substeps from `state` (reference layouts, see
    read_state) and return the new state. `f64` computes in double."""
    dt = np.float64 if f64 else np.float32
    real = C.c_double if f64 else C.c_float
    n = len(state["pos"])
    nc = int(params_words[7])
    out = {k: np.ascontiguousarray(state[k], dt).copy() for k in ("pos", "vel", "F", "aux")}
    L = state.get("L")
    out["L"] = np.zeros((n, 12), dt) if L is None else np.ascontiguousarray(L, dt).copy()
    out["sortedIdx"] = np.zeros(n, np.uint32)
    out["cellTab"] = np.zeros(nc, np.uint32)
    pw = np.ascontiguousarray(params_words, np.uint32)
    mw = np.ascontiguousarray(material_words, np.uint32)
    fn = lib().xo_substep_f64 if f64 else lib().xo_substep_f32
    rc = fn(_p(pw, C.c_uint32), _p(mw, C.c_uint32), n, _p(out["pos"], real), _p(out["vel"], real),
            _p(out["F"], real), _p(out["L"], real), _p(out["aux"], real), _p(out["sortedIdx"], C.c_uint32),
            _p(out["cellTab"], C.c_uint32), iterations, 1 if has_water else 0, pbf_iterations, substeps, threads)
    if rc != 0:
        raise RuntimeError(f"oracle substep failed ({rc})")
    return out


def svd3(F9):
    F = np.ascontiguousarray(F9, np.float32).reshape(9)
    U = np.zeros(9, np.float32)
    s = np.zeros(3, np.float32)
    V = np.zeros(9, np.float32)
    lib().xo_svd3_f32(_p(F, C.c_float), _p(U, C.c_float), _p(s, C.c_float), _p(V, C.c_float))
    return U.reshape(3, 3).T, s, V.reshape(3, 3).T  # rows = matrix rows


def return_map(mat16, dt, sig, state, f64=True):
    dtype, real = (np.float64, C.c_double) if f64 else (np.float32, C.c_float)
    sig = np.ascontiguousarray(sig, dtype).reshape(-1, 3)
    out = np.zeros_like(sig)
    st = np.ascontiguousarray(state, dtype).copy()
    mw = np.ascontiguousarray(mat16, np.uint32)
    fn = lib().xo_return_map_f64 if f64 else lib().xo_return_map_f32
    fn(_p(mw, C.c_uint32), dt, len(sig), _p(sig, real), _p(out, real), _p(st, real))
    return out, st


def stvk(mu, lam, sig):
    sig = np.ascontiguousarray(sig, np.float64).reshape(-1, 3)
    psi = np.zeros(len(sig))
    d = np.zeros_like(sig)
    lib().xo_stvk_f64(mu, lam, len(sig), _p(sig, C.c_double), _p(psi, C.c_double), _p(d, C.c_double))
    return psi, d


def wendland(h, dx):
    dx = np.ascontiguousarray(dx, np.float64).reshape(-1, 3)
    w = np.zeros(len(dx))
    g = np.zeros_like(dx)
    lib().xo_kernel_f64(h, len(dx), _p(dx, C.c_double), _p(w, C.c_double), _p(g, C.c_double))
    return w, g


def pbf_kernels(h, dx):
    dx = np.ascontiguousarray(dx, np.float64).reshape(-1, 3)
    w = np.zeros(len(dx))
    g = np.zeros_like(dx)
    lib().xo_pbf_kernels_f64(h, len(dx), _p(dx, C.c_double), _p(w, C.c_double), _p(g, C.c_double))
    return w, g


def initial_state(scene: dict) -> dict:
    """createBuffers' initial upload (sim.js:52-81) in the reference layouts."""
    p = np.asarray(scene["positions"], np.float32).reshape(-1, 3)
    n = len(p)
    seeds = scene.get("colorSeeds")
    seeds = np.zeros(n, np.float32) if seeds is None else np.asarray(seeds, np.float32)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = p
    pos[:, 3] = np.asarray(scene["matIds"], np.float32) + seeds
    vel = np.zeros((n, 4), np.float32)
    if scene.get("velocities") is not None:
        vel[:, :3] = np.asarray(scene["velocities"], np.float32).reshape(-1, 3)
    F = np.zeros((n, 12), np.float32)
    F[:, 0] = F[:, 5] = F[:, 10] = 1.0
    aux = np.zeros((n, 4), np.float32)
    aux[:, 0] = np.float32(float(scene["h"]) ** 3)
    st = scene.get("states")
    if st is not None:
        aux[:, 2] = np.asarray(st, np.float32)
    return dict(pos=pos, vel=vel, F=F, L=np.zeros((n, 12), np.float32), aux=aux)


if __name__ == "__main__":
    print(os.path.dirname(__file__))
