"""Scene sampling on the GPU (xpbi_sample_shapes): the lattice samplers of
web/js/scenes.js:7-38 for scenes too large to sample quickly on the host.

The lattice points equal scenes.sample_box / scenes.sample_sphere's bit for
bit; the jitter draws come from Philox-4x32-10 keyed by the seed instead of
the host sampler's NumPy generator, so a device-sampled scene is a
different (equally seeded) draw of the same lattice.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._abi import Shape, check, lib

BOX, SPHERE = 0, 1


def box(lo, hi, mat_id: int, jitter: float = 0.2, state0: float = 0.0) -> dict:
    return dict(kind=BOX, lo=lo, hi=hi, mat_id=mat_id, jitter=jitter, state0=state0)


def sphere(centre, radius: float, mat_id: int, jitter: float = 0.2, state0: float = 0.0) -> dict:
    return dict(kind=SPHERE, centre=centre, radius=radius, mat_id=mat_id, jitter=jitter, state0=state0)


def _shapes(shapes):
    arr = (Shape * len(shapes))()
    for k, d in enumerate(shapes):
        arr[k].kind = int(d["kind"])
        for a in range(3):
            arr[k].lo[a] = float(d.get("lo", [0, 0, 0])[a])
            arr[k].hi[a] = float(d.get("hi", [0, 0, 0])[a])
            arr[k].centre[a] = float(d.get("centre", [0, 0, 0])[a])
        arr[k].radius = float(d.get("radius", 0.0))
        arr[k].mat_id = int(d["mat_id"])
        arr[k].state0 = float(d.get("state0", 0.0))
        arr[k].jitter = float(d.get("jitter", 0.2))
    return arr


def sample_shapes(shapes, h: float, seed: int = 0):
    """(positions (N, 3) f32, mat_ids (N,) u32, states (N,) f32)."""
    arr = _shapes(shapes)
    n = C.c_uint32()
    check(lib().xpbi_sample_shapes(arr, len(shapes), float(h), int(seed), 0, None, None, None, C.byref(n)))
    pos = np.empty((n.value, 3), np.float32)
    mid = np.empty(n.value, np.uint32)
    st = np.empty(n.value, np.float32)
    f = C.POINTER(C.c_float)
    u = C.POINTER(C.c_uint32)
    check(lib().xpbi_sample_shapes(arr, len(shapes), float(h), int(seed), n.value, pos.ctypes.data_as(f),
                                   mid.ctypes.data_as(u), st.ctypes.data_as(f), C.byref(n)))
    return pos, mid, st


def philox(counter, key):
    """Philox-4x32-10 on the host (the library's own implementation)."""
    c = np.ascontiguousarray(counter, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    u = C.POINTER(C.c_uint32)
    check(lib().xpbi_philox4x32_10(c.ctypes.data_as(u), k.ctypes.data_as(u), out.ctypes.data_as(u)))
    return out
