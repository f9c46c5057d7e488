"""Uniform words of the reference's Simulation — TEST INFRASTRUCTURE ONLY.

A NumPy restatement of how web/js/sim.js turns a scene and the frame loop's
parameters into the two uniform buffers its kernels read, so that the CPU
paths (the oracle, the reference's kernels translated to C++) can be driven
without the library under test:
  - grid sizing, sim.js:20-26 (f64: origin = domainMin - 2 cs,
    dims = ceil(extent / cs) + 4, cs = support = 2 h);
  - writeMaterials, sim.js:84-99 (mu, lambda and mass in f64, stored in f32;
    kind as u32 bits; boundFriction defaults to 0.4);
  - writeParams, sim.js:159-186 (37 words of the 64-word Params block);
  - the frame loop's writeParams argument, main.js:385-402
    (dt = (1/60) timeScale / substeps unless the scene fixes dt).
Only tests, the smoke check and the benchmark's CPU leg use it; the ABI's
own packing (xpbi_pack_uniforms) is checked against it.
"""
from __future__ import annotations

import math

import numpy as np

PARAMS_WORDS = 64
MATERIAL_WORDS = 16
MAX_MATERIALS = 8


def _bits(x) -> np.uint32:
    return np.frombuffer(np.float32(x).tobytes(), np.uint32)[0]


def grid(scene: dict):
    """(origin[3] f64, support f64, dims[3], numCells), sim.js:20-26."""
    h = float(scene["h"])
    cs = 2 * h
    pad = 2
    lo, hi = scene["domainMin"], scene["domainMax"]
    origin = [float(lo[k]) - pad * cs for k in range(3)]
    dims = [int(math.ceil((float(hi[k]) - float(lo[k])) / cs)) + 2 * pad for k in range(3)]
    return origin, cs, dims, dims[0] * dims[1] * dims[2]


def frame_params(scene: dict, **over) -> dict:
    """The frame loop's writeParams argument for a scene (main.js:385-402)."""
    dt = scene["dt"] if "dt" in scene else (1 / 60) * scene["timeScale"] / scene["substeps"]
    p = dict(dt=dt, domainMin=scene["domainMin"], domainMax=scene["domainMax"], gravity=scene["gravity"],
             colliderPos=[0.0, 0.0, 0.0], colliderR=0.0, colliderVel=[0.0, 0.0, 0.0], colliderActive=False,
             xsphC=scene.get("xsphC", 0.01), omega=scene.get("omega", 0.5),
             contactOmega=scene.get("contactOmega", 0.4), pbfEps=scene.get("pbfEps", 100.0),
             sCorrK=scene.get("sCorrK", 1e-4), time=0.0, kDamp=scene.get("kDamp", 0.4),
             pbfIterations=scene.get("pbfIterations"))
    p.update(over)
    return p


def material_words(materials, V0: float) -> np.ndarray:
    """writeMaterials (sim.js:84-99): 8 x 16 words."""
    w = np.zeros(MAX_MATERIALS * MATERIAL_WORDS, np.uint32)
    for i, m in enumerate(materials):
        o = i * MATERIAL_WORDS
        E, nu = float(m["E"]), float(m["nu"])
        mu = E / (2 * (1 + nu))
        lam = E * nu / ((1 + nu) * (1 - 2 * nu))
        dens = float(m["density"])
        w[o + 0], w[o + 1], w[o + 2] = _bits(mu), _bits(lam), _bits(dens)
        w[o + 3] = np.uint32(int(m["kind"]))
        for k in range(4):
            v = m.get(f"p{k}")
            w[o + 4 + k] = _bits(0.0 if v is None else float(v))
        col = m.get("color", [0.0, 0.0, 0.0])
        for k in range(3):
            w[o + 8 + k] = _bits(float(col[k]))
        w[o + 11] = _bits(1.0)
        bf = m.get("boundFriction")
        w[o + 12] = _bits(0.4 if bf is None else float(bf))
        w[o + 13] = _bits(dens * V0)  # mass
    return w


def params_words(scene: dict, p: dict) -> np.ndarray:
    """writeParams (sim.js:159-186): the 64-word Params block."""
    origin, cs, dims, cells = grid(scene)
    h = float(scene["h"])
    n = len(np.asarray(scene["positions"]).reshape(-1)) // 3
    w = np.zeros(PARAMS_WORDS, np.uint32)
    for k in range(3):
        w[k] = _bits(origin[k])
        w[4 + k] = np.uint32(dims[k])
        w[8 + k] = _bits(float(p["domainMin"][k]))
        w[12 + k] = _bits(float(p["domainMax"][k]))
        w[16 + k] = _bits(float(p["gravity"][k]))
        w[20 + k] = _bits(float(p.get("colliderPos", [0, 0, 0])[k]))
        w[24 + k] = _bits(float(p.get("colliderVel", [0, 0, 0])[k]))
    w[3] = _bits(cs)
    w[7] = np.uint32(cells)
    w[11] = _bits(float(p["dt"]))
    w[15] = _bits(h)
    w[19] = _bits(cs)
    w[23] = _bits(float(p.get("colliderR", 0.0)))
    w[27] = _bits(1.0 if p.get("colliderActive") else 0.0)
    w[28] = np.uint32(n)
    w[29] = _bits(h ** 3)
    w[30] = _bits(float(p.get("xsphC", 0.01)))
    w[31] = _bits(float(p.get("omega", 0.5)))
    w[32] = _bits(float(p.get("pbfEps", 100.0)))
    w[33] = _bits(float(p.get("sCorrK", 1e-4)))
    w[34] = _bits(float(p.get("time", 0.0)))
    w[35] = _bits(float(p.get("contactOmega", 0.4)))
    kd = p.get("kDamp")
    w[36] = _bits(0.4 if kd is None else float(kd))  # sim.js:184
    return w


def pack(scene: dict, p: dict | None = None):
    """(params words, material words) of a scene and a writeParams argument."""
    if p is None:
        p = frame_params(scene)
    return params_words(scene, p), material_words(scene["materials"], float(scene["h"]) ** 3)
