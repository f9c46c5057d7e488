"""Generate golden substeps from the reference's own kernels.

Runs the reference's WGSL compute kernels (web/js/shaders/common.js and
simkernels.js of Chiplis/xpbi-webgpu, translated mechanically to C++ and
run in the dispatch order of web/js/sim.js:220-272 by oracle/wgsl_ref.py)
on five small seeded scenes that exercise every material model, contact,
the boundary, the collider and PBF: each is rolled forward by the reference
kernels until the motion has developed, and the fixture keeps that input
state and the reference's state one substep later (parity is defined per
substep from an identical input). The result is committed
as reference_substeps.npz; tests/test_oracle.py checks the oracle against
it wherever the reference itself is not at hand.

Usage: python tests/golden/make_reference_golden.py [reference checkout]
"""
from __future__ import annotations

import importlib
import os
import platform
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

IN_FIELDS = ("pos", "vel", "F", "aux")
OUT_FIELDS = ("pos", "vel", "F", "L", "aux", "sortedIdx", "cellTab")


def cases(xp):
    S = xp.scenes
    out = []

    def scene(h, parts, materials, has_water, vel=None, iterations=4, seed=0, **extra):
        rng = np.random.default_rng(seed)
        s = S.base(h)
        s.update(iterations=iterations, **extra)
        pos, mid, st = [], [], []
        for kind, args in parts:
            (S.sample_box if kind == "box" else S.sample_sphere)(rng, pos, mid, st, *args)
        return S._finish(s, rng, pos, mid, st, materials, has_water, vel)

    # 1. Drucker-Prager sand block thrown onto the floor
    sc = scene(0.03, [("box", ([0.4, 0.02, 0.4], [0.64, 0.2, 0.64], 0.03, 0))], [S.SAND(35)], False)
    n = len(sc["positions"])
    sc["velocities"] = np.tile(np.float32([0.5, -2.0, 0.0]), (n, 1))
    out.append(("sand_impact", sc, {}, 25, -1))
    # 2. NACC ball against the x = 0 wall
    sc = scene(0.025, [("sphere", ([0.12, 0.3, 0.5], 0.09, 0.025, 0, 0.2, -0.008))], [S.SNOW_NACC()], False)
    n = len(sc["positions"])
    sc["velocities"] = np.tile(np.float32([-3.0, -1.0, 0.0]), (n, 1))
    out.append(("nacc_wall", sc, {}, 40, -1))
    # 3. von Mises, Herschel-Bulkley (bisection branch) and snow blocks colliding
    mats = [S.PLASTICINE(30), S.GOO(0.5), S.SNOW_CLASSIC()]
    sc = scene(0.03, [("box", ([0.2, 0.02, 0.4], [0.38, 0.14, 0.58], 0.03, 0)),
                      ("box", ([0.42, 0.02, 0.4], [0.58, 0.14, 0.58], 0.03, 1, 0.2, 0.0)),
                      ("box", ([0.62, 0.02, 0.4], [0.8, 0.14, 0.58], 0.03, 2, 0.2, 1.0))], mats, False)
    p = sc["positions"]
    v = np.zeros((len(p), 3), np.float32)
    v[:, 0] = np.where(p[:, 0] < 0.4, 2.0, np.where(p[:, 0] > 0.6, -2.0, 0.0))
    sc["velocities"] = v
    out.append(("vm_hb_snow", sc, {}, 20, -1))
    # 4. water sampled ~7% closer than the kernel spacing (compressed, so
    #    PBF acts) against sand: PBF in the first 2 of 4 iterations, then in
    #    every iteration
    sc = scene(0.03, [("box", ([0.05, 0.02, 0.4], [0.33, 0.3, 0.52], 0.028, 1)),
                      ("box", ([0.34, 0.02, 0.4], [0.46, 0.16, 0.52], 0.03, 0))],
               [S.SAND(30, 0.004), S.WATER_MAT()], True)
    out.append(("water_sand_pbf2", sc, {"pbfIterations": 2}, 4, 2))
    out.append(("water_sand_every", sc, {"pbfIterations": None}, 4, -1))
    # 5. elastic block struck by the moving sphere collider
    sc = scene(0.03, [("box", ([0.4, 0.3, 0.4], [0.6, 0.5, 0.6], 0.03, 0))], [S.ELASTIC_MAT()], False)
    out.append(("elastic_collider", sc, {"colliderActive": True, "colliderPos": [0.5, 0.58, 0.5],
                                         "colliderR": 0.12, "colliderVel": [0.0, -1.0, 0.0]}, 10, -1))
    return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else None
    if ref:
        os.environ["XPBI_REFERENCE"] = ref
    from oracle import oracle as O
    from oracle import wgsl_ref as W
    W.build(force=True)
    xp = importlib.import_module("xpbi-webgpu_gb300")
    blob = {"machine": np.array(platform.machine())}
    names = []
    for name, sc, over, warm, pbf in cases(xp):
        p = xp.params_for(sc, **over)
        pw, mw = xp.pack_uniforms(sc, p)
        it, hw = sc["iterations"], sc["hasWater"]
        st = W.substep(pw, mw, O.initial_state(sc), it, hw, pbf, warm)
        st1 = W.substep(pw, mw, st, it, hw, pbf, 1)
        names.append(name)
        blob[f"{name}/params"] = pw
        blob[f"{name}/materials"] = mw
        blob[f"{name}/run"] = np.array([it, int(hw), pbf, 1], np.int32)
        for k in IN_FIELDS:
            blob[f"{name}/in/{k}"] = st[k]
        for k in OUT_FIELDS:
            blob[f"{name}/out/{k}"] = st1[k]
        print(name, len(sc["positions"]), "particles")
    blob["cases"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "reference_substeps.npz"), **blob)


if __name__ == "__main__":
    main()
