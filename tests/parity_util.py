"""Shared helpers for the GPU-vs-oracle parity tests.

Parity is defined per substep from an identical input state: the GPU state
is read back, the oracle runs one substep from it, the GPU runs the same
substep, and the two results are compared:
  - sort: cell table (cell starts after the scatter) and permutation
    bit-exact;
  - particle state (pos, vel, F, L, aux): normwise relative error
    max|gpu - oracle| / max|oracle| <= REL_TOL per field, FP32.
The error of both against the FP64 oracle of the same substep is reported.
"""
from __future__ import annotations

import numpy as np

REL_TOL = 1e-4
FIELDS = ("pos", "vel", "F", "L", "aux")


def rel(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.size == 0:
        return 0.0
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def run_pair(xp, O, scene, warm: int = 0, iterations=None, has_water=None, params=None, threads: int = 0):
    """(state before, GPU state after, f32 oracle after, f64 oracle after)."""
    p = xp.params_for(scene) if params is None else params
    it = scene["iterations"] if iterations is None else iterations
    hw = scene["hasWater"] if has_water is None else has_water
    pi = p.get("pbfIterations")
    pi = -1 if pi is None else int(pi)
    with xp.Simulation(scene) as sim:
        sim.write_params(p)
        if warm:
            sim.step(warm, it, hw)
        s0 = sim.read_state()
        pw, mw = sim.uniforms()
        ref = O.substep(pw, mw, s0, it, hw, pi, threads=threads)
        ref64 = O.substep(pw, mw, s0, it, hw, pi, threads=threads, f64=True)
        sim.encode_substep(it, hw)
        s1 = sim.read_state()
    return s0, s1, ref, ref64


def compare(s1, ref, ref64=None, has_pbf: bool = False) -> dict:
    """Per-field errors; raises AssertionError on a parity failure."""
    report = {}
    assert np.array_equal(s1["cellTab"], ref["cellTab"]), "cell table differs"
    assert np.array_equal(s1["sortedIdx"], ref["sortedIdx"]), "sort permutation differs"
    for f in FIELDS:
        a, b = s1[f], ref[f]
        if f == "aux" and not has_pbf:
            a, b = a[:, :3], b[:, :3]
        e = rel(a, b)
        report[f] = e
        if ref64 is not None:
            b64 = ref64[f] if not (f == "aux" and not has_pbf) else ref64[f][:, :3]
            report[f + "_gpu_vs_f64"] = rel(a, b64)
            report[f + "_f32oracle_vs_f64"] = rel(b, b64)
    bad = {f: report[f] for f in FIELDS if report[f] > REL_TOL}
    assert not bad, f"parity failure (normwise relative error > {REL_TOL}): {bad}"
    return report
