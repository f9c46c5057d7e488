"""Shared helpers for the GPU-vs-oracle parity tests.

Parity is defined per substep from an identical input state: the GPU state
is read back, the oracle runs one substep from it, the GPU runs the same
substep, and the two results are compared:
  - sort: cell table (cell starts after the scatter) and permutation
    bit-exact;
  - particle state (pos, vel, F, L, V^n = aux.x, plastic state = aux.z):
    normwise relative error max|gpu - oracle| / max|oracle| <= REL_TOL per
    field, FP32;
  - the solver's multipliers (XPBI lambda = aux.y, PBF lambda = aux.w):
    <= MULT_TOL. The PBF multiplier is -C / (...) with C = rho/rho0 - 1, a
    difference of two nearly equal f32 numbers: a rounding-level change of
    rho shifts C by ~1e-7 absolute, which is ~1e-4 relative to the largest
    C of a scene at rest. That conditioning, not the kernels, sets MULT_TOL.
The error of both against the FP64 oracle of the same substep is reported.

Wherever the reference's own kernels are available (oracle/wgsl_ref.py: the
reference's WGSL translated mechanically to C++ and run on the CPU),
run_pair also runs them on the same input and requires the f32 oracle to
equal them bit for bit, so every GPU comparison is against the reference's
code itself.

Where the reference algorithm itself is not reproducible to REL_TOL in f32 —
flowing granular material near F = I, where the Hencky strain log(sigma) of
sigma = 1 + O(1e-4) keeps only ~3 significant digits in f32 and the Jacobi
solve carries that into the velocities — the f32 oracle already differs from
the f64 oracle by more than REL_TOL on the same substep. There a field passes
if the GPU is no further from the f64 oracle than NOISE_FACTOR times the f32
noise envelope of the substep (and no further from the f32 oracle than that
plus the envelope). The envelope is the largest distance from the f64 oracle
over the f32 oracle run on the input and, where the case supplies them, on
inputs whose velocities (for crowded clumps, positions and F as well) carry
a 1e-7 relative perturbation: one f32 run is a single sample of rounding
noise that such a substep amplifies, and the GPU's own (equally valid)
rounding is another sample. The f64 response of such a
state to a 1e-7 input perturbation is 1e-7, so the spread is f32 rounding,
not physics.
"""
from __future__ import annotations

import json
import os

import numpy as np

REL_TOL = 1e-4
MULT_TOL = 1e-3
NOISE_FACTOR = 2.0
FIELDS = ("pos", "vel", "F", "L", "Vn", "state")


def rel(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.size == 0:
        return 0.0
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def run_pair(xp, O, scene, warm: int = 0, iterations=None, has_water=None, params=None, threads: int = 0,
             lanes: int = 0):
    """(state before, GPU state after, f32 oracle after, f64 oracle after);
    lanes: lanes per particle of solveA / solveB (0: the library's choice)."""
    p = xp.params_for(scene) if params is None else params
    it = scene["iterations"] if iterations is None else iterations
    hw = scene["hasWater"] if has_water is None else has_water
    pi = p.get("pbfIterations")
    pi = -1 if pi is None else int(pi)
    with xp.Simulation(scene) as sim:
        sim.write_params(p)
        sim.set_lanes(lanes)
        if warm:
            sim.step(warm, it, hw)
        s0 = sim.read_state()
        pw, mw = sim.uniforms()
        ref = O.substep(pw, mw, s0, it, hw, pi, threads=threads)
        ref64 = O.substep(pw, mw, s0, it, hw, pi, threads=threads, f64=True)
        sim.encode_substep(it, hw)
        s1 = sim.read_state()
    check_against_reference_kernels(pw, mw, s0, it, hw, pi, ref)
    return s0, s1, ref, ref64


def check_against_reference_kernels(pw, mw, s0, it, hw, pi, ref) -> bool:
    """Requires the f32 oracle's substep `ref` to equal the reference's own
    kernels bit for bit on the same input; False if they are unavailable."""
    from oracle import wgsl_ref as W
    if not W.available():
        return False
    wr = W.substep(pw, mw, s0, it, hw, pi)
    for k in ("pos", "vel", "F", "L", "aux", "sortedIdx", "cellTab"):
        assert np.array_equal(wr[k], ref[k]), f"oracle differs from the reference's kernels in {k}"
    return True


def perturbed_runs(O, scene, s0, iterations=None, has_water=None, params=None, xp=None, count: int = 3,
                   positions: bool = False):
    """f32 oracle runs of the substep run_pair checked, from inputs whose
    velocities (and with `positions`, positions and F too) carry a seeded
    1e-7 relative perturbation (the noise envelope of compare); returns a
    callable so the runs happen only when needed. Position perturbations
    suit states driven by overlaps (crowded clumps), whose response to
    rounding is through the contact distances; a sample whose perturbation
    moved a particle across a cell boundary is left out by compare."""
    p = xp.params_for(scene) if params is None else params
    it = scene["iterations"] if iterations is None else iterations
    hw = scene["hasWater"] if has_water is None else has_water
    pi = p.get("pbfIterations")
    pi = -1 if pi is None else int(pi)
    pw, mw = xp.pack_uniforms(scene, p)

    def runs():
        out = []
        for seed in range(count):
            rng = np.random.default_rng(1000 + seed)
            s = dict(s0)
            v = s0["vel"].copy()
            v[:, :3] *= (1.0 + 1e-7 * rng.uniform(-1.0, 1.0, size=(len(v), 3))).astype(np.float32)
            s["vel"] = v
            if positions:
                x = s0["pos"].copy()
                x[:, :3] *= (1.0 + 1e-7 * rng.uniform(-1.0, 1.0, size=(len(x), 3))).astype(np.float32)
                s["pos"] = x
                # F too: V^n = V0 det F weighs every neighbour sum, the
                # Bonet-Lok correction's included
                F = s0["F"].copy()
                F *= (1.0 + 1e-7 * rng.uniform(-1.0, 1.0, size=F.shape)).astype(np.float32)
                s["F"] = F
            out.append(O.substep(pw, mw, s, it, hw, pi))
        return out
    return runs


def _split(st):
    out = {k: st[k] for k in ("pos", "vel", "F", "L")}
    out["Vn"] = st["aux"][:, 0]
    out["lambda"] = st["aux"][:, 1]
    out["state"] = st["aux"][:, 2]
    out["pbf_lambda"] = st["aux"][:, 3]
    return out


def compare(s1, ref, ref64=None, has_pbf: bool = False, perturbed=None) -> dict:
    """Per-field errors; raises AssertionError on a parity failure.

    perturbed: optional callable returning f32 oracle results of the same
    substep from slightly perturbed inputs (called only if a field needs the
    noise envelope)."""
    report = {}
    assert np.array_equal(s1["cellTab"], ref["cellTab"]), "cell table differs"
    assert np.array_equal(s1["sortedIdx"], ref["sortedIdx"]), "sort permutation differs"
    a_, b_ = _split(s1), _split(ref)
    c_ = _split(ref64) if ref64 is not None else None
    mults = ("lambda", "pbf_lambda") if has_pbf else ("lambda",)
    for f in FIELDS + mults:
        report[f] = rel(a_[f], b_[f])
        if c_ is not None:
            report[f + "_gpu_vs_f64"] = rel(a_[f], c_[f])
            report[f + "_f32oracle_vs_f64"] = rel(b_[f], c_[f])
    bad = {}
    for f in FIELDS + mults:
        tol = REL_TOL if f in FIELDS else MULT_TOL
        if report[f] <= tol:
            continue
        if c_ is None:
            bad[f] = report[f]
            continue
        # f32 noise envelope of the reference algorithm on this very substep:
        # how far f32 runs of it land from the f64 oracle
        env = report[f + "_f32oracle_vs_f64"]
        if perturbed is not None:
            if "_pert" not in report:
                # samples sorted like the reference only (a perturbation that
                # moved a particle into another cell permutes the arrays)
                report["_pert"] = [_split(p) for p in perturbed()
                                   if np.array_equal(p["sortedIdx"], ref["sortedIdx"])]
            for p in report["_pert"]:
                env = max(env, rel(p[f], c_[f]))
            report[f + "_f32_envelope"] = env
        floor = max(tol, NOISE_FACTOR * env)
        if report[f + "_gpu_vs_f64"] > floor or report[f] > floor + env:
            bad[f] = report[f]
    report.pop("_pert", None)
    _record(report, bad)
    assert not bad, f"parity failure: {bad} (report {report})"
    return report


def _record(report: dict, bad: dict) -> None:
    """With XPBI_PARITY_REPORT=<file>, append this comparison's errors (GPU
    vs f32 oracle, GPU vs f64 oracle, f32 oracle vs f64 oracle) as one JSON
    line tagged with the running test."""
    path = os.environ.get("XPBI_PARITY_REPORT")
    if not path:
        return
    line = {"test": os.environ.get("PYTEST_CURRENT_TEST", "").split(" ")[0], "pass": not bad,
            "errors": {k: float(v) for k, v in report.items()}}
    with open(path, "a") as f:
        f.write(json.dumps(line) + "\n")
