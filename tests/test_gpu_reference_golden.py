"""The GPU against committed golden substeps of the reference's own kernels,
and size-independent properties of one substep at full benchmark size.

Golden substeps (tests/golden/reference_substeps.npz, made by
tests/golden/make_reference_golden.py from the reference's WGSL kernels):
five small scenes covering every material model, contact, walls, the
collider and both PBF schedules. The GPU starts from each stored input state
with the same uniforms, runs the same substep and must match the stored
result under the parity definition of parity_util (sort bit-exact, state
within 1e-4 relative, with the f32 noise envelope of the oracle where the
reference algorithm itself is ill-conditioned).

At full size (too large for the oracle in a test) — the 1M-particle dam
breach (plain solve), the 4M-particle dam-breach mix under the learned
solve as benchmarked, and the 256-scene mixed batch — one substep must give
every scene a valid counting sort (a permutation in cell order whose cell
table counts the cells of the positions it was sorted from), finite state
inside the domain, non-positive PBF multipliers, and the same bytes when
repeated from the same state; the learned solve must also end every scene
within both tolerances or re-solve it plainly.
"""
import importlib.util
import os

import numpy as np
import pytest

from parity_util import compare

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden():
    spec = importlib.util.spec_from_file_location("make_reference_golden",
                                                  os.path.join(HERE, "golden", "make_reference_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod, np.load(os.path.join(HERE, "golden", "reference_substeps.npz"))


def test_gpu_reproduces_reference_golden_substeps(xp, oracle, built_lib):
    mod, z = _golden()
    for name, sc, over, warm, pbf in mod.cases(xp):
        p = xp.params_for(sc, **over)
        it, hw, pbf_, steps = (int(x) for x in z[f"{name}/run"])
        inp = {k: z[f"{name}/in/{k}"] for k in ("pos", "vel", "F", "aux")}
        with xp.Simulation(sc) as sim:
            sim.write_params(p)
            pw, mw = sim.uniforms()
            assert np.array_equal(pw, z[f"{name}/params"]) and np.array_equal(mw, z[f"{name}/materials"]), name
            sim.write_state(0, pos=inp["pos"], vel=inp["vel"], F=inp["F"], aux=inp["aux"])
            for _ in range(steps):
                sim.encode_substep(it, bool(hw))
            s1 = sim.read_state()
        ref = {k: z[f"{name}/out/{k}"] for k in ("pos", "vel", "F", "L", "aux", "sortedIdx", "cellTab")}
        ref64 = oracle.substep(pw, mw, inp, it, bool(hw), pbf_, steps, f64=True)

        def perturbed():
            out = []
            for seed in range(3):
                rng = np.random.default_rng(2000 + seed)
                s = dict(inp)
                v = inp["vel"].copy()
                v[:, :3] *= (1.0 + 1e-7 * rng.uniform(-1.0, 1.0, size=(len(v), 3))).astype(np.float32)
                s["vel"] = v
                out.append(oracle.substep(pw, mw, s, it, bool(hw), pbf_, steps))
            return out

        rep = compare(s1, ref, ref64, has_pbf=bool(hw), perturbed=perturbed)
        print(name, {k: f"{v:.1e}" for k, v in rep.items() if "_" not in k})


def _check_substep(s0, a, pw, label=""):
    """One substep of a scene from state s0 to a: a counting sort (a
    permutation in cell order, within a cell by descending previous index,
    whose cell table counts the cells of the positions it was sorted from),
    finite state inside the domain, non-positive PBF multipliers."""
    n = len(s0["pos"])
    idx = a["sortedIdx"].astype(np.int64)
    assert np.array_equal(np.sort(idx), np.arange(n)), f"{label}: not a permutation"
    o = pw[0:3].view(np.float32)
    cs = pw[3:4].view(np.float32)[0]
    dims = pw[4:7].astype(np.int64)
    x = s0["pos"][:, :3]
    c = np.clip(np.floor((x - o) / cs), 0, dims - 1).astype(np.int64)
    key = c[:, 0] + c[:, 1] * dims[0] + c[:, 2] * dims[0] * dims[1]
    ks = key[idx]
    assert np.all(np.diff(ks) >= 0), f"{label}: not in cell order"
    same = np.diff(ks) == 0
    assert np.all(np.diff(idx)[same] < 0), f"{label}: within a cell, not by descending previous index"
    counts = np.bincount(key, minlength=int(pw[7]))
    assert np.array_equal(a["cellTab"].astype(np.int64), np.concatenate([[0], np.cumsum(counts)[:-1]])), label
    for k in ("pos", "vel", "F", "L", "aux"):
        assert np.all(np.isfinite(a[k])), f"{label}: {k}"
    lo = pw[8:11].view(np.float32)
    hi = pw[12:15].view(np.float32)
    assert np.all(a["pos"][:, :3] >= lo) and np.all(a["pos"][:, :3] <= hi), label
    assert np.all(a["aux"][:, 3] <= 0.0), label


def _same(a, b, label=""):
    for k in ("pos", "vel", "F", "L", "aux", "sortedIdx", "cellTab"):
        assert np.array_equal(a[k], b[k]), f"{label}: repeat differs in {k}"


def _restore(sim, states):
    for k, st in enumerate(states):
        sim.write_state(k, pos=st["pos"], vel=st["vel"], F=st["F"], aux=st["aux"])


def test_full_size_substep_properties(xp, built_lib):
    sc = xp.scenes.config_dam_breach()
    p = xp.params_for(sc)
    it = sc["iterations"]
    with xp.Simulation(sc) as sim:
        sim.write_params(p)
        sim.step(20, it, True)
        s0 = sim.read_state()
        sim.encode_substep(it, True)
        a = sim.read_state()
        _restore(sim, [s0])
        sim.encode_substep(it, True)
        b = sim.read_state()
        pw, _ = sim.uniforms()
    _same(a, b)
    _check_substep(s0, a, pw)


def test_full_size_learned_mix_properties(xp, built_lib):
    """The benchmark's headline path at its size: the 4M-particle dam-breach
    mix (four 1M scenes, one handle) under the learned solve as benchmarked
    (network warm start, active set share 0.25, iteration cap 30; in the
    substep's graph the device while-loop and the judge's conditional
    re-solve), one substep from the benchmark's state 100 plain substeps in
    (the solids loaded, the water flowing): every scene's sort
    and state valid, the same bytes when the graph substep is repeated from
    the same state (the worklists are appended by atomics in no fixed order;
    no result may depend on it), and every scene either within both
    tolerances — the plain solve's final relative residuals on the same
    substep, median over the scenes — or re-solved plainly by the judge."""
    import importlib
    tw = importlib.import_module("xpbi-webgpu_gb300.train_warm")
    scenes = xp.scenes.config_dam_mix()
    S = len(scenes)
    with xp.Simulation(scenes) as sim:
        for k, sc in enumerate(scenes):
            sim.write_params(xp.params_for(sc), scene=k)
            sim.set_schedule(k, sc["iterations"], sc["hasWater"])
        sim.set_solver(0, 0.0, False, True)  # carries the multipliers the warm start reads
        sim.step(100, -1, True)
        s0 = [sim.read_state(k) for k in range(S)]
        pw = [sim.uniforms(k)[0] for k in range(S)]

        def rel(k):
            r, _ = sim.read_residuals(k)
            c = sim.read_contact_residuals(k)
            return float(r[-1] / r[0]), float(c[-1] / c[0])

        sim.set_solver(0, 0.0, True, False)
        sim.step(1, -1, True)
        plain = [rel(k) for k in range(S)]
        tau = float(np.median([x[0] for x in plain]))
        tau_c = float(np.median([x[1] for x in plain]))
        assert 0.0 < tau <= 1.0 and 0.0 < tau_c <= 1.0, plain
        _restore(sim, s0)
        sim.set_network(tw.load_weights())
        sim.set_active_set(0.25)
        sim.set_max_iterations(30)
        sim.set_solver(1, tau, True, False, contact_rel_tol=tau_c)
        sim.step(1, -1, True)
        a = [sim.read_state(k) for k in range(S)]
        learned = [rel(k) for k in range(S)]
        resolved = [sim.read_fallback(k) for k in range(S)]
        _restore(sim, s0)
        sim.step(1, -1, True)
        b = [sim.read_state(k) for k in range(S)]
    print({"tau": tau, "tau_c": tau_c, "learned": learned, "resolved": resolved})
    for k in range(S):
        _same(a[k], b[k], f"scene {k}")
        _check_substep(s0[k], a[k], pw[k], f"scene {k}")
        reached = learned[k][0] <= tau * 1.0001 and learned[k][1] <= tau_c * 1.0001
        assert reached or resolved[k], (k, learned[k], tau, tau_c)


def test_full_size_batch_properties(xp, built_lib):
    """The 256-scene mixed batch (about 4M particles over 256 scenes of 2k to
    60k particles, every plasticity model, 10 to 20 iterations each) in one
    handle: after three graph substeps, one more gives every scene a valid
    sort and state, and the same bytes when repeated from the same state."""
    scenes = xp.scenes.config_batch(seed=0)
    S = len(scenes)
    hw = any(sc["hasWater"] for sc in scenes)
    with xp.Simulation(scenes) as sim:
        for k, sc in enumerate(scenes):
            sim.write_params(xp.params_for(sc), scene=k)
            sim.set_schedule(k, sc["iterations"], sc["hasWater"])
        sim.step(3, -1, hw)
        s0 = [sim.read_state(k) for k in range(S)]
        pw = [sim.uniforms(k)[0] for k in range(S)]
        sim.step(1, -1, hw)
        a = [sim.read_state(k) for k in range(S)]
        _restore(sim, s0)
        sim.step(1, -1, hw)
        b = [sim.read_state(k) for k in range(S)]
    assert sum(len(x["pos"]) for x in s0) > 3_000_000
    for k in range(S):
        _same(a[k], b[k], f"scene {k}")
        _check_substep(s0[k], a[k], pw[k], f"scene {k}")
