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

At full size (the 1M-particle dam breach, too large for the oracle in a
test) one substep must give a valid counting sort — a permutation in cell
order whose cell table counts the cells of the positions it was sorted
from — finite state inside the domain, non-positive PBF multipliers, and
the same bytes when repeated from the same state.
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
        sim.write_state(0, pos=s0["pos"], vel=s0["vel"], F=s0["F"], aux=s0["aux"])
        sim.encode_substep(it, True)
        b = sim.read_state()
        pw, _ = sim.uniforms()
    n = len(s0["pos"])
    for k in ("pos", "vel", "F", "L", "aux", "sortedIdx", "cellTab"):
        assert np.array_equal(a[k], b[k]), f"repeat differs in {k}"
    idx = a["sortedIdx"].astype(np.int64)
    assert np.array_equal(np.sort(idx), np.arange(n)), "not a permutation"
    o = pw[0:3].view(np.float32)
    cs = pw[3:4].view(np.float32)[0]
    dims = pw[4:7].astype(np.int64)
    x = s0["pos"][:, :3]
    c = np.clip(np.floor((x - o) / cs), 0, dims - 1).astype(np.int64)
    key = c[:, 0] + c[:, 1] * dims[0] + c[:, 2] * dims[0] * dims[1]
    ks = key[idx]
    assert np.all(np.diff(ks) >= 0), "not in cell order"
    same = np.diff(ks) == 0
    assert np.all(np.diff(idx)[same] < 0), "within a cell, not by descending previous index"
    counts = np.bincount(key, minlength=int(pw[7]))
    assert np.array_equal(a["cellTab"].astype(np.int64), np.concatenate([[0], np.cumsum(counts)[:-1]]))
    for k in ("pos", "vel", "F", "L", "aux"):
        assert np.all(np.isfinite(a[k])), k
    lo = pw[8:11].view(np.float32)
    hi = pw[12:15].view(np.float32)
    assert np.all(a["pos"][:, :3] >= lo) and np.all(a["pos"][:, :3] <= hi)
    assert np.all(a["aux"][:, 3] <= 0.0)
