"""GPU parity: libxpbi's substep vs the CPU oracle from identical state.

Every case calls the C ABI through the package's ctypes binding, runs the
same substep in the oracle, and checks the sort bit-exactly and the FP32
particle state within 1e-4 normwise relative error (parity_util.REL_TOL).
"""
import numpy as np
import pytest

from parity_util import REL_TOL, compare, perturbed_runs, rel, run_pair

pytestmark = pytest.mark.gpu


def _scene(xp, name, **kw):
    return getattr(xp.scenes, name)(**kw)


@pytest.mark.parametrize("warm", [0, 5])
def test_sand_column_config(xp, oracle, built_lib, warm):
    sc = xp.scenes.config_sand_column()
    s0, s1, ref, ref64 = run_pair(xp, oracle, sc, warm=warm)
    rep = compare(s1, ref, ref64, perturbed=perturbed_runs(oracle, sc, s0, xp=xp))
    print("sand_column", warm, rep)


def test_sand_column_after_collapse_starts(xp, oracle, built_lib):
    sc = xp.scenes.config_sand_column()
    # the column free-falls (uniform velocity, grad v = 0) until its base
    # reaches the floor after ~160 substeps; by 300 it is flowing
    s0, s1, ref, ref64 = run_pair(xp, oracle, sc, warm=300)
    assert np.abs(ref["aux"][:, 1]).max() > 0
    compare(s1, ref, ref64, perturbed=perturbed_runs(oracle, sc, s0, xp=xp))


@pytest.mark.parametrize("name", ["sand_column", "sand_two_blocks", "snowball_smash", "plasticine",
                                  "goo", "snow_classic", "dam_breach", "elastic_block"])
def test_reference_demo_scenes(xp, oracle, built_lib, name):
    sc = _scene(xp, name)
    s0, s1, ref, ref64 = run_pair(xp, oracle, sc, warm=12)
    rep = compare(s1, ref, ref64, has_pbf=sc["hasWater"], perturbed=perturbed_runs(oracle, sc, s0, xp=xp))
    print(name, len(sc["positions"]), rep)


def test_nacc_snowball_wall_impact(xp, oracle, built_lib):
    sc = xp.scenes.config_nacc_snowball()
    # ~120 substeps until the sphere reaches the wall; start near impact
    s0, s1, ref, ref64 = run_pair(xp, oracle, sc, warm=125)
    compare(s1, ref, ref64, perturbed=perturbed_runs(oracle, sc, s0, xp=xp))


def test_dam_breach_small(xp, oracle, built_lib):
    sc = xp.scenes.config_dam_breach(scale=0.05)
    s0, s1, ref, ref64 = run_pair(xp, oracle, sc, warm=10)
    compare(s1, ref, ref64, has_pbf=True, perturbed=perturbed_runs(oracle, sc, s0, xp=xp))


def test_dam_breach_fast_water(xp, oracle, built_lib):
    """Water pushed to 12 m/s before the substep: the PBF passes pair
    particles by predicted positions far from the current ones."""
    sc = xp.scenes.config_dam_breach(scale=0.05)
    p = xp.params_for(sc)
    it = sc["iterations"]
    with xp.Simulation(sc) as sim:
        sim.write_params(p)
        sim.step(10, it, True)
        st = sim.read_state()
        kinds = np.array([m["kind"] for m in sc["materials"]])
        water = kinds[np.abs(st["pos"][:, 3]).astype(int)] == 6
        vel = st["vel"].copy()
        vel[water, 0] += 12.0
        sim.write_state(0, vel=vel)
        s0 = sim.read_state()
        pw, mw = sim.uniforms()
        ref = oracle.substep(pw, mw, s0, it, True, 4)
        ref64 = oracle.substep(pw, mw, s0, it, True, 4, f64=True)
        sim.encode_substep(it, True)
        s1 = sim.read_state()
    assert water.sum() > 0
    compare(s1, ref, ref64, has_pbf=True)


def test_fast_solids_contact_reach(xp, oracle, built_lib):
    """Sand thrown in random directions at up to 4 m/s while it presses on
    the floor: solveB loads a neighbour's predicted position only within
    minD + dt |v_i| + the scene's largest solid displacement, so large and
    uneven displacements must still find every contact pair."""
    sc = xp.scenes.config_sand_column()
    p = xp.params_for(sc)
    it = sc["iterations"]
    with xp.Simulation(sc) as sim:
        sim.write_params(p)
        sim.step(200, it, False)
        st = sim.read_state()
        rng = np.random.default_rng(5)
        vel = st["vel"].copy()
        vel[:, :3] += rng.uniform(-4.0, 4.0, size=(len(vel), 3)).astype(np.float32)
        sim.write_state(0, vel=vel)
        s0 = sim.read_state()
        pw, mw = sim.uniforms()
        ref = oracle.substep(pw, mw, s0, it, False, -1)
        ref64 = oracle.substep(pw, mw, s0, it, False, -1, f64=True)
        sim.encode_substep(it, False)
        s1 = sim.read_state()
    compare(s1, ref, ref64, perturbed=perturbed_runs(oracle, sc, s0, xp=xp))


def test_reference_pbf_interleave(xp, oracle, built_lib):
    """pbfIterations unset: one PBF pass after every XPBI iteration."""
    sc = xp.scenes.config_dam_breach(scale=0.05)
    p = xp.params_for(sc, pbfIterations=None)
    s0, s1, ref, ref64 = run_pair(xp, oracle, sc, warm=3, params=p)
    compare(s1, ref, ref64, has_pbf=True, perturbed=perturbed_runs(oracle, sc, s0, params=p, xp=xp))


def test_collider_active(xp, oracle, built_lib):
    sc = xp.scenes.plasticine()
    p = xp.params_for(sc, colliderActive=True, colliderPos=[0.5, 0.45, 0.5], colliderR=0.08,
                      colliderVel=[0.3, -0.5, 0.0])
    s0, s1, ref, ref64 = run_pair(xp, oracle, sc, warm=4, params=p)
    compare(s1, ref, ref64, perturbed=perturbed_runs(oracle, sc, s0, params=p, xp=xp))


def test_zero_iterations(xp, oracle, built_lib):
    sc = xp.scenes.elastic_block()
    s0, s1, ref, ref64 = run_pair(xp, oracle, sc, warm=2, iterations=0)
    compare(s1, ref, ref64, perturbed=perturbed_runs(oracle, sc, s0, iterations=0, xp=xp))


def test_graph_step_matches_encode(xp, built_lib):
    """xpbi_step (graph replay) and xpbi_encode_substep give identical bytes."""
    sc = xp.scenes.snow_classic()
    p = xp.params_for(sc)
    out = []
    for use_graph in (True, False):
        with xp.Simulation(sc) as sim:
            sim.write_params(p)
            if use_graph:
                sim.step(7, sc["iterations"], False)
            else:
                for _ in range(7):
                    sim.encode_substep(sc["iterations"], False)
            out.append(sim.read_state())
    for k in ("pos", "vel", "F", "aux", "sortedIdx", "cellTab"):
        assert np.array_equal(out[0][k], out[1][k]), k


def test_deterministic_rerun(xp, built_lib):
    sc = xp.scenes.dam_breach()
    p = xp.params_for(sc)
    out = []
    for _ in range(2):
        with xp.Simulation(sc) as sim:
            sim.write_params(p)
            sim.step(10, sc["iterations"], True)
            out.append(sim.read_state())
    for k in ("pos", "vel", "F", "L", "aux", "sortedIdx", "cellTab"):
        assert np.array_equal(out[0][k], out[1][k]), k


def test_batched_scenes_match_single(xp, oracle, built_lib):
    """A batch of uneven scenes with mixed materials: every scene's substep
    matches its own oracle run (sort bit-exact, state within tolerance)."""
    scenes = [xp.scenes.plasticine(), xp.scenes.snowball_smash(), xp.scenes.goo(), xp.scenes.dam_breach(),
              xp.scenes.snow_classic()]
    iters = [4, 3, 5, 2, 6]
    with xp.Simulation(scenes) as sim:
        for k, sc in enumerate(scenes):
            sim.write_params(xp.params_for(sc), scene=k)
            sim.set_schedule(k, iters[k], sc["hasWater"])
        sim.step(3, -1, False)
        states = [sim.read_state(k) for k in range(len(scenes))]
        uni = [sim.uniforms(k) for k in range(len(scenes))]
        sim.encode_substep(-1, False)
        after = [sim.read_state(k) for k in range(len(scenes))]
    for k, sc in enumerate(scenes):
        pw, mw = uni[k]
        ref = oracle.substep(pw, mw, states[k], iters[k], sc["hasWater"], -1)
        ref64 = oracle.substep(pw, mw, states[k], iters[k], sc["hasWater"], -1, f64=True)
        compare(after[k], ref, ref64, has_pbf=sc["hasWater"])


@pytest.mark.parametrize("lanes", [0, 4])
def test_mixed_batch_sample_of_the_256_scene_config(xp, oracle, built_lib, lanes):
    """Twenty scenes of the batched config's distribution (seed 3: every
    plasticity model — Drucker-Prager, NACC, von Mises, Herschel-Bulkley,
    snow — and 10 to 20 iterations per scene; 2k-8k particles each), one
    handle, one launch per stage: after five substeps every scene's next
    substep matches its own oracle run. lanes 0 is the library's choice for
    this size (one lane per particle); 4 forces the small-scene path."""
    scenes = xp.scenes.config_batch(n_scenes=20, seed=3, n_lo=2000, n_hi=8000)
    kinds = {s["materials"][0]["kind"] for s in scenes}
    its = [s["iterations"] for s in scenes]
    assert kinds == {xp.scenes.DP, xp.scenes.NACC, xp.scenes.VM, xp.scenes.HB, xp.scenes.SNOW}
    assert min(its) == 10 and max(its) == 20
    with xp.Simulation(scenes) as sim:
        sim.set_lanes(lanes)
        for k, sc in enumerate(scenes):
            sim.write_params(xp.params_for(sc), scene=k)
            sim.set_schedule(k, sc["iterations"], sc["hasWater"])
        sim.step(5, -1, False)
        states = [sim.read_state(k) for k in range(len(scenes))]
        uni = [sim.uniforms(k) for k in range(len(scenes))]
        sim.encode_substep(-1, False)
        after = [sim.read_state(k) for k in range(len(scenes))]
    for k, sc in enumerate(scenes):
        pw, mw = uni[k]
        ref = oracle.substep(pw, mw, states[k], its[k], False, -1)
        ref64 = oracle.substep(pw, mw, states[k], its[k], False, -1, f64=True)
        compare(after[k], ref, ref64,
                perturbed=perturbed_runs(oracle, sc, states[k], iterations=its[k], has_water=False, xp=xp))


def test_profile_substep_labels(xp, built_lib):
    sc = xp.scenes.dam_breach()
    with xp.Simulation(sc) as sim:
        sim.write_params(xp.params_for(sc))
        text = sim.profile_substep(3, True)
        n = sim.launches_per_substep(3, True)
    lines = [l for l in text.splitlines() if l]
    assert len(lines) == n - 1  # the crowded-cell pass is timed with the reorder
    assert lines[0].startswith("count:") and lines[-1].startswith("updateF+integrate:")
    assert sum(1 for l in lines if l.startswith("pbfB:")) == 3


def _clump(xp, sc, oracle, warm, count, material_kind, lanes=0):
    """Move `count` particles of one material into a ball of radius 0.3 h:
    their neighbour lists overflow the 64-entry record (every list-driven
    pass falls back to the stencil walk) and their cell's bucket passes the
    64 members of the rank rule (the crowded-bucket sort)."""
    p = xp.params_for(sc)
    it = sc["iterations"]
    rng = np.random.default_rng(11)
    with xp.Simulation(sc) as sim:
        sim.write_params(p)
        sim.set_lanes(lanes)
        if warm:
            sim.step(warm, it, sc["hasWater"])
        st = sim.read_state()
        kinds = np.array([m["kind"] for m in sc["materials"]])
        idx = np.flatnonzero(kinds[np.abs(st["pos"][:, 3]).astype(int)] == material_kind)[:count]
        centre = st["pos"][idx, :3].mean(axis=0)
        u = rng.normal(size=(len(idx), 3))
        u *= (0.3 * sc["h"] * rng.uniform(0, 1, len(idx)) ** (1 / 3) / np.linalg.norm(u, axis=1))[:, None]
        pos = st["pos"].copy()
        pos[idx, :3] = (centre + u).astype(np.float32)
        sim.write_state(0, pos=pos)
        s0 = sim.read_state()
        pw, mw = sim.uniforms()
        pi = p.get("pbfIterations")
        pi = -1 if pi is None else int(pi)
        ref = oracle.substep(pw, mw, s0, it, sc["hasWater"], pi)
        ref64 = oracle.substep(pw, mw, s0, it, sc["hasWater"], pi, f64=True)
        sim.encode_substep(it, sc["hasWater"])
        s1 = sim.read_state()
    assert len(idx) == count
    return s0, s1, ref, ref64, p, centre.astype(np.float64)


# A clump of particles 0.3 h across is an ill-conditioned solve: inside it and
# within two kernel supports (2 h each) of it the f32 oracle is itself ~0.3 of
# the peak velocity away from the f64 oracle, so there the comparison runs
# through the noise envelope. Beyond that the substep is an ordinary one: at
# three supports and more the GPU must match the f32 oracle to FAR_TOL of each
# field's largest magnitude (measured: <= 1.4e-6 for the velocities).
FAR_SUPPORTS = 3.0
FAR_TOL = 1e-5


def _far_field(s1, ref, centre, h, min_count):
    d = np.linalg.norm(s1["pos"][:, :3].astype(np.float64) - centre, axis=1) / (2.0 * h)
    far = d >= FAR_SUPPORTS
    assert far.sum() >= min_count
    for k in ("pos", "vel", "F", "L"):
        a = s1[k].reshape(len(d), -1).astype(np.float64)
        b = ref[k].reshape(len(d), -1).astype(np.float64)
        if k in ("pos", "vel"):
            a, b = a[:, :3], b[:, :3]
        err = np.abs(a[far] - b[far]).max() / max(np.abs(b).max(), 1e-30)
        assert err <= FAR_TOL, (k, err)


@pytest.mark.parametrize("lanes", [1, 2, 4])
def test_crowded_clump_sand(xp, oracle, built_lib, lanes):
    sc = xp.scenes.config_sand_column()
    s0, s1, ref, ref64, p, centre = _clump(xp, sc, oracle, 0, 150, 1, lanes)
    compare(s1, ref, ref64, perturbed=perturbed_runs(oracle, sc, s0, xp=xp, count=6, positions=True))
    _far_field(s1, ref, centre, sc["h"], min_count=10000)


def test_crowded_clump_water(xp, oracle, built_lib):
    sc = xp.scenes.config_dam_breach(scale=0.05)
    s0, s1, ref, ref64, p, centre = _clump(xp, sc, oracle, 5, 150, 6)
    compare(s1, ref, ref64, has_pbf=True,
            perturbed=perturbed_runs(oracle, sc, s0, xp=xp, count=6, positions=True))
    _far_field(s1, ref, centre, sc["h"], min_count=40000)


def test_batch_with_an_empty_scene(xp, oracle, built_lib):
    """A batch whose first scene has no particles: the others step as alone."""
    empty = dict(xp.scenes.plasticine())
    empty["positions"] = np.zeros((0, 3), np.float32)
    empty["matIds"] = np.zeros(0, np.uint32)
    for k in ("states", "velocities", "colorSeeds"):
        empty.pop(k, None)
    scenes = [empty, xp.scenes.snowball_smash(), xp.scenes.goo()]
    with xp.Simulation(scenes) as sim:
        for k, sc in enumerate(scenes):
            sim.write_params(xp.params_for(sc), scene=k)
            sim.set_schedule(k, sc["iterations"], sc["hasWater"])
        sim.step(3, -1, False)
        states = [sim.read_state(k) for k in range(1, 3)]
        uni = [sim.uniforms(k) for k in range(1, 3)]
        sim.encode_substep(-1, False)
        after = [sim.read_state(k) for k in range(1, 3)]
        assert len(sim.read_state(0)["pos"]) == 0
    for k, sc in enumerate(scenes[1:]):
        pw, mw = uni[k]
        ref = oracle.substep(pw, mw, states[k], sc["iterations"], sc["hasWater"], -1)
        ref64 = oracle.substep(pw, mw, states[k], sc["iterations"], sc["hasWater"], -1, f64=True)
        compare(after[k], ref, ref64, has_pbf=sc["hasWater"])


@pytest.mark.parametrize("case", ["sand_flowing", "dam_breach", "snowball"])
def test_one_lane_per_particle(xp, oracle, built_lib, case):
    """The same substeps with one lane per particle in solveA / solveB (the
    path large handles take; small ones default to four lanes)."""
    if case == "sand_flowing":
        sc, warm = xp.scenes.config_sand_column(), 300
    elif case == "dam_breach":
        sc, warm = xp.scenes.config_dam_breach(scale=0.05), 10
    else:
        sc, warm = xp.scenes.config_nacc_snowball(), 125
    s0, s1, ref, ref64 = run_pair(xp, oracle, sc, warm=warm, lanes=1)
    compare(s1, ref, ref64, has_pbf=sc["hasWater"], perturbed=perturbed_runs(oracle, sc, s0, xp=xp))


@pytest.mark.parametrize("lanes", [2, 4])
def test_several_lanes_on_a_large_handle(xp, oracle, built_lib, lanes):
    """Two or four lanes forced on a handle above the automatic thresholds."""
    sc = xp.scenes.config_dam_breach(scale=0.3)
    s0, s1, ref, ref64 = run_pair(xp, oracle, sc, warm=5, lanes=lanes)
    compare(s1, ref, ref64, has_pbf=True, perturbed=perturbed_runs(oracle, sc, s0, xp=xp))
