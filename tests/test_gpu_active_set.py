"""The active set (work skipping of an early-stopped solve) on the GPU.

With a tolerance so small that no particle settles (and every velocity
change counts as a move), skipping only the particles whose inputs did not
change must reproduce the solve that visits every particle (a particle is
only skipped where the full solve would redo the same evaluation). With the plain solve's own
tolerance (and an iteration cap of twice the plain budget), the visited sets
shrink over the iterations and the solve ends within both residual
tolerances (re-measured on the final state by a pass over every
particle)."""
import json

import numpy as np
import pytest

from parity_util import rel

pytestmark = pytest.mark.gpu


def _state(xp, sc, warm):
    with xp.Simulation(sc) as sim:
        sim.write_params(xp.params_for(sc))
        sim.step(warm, sc["iterations"], sc["hasWater"])
        return sim.read_state()


def _run(xp, sc, s0, mode, tol, tol_c, share, net=None, cap=0):
    with xp.Simulation(sc) as sim:
        sim.write_params(xp.params_for(sc))
        sim.write_state(0, pos=s0["pos"], vel=s0["vel"], F=s0["F"], aux=s0["aux"])
        if net is not None:
            sim.set_network(net)
        sim.set_lanes(1)
        sim.set_active_set(share)
        sim.set_max_iterations(cap)
        sim.set_solver(mode, tol, True, False, contact_rel_tol=tol_c)
        sim.encode_substep(sc["iterations"], sc["hasWater"])
        r, used = sim.read_residuals()
        c = sim.read_contact_residuals()
        a, b = sim.read_active_counts()
        return sim.read_state(), r, c, used, a, b


@pytest.mark.parametrize("case", ["dam_breach", "sand_column"])
def test_nothing_settles_matches_the_full_solve(xp, built_lib, case):
    if case == "dam_breach":
        sc, warm = xp.scenes.config_dam_breach(scale=0.05), 100  # loaded: constraints active
    else:
        sc, warm = xp.scenes.config_sand_column(), 300
    s0 = _state(xp, sc, warm)
    full = _run(xp, sc, s0, 0, 1e-9, 1e-9, 0.0)
    act = _run(xp, sc, s0, 0, 1e-9, 1e-9, 0.25)
    errs = {k: rel(act[0][k], full[0][k]) for k in ("pos", "vel", "F")}
    print(json.dumps({"case": case, **errs, "visited_solveA": act[4][1:8].tolist()}))
    assert full[3] == act[3] == sc["iterations"]
    for k in ("pos", "vel", "F"):
        assert errs[k] <= 1e-6, (k, errs)
    assert np.array_equal(act[0]["sortedIdx"], full[0]["sortedIdx"])


def test_visited_particles_shrink_and_tolerances_hold(xp, built_lib):
    import importlib
    tw = importlib.import_module("xpbi-webgpu_gb300.train_warm")
    sc = xp.scenes.config_dam_breach(scale=0.1)
    K = sc["iterations"]
    s0 = _state(xp, sc, 100)
    plain = _run(xp, sc, s0, 0, 0.0, 0.0, 0.0)
    tau = float(plain[1][1 + K] / plain[1][0])
    tau_c = float(plain[2][1 + K] / plain[2][0])
    cap = 2 * K
    st, r, c, used, a, b = _run(xp, sc, s0, 1, tau, tau_c, 0.25, tw.load_weights(), cap)
    kinds = np.array([m["kind"] for m in sc["materials"]])
    n_solid = int((kinds[np.asarray(sc["matIds"])] != xp.scenes.WATER).sum())
    frac = (a[1:used] / n_solid).round(4).tolist()
    print(json.dumps({"tau": tau, "tau_c": tau_c, "used": used, "solveA_fraction": frac,
                      "solveB": b[1:used].tolist(), "final": float(r[-1] / r[0]),
                      "final_contact": float(c[-1] / c[0])}))
    assert len(r) == cap + 2
    assert 1 <= used <= cap
    # the final state's residuals, re-measured over every particle
    assert r[-1] / r[0] <= tau * 1.0001 and c[-1] / c[0] <= tau_c * 1.0001
    assert (a[1:used] <= n_solid).all() and (b[1:used] <= len(sc["positions"])).all()
    if used > 3:
        assert a[used - 1] < a[1]  # fewer solids revisited at the end than at iteration 1
    assert np.isfinite(st["vel"]).all()


def test_device_loop_graph_matches_enqueued_substep(xp, built_lib):
    """An early-stopped active-set solve replayed from its graph, whose last
    iterations run as a device loop until every scene stopped, gives the
    bytes of the same substep enqueued launch by launch (where iterations
    past the stop find nothing to do), and the same iterations and residual
    history."""
    import importlib
    tw = importlib.import_module("xpbi-webgpu_gb300.train_warm")
    sc = xp.scenes.config_dam_breach(scale=0.1)
    K = sc["iterations"]
    s0 = _state(xp, sc, 100)
    plain = _run(xp, sc, s0, 0, 0.0, 0.0, 0.0)
    tau = float(plain[1][1 + K] / plain[1][0])
    tau_c = float(plain[2][1 + K] / plain[2][0])
    out = []
    for graph in (False, True):
        with xp.Simulation(sc) as sim:
            sim.write_params(xp.params_for(sc))
            sim.write_state(0, pos=s0["pos"], vel=s0["vel"], F=s0["F"], aux=s0["aux"])
            sim.set_network(tw.load_weights())
            sim.set_lanes(1)
            sim.set_active_set(0.25)
            sim.set_max_iterations(2 * K)
            sim.set_solver(1, tau, True, False, contact_rel_tol=tau_c)
            for _ in range(2):  # the second substep starts from the first's multipliers
                if graph:
                    sim.step(1, K, True)
                else:
                    sim.encode_substep(K, True)
            r, used = sim.read_residuals()
            out.append((sim.read_state(), r, used, sim.read_active_counts()))
    (a, ra, ua, ca), (g, rg, ug, cg) = out
    assert ua == ug and 1 <= ua <= 2 * K
    for k in ("pos", "vel", "F", "aux", "sortedIdx"):
        assert np.array_equal(a[k], g[k]), k
    assert np.array_equal(np.nan_to_num(ra, nan=-2), np.nan_to_num(rg, nan=-2))
    assert np.array_equal(ca[0], cg[0]) and np.array_equal(ca[1], cg[1])
