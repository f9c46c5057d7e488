"""Solver modes on the GPU: residual tracking, early stop, and what the
trained warm-start network gains over the plain zero start and over the
previous-substep multiplier."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tw(built_lib):
    return importlib.import_module("xpbi-webgpu_gb300.train_warm")


def _rollout(xp, sc, warm):
    with xp.Simulation(sc) as sim:
        sim.write_params(xp.params_for(sc))
        sim.set_solver(0, 0.0, False, True)
        if warm:
            sim.step(warm, sc["iterations"], sc["hasWater"])
        return sim.read_state()


def _curves(xp, sc, st, mode, net=None, substeps=3, tol=0.0):
    it = sc["iterations"]
    out = []
    with xp.Simulation(sc) as sim:
        sim.write_params(xp.params_for(sc))
        sim.write_state(0, pos=st["pos"], vel=st["vel"], F=st["F"], aux=st["aux"])
        if net is not None:
            sim.set_network(net)
        sim.set_solver(mode, tol, True, False)
        for _ in range(substeps):
            sim.encode_substep(it, sc["hasWater"])
            r, used = sim.read_residuals()
            c = sim.read_contact_residuals()
            out.append((r[: it + 2] / r[0], used, c[: it + 2] / c[0] if c[0] > 0 else np.zeros(it + 2)))
        state = sim.read_state()
    return out, state


def test_tracking_does_not_change_the_solve(xp, built_lib):
    sc = xp.scenes.sand_two_blocks()
    res = []
    for track in (False, True):
        with xp.Simulation(sc) as sim:
            sim.write_params(xp.params_for(sc))
            sim.set_solver(0, 0.0, track, track)
            sim.step(6, sc["iterations"], False)
            res.append(sim.read_state())
    for k in ("pos", "vel", "F", "aux", "sortedIdx"):
        assert np.array_equal(res[0][k], res[1][k]), k


@pytest.mark.parametrize("lanes,track", [(0, False), (1, False), (1, True)])
def test_zero_network_is_the_previous_multiplier_start(xp, built_lib, lanes, track):
    """The network predicts an increment over the previous multiplier. With
    one lane per slot the network mode's iteration 0 reads the constraint
    computeL evaluated with the features (k_solveA_stored, with or without residual
    tracking), the previous-multiplier mode evaluates it in solveA: both must
    give the same bytes."""
    sc = xp.scenes.dam_breach()
    zero = np.zeros(9473, np.float32)
    res = []
    for mode in (2, 1):
        with xp.Simulation(sc) as sim:
            sim.write_params(xp.params_for(sc))
            sim.set_lanes(lanes)
            sim.set_network(zero)
            sim.set_solver(mode, 0.0, track, False)
            sim.step(5, sc["iterations"], True)
            res.append(sim.read_state())
    for k in ("pos", "vel", "F", "sortedIdx"):
        assert np.array_equal(res[0][k], res[1][k]), k


def test_plain_residual_history(xp, built_lib):
    sc = xp.scenes.config_sand_column()
    st = _rollout(xp, sc, 300)
    (curves, _), = [_curves(xp, sc, st, 0, substeps=1)]
    r, used, _ = curves[-1]
    assert used == sc["iterations"]
    assert r[0] == 1.0 and r[1] == pytest.approx(1.0, rel=1e-6)  # iteration 0 enters at lambda = 0
    assert r[-1] < 0.05 * r[1]  # ten damped Jacobi iterations remove >95% of it


def test_early_stop_skips_remaining_iterations(xp, built_lib):
    sc = xp.scenes.config_sand_column()
    st = _rollout(xp, sc, 300)
    curves, _ = _curves(xp, sc, st, 0, substeps=2, tol=0.2)
    for r, used, c in curves:
        # a stop found at iteration k (residuals of the state entering it)
        # takes effect after iteration k's update: k + 1 iterations applied
        assert 1 < used < sc["iterations"]
        k = used - 1
        assert r[1 + k] <= 0.2 * 1.0001 and c[1 + k] <= 0.2 * 1.0001  # constraint and contact
        assert r[k] > 0.2 or c[k] > 0.2  # and not one iteration earlier
        assert np.isnan(r[1 + used:-1]).all()  # iterations after the stop did not run


def test_network_warm_start_gains(xp, tw):
    """Held-out dam breach (a seed the training scenes never use), 150
    substeps in. What the trained network gains over the method without it:
    its multiplier starts the solve many times closer to convergence than the
    plain zero start and clearly closer than the previous substep's
    multiplier alone, and the early iterations stay ahead of the plain solve.
    What it does not gain: the contact correction that runs inside the same
    iterations converges at the same rate from any multiplier start, so the
    contact residual curves coincide and set the iterations an equal-residual
    stop needs (printed, not asserted)."""
    net = tw.load_weights()
    sc = xp.scenes.config_dam_breach(seed=0, scale=0.1)
    st = _rollout(xp, sc, 150)
    plain, _ = _curves(xp, sc, st, 0)
    prev, _ = _curves(xp, sc, st, 2)
    learned, _ = _curves(xp, sc, st, 1, net)
    it = sc["iterations"]
    for (rp, _, cp), (rv, _, _), (rl, _, cl) in zip(plain, prev, learned):
        assert rl[1] < 0.6 * rv[1] and rv[1] < 0.5 * rp[1]  # starting residual
        assert (rl[1:5] < rp[1:5]).all()              # ahead in the first iterations
        assert rl[-1] < 3.0 * rp[-1]                  # final residual no worse than 3x plain's
        print("contact residual after the budget: plain", float(cp[-1]), "network", float(cl[-1]))
        target = rp[-1] * 1.05                        # plain's final residual
        k_plain = int(np.argmax(rp[1:it + 1] <= target)) if (rp[1:it + 1] <= target).any() else it
        k_net = int(np.argmax(rl[1:it + 1] <= target)) if (rl[1:it + 1] <= target).any() else it
        print("iterations to the plain final residual: plain", k_plain, "network", k_net,
              "start", float(rl[1]), "vs previous", float(rv[1]))
