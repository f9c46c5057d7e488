"""Asynchronous position read-back: each step's positions copied behind the
work that produced them while the next substeps run (their position update
waits for the copy), equal to the synchronous read-back of the same steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_async_read_back_matches_sync(xp, built_lib):
    sc = xp.scenes.dam_breach()
    p = xp.params_for(sc)
    it = sc["iterations"]
    n = len(sc["positions"])
    got = [np.empty((n, 4), np.float32) for _ in range(5)]
    with xp.Simulation(sc) as sim:
        sim.write_params(p)
        for k in range(5):
            sim.step(1, it, True)
            sim.read_pos_async(0, got[k])
        sim.synchronize()
    with xp.Simulation(sc) as sim:
        sim.write_params(p)
        for k in range(5):
            sim.step(1, it, True)
            ref = sim.read_pos(0)
            assert np.array_equal(got[k], ref), k
    assert not np.array_equal(got[0], got[-1])


def test_params_written_every_step_are_the_ones_each_step_uses(xp, built_lib):
    """A frame's writeParams + step queue without waiting for the previous
    substep (the uniforms go through a ring of page-locked staging slots,
    each reused once its copy completed): twelve steps with a different
    gravity each, queued back to back, end in the state of the same steps
    run one at a time with a synchronize after each."""
    sc = xp.scenes.dam_breach()
    it = sc["iterations"]
    states = []
    for sync in (False, True):
        with xp.Simulation(sc) as sim:
            for k in range(12):
                p = dict(xp.params_for(sc))
                p["gravity"] = [0.3 * (k % 3 - 1), -9.8 - 0.5 * k, 0.2 * (k % 2)]
                sim.write_params(p)
                sim.step(1, it, True)
                if sync:
                    sim.synchronize()
            sim.synchronize()
            states.append(sim.read_state())
    for k in ("pos", "vel", "F", "aux", "sortedIdx"):
        assert np.array_equal(states[0][k], states[1][k]), k
