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
