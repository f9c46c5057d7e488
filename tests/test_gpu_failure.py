"""Failure detection on the GPU without a fault: a bounded device wait that
runs out is reported to the host as a status, and the handle stays usable.

The prefix scan's look-back waits on descriptors that earlier tiles
publish; every such wait gives up after a fixed number of polls and raises
the device error word. xpbi_test_wait_expiry runs that same wait on a
descriptor nothing publishes, so it expires after a short limit; nothing
faults, traps or spins without a limit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ERR_DEVICE = 4


def test_expired_wait_is_reported_and_the_handle_recovers(xp, built_lib):
    sc = xp.scenes.sand_column()
    p = xp.params_for(sc)
    it = sc["iterations"]
    with xp.Simulation(sc) as ref:
        ref.write_params(p)
        ref.step(3, it, False)
        want = ref.read_state()
    with xp.Simulation(sc) as sim:
        sim.write_params(p)
        sim.step(1, it, False)
        sim.synchronize()
        sim.test_wait_expiry(1000)
        with pytest.raises(xp.XpbiError) as e:
            sim.synchronize()
        assert e.value.code == ERR_DEVICE
        assert "bounded wait expired" in str(e.value)
        sim.synchronize()  # the error word was read and cleared
        # the expired wait touched no particle state: the next substeps give
        # the bytes of an undisturbed run
        sim.step(2, it, False)
        sim.synchronize()
        got = sim.read_state()
    for k in ("pos", "vel", "F", "aux", "sortedIdx"):
        assert np.array_equal(got[k], want[k]), k


def test_wait_expiry_polls_are_checked(xp, built_lib):
    sc = xp.scenes.sand_column()
    with xp.Simulation(sc) as sim:
        for bad in (0, (1 << 20) + 1):
            with pytest.raises(xp.XpbiError) as e:
                sim.test_wait_expiry(bad)
            assert e.value.code == 1
