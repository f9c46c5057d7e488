"""The autotuner: every register-allocation variant of solveA and solveB
computes the same substep bit for bit, and xpbi_autotune leaves the state
untouched while it times them."""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vel", "F", "L", "aux", "sortedIdx", "cellTab")


def _run(xp, sc, variants, substeps=4):
    with xp.Simulation(sc) as sim:
        sim.write_params(xp.params_for(sc))
        sim.set_lanes(1)  # the register variants are the one-lane kernels
        sim.step(3, sc["iterations"], sc["hasWater"])
        if variants is not None:
            sim.set_variants(*variants)
        sim.step(substeps, sc["iterations"], sc["hasWater"])
        return sim.read_state()


def test_every_variant_gives_the_same_substep(xp, built_lib):
    sc = xp.scenes.config_dam_breach(scale=0.05)
    ref = _run(xp, sc, None)
    combos = [(a, 0) for a in range(1, xp.Simulation.SOLVEA_VARIANTS)] + \
             [(0, bv) for bv in range(1, xp.Simulation.SOLVEB_VARIANTS)]
    for a, bv in combos:
        st = _run(xp, sc, (a, bv))
        for k in FIELDS:
            assert np.array_equal(st[k], ref[k]), (a, bv, k)


def test_autotune_keeps_the_state_and_picks_a_variant(xp, built_lib):
    sc = xp.scenes.config_dam_breach(scale=0.05)
    with xp.Simulation(sc) as sim:
        sim.write_params(xp.params_for(sc))
        sim.set_lanes(1)
        sim.step(5, sc["iterations"], True)
        before = sim.read_state()
        res = sim.autotune(sc["iterations"], True, repeats=3)
        after = sim.read_state()
        for k in FIELDS:
            assert np.array_equal(before[k], after[k]), k
        assert 0 <= res["solveA"] < xp.Simulation.SOLVEA_VARIANTS
        assert 0 <= res["solveB"] < xp.Simulation.SOLVEB_VARIANTS
        assert all(t > 0 for t in res["solveA_ms"] + res["solveB_ms"])
        sim.step(2, sc["iterations"], True)  # the chosen variants replay in a new graph
        tuned = sim.read_state()
    ref = _run(xp, sc, None, substeps=4)  # 3 + 4 = the 5 + 2 substeps above
    for k in FIELDS:
        assert np.array_equal(tuned[k], ref[k]), k
