"""The oracle against the reference's own kernels, on the CPU.

oracle/wgsl_ref.py translates the reference's WGSL (web/js/shaders/common.js
and simkernels.js) mechanically into C++ and runs it in the dispatch order of
Simulation.encodeSubstep (web/js/sim.js:220-272). The f32 oracle must equal
it bit for bit — sort, positions, velocities, F, L, V^n, multipliers and
plastic state — on every reference demo scene and on the benchmark configs,
fresh and after the motion has developed (flowing sand, NACC impact, water
over sand with the 4-pass PBF schedule and the reference's every-iteration
interleave). A mistake planted in the oracle's input (one ulp of the damping
parameter) must break the equality, so the comparison has teeth.
"""
import numpy as np
import pytest

FIELDS = ("pos", "vel", "F", "L", "aux", "sortedIdx", "cellTab")


@pytest.fixture(scope="module")
def wref():
    from oracle import wgsl_ref as W
    if not W.available():
        pytest.skip("the reference's WGSL is not available here")
    W.lib()
    return W


def _uniforms(xp, sc, pbf):
    p = xp.params_for(sc) if pbf >= 0 else xp.params_for(sc, pbfIterations=None)
    return xp.pack_uniforms(sc, p)


def _same(a, b):
    return [k for k in FIELDS if not np.array_equal(a[k], b[k])]


CASES = [
    # scene factory, kwargs, warm-up substeps (oracle), compared substeps, PBF passes (-1: every iteration)
    ("sand_column", {}, 0, 2, -1),
    ("sand_two_blocks", {}, 30, 2, -1),
    ("snowball_smash", {}, 60, 2, -1),
    ("plasticine", {}, 100, 2, -1),
    ("goo", {}, 100, 2, -1),
    ("snow_classic", {}, 150, 2, -1),
    ("dam_breach", {}, 40, 2, -1),
    ("elastic_block", {}, 40, 2, -1),
    ("config_sand_column", {}, 190, 2, -1),
    ("config_dam_breach", {"scale": 0.05}, 30, 1, 4),
    ("config_dam_breach", {"scale": 0.05}, 5, 1, -1),
]


@pytest.mark.parametrize("name,kw,warm,steps,pbf", CASES, ids=[f"{c[0]}-{c[2]}-{c[4]}" for c in CASES])
def test_oracle_equals_reference_kernels(xp, oracle, wref, name, kw, warm, steps, pbf):
    sc = getattr(xp.scenes, name)(**kw)
    pw, mw = _uniforms(xp, sc, pbf)
    it, hw = sc["iterations"], sc["hasWater"]
    st = oracle.initial_state(sc)
    if warm:
        st = oracle.substep(pw, mw, st, it, hw, pbf, warm)
    a = oracle.substep(pw, mw, st, it, hw, pbf, steps)
    b = wref.substep(pw, mw, st, it, hw, pbf, steps)
    assert not _same(a, b), _same(a, b)


def test_reference_kernels_thread_count_independent(xp, wref):
    sc = xp.scenes.dam_breach()
    pw, mw = _uniforms(xp, sc, -1)
    from oracle import oracle as O
    st = O.initial_state(sc)
    a = wref.substep(pw, mw, st, sc["iterations"], True, -1, 2, threads=1)
    b = wref.substep(pw, mw, st, sc["iterations"], True, -1, 2, threads=4)
    assert not _same(a, b)


def test_a_planted_mistake_breaks_the_equality(xp, oracle, wref):
    sc = xp.scenes.config_sand_column()
    pw, mw = _uniforms(xp, sc, -1)
    st = oracle.initial_state(sc)
    st = oracle.substep(pw, mw, st, sc["iterations"], False, -1, 170)
    bad = np.array(pw, np.uint32).copy()
    bad[36] += 1  # kDamp one ulp up, in the oracle's input only
    a = oracle.substep(bad, mw, st, sc["iterations"], False, -1, 1)
    b = wref.substep(pw, mw, st, sc["iterations"], False, -1, 1)
    assert "vel" in _same(a, b)
