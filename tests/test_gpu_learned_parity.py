"""The learned solve — the path the benchmark's headline number measures —
held to the plain solve's accuracy on the same substep.

Both solves approximate the same Jacobi fixed point: the plain one by its
fixed iteration budget from lambda = 0 (the reference's schedule), the
learned one from the network's warm start until its constraint and contact
residuals reach the plain solve's own final values (equal residual; it may
run up to ITERATION_CAP times the plain budget to get there). Each
is compared with the FP64 oracle's solve of that substep run to
convergence (CONVERGED_ITERATIONS Jacobi iterations, the same PBF schedule),
from the identical input state:
  - the learned state's solid velocities (max-norm) must be within
    ERR_FACTOR times the plain GPU state's error from it, or within
    SOLID_FLOOR of it where the plain solve already sits closer than that
    (solids at the water interface take half-weight PBF corrections in the
    first iterations, so like the water they follow the iterate there:
    measured 1.4e-4 against plain's 1.1e-5 on the 50k dam breach, 4.3e-4
    against 4.3e-4 on the 100k one); the root-mean-square velocity error
    over every particle must be within ERR_FACTOR times plain's plus
    RMS_FLOOR, and the positions within ERR_FACTOR times plain's plus FLOOR;
  - water is held to the RMS bound only: the PBF passes run inside the
    first iterations and see the solids' iterate there, which the start
    value changes, so near the interface a few water particles end
    elsewhere than on the zero-start path the converged solve follows
    (reported as the every-particle max-norm);
  - the learned solve must end with both residuals within their tolerances
    (the early stop's own criterion, re-measured on the final state);
and the plain GPU state is within the parity tolerance of the FP64 oracle
at the plain budget (its own parity). The learned solve runs with and
without the active set (share 0.25: particles whose inputs did not change
are not revisited, settled particles take no impulse).
"""
import json

import numpy as np
import pytest

from parity_util import rel

pytestmark = pytest.mark.gpu

CONVERGED_ITERATIONS = 120
ERR_FACTOR = 1.5
FLOOR = 2e-5       # positions, relative to the largest coordinate
SOLID_FLOOR = 2e-4  # solid velocities, relative to the largest speed: twice the 1e-4 parity tolerance
RMS_FLOOR = 1e-5   # relative to the root-mean-square speed
ITERATION_CAP = 2  # the learned solve may run up to twice the plain budget to reach the plain residual

CASES = {
    "dam_breach_50k": ("config_dam_breach", dict(scale=0.05), 100),
    "dam_breach_100k": ("config_dam_breach", dict(scale=0.1), 100),
    "sand_column_300": ("config_sand_column", dict(), 300),
}


def _solve(xp, sc, s0, mode, tol=0.0, tol_c=0.0, net=None, share=0.0, cap=0):
    it, hw = sc["iterations"], sc["hasWater"]
    with xp.Simulation(sc) as sim:
        sim.write_params(xp.params_for(sc))
        sim.write_state(0, pos=s0["pos"], vel=s0["vel"], F=s0["F"], aux=s0["aux"])
        if net is not None:
            sim.set_network(net)
        sim.set_lanes(1)
        sim.set_active_set(share)
        sim.set_max_iterations(cap)
        sim.set_solver(mode, tol, True, False, contact_rel_tol=tol_c)
        sim.encode_substep(it, hw)
        r, used = sim.read_residuals()
        c = sim.read_contact_residuals()
        st = sim.read_state()
    rel_r = float(r[-1] / r[0]) if r[0] > 0 else 0.0
    rel_c = float(c[-1] / c[0]) if c[0] > 0 else 0.0
    return st, rel_r, rel_c, used


@pytest.mark.parametrize("share", [0.0, 0.25])
@pytest.mark.parametrize("case", sorted(CASES))
def test_learned_solve_is_as_accurate_as_plain(xp, oracle, built_lib, case, share):
    import importlib
    tw = importlib.import_module("xpbi-webgpu_gb300.train_warm")
    fn, kw, warm = CASES[case]
    sc = getattr(xp.scenes, fn)(**kw)
    it, hw = sc["iterations"], sc["hasWater"]
    p = xp.params_for(sc)
    pbf = -1 if p.get("pbfIterations") is None else int(p["pbfIterations"])
    with xp.Simulation(sc) as sim:
        sim.write_params(p)
        sim.step(warm, it, hw)
        s0 = sim.read_state()
        pw, mw = sim.uniforms()
    plain, tau, tau_c, used_p = _solve(xp, sc, s0, 0)
    learned, rl, rlc, used_l = _solve(xp, sc, s0, 1, tau, tau_c, tw.load_weights(), share, ITERATION_CAP * it)
    conv = oracle.substep(pw, mw, s0, CONVERGED_ITERATIONS, hw, pbf, f64=True)
    at_budget = oracle.substep(pw, mw, s0, it, hw, pbf, f64=True)
    kinds = np.array([m["kind"] for m in sc["materials"]])
    solid = kinds[np.abs(learned["pos"][:, 3]).astype(int)] != xp.scenes.WATER
    vmax = float(np.abs(conv["vel"][:, :3]).max())
    vrms = float(np.sqrt((conv["vel"][:, :3].astype(np.float64) ** 2).sum(axis=1).mean()))

    def errs(st):
        d = np.abs(st["vel"][:, :3].astype(np.float64) - conv["vel"][:, :3])
        return (float(d[solid].max() / vmax) if solid.any() else 0.0,           # solids, max-norm
                float(np.sqrt((d ** 2).sum(axis=1).mean()) / vrms),             # every particle, RMS
                float(d.max() / vmax),                                          # every particle, max-norm
                rel(st["pos"], conv["pos"]))
    ep, el = errs(plain), errs(learned)
    e = dict(vel_solid_max_plain=ep[0], vel_solid_max_learned=el[0], vel_rms_plain=ep[1], vel_rms_learned=el[1],
             vel_max_plain=ep[2], vel_max_learned=el[2], pos_plain=ep[3], pos_learned=el[3],
             plain_vs_f64_at_budget=rel(plain["vel"], at_budget["vel"]), tau=tau, tau_c=tau_c,
             learned_rel=rl, learned_rel_contact=rlc, iterations_plain=used_p, iterations_learned=used_l)
    print(json.dumps({"case": case, "share": share, **e}))
    assert used_p == it
    assert used_l <= ITERATION_CAP * it
    assert rl <= tau * 1.0001 and rlc <= tau_c * 1.0001
    assert e["plain_vs_f64_at_budget"] <= 2e-4  # the plain GPU solve is the f64 solve at its budget
    assert el[0] <= max(ERR_FACTOR * ep[0], SOLID_FLOOR), e  # solid velocities
    assert el[1] <= ERR_FACTOR * ep[1] + RMS_FLOOR, e      # every particle, root mean square
    assert el[3] <= ERR_FACTOR * ep[3] + FLOOR, e          # positions
