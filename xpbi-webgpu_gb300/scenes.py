"""Seeded scene factories.

Restates web/js/scenes.js (lattice samplers, material presets, solver
defaults and the demo scenes) with a seeded generator in place of the
reference's unseeded ``Math.random()``, and adds the five benchmark
workloads (sand column, NACC snowball, dam breach, a batch of 256 mixed
scenes, and the 4-seed dam-breach mix).

A scene is a dict with the fields ``new Simulation(device, scene)`` reads
(sim.js:10-81) plus the frame-loop settings (main.js:385-402). The module
needs only NumPy, so CPU tools can load it without the library.
"""
from __future__ import annotations

import math

import numpy as np

# material kinds, MAT of web/js/sim.js:4-7 (the ABI's XPBI_* kinds have the same values)
ELASTIC, DP, NACC, VM, HB, SNOW, WATER = range(7)


def _jsround(x: float) -> int:
    """Math.round: halves round toward +infinity."""
    return int(math.floor(x + 0.5))


def sample_box(rng, out, mid, states, lo, hi, h, mat_idx, jitter=0.2, state0=0.0):
    """Lattice at cell centres with uniform jitter (scenes.js:7-20)."""
    n = [max(1, _jsround((hi[i] - lo[i]) / h)) for i in range(3)]
    k, j, i = np.meshgrid(np.arange(n[2]), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    base = np.stack([lo[0] + (i.ravel() + 0.5) * h, lo[1] + (j.ravel() + 0.5) * h,
                     lo[2] + (k.ravel() + 0.5) * h], axis=1)
    base = base + (rng.random(base.shape) - 0.5) * jitter * h
    out.append(base)
    mid.append(np.full(len(base), mat_idx, np.uint32))
    states.append(np.full(len(base), state0, np.float64))


def js_hypot3(a, b, c):
    """Math.hypot(a, b, c) as the reference's browser (Chrome's V8) evaluates
    it, elementwise in f64: the arguments scaled by the largest magnitude,
    their squares added with Kahan compensation, sqrt(sum) * max. Lattice
    points exactly on a sphere's surface (d == r up to rounding) land inside
    or outside by this rounding, so the membership test uses it rather than
    sqrt(a^2 + b^2 + c^2), which differs on ~1e-4 of the snowball's points."""
    v = [np.abs(np.asarray(x, np.float64)) for x in (a, b, c)]
    m = np.maximum(np.maximum(v[0], v[1]), v[2])
    safe = np.where(m > 0, m, 1.0)
    total = np.zeros_like(m)
    comp = np.zeros_like(m)
    for x in v:
        n = x / safe
        summand = n * n - comp
        prelim = total + summand
        comp = (prelim - total) - summand
        total = prelim
    return np.where(m > 0, np.sqrt(total) * m, 0.0)


def sample_sphere(rng, out, mid, states, c, r, h, mat_idx, jitter=0.2, state0=0.0):
    """Lattice points inside a sphere with uniform jitter (scenes.js:22-38)."""
    n = math.ceil(2 * r / h)
    k, j, i = np.meshgrid(np.arange(n + 1), np.arange(n + 1), np.arange(n + 1), indexing="ij")
    p = np.stack([c[0] - r + i.ravel() * h, c[1] - r + j.ravel() * h, c[2] - r + k.ravel() * h], axis=1)
    d = js_hypot3(p[:, 0] - c[0], p[:, 1] - c[1], p[:, 2] - c[2])
    p = p[d <= r]
    p = p + (rng.random(p.shape) - 0.5) * jitter * h
    out.append(p)
    mid.append(np.full(len(p), mat_idx, np.uint32))
    states.append(np.full(len(p), state0, np.float64))


def dp_alpha(phi_deg: float) -> float:
    """Drucker-Prager alpha from the friction angle (scenes.js:42)."""
    s = math.sin(phi_deg * math.pi / 180)
    return math.sqrt(2 / 3) * 2 * s / (3 - s)


# ---- material presets (scenes.js:40-80)
def SAND(phi_deg=35, cohesion=0.0):
    return dict(kind=DP, E=2000, nu=0.3, density=1.0, p0=dp_alpha(phi_deg), p1=cohesion,
                color=[0.85, 0.63, 0.28], boundFriction=0.5)


def SNOW_NACC():
    return dict(kind=NACC, E=2000, nu=0.3, density=4.0, p0=-0.008, p1=0.05, p2=5, p3=1.85,
                color=[0.93, 0.95, 0.98], boundFriction=0.35)


def PLASTICINE(sig_y=30):
    return dict(kind=VM, E=1200, nu=0.42, density=2.0, p0=sig_y, color=[0.36, 0.76, 0.72], boundFriction=0.4)


def GOO(h_exp=1.0):
    return dict(kind=HB, E=2250, nu=0.125, density=100.0, p0=45, p1=h_exp, p2=25,
                color=[0.91, 0.45, 0.62], boundFriction=0.2)


def SNOW_CLASSIC():
    return dict(kind=SNOW, E=9000, nu=0.2, density=4.0, p0=3.5e-2, p1=8e-3, p2=10,
                color=[0.96, 0.97, 1.0], boundFriction=0.35)


def WATER_MAT():
    return dict(kind=WATER, E=100, nu=0.3, density=1.0, color=[0.25, 0.55, 0.95], boundFriction=0.0)


def ELASTIC_MAT():
    return dict(kind=ELASTIC, E=900, nu=0.3, density=2.0, color=[0.62, 0.52, 0.86], boundFriction=0.3)


def base(h):
    """Solver defaults (scenes.js:82-92)."""
    return dict(h=h, domainMin=[0.0, 0.0, 0.0], domainMax=[1.0, 1.0, 1.0], gravity=[0.0, -9.8, 0.0],
                substeps=8, iterations=3, timeScale=0.42, omega=0.5, contactOmega=0.4, xsphC=0.01,
                pbfEps=100.0, sCorrK=0.0001, kDamp=0.4,
                camera=dict(theta=0.5, phi=0.32, dist=2.1, target=[0.5, 0.28, 0.5]))


def _finish(s, rng, pos, mid, st, materials, has_water, velocities=None):
    positions = np.concatenate(pos).astype(np.float32)
    n = len(positions)
    s.update(positions=positions, matIds=np.concatenate(mid), states=np.concatenate(st).astype(np.float32),
             velocities=None if velocities is None else np.asarray(velocities, np.float32).reshape(n, 3),
             materials=materials, hasWater=has_water,
             colorSeeds=(rng.random(n) * 0.49).astype(np.float32))
    return s


def frame_dt(scene) -> float:
    """Per-substep dt of the frame loop: (1/60) * timeScale / substeps (main.js:387)."""
    if "dt" in scene:
        return scene["dt"]
    return (1 / 60) * scene["timeScale"] / scene["substeps"]


# ---- demo scenes (scenes.js:94-176)
def sand_column(seed=0):
    rng = np.random.default_rng(seed)
    s = base(0.016)
    pos, mid, st = [], [], []
    sample_box(rng, pos, mid, st, [0.36, 0.015, 0.36], [0.64, 0.62, 0.64], s["h"], 0)
    return _finish(s, rng, pos, mid, st, [SAND(35)], False)


def sand_two_blocks(seed=0):
    rng = np.random.default_rng(seed)
    s = base(0.017)
    pos, mid, st = [], [], []
    sample_box(rng, pos, mid, st, [0.08, 0.015, 0.35], [0.38, 0.42, 0.65], s["h"], 0)
    n1 = len(pos[0])
    sample_box(rng, pos, mid, st, [0.62, 0.015, 0.35], [0.92, 0.42, 0.65], s["h"], 0)
    n = n1 + len(pos[1])
    vel = np.zeros((n, 3))
    vel[:n1, 0] = 1.6
    vel[n1:, 0] = -1.6
    return _finish(s, rng, pos, mid, st, [SAND(35)], False, vel)


def snowball_smash(seed=0):
    rng = np.random.default_rng(seed)
    s = base(0.018)
    s.update(substeps=9, iterations=3, timeScale=0.45)
    m = SNOW_NACC()
    pos, mid, st = [], [], []
    sample_box(rng, pos, mid, st, [0.1, 0.015, 0.1], [0.9, 0.14, 0.9], s["h"], 0, 0.2, m["p0"])
    n1 = len(pos[0])
    sample_sphere(rng, pos, mid, st, [0.2, 0.55, 0.5], 0.11, s["h"], 0, 0.2, m["p0"])
    n = n1 + len(pos[1])
    vel = np.zeros((n, 3))
    vel[n1:, 0] = 2.6
    vel[n1:, 1] = -3.2
    return _finish(s, rng, pos, mid, st, [m], False, vel)


def plasticine(seed=0):
    rng = np.random.default_rng(seed)
    s = base(0.013)
    s.update(substeps=8, iterations=6, timeScale=0.4)
    pos, mid, st = [], [], []
    sample_sphere(rng, pos, mid, st, [0.5, 0.4, 0.5], 0.16, s["h"], 0)
    return _finish(s, rng, pos, mid, st, [PLASTICINE(80)], False)


def goo(seed=0):
    rng = np.random.default_rng(seed)
    s = base(0.013)
    s.update(substeps=9, iterations=3, timeScale=0.5)
    pos, mid, st = [], [], []
    sample_sphere(rng, pos, mid, st, [0.5, 0.42, 0.5], 0.17, s["h"], 0)
    return _finish(s, rng, pos, mid, st, [GOO(1.0)], False)


def snow_classic(seed=0):
    rng = np.random.default_rng(seed)
    s = base(0.013)
    s.update(substeps=10, timeScale=0.38, iterations=4)
    pos, mid, st = [], [], []
    sample_sphere(rng, pos, mid, st, [0.35, 0.45, 0.42], 0.1, s["h"], 0, 0.2, 1.0)
    sample_sphere(rng, pos, mid, st, [0.65, 0.5, 0.58], 0.1, s["h"], 0, 0.2, 1.0)
    p = np.concatenate(pos)
    vel = np.zeros((len(p), 3))
    vel[:, 0] = np.where(p[:, 0] < 0.5, 1.5, -1.5)
    return _finish(s, rng, pos, mid, st, [SNOW_CLASSIC()], False, vel)


def dam_breach(seed=0):
    rng = np.random.default_rng(seed)
    s = base(0.019)
    s.update(substeps=6, iterations=3, timeScale=0.45)
    pos, mid, st = [], [], []
    sample_box(rng, pos, mid, st, [0.42, 0.015, 0.05], [0.6, 0.34, 0.95], s["h"], 0)
    sample_box(rng, pos, mid, st, [0.03, 0.015, 0.05], [0.36, 0.5, 0.95], s["h"], 1)
    return _finish(s, rng, pos, mid, st, [SAND(30, 0.004), WATER_MAT()], True)


def elastic_block(seed=0):
    rng = np.random.default_rng(seed)
    s = base(0.014)
    s.update(substeps=10, iterations=4, timeScale=0.5)
    pos, mid, st = [], [], []
    sample_box(rng, pos, mid, st, [0.38, 0.3, 0.38], [0.62, 0.54, 0.62], s["h"], 0)
    return _finish(s, rng, pos, mid, st, [ELASTIC_MAT()], False)


SCENES = {
    "Sand: column collapse": sand_column,
    "Sand: two blocks collide": sand_two_blocks,
    "Snow: snowball smash": snowball_smash,
    "Plasticine: drop & poke": plasticine,
    "Goo: Herschel-Bulkley": goo,
    "Snow: classic (Stomakhin)": snow_classic,
    "Dam breach: water + sand": dam_breach,
    "Elastic: StVK block": elastic_block,
}


# ---- benchmark workloads ------------------------------------------------
def _solver(s, dt, iterations, substeps, **kw):
    s.update(dt=dt, iterations=iterations, substeps=substeps, gravity=[0.0, -9.81, 0.0], **kw)
    return s


def config_sand_column(seed=0):
    """DP sand column: 20x20x40 lattice (16,000) at r=0.01, jitter +-0.1r,
    E=1e5, nu=0.3, rho=1600, phi=30 deg, floor friction 0.5; dt=2e-4,
    10 iterations, 200 substeps."""
    rng = np.random.default_rng(seed)
    s = base(0.01)
    s.update(domainMin=[0.0, 0.0, 0.0], domainMax=[1.0, 0.5, 1.0])
    pos, mid, st = [], [], []
    sample_box(rng, pos, mid, st, [0.4, 0.0, 0.4], [0.6, 0.4, 0.6], 0.01, 0)
    mat = dict(kind=DP, E=1e5, nu=0.3, density=1600.0, p0=dp_alpha(30), p1=0.0,
               color=[0.85, 0.63, 0.28], boundFriction=0.5)
    _finish(s, rng, pos, mid, st, [mat], False)
    return _solver(s, 2e-4, 10, 200)


def config_nacc_snowball(seed=0):
    """NACC sphere R=0.3 at r=0.01 (~113k) centred (0.36,0.5,0.5) moving at
    -5 m/s toward the x=0 wall; E=1.4e5, nu=0.3, rho=400, beta=0.5, xi=3,
    M=1.85, alpha0=-0.04; dt=1e-4, 20 iterations, 300 substeps."""
    rng = np.random.default_rng(seed)
    s = base(0.01)
    pos, mid, st = [], [], []
    sample_sphere(rng, pos, mid, st, [0.36, 0.5, 0.5], 0.3, 0.01, 0, 0.2, -0.04)
    n = len(pos[0])
    vel = np.zeros((n, 3))
    vel[:, 0] = -5.0
    mat = dict(kind=NACC, E=1.4e5, nu=0.3, density=400.0, p0=-0.04, p1=0.5, p2=3.0, p3=1.85,
               color=[0.93, 0.95, 0.98], boundFriction=0.35)
    _finish(s, rng, pos, mid, st, [mat], False, vel)
    return _solver(s, 1e-4, 20, 300)


def config_dam_breach(seed=0, scale=1.0):
    """Dam breach in a 2x1x1 m box at r=0.008: water 75x80x100 (600k, PBF
    rho0=1000, eps=100) beside a DP sand dam 50x80x100 (400k, phi=35, E=2e5,
    nu=0.3); 15 XPBI + 4 PBF iterations, dt=1e-4, 200 substeps.

    s_corr uses the reference's own k = 1e-4 (scenes.js:89). With k = 0.1 the
    reference's correction, (lambda_i + lambda_j + s_corr) gradW * m / rho0
    (simkernels.js:467), moves a pair ~0.8 m at this spacing and every
    particle hits the CFL cap in the first substep.
    ``scale`` < 1 shrinks the z extent (fewer particles) for quick checks."""
    rng = np.random.default_rng(seed)
    r = 0.008
    s = base(r)
    s.update(domainMin=[0.0, 0.0, 0.0], domainMax=[2.0, 1.0, 1.0])
    z0, z1 = 0.1, 0.1 + 0.8 * scale
    pos, mid, st = [], [], []
    sample_box(rng, pos, mid, st, [0.008, 0.0, z0], [0.608, 0.64, z1], r, 1)
    sample_box(rng, pos, mid, st, [0.70, 0.0, z0], [1.10, 0.64, z1], r, 0)
    sand = dict(kind=DP, E=2e5, nu=0.3, density=1600.0, p0=dp_alpha(35), p1=0.0,
                color=[0.85, 0.63, 0.28], boundFriction=0.5)
    water = dict(kind=WATER, E=100, nu=0.3, density=1000.0, color=[0.25, 0.55, 0.95], boundFriction=0.0)
    _finish(s, rng, pos, mid, st, [sand, water], True)
    return _solver(s, 1e-4, 15, 200, pbfIterations=4, sCorrK=1e-4, pbfEps=100.0)


def config_batch(n_scenes=256, seed=0, n_lo=2000, n_hi=60000):
    """Batch of independent scenes: sizes log-uniform in [n_lo, n_hi], box or
    sphere lattice at r=0.01, material uniform over {DP, NACC, VM, HB, SNOW},
    E log-uniform in [5e4, 5e5], nu=0.3, 10..20 iterations each; each scene's
    domain is its body's bounding box padded by 4 cells."""
    rng = np.random.default_rng(seed)
    r = 0.01
    out = []
    for si in range(n_scenes):
        target = int(math.floor(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        E = float(math.exp(rng.uniform(math.log(5e4), math.log(5e5))))
        kind = int(rng.choice([DP, NACC, VM, HB, SNOW]))
        state0 = 0.0
        if kind == DP:
            mat = dict(kind=DP, E=E, nu=0.3, density=1000.0, p0=dp_alpha(float(rng.uniform(25, 40))), p1=0.0)
        elif kind == NACC:
            mat = dict(kind=NACC, E=E, nu=0.3, density=400.0, p0=-0.04, p1=0.5, p2=3.0, p3=1.85)
            state0 = -0.04
        elif kind == VM:
            mat = dict(kind=VM, E=E, nu=0.3, density=1000.0,
                       p0=float(math.exp(rng.uniform(math.log(1e3), math.log(1e4)))))
        elif kind == HB:
            mat = dict(kind=HB, E=E, nu=0.3, density=1000.0, p0=float(rng.uniform(50, 500)),
                       p1=float(rng.uniform(0.3, 1.0)), p2=float(rng.uniform(1, 50)))
        else:
            mat = dict(kind=SNOW, E=E, nu=0.3, density=400.0, p0=2.5e-2, p1=7.5e-3, p2=10.0)
            state0 = 1.0
        mat.update(color=[0.8, 0.8, 0.8], boundFriction=0.4)
        s = base(r)
        pos, mid, st = [], [], []
        if rng.random() < 0.5:
            side = max(2, _jsround((target / 2) ** (1 / 3)))
            ny = max(2, _jsround(target / (side * side)))
            lo = [0.1, 0.1, 0.1]
            hi = [0.1 + side * r, 0.1 + ny * r, 0.1 + side * r]
            sample_box(rng, pos, mid, st, lo, hi, r, 0, 0.2, state0)
        else:
            R = r * (3 * target / (4 * math.pi)) ** (1 / 3)
            sample_sphere(rng, pos, mid, st, [0.1 + R, 0.1 + R, 0.1 + R], R, r, 0, 0.2, state0)
        p = pos[0]
        cs = 2 * r
        dmin = [float(p[:, k].min() - 4 * cs) for k in range(3)]
        dmax = [float(p[:, k].max() + 4 * cs) for k in range(3)]
        dmin[1] = float(p[:, 1].min() - 0.5 * r)
        s.update(domainMin=dmin, domainMax=dmax)
        _finish(s, rng, pos, mid, st, [mat], False)
        _solver(s, 1e-4, int(rng.integers(10, 21)), 200)
        out.append(s)
    return out


def config_dam_mix(seeds=(0, 1, 2, 3), scale=1.0):
    """The dam-breach scene mix at 4M particles: one scene per seed."""
    return [config_dam_breach(seed=s, scale=scale) for s in seeds]


CONFIGS = {
    "sand_column": config_sand_column,
    "nacc_snowball": config_nacc_snowball,
    "dam_breach": config_dam_breach,
    "batch256": config_batch,
    "dam_mix4": config_dam_mix,
}
