"""The host samplers against the reference's sampling loops (no GPU).

`sample_box` / `sample_sphere` (scenes.py) are vectorised NumPy; every
benchmark input comes from them. Here they are pinned to a scalar,
loop-for-loop restatement of web/js/scenes.js:7-38 driven by the same
random stream one draw at a time (the reference's Math.random() replaced by
the seeded generator, drawn in the reference's order: k, j, i loops, then x,
y, z per particle, and for the sphere only for accepted lattice points).
"""
import importlib
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def S():
    return importlib.import_module("xpbi-webgpu_gb300.scenes")


def js_round(x):
    return math.floor(x + 0.5)  # Math.round: halves toward +infinity


def js_hypot(*args):
    """Math.hypot as Chrome's V8 computes it (the browser the reference's
    README measures in): magnitudes scaled by the largest, squares summed with
    Kahan compensation in argument order, sqrt(sum) * max."""
    a = [abs(x) for x in args]
    m = max(a)
    if m == 0:
        return 0.0
    total = comp = 0.0
    for x in a:
        n = x / m
        summand = n * n - comp
        prelim = total + summand
        comp = (prelim - total) - summand
        total = prelim
    return math.sqrt(total) * m


def js_sample_box(random, lo, hi, h, mat, jitter=0.2, state0=0.0):
    """web/js/scenes.js:7-20, statement for statement."""
    out, mid, states = [], [], []
    n = [max(1, js_round((hi[i] - lo[i]) / h)) for i in range(3)]
    for k in range(n[2]):
        for j in range(n[1]):
            for i in range(n[0]):
                out.append((lo[0] + (i + 0.5) * h + (random() - 0.5) * jitter * h,
                            lo[1] + (j + 0.5) * h + (random() - 0.5) * jitter * h,
                            lo[2] + (k + 0.5) * h + (random() - 0.5) * jitter * h))
                mid.append(mat)
                states.append(state0)
    return np.array(out), np.array(mid), np.array(states)


def js_sample_sphere(random, c, r, h, mat, jitter=0.2, state0=0.0):
    """web/js/scenes.js:22-38, statement for statement."""
    out, mid, states = [], [], []
    n = math.ceil(2 * r / h)
    for k in range(n + 1):
        for j in range(n + 1):
            for i in range(n + 1):
                p = (c[0] - r + i * h, c[1] - r + j * h, c[2] - r + k * h)
                d = js_hypot(p[0] - c[0], p[1] - c[1], p[2] - c[2])
                if d <= r:
                    out.append((p[0] + (random() - 0.5) * jitter * h,
                                p[1] + (random() - 0.5) * jitter * h,
                                p[2] + (random() - 0.5) * jitter * h))
                    mid.append(mat)
                    states.append(state0)
    return np.array(out).reshape(-1, 3), np.array(mid), np.array(states)


def _host_box(S, seed, *args, **kw):
    out, mid, st = [], [], []
    S.sample_box(np.random.default_rng(seed), out, mid, st, *args, **kw)
    return out[0], mid[0], st[0]


def _host_sphere(S, seed, *args, **kw):
    out, mid, st = [], [], []
    S.sample_sphere(np.random.default_rng(seed), out, mid, st, *args, **kw)
    return out[0], mid[0], st[0]


@pytest.mark.parametrize("lo, hi, h", [
    ([0.0, 0.0, 0.0], [0.2, 0.1, 0.05], 0.01),       # 20 x 10 x 5
    ([0.4, 0.0, 0.4], [0.6, 0.4, 0.6], 0.01),        # the sand column's 20 x 40 x 20
    ([0.0, 0.0, 0.0], [1.25, 0.75, 0.5], 0.5),       # halves: Math.round(2.5) = 3, (1.5) = 2, (1) = 1
    ([0.0, 0.0, 0.0], [0.001, 0.3, 0.002], 0.01),    # Math.max(1, ...) on thin extents
])
def test_sample_box_follows_scenes_js(S, lo, hi, h):
    rng = np.random.default_rng(11)
    want, wmid, wst = js_sample_box(rng.random, lo, hi, h, 3, state0=-0.04)
    got, mid, st = _host_box(S, 11, lo, hi, h, 3, state0=-0.04)
    n = [max(1, js_round((hi[i] - lo[i]) / h)) for i in range(3)]
    assert len(got) == len(want) == n[0] * n[1] * n[2]
    assert np.array_equal(got, want)  # same lattice, same draws, same arithmetic
    assert (mid == 3).all() and (wmid == 3).all() and np.array_equal(st, wst)


def test_box_lattice_offsets_and_jitter(S):
    """Cell-centre lattice (i + 0.5) h with jitter (rand - 0.5) 0.2 h: each
    particle lies within +-0.1 h of its lattice point, and the jitter covers
    that range."""
    lo, hi, h = [0.1, 0.2, 0.3], [0.5, 0.4, 0.4], 0.02
    got, _, _ = _host_box(S, 5, lo, hi, h, 0)
    n = [20, 10, 5]
    k, j, i = np.meshgrid(np.arange(n[2]), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    lattice = np.stack([lo[0] + (i.ravel() + 0.5) * h, lo[1] + (j.ravel() + 0.5) * h,
                        lo[2] + (k.ravel() + 0.5) * h], axis=1)
    off = (got - lattice) / h
    assert np.abs(off).max() <= 0.1 + 1e-12
    assert off.min() < -0.099 and off.max() > 0.099
    assert abs(off.mean()) < 0.01
    zero = _host_box(S, 5, lo, hi, h, 0, jitter=0.0)[0]
    assert np.array_equal(zero, lattice)


@pytest.mark.parametrize("c, r, h", [
    ([0.36, 0.5, 0.5], 0.05, 0.01),    # the snowball's lattice at a tenth of its radius
    ([0.5, 0.5, 0.5], 0.1, 0.02),
    ([0.0, 0.0, 0.0], 1.0, 0.25),      # lattice points exactly on the sphere (d == r)
])
def test_sample_sphere_follows_scenes_js(S, c, r, h):
    rng = np.random.default_rng(3)
    want, _, _ = js_sample_sphere(rng.random, c, r, h, 2, state0=-0.04)
    got, mid, st = _host_sphere(S, 3, c, r, h, 2, state0=-0.04)
    assert len(got) == len(want)
    assert np.array_equal(got, want)
    assert (mid == 2).all() and (st == -0.04).all()
    # membership: every accepted lattice point within r of the centre, and
    # every rejected one outside
    n = math.ceil(2 * r / h)
    pts = [(c[0] - r + i * h, c[1] - r + j * h, c[2] - r + kk * h)
           for kk in range(n + 1) for j in range(n + 1) for i in range(n + 1)]
    inside = sum(1 for p in pts if js_hypot(p[0] - c[0], p[1] - c[1], p[2] - c[2]) <= r)
    assert inside == len(got)


def test_sphere_count_at_the_snowball_size(S):
    """The NACC snowball config's sphere (R = 0.3 at r = 0.01): the lattice
    count the reference's loop gives (its membership test in f64)."""
    c, r, h = [0.36, 0.5, 0.5], 0.3, 0.01
    n = math.ceil(2 * r / h)
    ax = np.arange(n + 1)
    k, j, i = np.meshgrid(ax, ax, ax, indexing="ij")
    p = np.stack([c[0] - r + i.ravel() * h, c[1] - r + j.ravel() * h, c[2] - r + k.ravel() * h], axis=1)
    d = np.array([js_hypot(*(q - np.asarray(c))) for q in p])
    got, _, _ = _host_sphere(S, 0, c, r, h, 0)
    assert len(got) == int((d <= r).sum())
    # the naive norm puts some of the surface points on the other side
    naive = np.sqrt(((p - np.asarray(c)) ** 2).sum(axis=1))
    assert int((naive <= r).sum()) != len(got)
    assert abs(len(got) - 4 / 3 * math.pi * 30 ** 3) < 0.01 * 4 / 3 * math.pi * 30 ** 3
