"""Scene sampling on the device (xpbi_sample_shapes) against the host
sampler (scenes.py, itself pinned to web/js/scenes.js:7-38): the same
lattice bit for bit, in the same order, with jitter drawn from the
Philox-4x32-10 stream the oracle restates."""
import importlib
import json
import time

import numpy as np
import pytest

from oracle import philox as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ds(built_lib):
    return importlib.import_module("xpbi-webgpu_gb300.device_sample")


def _host(xp, shapes, h, seed=0):
    S = xp.scenes
    rng = np.random.default_rng(seed)
    out, mid, st = [], [], []
    for d in shapes:
        if d["kind"] == 0:
            S.sample_box(rng, out, mid, st, d["lo"], d["hi"], h, d["mat_id"], d["jitter"], d["state0"])
        else:
            S.sample_sphere(rng, out, mid, st, d["centre"], d["radius"], h, d["mat_id"], d["jitter"], d["state0"])
    return np.concatenate(out), np.concatenate(mid), np.concatenate(st)


def _shapes(ds, jitter):
    return [ds.box([0.008, 0.0, 0.1], [0.608, 0.64, 0.18], 1, jitter),      # the dam breach's water, 10% of z
            ds.box([0.4, 0.0, 0.4], [0.6, 0.4, 0.6], 0, jitter, -0.04),       # the sand column
            ds.sphere([0.36, 0.5, 0.5], 0.3, 2, jitter, -0.04),             # the snowball (d == r points included)
            ds.box([0.0, 0.0, 0.0], [0.001, 0.3, 0.002], 3, jitter)]        # Math.max(1, ...) on thin extents


def test_lattice_equals_the_host_sampler(xp, ds):
    for h in (0.008, 0.01):
        shapes = _shapes(ds, 0.0)
        pos, mid, st = ds.sample_shapes(shapes, h, seed=3)
        hp, hm, hs = _host(xp, shapes, h)
        assert len(pos) == len(hp)
        assert np.array_equal(pos, hp.astype(np.float32))  # point for point, in the reference's order
        assert np.array_equal(mid, hm) and np.array_equal(st, hs.astype(np.float32))


def test_jitter_follows_the_generator(xp, ds):
    h, seed = 0.01, 0x1234_5678_9ABC
    shapes = _shapes(ds, 0.2)
    pos, _, _ = ds.sample_shapes(shapes, h, seed)
    lattice, _, _ = _host(xp, _shapes(ds, 0.0), h)
    rng = np.random.default_rng(0)
    for q in rng.choice(len(pos), 300, replace=False).tolist() + [0, len(pos) - 1]:
        want = np.array(P.jitter(lattice[q], q, seed, 0.2 * h), np.float32)
        assert np.array_equal(pos[q], want), q
    off = (pos.astype(np.float64) - lattice) / h
    assert np.abs(off).max() <= 0.1 + 2e-5  # +- 0.1 h, plus the f32 rounding of coordinates up to 1 m
    assert abs(off.mean()) < 2e-3 and abs(off.std() - 0.2 / np.sqrt(12)) < 2e-3
    again, _, _ = ds.sample_shapes(shapes, h, seed)
    other, _, _ = ds.sample_shapes(shapes, h, seed + 1)
    assert np.array_equal(again, pos) and not np.array_equal(other, pos)


def test_large_scene_on_the_device(xp, ds):
    """The 4M-particle dam-breach mix's shapes: sampled on the device against
    the host sampler's time (printed), same lattice counts."""
    shapes, host_n = [], 0
    for k in range(4):
        shapes += [ds.box([0.008, 0.0, 0.1], [0.608, 0.64, 0.9], 1), ds.box([0.70, 0.0, 0.1], [1.10, 0.64, 0.9], 0)]
    ds.sample_shapes(shapes[:1], 0.008)  # context and module loading out of the timing
    t0 = time.perf_counter()
    pos, mid, _ = ds.sample_shapes(shapes, 0.008, seed=1)
    t_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    mix = xp.scenes.config_dam_mix()
    t_host = time.perf_counter() - t0
    host_n = sum(len(s["positions"]) for s in mix)
    print(json.dumps({"particles": len(pos), "device_s": round(t_dev, 4), "host_s": round(t_host, 4)}))
    assert len(pos) == host_n == 4_000_000
    assert (mid[:600_000] == 1).all() and (mid[600_000:1_000_000] == 0).all()
