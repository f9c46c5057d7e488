"""Host-side checks of libxpbi (no GPU): every declared symbol is exported,
uniform packing follows sim.js, and invalid scenes are rejected."""
import ctypes as C
import math
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "xpbi.h")).read()
    return sorted(set(re.findall(r"\b(xpbi_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(xp, built_lib):
    from importlib import import_module
    abi = import_module("xpbi-webgpu_gb300._abi")
    declared = _declared_symbols()
    assert declared == sorted(abi.EXPORTS)
    lib = C.CDLL(abi.LIB_PATH)
    for name in declared:
        assert hasattr(lib, name), name


def _f(words, k):
    return float(np.frombuffer(np.asarray(words, np.uint32)[k:k + 1].tobytes(), np.float32)[0])


def test_pack_uniforms_matches_sim_js_layout(xp, built_lib):
    sc = xp.scenes.config_dam_breach(scale=0.05)
    p = xp.params_for(sc, colliderActive=True, colliderPos=[0.1, 0.2, 0.3], colliderR=0.05,
                      colliderVel=[1.0, 2.0, 3.0], time=1.5)
    pw, mw = xp.pack_uniforms(sc, p)
    h = 0.008
    cs = 2 * h
    # grid sizing, sim.js:20-26 (f64)
    dims = [math.ceil((sc["domainMax"][k] - sc["domainMin"][k]) / cs) + 4 for k in range(3)]
    assert list(pw[4:7]) == dims == [129, 67, 67]
    assert int(pw[7]) == 129 * 67 * 67 == 579081
    for k in range(3):
        assert _f(pw, k) == np.float32(sc["domainMin"][k] - 2 * cs)
    assert _f(pw, 3) == np.float32(cs) and _f(pw, 19) == np.float32(cs)
    assert _f(pw, 11) == np.float32(1e-4)
    assert _f(pw, 15) == np.float32(h)
    assert _f(pw, 17) == np.float32(-9.81)
    assert [_f(pw, 20 + k) for k in range(3)] == [np.float32(x) for x in (0.1, 0.2, 0.3)]
    assert _f(pw, 23) == np.float32(0.05) and _f(pw, 27) == 1.0
    assert [_f(pw, 24 + k) for k in range(3)] == [1.0, 2.0, 3.0]
    assert int(pw[28]) == len(sc["positions"])
    assert _f(pw, 29) == np.float32(h ** 3)
    assert _f(pw, 30) == np.float32(0.01) and _f(pw, 31) == np.float32(0.5)
    assert _f(pw, 32) == np.float32(100.0) and _f(pw, 33) == np.float32(1e-4)
    assert _f(pw, 34) == np.float32(1.5) and _f(pw, 35) == np.float32(0.4) and _f(pw, 36) == np.float32(0.4)
    # materials, sim.js:84-99: mu, lam from E, nu in f64; mass = rho * V0
    E, nu = 2e5, 0.3
    assert _f(mw, 0) == np.float32(E / (2 * (1 + nu)))
    assert _f(mw, 1) == np.float32(E * nu / ((1 + nu) * (1 - 2 * nu)))
    assert _f(mw, 2) == 1600.0 and int(mw[3]) == xp.scenes.DP
    assert _f(mw, 4) == np.float32(xp.scenes.dp_alpha(35))
    assert _f(mw, 12) == np.float32(0.5) and _f(mw, 13) == np.float32(1600.0 * h ** 3)
    assert int(mw[16 + 3]) == xp.scenes.WATER and _f(mw, 16 + 2) == 1000.0
    assert _f(mw, 11) == 1.0  # colour alpha
    assert not mw[32:].any()


def test_bound_friction_default(xp, built_lib):
    sc = xp.scenes.elastic_block()
    sc["materials"][0]["boundFriction"] = None
    _, mw = xp.pack_uniforms(sc, xp.params_for(sc))
    assert _f(mw, 12) == np.float32(0.4)


@pytest.mark.parametrize("mutate, msg", [
    (lambda s: s.update(h=0.0), "h must be positive"),
    (lambda s: s.update(domainMax=[0.0, 1.0, 1.0]), "domain_max"),
    (lambda s: s.update(materials=[]), "n_materials"),
    (lambda s: s.update(matIds=np.full(len(s["matIds"]), 3, np.uint32)), "mat_ids"),
    (lambda s: s["materials"][0].update(kind=9), "kind out of range"),
])
def test_invalid_scenes_rejected(xp, built_lib, mutate, msg):
    sc = xp.scenes.elastic_block()
    mutate(sc)
    with pytest.raises(xp.XpbiError) as e:
        xp.pack_uniforms(sc, xp.params_for(sc))
    assert e.value.code == 1 and msg in str(e.value)


def test_empty_scene_packs(xp, built_lib):
    sc = xp.scenes.elastic_block()
    sc["positions"] = np.zeros((0, 3), np.float32)
    sc["matIds"] = np.zeros(0, np.uint32)
    sc["states"] = np.zeros(0, np.float32)
    sc["colorSeeds"] = np.zeros(0, np.float32)
    pw, _ = xp.pack_uniforms(sc, xp.params_for(sc))
    assert int(pw[28]) == 0


def test_render_camera_follows_main_js(xp):
    import math
    cam = xp.render.camera()  # scenes.js:90 orbit
    t, p, d, tgt = 0.5, 0.32, 2.1, [0.5, 0.28, 0.5]
    want = [tgt[0] + d * math.cos(p) * math.sin(t), tgt[1] + d * math.sin(p), tgt[2] + d * math.cos(p) * math.cos(t)]
    assert np.allclose(list(cam.eye), want, rtol=1e-6)
    assert cam.fov_y == pytest.approx(math.pi / 4) and cam.near_z == pytest.approx(0.02) and cam.far_z == 50


def test_ppm_writer(xp, tmp_path):
    img = np.zeros((2, 3, 4), np.uint8)
    img[0, 1, :3] = (10, 20, 30)
    xp.render.write_ppm(str(tmp_path / "a.ppm"), img)
    data = (tmp_path / "a.ppm").read_bytes()
    assert data.startswith(b"P6\n3 2\n255\n") and data[len(b"P6\n3 2\n255\n") + 3:][:3] == bytes((10, 20, 30))


def test_oracle_packing_equals_the_abi(xp, built_lib):
    """The CPU paths pack their uniforms with oracle/uniforms.py (no library);
    it must give the ABI's words for every demo scene and benchmark config,
    including a collider and explicit damping."""
    from oracle import uniforms as U
    scenes = [f() for f in xp.scenes.SCENES.values()]
    scenes += [xp.scenes.config_sand_column(), xp.scenes.config_nacc_snowball(),
               xp.scenes.config_dam_breach(scale=0.05)]
    scenes += xp.scenes.config_batch(n_scenes=12, seed=3)
    for sc in scenes:
        for over in ({}, dict(colliderActive=True, colliderPos=[0.1, 0.2, 0.3], colliderR=0.05,
                              colliderVel=[1.0, -2.0, 0.5], time=0.25, kDamp=0.3)):
            p = xp.params_for(sc, **over)
            assert p == U.frame_params(sc, **over)
            pw, mw = xp.pack_uniforms(sc, p)
            opw, omw = U.pack(sc, p)
            assert np.array_equal(pw, opw)
            assert np.array_equal(mw, omw)
