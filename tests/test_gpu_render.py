"""The headless renderer (xpbi_render) against the CPU restatement of the
reference's frame (oracle/render_ref.py): background, gridded ground and
sphere impostors of sand and water particles."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tiny_scene(xp):
    rng = np.random.default_rng(3)
    n = 60
    s = xp.scenes.dam_breach()
    pos = np.column_stack([rng.uniform(0.3, 0.7, n), rng.uniform(0.05, 0.5, n), rng.uniform(0.3, 0.7, n)])
    kinds = [m["kind"] for m in s["materials"]]
    sand, water = kinds.index(1), kinds.index(6)
    mat = np.where(np.arange(n) % 2 == 0, sand, water).astype(np.uint32)
    vel = np.column_stack([np.zeros(n), -rng.uniform(0, 3, n), np.zeros(n)])
    return dict(s, positions=pos.astype(np.float32), matIds=mat, states=np.zeros(n, np.float32),
                velocities=vel.astype(np.float32), colorSeeds=rng.uniform(0, 0.49, n).astype(np.float32))


def test_render_matches_the_cpu_restatement(xp, built_lib):
    from oracle import render_ref
    sc = _tiny_scene(xp)
    W, H = 96, 64
    with xp.Simulation(sc) as sim:
        sim.write_params(xp.params_for(sc))
        cam = xp.render.camera(sc["camera"], draw_box=False, particle_radius=0.03)
        img = xp.render.render(sim, 0, cam, W, H)
        again = xp.render.render(sim, 0, cam, W, H)
        st = sim.read_state()
        _, mw = sim.uniforms()
    assert np.array_equal(img, again)  # deterministic
    ref = render_ref.render(st["pos"], st["vel"], mw, list(cam.eye), list(cam.target), W, H, 0.03,
                            sc["domainMin"][1])
    diff = np.abs(img.astype(int) - ref.astype(int)).max(axis=2)
    assert (diff <= 1).mean() >= 0.995, (diff > 1).sum()
    particles = (ref != render_ref.render(st["pos"][:0], st["vel"][:0], mw, list(cam.eye), list(cam.target),
                                          W, H, 0.03, sc["domainMin"][1])).any(axis=2)
    assert particles.sum() > 100  # the particles cover part of the frame


def test_render_demo_scene_frame(xp, built_lib, tmp_path):
    sc = xp.scenes.sand_column()
    with xp.Simulation(sc) as sim:
        sim.write_params(xp.params_for(sc))
        empty = xp.render.render(sim, 0, xp.render.camera(sc["camera"]), 320, 180)
        sim.step(20, sc["iterations"], sc["hasWater"])
        img = xp.render.render(sim, 0, xp.render.camera(sc["camera"]), 320, 180)
    xp.render.write_ppm(str(tmp_path / "frame.ppm"), img)
    assert (tmp_path / "frame.ppm").stat().st_size == 320 * 180 * 3 + len(b"P6\n320 180\n255\n")
    assert img.shape == (180, 320, 4) and (img[..., 3] == 255).all()
    assert (np.abs(img.astype(int) - empty.astype(int)).max(axis=2) > 0).sum() > 1000
