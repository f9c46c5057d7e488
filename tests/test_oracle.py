"""The oracle itself: pinned against the reference prototype's golden
vectors, then checked against known answers derived from the mathematics
(the reference ships no tests or fixtures of its own)."""
import json
import math
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _mat_words(kind, E, nu, density=1000.0, p=(0, 0, 0, 0), h=0.01, bf=0.4):
    """One material packed like sim.js:84-99 (f32 words)."""
    mu = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    w = np.zeros(16, np.float32)
    w[0], w[1], w[2] = mu, lam, density
    w[4:8] = p
    w[12], w[13] = bf, density * h ** 3
    u = w.view(np.uint32).copy()
    u[3] = kind
    return u


# ------------------------------------------------------------ golden vectors
def test_drucker_prager_matches_reference_prototype(oracle):
    gold = json.load(open(os.path.join(HERE, "golden", "dp_stvk_prototype.json")))
    for c in gold["cases"]:
        S = np.array(c["sigma"])
        mw = _mat_words(1, c["E"], c["nu"], p=(c["alpha"], 0, 0, 0))
        # the oracle reads mu, lambda, alpha from f32 words: feed the f64
        # prototype the same rounded values
        mu = float(mw[:1].view(np.float32)[0])
        out, _ = oracle.return_map(mw, 1e-4, S, np.zeros(len(S)))
        ref = np.array(c["dp"])
        # the prototype evaluates with f64 mu/lambda/alpha, the words are f32
        np.testing.assert_allclose(out, ref, rtol=2e-6, atol=2e-6)
        assert mu > 0


def test_stvk_matches_reference_prototype(oracle):
    gold = json.load(open(os.path.join(HERE, "golden", "dp_stvk_prototype.json")))
    for c in gold["cases"]:
        S = np.array(c["sigma"])
        psi, dpsi = oracle.stvk(c["mu"], c["lam"], S)
        np.testing.assert_allclose(psi, c["psi"], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(dpsi, c["dpsi"], rtol=1e-12, atol=1e-9)


# ------------------------------------------------------------ SPH kernels
def test_wendland_normalised_and_gradient(oracle):
    h = 0.01
    n = 64
    x = (np.arange(n) + 0.5) / n * 4 * h - 2 * h
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    d = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    w, g = oracle.wendland(h, d)
    integral = w.sum() * (4 * h / n) ** 3
    assert abs(integral - 1.0) < 2e-3
    # gradient vs central differences of W
    pts = np.random.default_rng(0).uniform(-1.8 * h, 1.8 * h, (200, 3))
    eps = 1e-7
    for k in range(3):
        dp = pts.copy(); dp[:, k] += eps
        dm = pts.copy(); dm[:, k] -= eps
        fd = (oracle.wendland(h, dp)[0] - oracle.wendland(h, dm)[0]) / (2 * eps)
        np.testing.assert_allclose(oracle.wendland(h, pts)[1][:, k], fd, rtol=1e-5, atol=1e-2)


def test_poly6_normalised_and_spiky_gradient(oracle):
    h = 0.01
    H = 2 * h
    n = 64
    x = (np.arange(n) + 0.5) / n * 2 * H - H
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    d = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    w, _ = oracle.pbf_kernels(h, d)
    assert abs(w.sum() * (2 * H / n) ** 3 - 1.0) < 2e-3
    pts = np.random.default_rng(1).uniform(-0.9 * H, 0.9 * H, (300, 3))
    pts = pts[np.linalg.norm(pts, axis=1) < 0.95 * H]
    r = np.linalg.norm(pts, axis=1)
    _, g = oracle.pbf_kernels(h, pts)
    # spiky W = 15/(pi H^6) (H - r)^3  ->  grad = -45/(pi H^6) (H - r)^2 x/r
    want = (-45 / (math.pi * H ** 6) * (H - r) ** 2 / r)[:, None] * pts
    np.testing.assert_allclose(g, want, rtol=1e-6)


# ------------------------------------------------------------ svd3
@pytest.mark.parametrize("seed", range(4))
def test_svd3_reconstructs(oracle, seed):
    rng = np.random.default_rng(seed)
    for _ in range(200):
        F = np.eye(3) + 0.3 * rng.standard_normal((3, 3))
        Fc = F.T.reshape(9).astype(np.float32)  # column-major
        U, s, V = oracle.svd3(Fc)
        assert s[0] >= s[1] >= abs(s[2]) - 1e-6
        np.testing.assert_allclose(U @ np.diag(s) @ V.T, F, atol=2e-5)
        np.testing.assert_allclose(U.T @ U, np.eye(3), atol=1e-5)
        np.testing.assert_allclose(V.T @ V, np.eye(3), atol=1e-5)
        assert np.linalg.det(U) > 0 and np.linalg.det(V) > 0
        if np.linalg.det(F) < 0:
            assert s[2] < 0


def test_svd3_degenerate_identity(oracle):
    U, s, V = oracle.svd3(np.eye(3, dtype=np.float32).reshape(9))
    np.testing.assert_allclose(s, [1, 1, 1], atol=1e-7)
    np.testing.assert_allclose(U @ np.diag(s) @ V.T, np.eye(3), atol=1e-6)


# ------------------------------------------------------------ return maps
def _dev_norm(s):
    e = np.log(s)
    return np.linalg.norm(e - e.sum(1, keepdims=True) / 3, axis=1), e.sum(1)


def test_von_mises_projects_onto_yield_surface(oracle):
    E, nu, sy = 1e5, 0.3, 2000.0
    mw = _mat_words(3, E, nu, p=(sy, 0, 0, 0))
    mu = float(mw[:1].view(np.float32)[0])
    S = np.random.default_rng(3).uniform(0.8, 1.25, (500, 3))
    out, _ = oracle.return_map(mw, 1e-4, S, np.zeros(len(S)))
    dn0, tr0 = _dev_norm(S)
    dn1, tr1 = _dev_norm(out)
    yielded = dn0 > sy / (2 * mu)
    assert yielded.any() and (~yielded).any()
    np.testing.assert_allclose(dn1[yielded], sy / (2 * mu), rtol=1e-6)
    np.testing.assert_allclose(tr1, tr0, atol=1e-12)
    np.testing.assert_array_equal(out[~yielded], S[~yielded])


def test_drucker_prager_cases(oracle):
    E, nu = 1e5, 0.3
    a = math.sqrt(2 / 3) * 2 * math.sin(math.radians(30)) / (3 - math.sin(math.radians(30)))
    mw = _mat_words(1, E, nu, p=(a, 0, 0, 0))
    w = mw.view(np.float32)
    mu, lam, af = float(w[0]), float(w[1]), float(w[4])
    S = np.random.default_rng(4).uniform(0.8, 1.2, (600, 3))
    out, _ = oracle.return_map(mw, 1e-4, S, np.zeros(len(S)))
    dn, tr = _dev_norm(S)
    dg = dn + af * (3 * lam + 2 * mu) / (2 * mu) * tr
    tip = tr > 0
    np.testing.assert_allclose(out[tip], 1.0, atol=1e-12)
    el = (~tip) & (dg <= 0)
    np.testing.assert_array_equal(out[el], S[el])
    cone = (~tip) & (dg > 0)
    assert tip.any() and el.any() and cone.any()
    dn1, tr1 = _dev_norm(out[cone])
    np.testing.assert_allclose(tr1, tr[cone], atol=1e-12)
    np.testing.assert_allclose(dn1 + af * (3 * lam + 2 * mu) / (2 * mu) * tr1, 0.0, atol=1e-10)


def test_drucker_prager_zero_deviator_goes_to_tip(oracle):
    """WGSL quirk (common.js:213): a pure compression with no deviator is
    projected to the tip (sigma = exp(cohesion)), not left elastic."""
    mw = _mat_words(1, 1e5, 0.3, p=(0.3, 0, 0, 0))
    out, _ = oracle.return_map(mw, 1e-4, np.full((1, 3), 0.9), np.zeros(1))
    np.testing.assert_allclose(out, 1.0)


def test_herschel_bulkley_analytic_and_bisection(oracle):
    E, nu, sy, eta, dt = 2250.0, 0.125, 45.0, 25.0, 1e-3
    S = np.random.default_rng(5).uniform(0.7, 1.4, (300, 3))
    for hexp in (1.0, 0.5, 0.3):
        mw = _mat_words(4, E, nu, p=(sy, hexp, eta, 0))
        mu = float(mw[:1].view(np.float32)[0])
        out, _ = oracle.return_map(mw, dt, S, np.zeros(len(S)))
        J = S.prod(1)
        np.testing.assert_allclose(out.prod(1), J, rtol=1e-9)  # volume kept
        bb = S ** 2 * J[:, None] ** (-2 / 3)
        s_pre = mu * np.linalg.norm(bb - bb.sum(1, keepdims=True) / 3, axis=1)
        sY = math.sqrt(2 / 3) * sy
        ob = out ** 2 * J[:, None] ** (-2 / 3)
        s_new = mu * np.linalg.norm(ob - ob.sum(1, keepdims=True) / 3, axis=1)
        flow = s_pre > sY
        assert flow.any() and (~flow).any()
        np.testing.assert_array_equal(out[~flow], S[~flow])
        # viscoplastic relaxation: strictly between the yield stress and the
        # trial stress (up to the det-1 renormalisation of b-bar)
        assert np.all(s_new[flow] < s_pre[flow])
        assert np.all(s_new[flow] > sY * 0.98)


def test_herschel_bulkley_inviscid_limit_is_yield_projection(oracle):
    """eta -> 0 (Bingham limit, common.js:258-259): s_new = sqrt(2/3) sigmaY."""
    E, nu, sy = 2250.0, 0.125, 45.0
    mw = _mat_words(4, E, nu, p=(sy, 1.0, 0.0, 0))
    mu = float(mw[:1].view(np.float32)[0])
    S = np.random.default_rng(9).uniform(0.8, 1.25, (200, 3))
    out, _ = oracle.return_map(mw, 1e-3, S, np.zeros(len(S)))
    J = S.prod(1)
    bb = S ** 2 * J[:, None] ** (-2 / 3)
    s_pre = mu * np.linalg.norm(bb - bb.sum(1, keepdims=True) / 3, axis=1)
    flow = s_pre > math.sqrt(2 / 3) * sy
    ob = out ** 2 * J[:, None] ** (-2 / 3)
    s_new = mu * np.linalg.norm(ob - ob.sum(1, keepdims=True) / 3, axis=1)
    # the deviator is scaled to the yield stress at fixed trace, then b-bar is
    # renormalised to det 1 (common.js:274-277), which rescales the deviator
    sY = math.sqrt(2 / 3) * sy
    tr3 = bb.sum(1, keepdims=True) / 3
    b_new = (bb - tr3) * (sY / s_pre)[:, None] + tr3
    np.testing.assert_allclose(s_new[flow], (sY * b_new.prod(1) ** (-1 / 3))[flow], rtol=1e-9)


def test_snow_clamp_and_hardening_state(oracle):
    mw = _mat_words(5, 9000.0, 0.2, p=(3.5e-2, 8e-3, 10, 0))
    S = np.random.default_rng(6).uniform(0.9, 1.1, (300, 3))
    st = np.full(len(S), 1.0)
    out, st2 = oracle.return_map(mw, 1e-3, S, st)
    lo, hi = 1 - np.float32(3.5e-2), 1 + np.float32(8e-3)
    assert out.min() >= lo - 1e-12 and out.max() <= hi + 1e-12
    np.testing.assert_allclose(st2, np.clip(S.prod(1) / out.prod(1), 0.2, 2.0), rtol=1e-12)


def test_nacc_compression_tip(oracle):
    """Strong compression (p > p0) projects to the (p0, 0) tip: all three
    singular values equal J_n^(1/3), and alpha += log(J_tr / J_n)."""
    E, nu, beta, xi, M = 1.4e5, 0.3, 0.5, 3.0, 1.85
    mw = _mat_words(2, E, nu, p=(-0.04, beta, xi, M))
    w = mw.view(np.float32)
    mu, lam = float(w[0]), float(w[1])
    kappa = 2 / 3 * mu + lam
    alpha0 = -0.04
    S = np.array([[0.7, 0.72, 0.75]])
    out, a = oracle.return_map(mw, 1e-4, S, np.array([alpha0]))
    p0 = kappa * (1e-5 + math.sinh(min(xi * max(-alpha0, 0), 4)))
    Jn = math.sqrt(max(-2 * p0 / kappa + 1, 1e-6))
    np.testing.assert_allclose(out, Jn ** (1 / 3), rtol=1e-12)
    np.testing.assert_allclose(a, alpha0 + math.log(S.prod() / Jn), rtol=1e-12)


def test_nacc_elastic_inside_ellipse(oracle):
    mw = _mat_words(2, 1.4e5, 0.3, p=(-0.04, 0.5, 3.0, 1.85))
    S = np.array([[1.0, 1.0, 1.0]])
    out, a = oracle.return_map(mw, 1e-4, S, np.array([-0.04]))
    np.testing.assert_array_equal(out, S)
    assert a[0] == -0.04


def test_nacc_hardening_state_clamped(oracle):
    mw = _mat_words(2, 1.4e5, 0.3, p=(-0.04, 0.5, 3.0, 1.85))
    out, a = oracle.return_map(mw, 1e-4, np.array([[1.0, 1.0, 1.0]]), np.array([-3.0]))
    assert a[0] == pytest.approx(-0.25)


def test_elastic_and_water_pass_through(oracle):
    S = np.random.default_rng(7).uniform(0.5, 1.5, (50, 3))
    for kind in (0, 6):
        out, st = oracle.return_map(_mat_words(kind, 1e4, 0.3), 1e-3, S, np.full(len(S), 0.3))
        np.testing.assert_array_equal(out, S)
        np.testing.assert_array_equal(st, 0.3)


def test_stvk_rest_state_and_gradient(oracle):
    psi, d = oracle.stvk(1000.0, 2000.0, np.ones((1, 3)))
    assert psi[0] == 0 and not d.any()
    S = np.random.default_rng(8).uniform(0.6, 1.6, (100, 3))
    psi, d = oracle.stvk(1000.0, 2000.0, S)
    eps = 1e-7
    for k in range(3):
        Sp = S.copy(); Sp[:, k] += eps
        Sm = S.copy(); Sm[:, k] -= eps
        fd = (oracle.stvk(1000.0, 2000.0, Sp)[0] - oracle.stvk(1000.0, 2000.0, Sm)[0]) / (2 * eps)
        np.testing.assert_allclose(d[:, k], fd, rtol=1e-5)


# ------------------------------------------------------------ full substep
def _small_scene(xp):
    sc = xp.scenes.dam_breach()
    return sc, xp.pack_uniforms(sc, xp.params_for(sc))


def test_substep_sort_invariants(xp, oracle, built_lib):
    sc, (pw, mw) = _small_scene(xp)
    st = oracle.initial_state(sc)
    out = oracle.substep(pw, mw, st, 2, True)
    n = len(st["pos"])
    idx = out["sortedIdx"].astype(np.int64)
    assert np.array_equal(np.sort(idx), np.arange(n))  # a permutation
    ct = out["cellTab"].astype(np.int64)
    assert ct[0] == 0 and np.all(np.diff(ct) >= 0) and ct[-1] <= n
    # cell of every pre-sort particle, recomputed in f32 like cellCoord
    o = pw[0:3].view(np.float32)
    cs = pw[3:4].view(np.float32)[0]
    dims = pw[4:7].astype(np.int64)
    p = st["pos"][:, :3]
    c = np.clip(np.floor((p - o) / cs), 0, dims - 1).astype(np.int64)
    key = c[:, 0] + c[:, 1] * dims[0] + c[:, 2] * dims[0] * dims[1]
    k_sorted = key[idx]
    assert np.all(np.diff(k_sorted) >= 0)  # cell order
    # within a cell: descending previous index (serial atomicSub semantics)
    same = np.diff(k_sorted) == 0
    assert np.all(np.diff(idx)[same] < 0)
    counts = np.bincount(key, minlength=int(pw[7]))
    np.testing.assert_array_equal(ct, np.concatenate([[0], np.cumsum(counts)[:-1]]))


def test_substep_thread_count_independent(xp, oracle, built_lib):
    sc, (pw, mw) = _small_scene(xp)
    st = oracle.initial_state(sc)
    a = oracle.substep(pw, mw, st, 3, True, substeps=2, threads=1)
    b = oracle.substep(pw, mw, st, 3, True, substeps=2, threads=4)
    for k in ("pos", "vel", "F", "L", "aux", "sortedIdx", "cellTab"):
        assert np.array_equal(a[k], b[k]), k


def test_substep_f32_close_to_f64(xp, oracle, built_lib):
    sc, (pw, mw) = _small_scene(xp)
    st = oracle.initial_state(sc)
    a = oracle.substep(pw, mw, st, 3, True, substeps=1)
    b = oracle.substep(pw, mw, st, 3, True, substeps=1, f64=True)
    for k in ("pos", "vel", "F"):
        err = np.abs(a[k] - b[k]).max() / np.abs(b[k]).max()
        assert err < 1e-4, (k, err)


def test_gravity_only_first_substep(xp, oracle, built_lib):
    """At rest with F = I nothing but gravity acts in the first substep of a
    well-separated lattice: v = g dt for every particle, x += dt v."""
    sc = xp.scenes.config_sand_column()
    pw, mw = xp.pack_uniforms(sc, xp.params_for(sc))
    st = oracle.initial_state(sc)
    out = oracle.substep(pw, mw, st, 10, False)
    dt = np.float32(2e-4)
    np.testing.assert_allclose(out["vel"][:, 1], np.float32(-9.81) * dt, rtol=1e-6)
    np.testing.assert_allclose(out["vel"][:, [0, 2]], 0.0, atol=1e-12)
    assert np.all(out["aux"][:, 1] == 0)


# ------------------------------------------------------------ reference golden substeps
def test_oracle_matches_reference_golden_substeps(oracle):
    """Golden substeps of the reference's own kernels (tests/golden/
    make_reference_golden.py: its WGSL translated to C++, five small scenes
    covering every material model, contact, walls, the collider and both PBF
    schedules). The oracle reproduces them: the sort bit-exactly, the state
    bit-exactly on the machine type that generated them and within 1e-5
    relative elsewhere (libm's exp / log / pow may round differently)."""
    import os
    import platform

    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_substeps.npz"))
    exact = str(z["machine"]) == platform.machine()
    for name in z["cases"]:
        it, hw, pbf, steps = (int(x) for x in z[f"{name}/run"])
        st = {k: z[f"{name}/in/{k}"] for k in ("pos", "vel", "F", "aux")}
        out = oracle.substep(z[f"{name}/params"], z[f"{name}/materials"], st, it, bool(hw), pbf, steps)
        for k in ("sortedIdx", "cellTab"):
            assert np.array_equal(out[k], z[f"{name}/out/{k}"]), (name, k)
        for k in ("pos", "vel", "F", "L", "aux"):
            ref = z[f"{name}/out/{k}"]
            if exact:
                assert np.array_equal(out[k], ref), (name, k)
            else:
                err = np.abs(out[k].astype(np.float64) - ref).max() / max(np.abs(ref).max(), 1e-30)
                assert err <= 1e-5, (name, k, err)
