"""Host mirror of the reference ``Simulation`` class (web/js/sim.js:9-273).

Method names follow the JS surface (``writeMaterials`` -> ``write_materials``
and so on) with the same argument meaning. Every compute call goes through
libxpbi's C ABI (include/xpbi.h); there is no other path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import Material, Params, SceneDesc, check, lib
from .scenes import frame_dt


def _fptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def _uptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_uint32))


def _written(out):
    """The entries a residual read-back filled (the buffer starts at -1, a
    value no norm takes; skipped iterations are NaN)."""
    filled = np.flatnonzero(~(out == -1.0))
    return out[: filled[-1] + 1] if len(filled) else out[:0]


def make_materials(materials) -> C.Array:
    arr = (Material * max(1, len(materials)))()
    for k, m in enumerate(materials):
        arr[k].kind = int(m["kind"])
        arr[k].E = float(m.get("E", 0.0))
        arr[k].nu = float(m.get("nu", 0.0))
        arr[k].density = float(m.get("density", 0.0))
        for p in ("p0", "p1", "p2", "p3"):
            setattr(arr[k], p, float(m.get(p, 0.0) or 0.0))
        col = m.get("color", [0.0, 0.0, 0.0])
        for c in range(3):
            arr[k].color[c] = float(col[c])
        bf = m.get("boundFriction")
        arr[k].bound_friction = 0.4 if bf is None else float(bf)  # sim.js:95
    return arr


class _SceneArgs:
    """Keeps the numpy buffers of a descriptor alive for one ABI call."""

    def __init__(self, scene: dict):
        self.pos = np.ascontiguousarray(scene["positions"], np.float32).reshape(-1)
        n = len(self.pos) // 3
        self.mid = np.ascontiguousarray(scene["matIds"], np.uint32).reshape(-1)
        st = scene.get("states")
        self.states = None if st is None else np.ascontiguousarray(st, np.float32).reshape(-1)
        v = scene.get("velocities")
        self.vel = None if v is None else np.ascontiguousarray(v, np.float32).reshape(-1)
        cs = scene.get("colorSeeds")
        self.seeds = None if cs is None else np.ascontiguousarray(cs, np.float32).reshape(-1)
        self.mats = make_materials(scene["materials"])
        d = SceneDesc()
        d.n = n
        d.positions = _fptr(self.pos)
        d.mat_ids = _uptr(self.mid)
        d.states = _fptr(self.states)
        d.velocities = _fptr(self.vel)
        d.color_seeds = _fptr(self.seeds)
        d.h = float(scene["h"])
        for k in range(3):
            d.domain_min[k] = float(scene["domainMin"][k])
            d.domain_max[k] = float(scene["domainMax"][k])
        d.n_materials = len(scene["materials"])
        d.materials = C.cast(self.mats, C.POINTER(Material))
        self.desc = d


def make_params(p: dict) -> Params:
    """writeParams argument (main.js:392-402) as the ABI struct."""
    q = Params()
    q.dt = float(p["dt"])
    for k in range(3):
        q.domain_min[k] = float(p["domainMin"][k])
        q.domain_max[k] = float(p["domainMax"][k])
        q.gravity[k] = float(p["gravity"][k])
        q.collider_pos[k] = float(p.get("colliderPos", [0, 0, 0])[k])
        q.collider_vel[k] = float(p.get("colliderVel", [0, 0, 0])[k])
    q.collider_r = float(p.get("colliderR", 0.0))
    q.collider_active = 1 if p.get("colliderActive") else 0
    q.xsph_c = float(p.get("xsphC", 0.01))
    q.omega = float(p.get("omega", 0.5))
    q.contact_omega = float(p.get("contactOmega", 0.4))
    q.pbf_eps = float(p.get("pbfEps", 100.0))
    q.s_corr_k = float(p.get("sCorrK", 1e-4))
    q.time = float(p.get("time", 0.0))
    kd = p.get("kDamp")
    q.k_damp = 0.4 if kd is None else float(kd)  # sim.js:184
    pi = p.get("pbfIterations")
    q.pbf_iterations = -1 if pi is None else int(pi)
    return q


def params_for(scene: dict, **over) -> dict:
    """The frame loop's writeParams argument for a scene (main.js:392-402)."""
    p = dict(dt=frame_dt(scene), domainMin=scene["domainMin"], domainMax=scene["domainMax"],
             gravity=scene["gravity"], colliderPos=[0.0, 0.0, 0.0], colliderR=0.0, colliderVel=[0.0, 0.0, 0.0],
             colliderActive=False, xsphC=scene.get("xsphC", 0.01), omega=scene.get("omega", 0.5),
             contactOmega=scene.get("contactOmega", 0.4), pbfEps=scene.get("pbfEps", 100.0),
             sCorrK=scene.get("sCorrK", 1e-4), time=0.0, kDamp=scene.get("kDamp", 0.4),
             pbfIterations=scene.get("pbfIterations"))
    p.update(over)
    return p


def pack_uniforms(scene: dict, params: dict | None = None):
    """Host-only packing of the Params and Material uniform words."""
    a = _SceneArgs(scene)
    pw = np.zeros(_abi.PARAMS_WORDS, np.uint32)
    mw = np.zeros(_abi.MAX_MATERIALS * _abi.MATERIAL_WORDS, np.uint32)
    q = make_params(params) if params is not None else None
    check(lib().xpbi_pack_uniforms(C.byref(a.desc), None if q is None else C.byref(q), _uptr(pw), _uptr(mw)))
    return pw, mw


class Simulation:
    """One handle over one scene, or over a batch of independent scenes.

    ``Simulation(scene)`` mirrors ``new Simulation(device, scene)``;
    ``Simulation([scene, ...])`` builds a batched handle.
    """

    def __init__(self, scene):
        self._h = C.c_void_p()
        scenes = scene if isinstance(scene, (list, tuple)) else [scene]
        self.scenes = list(scenes)
        args = [_SceneArgs(s) for s in scenes]
        if len(args) == 1:
            check(lib().xpbi_create(C.byref(args[0].desc), C.byref(self._h)))
        else:
            descs = (SceneDesc * len(args))(*[a.desc for a in args])
            check(lib().xpbi_batch_create(descs, len(args), C.byref(self._h)))
        n, c, s = C.c_uint32(), C.c_uint32(), C.c_uint32()
        dims = (C.c_int32 * 3)()
        check(lib().xpbi_info(self._h, C.byref(n), C.byref(c), C.byref(s), dims))
        self.N, self.num_cells, self.n_scenes = n.value, c.value, s.value
        self.grid_dims = tuple(dims)
        self.scene_sizes = [len(a.pos) // 3 for a in args]

    # -- lifetime
    def close(self):
        if self._h:
            lib().xpbi_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- sim.js surface
    def write_materials(self, materials, scene: int = -1):
        arr = make_materials(materials)
        check(lib().xpbi_write_materials(self._h, scene, arr, len(materials)))

    def write_params(self, p: dict, scene: int = -1):
        q = make_params(p)
        check(lib().xpbi_write_params(self._h, scene, C.byref(q)))

    def set_schedule(self, scene: int, iterations: int, has_water: bool):
        check(lib().xpbi_set_schedule(self._h, scene, iterations, 1 if has_water else 0))

    def encode_substep(self, iterations: int, has_water: bool):
        check(lib().xpbi_encode_substep(self._h, iterations, 1 if has_water else 0))

    def step(self, substeps: int, iterations: int, has_water: bool):
        check(lib().xpbi_step(self._h, substeps, iterations, 1 if has_water else 0))

    def synchronize(self):
        check(lib().xpbi_synchronize(self._h))

    def set_stream(self, stream_handle: int | None):
        check(lib().xpbi_set_stream(self._h, C.c_void_p(stream_handle or 0)))

    def profile_substep(self, iterations: int, has_water: bool) -> str:
        cap = 4096
        ms = np.zeros(cap, np.float32)
        cnt = C.c_int32()
        buf = C.create_string_buffer(1 << 16)
        check(lib().xpbi_profile_substep(self._h, iterations, 1 if has_water else 0, _fptr(ms), cap,
                                         C.byref(cnt), buf, len(buf)))
        self.last_profile_ms = ms[: cnt.value].copy()
        return buf.value.decode()

    def launches_per_substep(self, iterations: int, has_water: bool) -> int:
        out = C.c_int32()
        check(lib().xpbi_launches_per_substep(self._h, iterations, 1 if has_water else 0, C.byref(out)))
        return out.value

    def test_wait_expiry(self, polls: int = 1000):
        """Enqueue the scan's bounded wait on a descriptor nothing publishes:
        the next synchronize() raises XpbiError (ERR_DEVICE) and the handle
        stays usable."""
        check(lib().xpbi_test_wait_expiry(self._h, polls))

    # -- readback (main.js:291-312) and state access
    def read_pos(self, scene: int = 0, out=None):
        n = self.scene_sizes[scene]
        a = out if out is not None else np.empty((n, 4), np.float32)
        check(lib().xpbi_read_positions(self._h, scene, _fptr(a)))
        return a

    def read_pos_async(self, scene: int, out):
        """Enqueue the read-back of the scene's positions into `out` (an
        (n, 4) float32 array, ideally in page-locked memory); the values are
        there once synchronize() returns. Keep `out` alive until then."""
        n = self.scene_sizes[scene]
        if out.shape != (n, 4) or out.dtype != np.float32 or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a C-contiguous (n, 4) float32 array")
        check(lib().xpbi_read_positions_async(self._h, scene, _fptr(out)))
        return out

    def read_vel(self, scene: int = 0, out=None):
        n = self.scene_sizes[scene]
        a = out if out is not None else np.empty((n, 4), np.float32)
        check(lib().xpbi_read_velocities(self._h, scene, _fptr(a)))
        return a

    def read_state(self, scene: int = 0) -> dict:
        n = self.scene_sizes[scene]
        _, mw = self.uniforms(scene)
        pw, _ = self.uniforms(scene)
        nc = int(pw[7])
        st = dict(pos=np.empty((n, 4), np.float32), vel=np.empty((n, 4), np.float32),
                  F=np.empty((n, 12), np.float32), L=np.empty((n, 12), np.float32),
                  aux=np.empty((n, 4), np.float32), sortedIdx=np.empty(n, np.uint32),
                  cellTab=np.empty(nc, np.uint32))
        check(lib().xpbi_read_state(self._h, scene, _fptr(st["pos"]), _fptr(st["vel"]), _fptr(st["F"]),
                                    _fptr(st["L"]), _fptr(st["aux"]), _uptr(st["sortedIdx"]),
                                    _uptr(st["cellTab"])))
        return st

    def write_state(self, scene: int = 0, pos=None, vel=None, F=None, aux=None):
        def f(a):
            return None if a is None else np.ascontiguousarray(a, np.float32)
        pos, vel, F, aux = f(pos), f(vel), f(F), f(aux)
        check(lib().xpbi_write_state(self._h, scene, _fptr(pos), _fptr(vel), _fptr(F), _fptr(aux)))

    def uniforms(self, scene: int = 0):
        pw = np.zeros(_abi.PARAMS_WORDS, np.uint32)
        mw = np.zeros(_abi.MAX_MATERIALS * _abi.MATERIAL_WORDS, np.uint32)
        check(lib().xpbi_read_uniforms(self._h, scene, _uptr(pw), _uptr(mw)))
        return pw, mw

    # -- solver modes and the warm-start network (not in the reference)
    PLAIN, NETWORK, PREVIOUS = 0, 1, 2

    def set_solver(self, mode: int = 0, rel_tol: float = 0.0, track_residual: bool = False,
                   log_features: bool = False, contact_rel_tol: float = -1.0):
        check(lib().xpbi_set_solver(self._h, mode, rel_tol, contact_rel_tol, 1 if track_residual else 0,
                                    1 if log_features else 0))

    def set_network(self, params):
        p = np.ascontiguousarray(params, np.float32)
        check(lib().xpbi_set_network(self._h, _fptr(p), len(p)))

    def read_residuals(self, scene: int = 0):
        """(norms, iterations run): norms[0] = |C(v_pred)|, norms[1+k] =
        |r_k| (NaN after an early stop), norms[-1] = residual of the final
        state (with track_residual). The length is the scene's iteration
        count (or an early-stopped solve's cap) + 2."""
        out = np.full(256, -1.0)
        used = C.c_int32()
        check(lib().xpbi_read_residuals(self._h, scene, out.ctypes.data_as(C.POINTER(C.c_double)), 256,
                                        C.byref(used)))
        return _written(out), used.value

    SOLVEA_VARIANTS, SOLVEB_VARIANTS = 6, 5

    def autotune(self, iterations: int = -1, has_water: bool = True, repeats: int = 5) -> dict:
        """Time every solveA / solveB variant on this handle's data and keep
        the fastest (xpbi_autotune); returns the choice and the timings."""
        chosen = (C.c_int32 * 2)()
        ms = np.zeros(self.SOLVEA_VARIANTS + self.SOLVEB_VARIANTS, np.float32)
        check(lib().xpbi_autotune(self._h, iterations, 1 if has_water else 0, repeats, chosen, _fptr(ms), len(ms)))
        return {"solveA": int(chosen[0]), "solveB": int(chosen[1]),
                "solveA_ms": ms[:self.SOLVEA_VARIANTS].tolist(), "solveB_ms": ms[self.SOLVEA_VARIANTS:].tolist()}

    def set_variants(self, solve_a: int = -1, solve_b: int = -1):
        check(lib().xpbi_set_variants(self._h, solve_a, solve_b))

    def set_lanes(self, lanes: int = 0):
        """Lanes per particle in solveA / solveB (0: four for small handles)."""
        check(lib().xpbi_set_lanes(self._h, lanes))

    def read_contact_residuals(self, scene: int = 0):
        """Contact residual norms in the slots of read_residuals."""
        out = np.full(256, -1.0)
        check(lib().xpbi_read_contact_residuals(self._h, scene, out.ctypes.data_as(C.POINTER(C.c_double)), 256))
        return _written(out)

    def read_fallback(self, scene: int = 0) -> bool:
        """Whether the last substep re-solved the scene plainly (its
        early-stopped solve missed the tolerances within its cap)."""
        r = C.c_int32()
        check(lib().xpbi_read_fallback(self._h, scene, C.byref(r)))
        return bool(r.value)

    def set_max_iterations(self, max_iterations: int):
        """Iteration cap of an early-stopped solve (0: the scene's count)."""
        check(lib().xpbi_set_max_iterations(self._h, int(max_iterations)))

    def read_training(self, scene: int = 0):
        n = self.scene_sizes[scene]
        f = np.empty((n, 16), np.float32)
        t = np.empty(n, np.float32)
        a = np.zeros(1, np.float32)
        check(lib().xpbi_read_training(self._h, scene, _fptr(f), _fptr(t), _fptr(a)))
        return f, t, float(a[0])

    def set_active_set(self, share: float):
        """Work skipping in an early-stopped solve (0 turns it off); see
        xpbi_set_active_set."""
        check(lib().xpbi_set_active_set(self._h, float(share)))

    def read_active_counts(self, cap: int = 129):
        """(solveA re-evaluations, solveB updates) per iteration of the last
        substep, summed over scenes (iterations 0 and 1 visit everything: 0)."""
        a = np.zeros(cap, np.uint32)
        b = np.zeros(cap, np.uint32)
        check(lib().xpbi_read_active_counts(self._h, _uptr(a), _uptr(b), cap))
        return a, b

    def read_particle_residuals(self, scene: int = 0):
        """(r2, c2, r0sq) per particle of the last substep (cell order):
        squared constraint residual and contact correction of the last
        recording pass, squared constraint residual at lambda = 0."""
        n = self.scene_sizes[scene]
        r2, c2, r0 = (np.empty(n, np.float32) for _ in range(3))
        check(lib().xpbi_read_particle_residuals(self._h, scene, _fptr(r2), _fptr(c2), _fptr(r0)))
        return r2, c2, r0

    def device_ptrs(self):
        p, v, m = C.c_void_p(), C.c_void_p(), C.c_void_p()
        check(lib().xpbi_device_ptrs(self._h, C.byref(p), C.byref(v), C.byref(m)))
        return p.value, v.value, m.value
