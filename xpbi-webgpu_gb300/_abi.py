"""ctypes binding of libxpbi (include/xpbi.h).

The library is the only compute path: if ``libxpbi.so`` is missing the
import of the package still works (host-only helpers), but every call that
needs it raises ``XpbiError`` instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# XPBI_LIB selects another build of the same library (a tuning variant)
LIB_PATH = os.environ.get("XPBI_LIB") or os.path.join(HERE, "libxpbi.so")

PARAMS_WORDS = 64
MATERIAL_WORDS = 16
MAX_MATERIALS = 8

OK, ERR_INVALID, ERR_CUDA, ERR_OOM, ERR_DEVICE = 0, 1, 2, 3, 4
ELASTIC, DP, NACC, VM, HB, SNOW, WATER = range(7)

# Every symbol include/xpbi.h declares (checked by the ABI tests).
EXPORTS = (
    "xpbi_last_error", "xpbi_pack_uniforms", "xpbi_create", "xpbi_batch_create", "xpbi_destroy",
    "xpbi_write_materials", "xpbi_write_params", "xpbi_set_schedule", "xpbi_encode_substep",
    "xpbi_step", "xpbi_synchronize", "xpbi_set_stream", "xpbi_read_positions",
    "xpbi_read_velocities", "xpbi_read_state", "xpbi_write_state", "xpbi_read_uniforms",
    "xpbi_info", "xpbi_profile_substep", "xpbi_device_ptrs", "xpbi_launches_per_substep",
    "xpbi_mlp_param_count", "xpbi_mlp_forward", "xpbi_mlp_grad", "xpbi_mlp_train",
    "xpbi_set_solver", "xpbi_set_network", "xpbi_read_residuals", "xpbi_read_training",
    "xpbi_sort_cells_noalloc", "xpbi_read_contact_residuals", "xpbi_autotune", "xpbi_set_variants",
    "xpbi_render", "xpbi_set_lanes", "xpbi_read_positions_async", "xpbi_test_wait_expiry",
    "xpbi_sort_cells_noalloc_status", "xpbi_test_noalloc_wait_expiry", "xpbi_read_particle_residuals",
    "xpbi_set_active_set", "xpbi_read_active_counts", "xpbi_set_max_iterations",
    "xpbi_read_fallback", "xpbi_sample_shapes", "xpbi_philox4x32_10",
)


class XpbiError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"xpbi error {code}: {msg}")
        self.code = code


class Material(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("E", C.c_double), ("nu", C.c_double), ("density", C.c_double),
                ("p0", C.c_double), ("p1", C.c_double), ("p2", C.c_double), ("p3", C.c_double),
                ("color", C.c_float * 3), ("bound_friction", C.c_double)]


class SceneDesc(C.Structure):
    _fields_ = [("n", C.c_uint32), ("positions", C.POINTER(C.c_float)), ("mat_ids", C.POINTER(C.c_uint32)),
                ("states", C.POINTER(C.c_float)), ("velocities", C.POINTER(C.c_float)),
                ("color_seeds", C.POINTER(C.c_float)), ("h", C.c_double),
                ("domain_min", C.c_double * 3), ("domain_max", C.c_double * 3),
                ("n_materials", C.c_uint32), ("materials", C.POINTER(Material))]


class Camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("target", C.c_float * 3), ("fov_y", C.c_float), ("near_z", C.c_float),
                ("far_z", C.c_float), ("light_dir", C.c_float * 3), ("particle_radius", C.c_float),
                ("draw_ground", C.c_int32), ("draw_box", C.c_int32)]


class Params(C.Structure):
    _fields_ = [("dt", C.c_float), ("domain_min", C.c_float * 3), ("domain_max", C.c_float * 3),
                ("gravity", C.c_float * 3), ("collider_pos", C.c_float * 3), ("collider_r", C.c_float),
                ("collider_vel", C.c_float * 3), ("collider_active", C.c_int32), ("xsph_c", C.c_float),
                ("omega", C.c_float), ("contact_omega", C.c_float), ("pbf_eps", C.c_float),
                ("s_corr_k", C.c_float), ("time", C.c_float), ("k_damp", C.c_float),
                ("pbf_iterations", C.c_int32)]


class Shape(C.Structure):
    _fields_ = [("kind", C.c_int32), ("lo", C.c_double * 3), ("hi", C.c_double * 3), ("centre", C.c_double * 3),
                ("radius", C.c_double), ("mat_id", C.c_uint32), ("state0", C.c_float), ("jitter", C.c_double)]


_lib = None

_P = C.c_void_p
_U32P = C.POINTER(C.c_uint32)
_F32P = C.POINTER(C.c_float)

_SIGS = {
    "xpbi_last_error": (C.c_char_p, []),
    "xpbi_pack_uniforms": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(Params), _U32P, _U32P]),
    "xpbi_create": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(_P)]),
    "xpbi_batch_create": (C.c_int, [C.POINTER(SceneDesc), C.c_uint32, C.POINTER(_P)]),
    "xpbi_destroy": (None, [_P]),
    "xpbi_write_materials": (C.c_int, [_P, C.c_int32, C.POINTER(Material), C.c_uint32]),
    "xpbi_write_params": (C.c_int, [_P, C.c_int32, C.POINTER(Params)]),
    "xpbi_set_schedule": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "xpbi_encode_substep": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "xpbi_step": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "xpbi_synchronize": (C.c_int, [_P]),
    "xpbi_set_stream": (C.c_int, [_P, _P]),
    "xpbi_read_positions": (C.c_int, [_P, C.c_uint32, _F32P]),
    "xpbi_read_velocities": (C.c_int, [_P, C.c_uint32, _F32P]),
    "xpbi_read_state": (C.c_int, [_P, C.c_uint32, _F32P, _F32P, _F32P, _F32P, _F32P, _U32P, _U32P]),
    "xpbi_write_state": (C.c_int, [_P, C.c_uint32, _F32P, _F32P, _F32P, _F32P]),
    "xpbi_read_uniforms": (C.c_int, [_P, C.c_uint32, _U32P, _U32P]),
    "xpbi_info": (C.c_int, [_P, _U32P, _U32P, _U32P, C.POINTER(C.c_int32)]),
    "xpbi_profile_substep": (C.c_int, [_P, C.c_int32, C.c_int32, _F32P, C.c_int32, C.POINTER(C.c_int32),
                                       C.c_char_p, C.c_size_t]),
    "xpbi_device_ptrs": (C.c_int, [_P, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P)]),
    "xpbi_launches_per_substep": (C.c_int, [_P, C.c_int32, C.c_int32, C.POINTER(C.c_int32)]),
    "xpbi_test_wait_expiry": (C.c_int, [_P, C.c_uint32]),
    "xpbi_mlp_param_count": (C.c_int, []),
    "xpbi_mlp_forward": (C.c_int, [_F32P, C.c_uint32, _F32P, _F32P]),
    "xpbi_mlp_grad": (C.c_int, [_F32P, _F32P, C.c_uint32, _F32P, _F32P, _F32P]),
    "xpbi_mlp_train": (C.c_int, [_F32P, _F32P, C.c_uint32, _F32P, C.c_int32, C.c_uint32, C.c_float, _F32P]),
    "xpbi_set_solver": (C.c_int, [_P, C.c_int32, C.c_float, C.c_float, C.c_int32, C.c_int32]),
    "xpbi_set_network": (C.c_int, [_P, _F32P, C.c_uint32]),
    "xpbi_read_residuals": (C.c_int, [_P, C.c_uint32, C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_int32)]),
    "xpbi_read_training": (C.c_int, [_P, C.c_uint32, _F32P, _F32P, _F32P]),
    "xpbi_read_particle_residuals": (C.c_int, [_P, C.c_uint32, _F32P, _F32P, _F32P]),
    "xpbi_set_active_set": (C.c_int, [_P, C.c_float]),
    "xpbi_set_max_iterations": (C.c_int, [_P, C.c_int32]),
    "xpbi_read_fallback": (C.c_int, [_P, C.c_uint32, C.POINTER(C.c_int32)]),
    "xpbi_sample_shapes": (C.c_int, [C.POINTER(Shape), C.c_uint32, C.c_double, C.c_uint64, C.c_uint32, _F32P,
                                     _U32P, _F32P, _U32P]),
    "xpbi_philox4x32_10": (C.c_int, [_U32P, _U32P, _U32P]),
    "xpbi_read_active_counts": (C.c_int, [_P, _U32P, _U32P, C.c_int32]),
    "xpbi_read_contact_residuals": (C.c_int, [_P, C.c_uint32, C.POINTER(C.c_double), C.c_int32]),
    "xpbi_autotune": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int32), _F32P, C.c_int32]),
    "xpbi_set_variants": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "xpbi_set_lanes": (C.c_int, [_P, C.c_int32]),
    "xpbi_read_positions_async": (C.c_int, [_P, C.c_uint32, _F32P]),
    "xpbi_render": (C.c_int, [_P, C.c_uint32, C.POINTER(Camera), C.c_uint32, C.c_uint32, C.POINTER(C.c_uint8),
                              C.POINTER(_P)]),
    "xpbi_sort_cells_noalloc": (C.c_int, [_P, C.c_uint32, _F32P, C.c_float, C.POINTER(C.c_int32), _P, _P, _P]),
    "xpbi_sort_cells_noalloc_status": (C.c_int, [_P]),
    "xpbi_test_noalloc_wait_expiry": (C.c_int, [C.c_uint32, _P]),
}


def lib():
    """Load libxpbi.so (built in-tree); raise if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise XpbiError(ERR_CUDA, f"libxpbi.so not built at {LIB_PATH}; run the package build first")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != OK:
        raise XpbiError(rc, lib().xpbi_last_error().decode(errors="replace"))
