"""ctypes declarations of the C ABI in include/sfgpu.h.

Loading fails loudly: there is no CPU fallback behind these entry points.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsfgpu.so")

SF_OK = 0
SF_NOT_CONVERGED = 1
SF_BAD_ARG = 2
SF_CUDA_ERROR = 3
SF_NO_DEVICE = 4
SF_OUT_OF_MEMORY = 5
SF_STALLED_FALLBACK = 6
SF_NOT_READY = 7
SF_TOO_LARGE = 8
SF_NOALLOC_MAX_BLOCKS = 8192

SF_PREC_FP64 = 0
SF_PREC_MIXED = 1
SF_PREC_LEARNED = 2

EXPORTED = [
    "sf_create", "sf_destroy", "sf_status_string", "sf_last_error", "sf_abi_version", "sf_default_opts",
    "sf_device_bytes", "sf_pressure_project", "sf_pressure_project_dev", "sf_pressure_reproject",
    "sf_pressure_reproject_dev", "sf_magnetic_solve", "sf_magnetic_solve_dev", "sf_magnetic_reset",
    "sf_collider_upload", "sf_levelset_upload", "sf_applied_field_prefetch", "sf_selftest_bounded_wait",
    "sf_collider_box_fractions", "sf_collider_face_fractions",
    "sf_unet_create", "sf_unet_destroy", "sf_unet_num_params", "sf_unet_set_params", "sf_unet_get_params",
    "sf_unet_forward_dev", "sf_unet_backward_dev", "sf_unet_train_step_dev", "sf_set_network",
    "sf_system_features_dev", "sf_unet_set_mode", "sf_unet_tc_launches", "sf_magnetic_residual_noalloc",
    "sf_system_operator",
    "sf_extrapolate_velocity", "sf_extrapolate_velocity_dev", "sf_collider_enforce", "sf_collider_enforce_dev",
    "sf_collider_face_normals", "sf_magnetic_vertex_pressures", "sf_magnetic_vertex_pressures_dev",
    "sf_pressure_jump", "sf_pressure_jump_dev", "sf_advect_levelset", "sf_advect_levelset_dev",
    "sf_advect_velocity", "sf_advect_velocity_dev", "sf_reinitialize", "sf_reinitialize_dev",
]


class sf_grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("h", C.c_double), ("origin", C.c_double * 3)]


class sf_solve_opts(C.Structure):
    _fields_ = [("precision", C.c_int), ("tol", C.c_double), ("max_iters", C.c_int), ("pre_smooth", C.c_int),
                ("post_smooth", C.c_int), ("coarse_sweeps", C.c_int), ("max_levels", C.c_int),
                ("coarse_dim", C.c_int), ("warm_start", C.c_int), ("use_graph", C.c_int),
                ("check_every", C.c_int), ("report_ref_residual", C.c_int), ("inner_tol", C.c_double),
                ("profile", C.c_int), ("smoother", C.c_int), ("coarse_pre", C.c_int), ("coarse_post", C.c_int),
                ("coarse_tail", C.c_int), ("full_sweeps", C.c_int), ("reserved", C.c_int * 2)]


class sf_solve_stats(C.Structure):
    _fields_ = [("iters", C.c_int), ("outer_iters", C.c_int), ("levels", C.c_int), ("converged", C.c_int),
                ("unknowns", C.c_longlong), ("rel_residual", C.c_double), ("rel_residual_ref", C.c_double),
                ("ms_build", C.c_double), ("ms_solve", C.c_double), ("ms_post", C.c_double),
                ("ms_total", C.c_double), ("h2d_bytes", C.c_longlong), ("d2h_bytes", C.c_longlong),
                ("status_detail", C.c_int), ("smooth_launches", C.c_int), ("smooth_ms", C.c_double),
                ("kernel_launches", C.c_longlong), ("smooth_bytes", C.c_double),
                ("guess_rel_residual", C.c_double), ("guess_energy_ratio", C.c_double),
                ("learned_steps", C.c_int), ("reserved_stats", C.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if not f.startswith("reserved")}


_P3 = C.c_void_p * 3
_lib = None


def load(path: str | None = None):
    """Load libsfgpu.so (built by build.py).  Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(f"libsfgpu.so not found at {path}: run __graft_entry__.build() (nvcc, sm_103a)")
    L = C.CDLL(path)
    V = C.c_void_p
    G = C.POINTER(sf_grid)
    O = C.POINTER(sf_solve_opts)
    S = C.POINTER(sf_solve_stats)
    L.sf_abi_version.argtypes = []
    L.sf_create.argtypes = [C.c_int, V, C.POINTER(V)]
    L.sf_create.restype = C.c_int
    L.sf_destroy.argtypes = [V]
    L.sf_destroy.restype = None
    L.sf_status_string.argtypes = [C.c_int]
    L.sf_status_string.restype = C.c_char_p
    L.sf_last_error.argtypes = [V]
    L.sf_last_error.restype = C.c_char_p
    L.sf_abi_version.restype = C.c_int
    L.sf_default_opts.argtypes = [O, C.c_int]
    L.sf_default_opts.restype = None
    L.sf_device_bytes.argtypes = [V]
    L.sf_device_bytes.restype = C.c_longlong
    for name in ("sf_pressure_project", "sf_pressure_project_dev", "sf_pressure_reproject",
                 "sf_pressure_reproject_dev"):
        f = getattr(L, name)
        f.argtypes = [V, G, _P3, V, V, V, V, C.c_double, V, O, S]
        f.restype = C.c_int
    for name in ("sf_magnetic_solve", "sf_magnetic_solve_dev"):
        f = getattr(L, name)
        f.argtypes = [V, G, V, C.c_double, C.c_double, V, V, V, O, S]  # hext: p3_ref (nullable)
        f.restype = C.c_int
    L.sf_magnetic_reset.argtypes = [V]
    L.sf_magnetic_reset.restype = C.c_int
    L.sf_collider_upload.argtypes = [V, G, _P3, V]
    L.sf_collider_upload.restype = C.c_int
    L.sf_levelset_upload.argtypes = [V, G, V]
    L.sf_levelset_upload.restype = C.c_int
    L.sf_applied_field_prefetch.argtypes = [V, G, _P3]
    L.sf_applied_field_prefetch.restype = C.c_int
    L.sf_selftest_bounded_wait.argtypes = [V, C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    L.sf_selftest_bounded_wait.restype = C.c_int
    for name in ("sf_extrapolate_velocity", "sf_extrapolate_velocity_dev"):
        f = getattr(L, name)
        f.argtypes = [V, G, _P3, V, _P3, C.c_double, C.c_int]
        f.restype = C.c_int
    for name in ("sf_collider_enforce", "sf_collider_enforce_dev"):
        f = getattr(L, name)
        f.argtypes = [V, G, _P3, _P3, _P3, V]
        f.restype = C.c_int
    for name in ("sf_magnetic_vertex_pressures", "sf_magnetic_vertex_pressures_dev"):
        f = getattr(L, name)
        f.argtypes = [V, G, C.c_double, _P3, V, V, C.c_longlong, V]
        f.restype = C.c_int
    for name in ("sf_pressure_jump", "sf_pressure_jump_dev"):
        f = getattr(L, name)
        f.argtypes = [V, G, _P3, V, V, C.c_longlong, C.c_double, C.c_double, C.c_double, _P3]
        f.restype = C.c_int
    for name in ("sf_advect_levelset", "sf_advect_levelset_dev"):
        f = getattr(L, name)
        f.argtypes = [V, G, V, _P3, C.c_double]
        f.restype = C.c_int
    for name in ("sf_advect_velocity", "sf_advect_velocity_dev"):
        f = getattr(L, name)
        f.argtypes = [V, G, _P3, C.c_double]
        f.restype = C.c_int
    for name in ("sf_reinitialize", "sf_reinitialize_dev"):
        f = getattr(L, name)
        f.argtypes = [V, G, V, C.c_int]
        f.restype = C.c_int
    L.sf_collider_face_normals.argtypes = [G, V, _P3]
    L.sf_collider_face_normals.restype = C.c_int
    L.sf_magnetic_residual_noalloc.argtypes = [V, G, V, C.c_double, C.c_double, _P3, V, V]
    L.sf_magnetic_residual_noalloc.restype = C.c_int
    L.sf_collider_box_fractions.argtypes = [G, C.c_int, _P3, V]
    L.sf_collider_box_fractions.restype = C.c_int
    L.sf_collider_face_fractions.argtypes = [G, V, _P3]
    L.sf_collider_face_fractions.restype = C.c_int
    L.sf_unet_create.argtypes = [V, C.POINTER(V)]
    L.sf_unet_create.restype = C.c_int
    L.sf_unet_destroy.argtypes = [V]
    L.sf_unet_destroy.restype = None
    L.sf_unet_num_params.argtypes = [V]
    L.sf_unet_num_params.restype = C.c_longlong
    L.sf_unet_set_params.argtypes = [V, V, C.c_longlong]
    L.sf_unet_set_params.restype = C.c_int
    L.sf_unet_get_params.argtypes = [V, V, C.c_longlong]
    L.sf_unet_get_params.restype = C.c_int
    L.sf_unet_forward_dev.argtypes = [V, G, V, V]
    L.sf_unet_forward_dev.restype = C.c_int
    L.sf_unet_backward_dev.argtypes = [V, G, V, V, V]
    L.sf_unet_backward_dev.restype = C.c_int
    L.sf_unet_train_step_dev.argtypes = [V, G, V, V, C.c_float, C.POINTER(C.c_double)]
    L.sf_unet_train_step_dev.restype = C.c_int
    L.sf_unet_set_mode.argtypes = [V, C.c_int]
    L.sf_unet_set_mode.restype = C.c_int
    L.sf_unet_tc_launches.argtypes = [V]
    L.sf_unet_tc_launches.restype = C.c_longlong
    L.sf_set_network.argtypes = [V, V]
    L.sf_set_network.restype = C.c_int
    L.sf_system_features_dev.argtypes = [V, C.c_int, V, V]
    L.sf_system_features_dev.restype = C.c_int
    L.sf_system_operator.argtypes = [V, C.c_int, V, V, V]
    L.sf_system_operator.restype = C.c_int
    _lib = L
    return L


def p3(ptrs):
    """Array of three pointers (or NULL when ptrs is None)."""
    if ptrs is None:
        return None
    return _P3(*[C.c_void_p(int(p)) for p in ptrs])


def p3_ref(ptrs):
    """Pointer to an array of three pointers for nullable `const double *const x[3]` arguments."""
    if ptrs is None:
        return None
    arr = p3(ptrs)
    return C.cast(C.pointer(arr), C.c_void_p), arr
