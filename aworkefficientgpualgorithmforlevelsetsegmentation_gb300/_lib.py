"""ctypes binding of liblss.so (include/lss.h).

The library is built in-tree by build.py; loading fails loudly when it is
missing (there is no CPU fallback anywhere in the product).
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_lib: C.CDLL | None = None
_phantom: C.CDLL | None = None


class lss_config(C.Structure):
    _fields_ = [("mode", C.c_int32), ("device", C.c_int32), ("brick_x", C.c_int32),
                ("brick_y", C.c_int32), ("brick_z", C.c_int32), ("threads_per_brick", C.c_int32),
                ("ref_quirk_i3", C.c_int32), ("use_graph", C.c_int32),
                ("hbm_budget_bytes", C.c_uint64), ("brick_workers", C.c_int32), ("pad_", C.c_int32)]


class lss_params(C.Structure):
    _fields_ = [("target", C.c_float), ("window", C.c_float), ("curvature", C.c_float),
                ("time_step", C.c_float), ("phi_min", C.c_float), ("phi_max", C.c_float),
                ("temporal_threshold", C.c_float), ("spatial_threshold", C.c_float),
                ("convergence_threshold", C.c_float), ("neighbourhood", C.c_int32),
                ("alpha_role", C.c_int32), ("data_term", C.c_int32)]


class lss_conv(C.Structure):
    _fields_ = [("rel_threshold", C.c_double), ("patience", C.c_int32),
                ("max_iterations", C.c_int32), ("abs_threshold", C.c_uint64)]


class lss_stats(C.Structure):
    _fields_ = [("iterations", C.c_uint64), ("active_count", C.c_uint64),
                ("initial_active_count", C.c_uint64), ("voxel_updates", C.c_uint64),
                ("brick_updates", C.c_uint64), ("device_bytes", C.c_uint64),
                ("last_step_ms", C.c_double), ("padded_x", C.c_uint32), ("padded_y", C.c_uint32),
                ("padded_z", C.c_uint32), ("brick_x", C.c_uint32), ("brick_y", C.c_uint32),
                ("brick_z", C.c_uint32), ("threads_per_brick", C.c_uint32), ("mode", C.c_int32),
                ("error_flags", C.c_int32), ("update_ms", C.c_double), ("barrier_ms", C.c_double),
                ("kernel_launches", C.c_uint64), ("grid_blocks", C.c_uint32),
                ("block_threads", C.c_uint32)]


class lss_grads(C.Structure):
    _fields_ = [("loss", C.c_double), ("d_target", C.c_double), ("d_window", C.c_double),
                ("d_curvature", C.c_double), ("active_voxel_iterations", C.c_uint64)]


P = C.c_void_p
u32, i32, u64, f32 = C.c_uint32, C.c_int32, C.c_uint64, C.c_float

# name: (restype, argtypes) of every entry point declared in include/lss.h and
# include/lss_phantom.h.
SIGNATURES = {
    "lss_version": (C.c_char_p, []),
    "lss_config_default": (i32, [C.POINTER(lss_config)]),
    "lss_params_default": (i32, [i32, C.POINTER(lss_params)]),
    "lss_create": (i32, [C.POINTER(P), C.POINTER(lss_config)]),
    "lss_destroy": (i32, [P]),
    "lss_last_error_string": (C.c_char_p, [P]),
    "lss_set_stream": (i32, [P, P]),
    "lss_load_volume": (i32, [P, P, i32, i32, i32, i32, f32]),
    "lss_load_volume_raw": (i32, [P, C.c_char_p, i32, i32, i32, i32, f32]),
    "lss_unload_volume": (i32, [P]),
    "lss_set_params": (i32, [P, C.POINTER(lss_params)]),
    "lss_get_params": (i32, [P, C.POINTER(lss_params)]),
    "lss_initialize_seed": (i32, [P, f32, f32, f32, f32]),
    "lss_set_seed_spheres": (i32, [P, P, i32]),
    "lss_set_phi": (i32, [P, P]),
    "lss_step": (i32, [P, i32, C.POINTER(i32)]),
    "lss_step_dense": (i32, [P, i32, C.POINTER(C.c_double)]),
    "lss_step_until_converged": (i32, [P, C.POINTER(lss_conv), C.POINTER(i32)]),
    "lss_is_finished": (i32, [P, C.POINTER(i32)]),
    "lss_active_count": (i32, [P, C.POINTER(u64)]),
    "lss_read_active": (i32, [P, P, u64, C.POINTER(u64)]),
    "lss_read_active_packed": (i32, [P, P, u64, C.POINTER(u64)]),
    "lss_read_phi": (i32, [P, P]),
    "lss_read_mask": (i32, [P, P]),
    "lss_save_mask_raw": (i32, [P, C.c_char_p]),
    "lss_read_export": (i32, [P, P]),
    "lss_read_active_volume": (i32, [P, P]),
    "lss_freeze_current": (i32, [P]),
    "lss_clear_current": (i32, [P]),
    "lss_clear_all": (i32, [P]),
    "lss_estimate_params": (i32, [P, C.POINTER(f32), C.POINTER(f32)]),
    "lss_get_stats": (i32, [P, C.POINTER(lss_stats)]),
    "lss_batch_create": (i32, [C.POINTER(P), C.POINTER(lss_config)]),
    "lss_batch_destroy": (i32, [P]),
    "lss_batch_add_volume": (i32, [P, P, i32, i32, i32, C.POINTER(lss_params), P, i32,
                                   C.POINTER(i32)]),
    "lss_batch_run": (i32, [P, C.POINTER(lss_conv), C.POINTER(i32)]),
    "lss_batch_read_phi": (i32, [P, i32, P]),
    "lss_batch_read_mask": (i32, [P, i32, P]),
    "lss_batch_get_stats": (i32, [P, i32, C.POINTER(lss_stats)]),
    "lss_batch_last_error_string": (C.c_char_p, [P]),
    "lss_adjoint_run": (i32, [P, i32, i32, P, f32, P, P, C.POINTER(lss_grads)]),
    "lss_compact_u32": (i32, [P, P, P, u64, P, P]),
    "lss_compact_u32_noalloc": (i32, [P, P, P, u64, P, P]),
    "lss_phantom_ellipsoid": (i32, [i32, i32, i32, P, P, f32, f32, f32, u64, P]),
    "lss_phantom_shells": (i32, [i32, i32, i32, i32, P, P, f32, f32, i32, u64, f32, f32, u64, P]),
    "lss_phantom_sdf_spheres": (i32, [i32, i32, i32, P, i32, f32, f32, P]),
    "lss_phantom_uniform": (C.c_double, [u64, u64]),
}

STATUS = {0: "LSS_OK", 1: "LSS_ERR_INVALID_ARGUMENT", 2: "LSS_ERR_STATE",
          3: "LSS_ERR_OUT_OF_MEMORY", 4: "LSS_ERR_CUDA", 5: "LSS_ERR_TIMEOUT",
          6: "LSS_ERR_UNSUPPORTED", 7: "LSS_ERR_NO_DEVICE", 8: "LSS_ERR_INJECTED",
          9: "LSS_ERR_CAPACITY"}


class LssError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Loads liblss.so (building it first if it is absent and nvcc exists)."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"{path} is missing: run the package build first")
            _build.build()
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


PHANTOM_FUNCTIONS = ("lss_phantom_ellipsoid", "lss_phantom_shells", "lss_phantom_sdf_spheres",
                     "lss_phantom_uniform")


def load_phantom(build_if_missing: bool = True) -> C.CDLL:
    """Loads libphantom.so, the host-only build of the include/lss_phantom.h
    generators (building it first if it is absent)."""
    global _phantom
    if _phantom is None:
        path = _build.PHANTOM_LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"{path} is missing: run the package build first")
            _build.build_phantom()
        L = C.CDLL(path)
        for name in PHANTOM_FUNCTIONS:
            res, args = SIGNATURES[name]
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _phantom = L
    return _phantom
