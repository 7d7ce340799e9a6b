"""ctypes binding of libplgpu.so (the C ABI of include/plgpu.h).

Loading fails loudly when the library is missing: there is no CPU fallback
for the physics step.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import _build

PLG_OK = 0
PLG_E_INVALID_ARG = 1
PLG_E_UNSUPPORTED = 2
PLG_E_STATE = 3
PLG_E_NO_MEMORY = 4
PLG_E_CUDA = 5
PLG_E_TIMEOUT = 6
PLG_E_STOPPED = 7
PLG_E_DEVICE = 8
PLG_E_CAPACITY = 9

PLG_ACCEL_PARTICLE_LIFE = 1
PLG_TILE_VARIANTS = 3
PLG_NOALLOC_MAX_PARTICLES = 1 << 18
PLG_NOALLOC_MAX_CELLS = 1 << 18

KERNELS = ["scan", "scatter", "gather", "force"]


class plg_settings(C.Structure):
    _fields_ = [
        ("rmax", C.c_double),
        ("friction", C.c_double),
        ("force", C.c_double),
        ("dt", C.c_double),
        ("beta", C.c_double),
        ("wrap", C.c_int32),
        ("accel_kind", C.c_int32),
    ]


class plg_world_desc(C.Structure):
    _fields_ = [
        ("settings", plg_settings),
        ("ntypes", C.c_int32),
        ("matrix", C.POINTER(C.c_double)),
        ("n", C.c_int64),
        ("pos", C.POINTER(C.c_double)),
        ("vel", C.POINTER(C.c_double)),
        ("type", C.POINTER(C.c_int32)),
    ]


class plg_cursor(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double), ("size", C.c_double),
                ("shape", C.c_int32), ("reserved", C.c_int32)]


POSITION_SETTERS = ["uniform", "centered", "uniform circle", "centered circle", "ring", "rainbow ring",
                    "color battle", "color wheel", "line", "spiral", "rainbow spiral"]
TYPE_SETTERS = ["random", "randomize 10%", "slices", "onion", "rotate", "flip", "more of first", "kill still"]
MATRIX_GENERATORS = ["random", "symmetry", "chains", "chains 2", "chains 3", "snakes", "zero"]

PLG_CURSOR_CIRCLE = 0
PLG_CURSOR_SQUARE = 1
PLG_CURSOR_INFINITY = 2


class plg_render_params(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("cam_x", C.c_double), ("cam_y", C.c_double),
                ("cam_w", C.c_double), ("cam_h", C.c_double), ("top_left_x", C.c_double), ("top_left_y", C.c_double),
                ("size", C.c_double), ("wrap", C.c_int32), ("reserved", C.c_int32)]


class plg_server_config(C.Structure):
    _fields_ = [
        ("memory_budget_bytes", C.c_int64),
        ("particle_capacity", C.c_int64 * 2),
        ("cell_capacity", C.c_int64 * 2),
        ("max_worlds_per_batch", C.c_int32),
        ("max_chunk_steps", C.c_int32),
        ("tile_variant", C.c_int32),
        ("autotune_interval_ms", C.c_int32),
    ]


class plg_server_stats_t(C.Structure):
    _fields_ = [
        ("submitted", C.c_int64),
        ("completed", C.c_int64),
        ("queued", C.c_int64),
        ("running", C.c_int64),
        ("resident_bytes", C.c_int64),
        ("peak_resident_bytes", C.c_int64),
        ("particle_steps", C.c_double),
        ("busy_s", C.c_double),
        ("wall_s", C.c_double),
        ("latency_p50_ms", C.c_double),
        ("latency_p99_ms", C.c_double),
        ("latency_mean_ms", C.c_double),
        ("busy_dim_s", C.c_double * 2),
        ("compactions", C.c_int64),
        ("autotunes", C.c_int64),
    ]


class plg_world_gen(C.Structure):
    _fields_ = [("world", plg_world_desc), ("position_setter", C.c_int32), ("type_setter", C.c_int32),
                ("seed", C.c_uint64)]


PLG_REQ_QUEUED = 0
PLG_REQ_RUNNING = 1
PLG_REQ_DONE = 2


class PlgError(RuntimeError):
    """A plg_* call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


_P = C.c_void_p
_I32P = C.POINTER(C.c_int32)
_I64P = C.POINTER(C.c_int64)
_DP = C.POINTER(C.c_double)
_FP = C.POINTER(C.c_float)
_U64P = C.POINTER(C.c_uint64)

# name -> (restype, argtypes)
SIGNATURES = {
    "plg_version": (C.c_char_p, []),
    "plg_status_string": (C.c_char_p, [C.c_int]),
    "plg_validate_settings": (C.c_int, [C.c_int, C.POINTER(plg_settings)]),
    "plg_cell_bounds": (C.c_int, [C.c_double, _I32P, _FP, C.c_int64]),
    "plg_create": (C.c_int, [C.c_int, C.c_int64, C.POINTER(_P)]),
    "plg_destroy": (C.c_int, [_P]),
    "plg_set_settings": (C.c_int, [_P, C.POINTER(plg_settings)]),
    "plg_get_settings": (C.c_int, [_P, C.POINTER(plg_settings)]),
    "plg_set_matrix": (C.c_int, [_P, C.c_int32, _DP]),
    "plg_upload": (C.c_int, [_P, C.c_int64, _DP, _DP, _I32P]),
    "plg_step": (C.c_int, [_P, C.c_int32]),
    "plg_step_async": (C.c_int, [_P, C.c_int32]),
    "plg_sync": (C.c_int, [_P, C.c_double]),
    "plg_download": (C.c_int, [_P, _DP, _DP, _I32P, _I32P]),
    "plg_step_download": (C.c_int, [_P, C.c_int32, _DP, _DP, _I32P, _I32P]),
    "plg_step_download_fuses": (C.c_int, [_P, _DP, _DP, _I32P, _I32P, C.POINTER(C.c_int32)]),
    "plg_set_tile": (C.c_int, [_P, C.c_int32]),
    "plg_get_tile": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "plg_autotune": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_int32), _DP]),
    "plg_test_scan_wait": (C.c_int, [C.POINTER(C.c_uint32), _DP]),
    "plg_particle_count": (C.c_int, [_P, _I64P]),
    "plg_request_stop": (C.c_int, [_P]),
    "plg_last_error": (C.c_char_p, [_P]),
    "plg_get_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "plg_set_use_graph": (C.c_int, [_P, C.c_int32]),
    "plg_profile_enable": (C.c_int, [_P, C.c_int32]),
    "plg_profile_read": (C.c_int, [_P, C.c_int32, _DP, _I64P]),
    "plg_kernel_name": (C.c_char_p, [C.c_int32]),
    "plg_debug_step": (C.c_int, [_P, _I32P, _I32P, _U64P, _U64P, _FP, _I64P]),
    "plg_probe_fp32_peak": (C.c_int, [_DP]),
    "plg_probe_sfu_peak": (C.c_int, [_DP]),
    "plg_step_stats": (C.c_int, [_P, _I64P]),
    "plg_sort_cells_noalloc": (C.c_int, [C.c_int32, C.c_double, C.c_int64, _P, _P, _P, _P, _P]),
    "plg_batch_create": (C.c_int, [C.c_int32, C.c_int64, C.c_int32, C.c_int64, C.POINTER(_P)]),
    "plg_batch_destroy": (C.c_int, [_P]),
    "plg_batch_update": (C.c_int, [_P, C.c_int32, _I32P, C.c_int32, C.POINTER(plg_world_desc), _I32P]),
    "plg_batch_step": (C.c_int, [_P, C.c_int32]),
    "plg_batch_step_async": (C.c_int, [_P, C.c_int32]),
    "plg_batch_sync": (C.c_int, [_P, C.c_double]),
    "plg_batch_download": (C.c_int, [_P, C.c_int32, _DP, _DP, _I32P, _I32P]),
    "plg_batch_world_info": (C.c_int, [_P, C.c_int32, _I64P, _I64P, _I64P]),
    "plg_batch_counts": (C.c_int, [_P, _I32P, _I64P, _I64P]),
    "plg_batch_set_use_graph": (C.c_int, [_P, C.c_int32]),
    "plg_batch_get_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "plg_batch_last_error": (C.c_char_p, [_P]),
    "plg_batch_step_stats": (C.c_int, [_P, _I64P]),
    "plg_batch_debug_step": (C.c_int, [_P, _I32P, _I32P, _U64P, _U64P, _FP, _I64P]),
    "plg_batch_set_tile": (C.c_int, [_P, C.c_int32]),
    "plg_batch_get_tile": (C.c_int, [_P, _I32P]),
    "plg_batch_autotune": (C.c_int, [_P, C.c_int32, _I32P, _DP]),
    "plg_batch_autotune_worlds": (C.c_int, [_P, C.c_int32, _I32P, _DP]),
    "plg_batch_set_world_tile": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "plg_batch_get_world_tile": (C.c_int, [_P, C.c_int32, _I32P]),
    "plg_batch_world_ids": (C.c_int, [_P, _I32P]),
    "plg_batch_set_steps": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "plg_batch_steps_left": (C.c_int, [_P, C.c_int32, _I32P]),
    "plg_cursor_count": (C.c_int, [_P, C.POINTER(plg_cursor), _I64P]),
    "plg_cursor_move": (C.c_int, [_P, C.POINTER(plg_cursor), C.c_double, C.c_double, C.c_double, _I64P]),
    "plg_cursor_delete": (C.c_int, [_P, C.POINTER(plg_cursor), _I64P]),
    "plg_append": (C.c_int, [_P, C.c_int64, _DP, _DP, _I32P]),
    "plg_permute": (C.c_int, [_P, C.c_int64, _I32P]),
    "plg_set_types": (C.c_int, [_P, _I32P]),
    "plg_generate": (C.c_int, [_P, C.c_int64, C.c_int32, C.c_int32, C.c_uint64]),
    "plg_apply_position_setter": (C.c_int, [_P, C.c_int32, C.c_uint64]),
    "plg_apply_type_setter": (C.c_int, [_P, C.c_int32, C.c_uint64]),
    "plg_generate_matrix": (C.c_int, [C.c_int32, C.c_int32, C.c_uint64, _DP]),
    "plg_render": (C.c_int, [_P, C.POINTER(plg_render_params), C.c_int32, _FP, C.POINTER(C.c_uint8)]),
    "plg_world_check": (C.c_int, [C.c_int32, C.POINTER(plg_world_desc)]),
    "plg_world_device_bytes": (C.c_int64, [C.c_int32, C.POINTER(plg_world_desc)]),
    "plg_server_create": (C.c_int, [C.POINTER(plg_server_config), C.POINTER(_P)]),
    "plg_server_submit": (C.c_int, [_P, C.c_int32, C.POINTER(plg_world_desc), C.c_int32, _I64P]),
    "plg_server_submit_generated": (C.c_int, [_P, C.c_int32, C.POINTER(plg_world_gen), C.c_int32, _I64P]),
    "plg_server_wait": (C.c_int, [_P, C.c_int64, C.c_double, _I32P]),
    "plg_server_wait_any": (C.c_int, [_P, C.c_double, _I64P]),
    "plg_server_result": (C.c_int, [_P, C.c_int64, _DP, _DP, _I32P, _I32P, _I64P, _DP]),
    "plg_server_stats": (C.c_int, [_P, C.POINTER(plg_server_stats_t)]),
    "plg_server_last_error": (C.c_char_p, [_P]),
    "plg_server_destroy": (C.c_int, [_P]),
}

_lib = None


def library_path() -> Path:
    return Path(os.environ.get("PLGPU_LIB", _build.LIB_PATH))


def load(build_if_missing: bool = True) -> C.CDLL:
    """Loads libplgpu.so (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: build it with plgpu._build.build()")
        _build.build()
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def ptr(a: np.ndarray | None, ctype):
    """ctypes pointer to a C-contiguous numpy array (or NULL)."""
    if a is None:
        return None
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data_as(C.POINTER(ctype))


def status_string(status: int) -> str:
    return load().plg_status_string(status).decode()
