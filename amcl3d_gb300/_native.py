"""ctypes binding of ``libamcl3d_gpu.so`` (the C ABI in ``include/amcl3d_gpu.h``).

The library is the only implementation: when it is missing or cannot be loaded,
importing this module raises ``ImportError`` (there is no CPU fallback).
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_LIB_PATH = Path(os.environ.get("AMCL3D_GPU_LIB", Path(__file__).resolve().parent / "_lib" / "libamcl3d_gpu.so"))

AMCL_OK = 0
STATUS = {
    0: "AMCL_OK",
    1: "AMCL_EINVAL",
    2: "AMCL_ENOMEM",
    3: "AMCL_ECUDA",
    4: "AMCL_ETIMEDOUT",
    5: "AMCL_ESTATE",
    6: "AMCL_EIO",
    7: "AMCL_ERANGE",
    8: "AMCL_ENOTSUP",
}
GRID_F32, GRID_F16, GRID_U8 = 0, 1, 2
OPT_CLOUD_SUM, OPT_RESAMPLE_PREFIX, OPT_WEIGHT_KERNEL, OPT_SEED, OPT_WAIT_PROBE = 1, 2, 3, 4, 5
PROF_NAMES = ("cloud_weight", "normalize", "resample", "predict", "distance_field")


class AmclError(RuntimeError):
    def __init__(self, status: int, func: str, detail: str):
        self.status = status
        super().__init__(f"{func}: {STATUS.get(status, status)}: {detail}")


class GridInfo(C.Structure):
    _fields_ = [
        ("min", C.c_double * 3),
        ("max", C.c_double * 3),
        ("resolution", C.c_double),
        ("sensor_dev", C.c_double),
        ("size", C.c_uint32 * 3),
        ("storage", C.c_uint32),
        ("u8_scale", C.c_float),
        ("reserved", C.c_uint32),
    ]


if not _LIB_PATH.exists():
    raise ImportError(
        f"amcl3d_gb300: native library {_LIB_PATH} is missing; build it with "
        "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)"
    )
lib = C.CDLL(str(_LIB_PATH))

_vp, _u32, _u64, _i32, _i64 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int32, C.c_int64
_f, _d, _int = C.c_float, C.c_double, C.c_int
_fp, _dp = C.POINTER(C.c_float), C.POINTER(C.c_double)

_SIGS = {
    "amcl_grid_create": [C.POINTER(_vp), _vp],
    "amcl_grid_destroy": [_vp],
    "amcl_grid_build": [_vp, _fp, _u64, _u32, _dp, _dp, _d, _d],
    "amcl_grid_load_cells": [_vp, C.POINTER(GridInfo), _fp, _fp],
    "amcl_grid_save": [_vp, C.c_char_p],
    "amcl_grid_load": [_vp, C.c_char_p, _dp, _dp, _d, _d],
    "amcl_grid_info_get": [_vp, C.POINTER(GridInfo)],
    "amcl_grid_weight_loop": [_vp, C.POINTER(_int)],
    "amcl_grid_read_cells": [_vp, _u64, _u64, _fp, _fp],
    "amcl_grid_set_storage": [_vp, _int],
    "amcl_grid_set_l2_window": [_vp, _int],
    "amcl_grid_is_into_map": [_vp, _f, _f, _f, C.POINTER(_int)],
    "amcl_grid_cloud_weights": [_vp, _fp, _u32, _fp, _u32, _u32, _f, _f, _fp],
    "amcl_grid_cloud_weights_noalloc": [_vp, _vp, _u32, _vp, _u32, _f, _f, _vp, _vp],
    "amcl_octomap_read": [C.c_char_p, _fp, _u64, C.POINTER(_u64), _dp, _dp, _dp, C.POINTER(_u64)],
    "amcl_grid_open": [_vp, C.c_char_p, _d, C.POINTER(_u64)],
    "amcl_grid_slice": [_vp, _d, C.POINTER(C.c_int8), _u64, C.POINTER(_u64), C.POINTER(_u32), C.POINTER(_u32)],
    "amcl_grid_stream": [_vp, C.POINTER(_vp)],
    "amcl_pf_create": [C.POINTER(_vp), _u64, _vp],
    "amcl_pf_destroy": [_vp],
    "amcl_pf_init": [_vp, _int, _f, _f, _f, _f, _f, _f, _f, _f],
    "amcl_pf_predict": [_vp, _d, _d, _d, _d, _d, _d, _d, _d],
    "amcl_pf_update": [_vp, _vp, _fp, _u32, _u32, _fp, _u32, _d, _d, _d, _d],
    "amcl_pf_update_dev": [_vp, _vp, _vp, _u32, _fp, _u32, _d, _d, _d, _d],
    "amcl_pf_update_ranges": [_vp, _fp, _u32, _d, _d],
    "amcl_pf_resample": [_vp],
    "amcl_pf_resample_with": [_vp, _f],
    "amcl_pf_get_mean": [_vp, _fp, _dp],
    "amcl_pf_is_initialized": [_vp, C.POINTER(_int)],
    "amcl_pf_size": [_vp, C.POINTER(_u32)],
    "amcl_pf_get_particles": [_vp, _fp, _u32],
    "amcl_pf_set_particles": [_vp, _fp, _u32],
    "amcl_pf_set_option": [_vp, _int, _i64],
    "amcl_pf_record_draws": [_vp, _int],
    "amcl_pf_get_draws": [_vp, _fp, _u32],
    "amcl_pf_get_resample_index": [_vp, C.POINTER(_i32), _u32],
    "amcl_pf_stream": [_vp, C.POINTER(_vp)],
    "amcl_batch_create": [C.POINTER(_vp), _u32, _u64, _u64, _vp],
    "amcl_batch_destroy": [_vp],
    "amcl_batch_add": [_vp, _vp, _u32, _u64, C.POINTER(_int)],
    "amcl_batch_remove": [_vp, _int],
    "amcl_batch_set_grid": [_vp, _int, _vp],
    "amcl_batch_init": [_vp, _int, _int, _f, _f, _f, _f, _f, _f, _f, _f],
    "amcl_batch_set_particles": [_vp, _int, _fp, _u32],
    "amcl_batch_get_particles": [_vp, _int, _fp, _u32],
    "amcl_batch_stage": [_vp, _int, _fp, _u32, _u32, _fp, _u32, _dp, _d, _d, _d, _d, _int],
    "amcl_batch_stage_many": [_vp, _u32, C.POINTER(_int), C.POINTER(_vp), C.POINTER(_u32), _u32, C.POINTER(_vp),
                              C.POINTER(_u32), _dp, _d, _d, _d, _d, _int],
    "amcl_batch_stage_packed": [_vp, _u32, C.POINTER(_int), _fp, C.POINTER(_u32), _u32, _fp, C.POINTER(_u32), _dp,
                                _d, _d, _d, _d, _int],
    "amcl_batch_step": [_vp],
    "amcl_batch_wait": [_vp],
    "amcl_batch_get_mean": [_vp, _int, _fp, _dp],
    "amcl_batch_set_tuning": [_vp, _int, _int],
    "amcl_batch_set_split": [_vp, _int, _u64],
    "amcl_batch_get_tuning": [_vp, C.POINTER(_int), C.POINTER(_int)],
    "amcl_batch_autotune": [_vp, _int, C.POINTER(_int), C.POINTER(_int), C.POINTER(_d)],
    "amcl_batch_capacity": [_vp, C.POINTER(_u64), C.POINTER(_u32)],
    "amcl_batch_stream": [_vp, C.POINTER(_vp)],
    "amcl_server_create": [C.POINTER(_vp), _u32, _u64, _u64, _vp],
    "amcl_server_create_lanes": [C.POINTER(_vp), _u32, _u64, _u64, _u32, _vp],
    "amcl_server_destroy": [_vp],
    "amcl_server_open_session": [_vp, _vp, _u32, _u64, _int, _fp, C.POINTER(_i64)],
    "amcl_server_close_session": [_vp, _i64],
    "amcl_server_submit": [_vp, _i64, _fp, _u32, _u32, _fp, _u32, _dp, _d, _d, _d, _d, _int, C.POINTER(_u64)],
    "amcl_server_poll": [_vp, _vp, _u32, C.POINTER(_u32)],
    "amcl_batch_counters": [_vp, C.POINTER(_u64), C.POINTER(_u64), C.POINTER(_u64)],
    "amcl_server_counters": [_vp, C.POINTER(_u64), C.POINTER(_u64)],
    "amcl_server_stats": [_vp, C.POINTER(_u64), C.POINTER(_u64), C.POINTER(_d), C.POINTER(_u32), C.POINTER(_u32)],
    "amcl_server_batch": [_vp, C.POINTER(_vp)],
    "amcl_pf_profile": [_vp, _int],
    "amcl_voxel_create": [C.POINTER(_vp), _vp],
    "amcl_voxel_destroy": [_vp],
    "amcl_voxel_stream": [_vp, C.POINTER(_vp)],
    "amcl_voxel_filter": [_vp, _fp, _u64, _u32, _f, _f, _f, _fp, _u64, C.POINTER(_u64)],
    "amcl_voxel_filter_dev": [_vp, _vp, _u64, _f, _f, _f, _vp, C.POINTER(_u64)],
    "amcl_pf_update_voxel": [_vp, _vp, _vp, _fp, _u32, _u32, _f, _f, _f, _fp, _u32, _d, _d, _d, _d, _fp, _u64,
                             C.POINTER(_u64)],
    "amcl_pf_profile_read": [_vp, _dp, C.POINTER(_u64), _int],
}
for _name, _args in _SIGS.items():
    _fn = getattr(lib, _name)
    _fn.argtypes = _args
    _fn.restype = _int
lib.amcl_status_string.argtypes = [_int]
lib.amcl_status_string.restype = C.c_char_p
lib.amcl_last_error.argtypes = []
lib.amcl_last_error.restype = C.c_char_p
lib.amcl_kernel_launches.argtypes = []
lib.amcl_kernel_launches.restype = _u64


def call(name: str, *args) -> None:
    rc = getattr(lib, name)(*args)
    if rc != AMCL_OK:
        raise AmclError(rc, name, lib.amcl_last_error().decode(errors="replace"))


def kernel_launches() -> int:
    return int(lib.amcl_kernel_launches())


def fptr(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_fp)


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def exported_symbols() -> list[str]:
    return sorted(list(_SIGS) + ["amcl_status_string", "amcl_last_error", "amcl_kernel_launches", "amcl_version"])
