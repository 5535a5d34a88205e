"""ctypes binding of liblbm_gb300.so (the C ABI in include/lbm_gb300.h).

The library is the product's compute path; there is no CPU fallback.  ``lib()`` raises
if the shared library has not been built (``build_native.build()``) or cannot be loaded.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build_native

MAX_Q = 37
MAX_BC = 8

LBM_OK, LBM_ERR_INVALID, LBM_ERR_CUDA, LBM_ERR_NOMEM, LBM_ERR_UNSUPPORTED, LBM_ERR_STATE, LBM_ERR_NONFINITE = \
    0, -1, -2, -3, -4, -5, -6

QUAD_IDS = {"D2Q4": 0, "D2Q5": 1, "D2Q9": 2, "D2Q13": 3, "D2Q17": 4, "D2Q21": 5, "D2Q37": 6}
SRT, TRT, MRT, ITERATIVE_INIT = 0, 1, 2, 3
STORE_F64, STORE_F32_DEV, STORE_F16_DEV, STORE_DF64_DEV, STORE_F32_DEV_SR, STORE_F64_DD = 0, 1, 2, 3, 4, 5
STORAGE_IDS = {"f64": STORE_F64, "f32dev": STORE_F32_DEV, "f16dev": STORE_F16_DEV, "df64dev": STORE_DF64_DEV,
               "f32sr": STORE_F32_DEV_SR, "f64dd": STORE_F64_DD}
FORCE_NONE, FORCE_CONSTANT, FORCE_FIELD, FORCE_SHEAR = 0, 1, 2, 3
BOUNCE_BACK, MOVING_WALL = 0, 1
NORTH, EAST, SOUTH, WEST = 0, 1, 2, 3
REDUCE_TRACK_ERRORS, REDUCE_COMPARE, REDUCE_MEAN_VELOCITY, REDUCE_VELOCITY_CONVERGENCE, \
    REDUCE_DENSITY_AT, REDUCE_CONSERVED = 0, 1, 2, 3, 4, 5
REDUCE_K = {0: 16, 1: 12, 2: 2, 3: 3, 4: 1, 5: 4}

_DP = C.POINTER(C.c_double)


class LbmBC(C.Structure):
    _fields_ = [("kind", C.c_int32), ("direction", C.c_int32), ("x_lo", C.c_int32), ("x_hi", C.c_int32),
                ("y_lo", C.c_int32), ("y_hi", C.c_int32), ("u", C.c_double * 2), ("rho", C.c_double),
                ("T", C.c_double)]


class LbmDesc(C.Structure):
    _fields_ = [("quadrature", C.c_int32), ("weights", C.c_double * MAX_Q),
                ("speed_of_sound_squared", C.c_double), ("collision", C.c_int32), ("tau", C.c_double * 4),
                ("force_kind", C.c_int32), ("force", C.c_double * 2), ("force_field", _DP),
                ("shear", C.c_double * 6), ("x_coords", _DP), ("y_coords", _DP), ("nonlinear", _DP),
                ("nbc", C.c_int32), ("bcs", C.POINTER(LbmBC)), ("nx", C.c_int64), ("ny", C.c_int64),
                ("storage", C.c_int32)]


class LbmAnalytic(C.Structure):
    _fields_ = [("rho", _DP), ("ux", _DP), ("uy", _DP), ("p", _DP), ("sxx", _DP), ("syx", _DP),
                ("sxy", _DP), ("syy", _DP), ("on_device", C.c_int32), ("tau", C.c_double),
                ("u_max", C.c_double), ("area", C.c_double)]


class LbmBatchSchedule(C.Structure):
    _fields_ = [("resident_max_nodes", C.c_int64 * 7), ("nodes_per_block", C.c_int32 * 7), ("split", C.c_int32 * 7)]


_lock = threading.Lock()
_lib = None


class LbmError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"liblbm_gb300 status {status}: {message}")
        self.status = status


def library_path() -> str:
    return build_native.LIB


def lib():
    """Load liblbm_gb300.so.  Raises if it is missing: the product has no CPU fallback."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(
                f"liblbm_gb300.so not found at {path}; build it first (build_native.build()). "
                "The collide-stream path runs only on the CUDA library.")
        L = C.CDLL(path)
        vp = C.c_void_p
        L.lbm_abi_version.restype = C.c_int32
        L.lbm_status_string.restype = C.c_char_p
        L.lbm_status_string.argtypes = [C.c_int32]
        L.lbm_create.argtypes = [C.POINTER(vp), C.POINTER(LbmDesc)]
        L.lbm_create.restype = C.c_int32
        L.lbm_destroy.argtypes = [vp]
        L.lbm_destroy.restype = None
        L.lbm_last_error.argtypes = [vp]
        L.lbm_last_error.restype = C.c_char_p
        L.lbm_set_stream.argtypes = [vp, vp]
        L.lbm_synchronize.argtypes = [vp]
        for name in ("lbm_upload", "lbm_download", "lbm_upload_device", "lbm_download_device"):
            getattr(L, name).argtypes = [vp, vp]
            getattr(L, name).restype = C.c_int32
        L.lbm_step.argtypes = [vp, C.c_int64, C.c_int64, C.c_double]
        L.lbm_step.restype = C.c_int32
        L.lbm_last_launch_count.argtypes = [vp]
        L.lbm_last_launch_count.restype = C.c_int64
        L.lbm_reduce.argtypes = [vp, C.c_int32, C.POINTER(LbmAnalytic), _DP]
        L.lbm_reduce.restype = C.c_int32
        L.lbm_macroscopic.argtypes = [vp, vp, vp, vp]
        L.lbm_macroscopic.restype = C.c_int32
        L.lbm_collide_device.argtypes = [vp, vp, vp, C.c_double]
        L.lbm_collide_device.restype = C.c_int32
        L.lbm_stream_device.argtypes = [vp, vp, vp]
        L.lbm_stream_device.restype = C.c_int32
        L.lbm_apply_bcs_device.argtypes = [vp, vp, vp]
        L.lbm_apply_bcs_device.restype = C.c_int32
        L.lbm_batch_create.argtypes = [C.POINTER(vp), C.POINTER(vp), C.c_int32]
        L.lbm_batch_create.restype = C.c_int32
        L.lbm_batch_destroy.argtypes = [vp]
        L.lbm_batch_destroy.restype = None
        L.lbm_batch_step.argtypes = [vp, C.POINTER(C.c_int64)]
        L.lbm_batch_step.restype = C.c_int32
        L.lbm_batch_step_timed.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), _DP]
        L.lbm_batch_step_timed.restype = C.c_int32
        L.lbm_batch_set_stream.argtypes = [vp, vp]
        L.lbm_batch_set_stream.restype = C.c_int32
        L.lbm_batch_synchronize.argtypes = [vp]
        L.lbm_batch_synchronize.restype = C.c_int32
        L.lbm_batch_last_launch_count.argtypes = [vp]
        L.lbm_batch_last_launch_count.restype = C.c_int64
        L.lbm_batch_last_error.argtypes = [vp]
        L.lbm_batch_last_error.restype = C.c_char_p
        L.lbm_initialize_fields.argtypes = [vp] + [_DP] * 7 + [C.c_double, C.c_int32]
        L.lbm_initialize_fields.restype = C.c_int32
        L.lbm_batch_reduce.argtypes = [vp, C.c_int32, C.POINTER(C.c_uint8), _DP]
        L.lbm_batch_reduce.restype = C.c_int32
        L.lbm_batch_reduce_fields.argtypes = [vp, C.c_int32, C.POINTER(C.c_uint8), C.POINTER(LbmAnalytic), _DP]
        L.lbm_batch_reduce_fields.restype = C.c_int32
        L.lbm_batch_share_stream.argtypes = [vp]
        L.lbm_batch_share_stream.restype = C.c_int32
        L.lbm_batch_set_schedule.argtypes = [vp, C.POINTER(LbmBatchSchedule)]
        L.lbm_batch_set_schedule.restype = C.c_int32
        L.lbm_adjoint_create.argtypes = [C.POINTER(vp), vp, C.c_int64, C.c_int64]
        L.lbm_adjoint_create.restype = C.c_int32
        L.lbm_adjoint_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.lbm_adjoint_info.restype = C.c_int32
        L.lbm_adjoint_destroy.argtypes = [vp]
        L.lbm_adjoint_destroy.restype = None
        L.lbm_adjoint_run.argtypes = [vp, _DP, _DP, _DP, _DP]
        L.lbm_adjoint_run.restype = C.c_int32
        L.lbm_adjoint_last_error.argtypes = [vp]
        L.lbm_adjoint_last_error.restype = C.c_char_p
        _lib = L
        return L


EXPORTED_SYMBOLS = [
    "lbm_abi_version", "lbm_status_string", "lbm_create", "lbm_destroy", "lbm_last_error",
    "lbm_set_stream", "lbm_synchronize", "lbm_upload", "lbm_download", "lbm_upload_device",
    "lbm_download_device", "lbm_step", "lbm_last_launch_count", "lbm_reduce", "lbm_macroscopic",
    "lbm_collide_device", "lbm_stream_device", "lbm_apply_bcs_device", "lbm_batch_create", "lbm_batch_destroy",
    "lbm_batch_step", "lbm_batch_step_timed", "lbm_batch_set_stream", "lbm_batch_synchronize", "lbm_batch_last_launch_count",
    "lbm_batch_last_error", "lbm_batch_reduce", "lbm_batch_reduce_fields", "lbm_batch_share_stream", "lbm_batch_set_schedule", "lbm_initialize_fields", "lbm_adjoint_create", "lbm_adjoint_info", "lbm_adjoint_destroy", "lbm_adjoint_run",
    "lbm_adjoint_last_error",
]


def ptr(a) -> int:
    """Address of a numpy array, a torch tensor, or an int."""
    if a is None:
        return 0
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


def check(ctx_handle, status):
    if status != LBM_OK:
        L = lib()
        msg = L.lbm_last_error(ctx_handle).decode() if ctx_handle else ""
        raise LbmError(status, f"{L.lbm_status_string(status).decode()} ({msg})")
    return status
