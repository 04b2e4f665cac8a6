"""ctypes binding of libqio_gb300.so (the C ABI in include/qio_gb300.h).

The library is the only compute path: if it is missing or no CUDA device is
present, calls fail loudly (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

QIO_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARGUMENT", 2: "OUT_OF_MEMORY", 3: "CUDA_ERROR",
                4: "TIMEOUT", 5: "NO_DEVICE", 6: "INTERNAL"}


class QioError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
        self.message = message


class ModelInfo(C.Structure):
    _fields_ = [("kind", C.c_int32), ("integer_weights", C.c_int32),
                ("n_vars", C.c_int64), ("n_terms", C.c_int64),
                ("n_incidences", C.c_int64), ("max_locality", C.c_int32),
                ("min_locality", C.c_int32), ("const_cost", C.c_double),
                ("scale_factor", C.c_double), ("max_coupling", C.c_double),
                ("device_bytes", C.c_int64), ("n_levels", C.c_int32),
                ("max_level_width", C.c_int32), ("level_kernel", C.c_int32),
                ("avg_locality", C.c_double), ("sum_coefficient_degrees_total", C.c_int64),
                ("accumulated_dependent_vars", C.c_int64), ("min_coupling", C.c_double)]


class SolverStats(C.Structure):
    _fields_ = [("replicas", C.c_int64), ("last_step", C.c_int64),
                ("attempts", C.c_uint64), ("accepts", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("sweep_kernel_ms", C.c_double),
                ("run_ms", C.c_double), ("near_ties", C.c_uint64),
                ("device_bytes", C.c_int64), ("windows", C.c_uint64),
                ("sweep_kernel", C.c_int32)]


class BatchStats(C.Structure):
    _fields_ = [("run_ms", C.c_double), ("launches", C.c_int64), ("walkers", C.c_int64),
                ("device_bytes", C.c_int64), ("kernel", C.c_int32),
                ("warps_per_block", C.c_int32), ("smem", C.c_int32), ("graph", C.c_int32),
                ("sweep_kernel_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
                ("active", C.c_int64), ("pending", C.c_int64), ("used_bytes", C.c_int64),
                ("budget_bytes", C.c_int64), ("peak_active", C.c_int64), ("elapsed_s", C.c_double),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("max_ms", C.c_double)]


# every symbol include/qio_gb300.h declares, with its ctypes signature
def _signatures():
    vp, i32, i64, dbl, cp = C.c_void_p, C.c_int32, C.c_int64, C.c_double, C.c_char_p
    P = C.POINTER
    st = C.c_int
    return {
        "qio_last_error_message": (cp, []),
        "qio_version": (cp, []),
        "qio_free": (None, [vp]),
        "qio_model_create": (st, [i32, i64, P(i64), P(C.c_int32), P(dbl), P(vp)]),
        "qio_model_create_json": (st, [cp, i32, P(vp)]),
        "qio_model_create_dimacs": (st, [cp, P(vp)]),
        "qio_model_create_proto_folder": (st, [cp, P(vp)]),
        "qio_model_cost_diff_bounds": (st, [vp, P(C.c_double), P(C.c_double)]),
        "qio_bayes_recommend": (st, [C.c_int32, P(C.c_double), P(C.c_double), C.c_int32, P(C.c_double),
                                     P(C.c_double), C.c_uint32, C.c_int32, P(C.c_double)]),
        "qio_model_get_info": (st, [vp, P(ModelInfo)]),
        "qio_model_get_var_names": (st, [vp, P(C.c_int32)]),
        "qio_model_destroy": (st, [vp]),
        "qio_states_cost": (st, [vp, i64, P(C.c_uint8), P(dbl), vp]),
        "qio_states_cost_noalloc": (st, [vp, i64, vp, vp, vp]),
        "qio_states_cost_difference": (st, [vp, i64, P(C.c_uint8), P(i64), P(dbl), vp]),
        "qio_states_apply": (st, [vp, i64, P(C.c_uint8), P(i64)]),
        "qio_solver_create": (st, [vp, cp, cp, P(vp)]),
        "qio_solver_init": (st, [vp, vp]),
        "qio_solver_run": (st, [vp, vp]),
        "qio_solver_result_json": (st, [vp, P(C.c_void_p)]),
        "qio_solver_replicas": (st, [vp, P(i64), P(dbl), P(dbl), P(C.c_uint64),
                                     P(C.c_uint64), P(C.c_uint8), P(C.c_uint8)]),
        "qio_solver_best": (st, [vp, P(dbl), P(C.c_uint8)]),
        "qio_solver_get_stats": (st, [vp, P(SolverStats)]),
        "qio_solver_pt_observables": (st, [vp, P(dbl)]),
        "qio_solver_destroy": (st, [vp]),
        "qio_batch_create": (st, [P(vp), i32, cp, cp, P(vp)]),
        "qio_batch_run": (st, [vp, vp]),
        "qio_batch_result_json": (st, [vp, i32, P(C.c_void_p)]),
        "qio_batch_lowest": (st, [vp, P(dbl)]),
        "qio_batch_get_stats": (st, [vp, P(BatchStats)]),
        "qio_batch_destroy": (st, [vp]),
        "qio_server_create": (st, [cp, P(vp)]),
        "qio_server_submit": (st, [vp, vp, cp, cp, P(i64)]),
        "qio_server_poll": (st, [vp, i64, P(i32), P(C.c_void_p)]),
        "qio_server_wait": (st, [vp, i64, dbl, P(i32), P(C.c_void_p)]),
        "qio_server_forget": (st, [vp, i64]),
        "qio_server_request_bytes": (st, [vp, i64, P(i64)]),
        "qio_server_get_stats": (st, [vp, P(ServerStats)]),
        "qio_server_destroy": (st, [vp]),
        "qio_run_json": (st, [cp, cp, cp, P(C.c_void_p)]),
    }


SYMBOLS = tuple(_signatures().keys())


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) the C-ABI library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build_if_missing and _build.needs_build():
            _build.build()
        if not os.path.exists(_build.LIB):
            raise ImportError(f"libqio_gb300.so not found at {_build.LIB}; run "
                              "qiotoolkit_gb300.build.build()")
        L = C.CDLL(_build.LIB)
        for name, (res, args) in _signatures().items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
        return _lib


def check(status: int) -> None:
    if status != QIO_OK:
        msg = load().qio_last_error_message()
        raise QioError(status, msg.decode() if msg else "")
