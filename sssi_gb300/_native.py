"""ctypes binding of libsssi_gb300.so (the C ABI declared in include/sssi_gb300.h).

The library is built in-tree by :func:`sssi_gb300.build.build_library`.  There
is no fallback: if the shared library is missing or cannot be loaded, every
entry point raises, so a GPU run can never silently compute on the CPU.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

from .build import LIB

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None

c_i64 = ctypes.c_int64
c_dp = ctypes.c_void_p  # double* / int64_t* passed as raw addresses (host or device)



class PlanConfig(ctypes.Structure):
    """sssi_plan_config"""
    _fields_ = [("mode", ctypes.c_int), ("nDiffOrder", ctypes.c_int), ("dz", ctypes.c_double),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("device_bytes", ctypes.c_size_t),
                ("steps_per_round", ctypes.c_int)]


class ShotDesc(ctypes.Structure):
    """sssi_shot_desc"""
    _fields_ = [("kind", ctypes.c_int), ("v", ctypes.c_void_p), ("vs", ctypes.c_void_p), ("nz", c_i64),
                ("nx", c_i64), ("ny", c_i64), ("nt", c_i64), ("nBoundary", ctypes.c_int), ("dt", ctypes.c_double),
                ("nsrc", ctypes.c_int), ("src_iz", ctypes.c_void_p), ("src_ix", ctypes.c_void_p),
                ("src_iy", ctypes.c_void_p), ("wavelets", ctypes.c_void_p), ("epsilon", ctypes.c_double),
                ("snap_stride", ctypes.c_int), ("data", ctypes.c_void_p), ("image", ctypes.c_void_p),
                ("stack", c_i64), ("stack_z0", c_i64), ("stack_x0", c_i64)]


class ShotInfo(ctypes.Structure):
    """sssi_shot_info"""
    _fields_ = [("state", ctypes.c_int), ("status", ctypes.c_int), ("submit_s", ctypes.c_double),
                ("start_s", ctypes.c_double), ("done_s", ctypes.c_double), ("cell_updates", c_i64)]


class PlanStats(ctypes.Structure):
    """sssi_plan_stats"""
    _fields_ = [("queued", c_i64), ("running", c_i64), ("done", c_i64), ("failed", c_i64),
                ("device_bytes_in_use", ctypes.c_size_t), ("device_bytes_budget", ctypes.c_size_t),
                ("batch_steps", c_i64), ("cell_updates", ctypes.c_double), ("admit_s", ctypes.c_double),
                ("round_s", ctypes.c_double), ("gpu_wait_s", ctypes.c_double), ("deliver_s", ctypes.c_double),
                ("batch2d_gpu_s", ctypes.c_double), ("batch2d_cell_updates", ctypes.c_double),
                ("batch2d_tile_shape", ctypes.c_int), ("batch2d_tune_ms", ctypes.c_double * 3)]


# name -> (restype, argtypes)
SIGNATURES = {
    "sssi_plan_create": (ctypes.c_int, [ctypes.POINTER(PlanConfig), ctypes.POINTER(ctypes.c_void_p)]),
    "sssi_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "sssi_shot_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ShotDesc), ctypes.POINTER(c_i64)]),
    "sssi_poll": (ctypes.c_int, [ctypes.c_void_p, c_i64, ctypes.POINTER(ShotInfo)]),
    "sssi_cancel": (ctypes.c_int, [ctypes.c_void_p, c_i64]),
    "sssi_plan_stack_create": (ctypes.c_int, [ctypes.c_void_p, c_i64, c_i64, ctypes.POINTER(c_i64)]),
    "sssi_plan_stack_get": (ctypes.c_int, [ctypes.c_void_p, c_i64, c_dp]),
    "sssi_debug_withhold_copy": (ctypes.c_int, [ctypes.c_int, ctypes.c_uint]),
    "sssi_debug_tile_shape": (ctypes.c_int, [ctypes.c_int]),
    "sssi_debug_schedule3d": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float)]),
    "sssi_debug_divide": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p,
                                         ctypes.c_void_p]),
    "sssi_wait": (ctypes.c_int, [ctypes.c_void_p, c_i64, ctypes.POINTER(ShotInfo)]),
    "sssi_plan_stats_get": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(PlanStats)]),
    "sssi_last_error": (ctypes.c_char_p, []),
    "sssi_version": (ctypes.c_int, []),
    "sssi_launch_count": (c_i64, []),
    "sssi_release_cache": (ctypes.c_int, []),
    "sssi_set_stream": (ctypes.c_int, [ctypes.c_void_p]),
    "sssi_enable_timing": (ctypes.c_int, [ctypes.c_int]),
    "sssi_last_timing": (ctypes.c_int, [c_dp, c_dp, ctypes.c_int, c_dp]),
    "sssi_measure_fp64_rate": (ctypes.c_int, [c_dp]),
    "sssi_dCoef": (ctypes.c_int, [ctypes.c_int, c_dp]),
    "sssi_diffOperator": (ctypes.c_int, [c_dp, ctypes.c_int, c_dp, c_dp, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                         c_dp, ctypes.c_int]),
    "sssi_dampPml": (ctypes.c_int, [c_dp, c_dp, c_i64, ctypes.c_double, c_dp]),
    "sssi_fwdTimeCpmlFor2dAw": (ctypes.c_int, [c_dp, c_dp, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_double, ctypes.c_double, ctypes.c_double, c_dp, c_dp,
                                                ctypes.c_int]),
    "sssi_rvsTimeCpmlFor2dAw": (ctypes.c_int, [c_dp, c_dp, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_double, ctypes.c_double, ctypes.c_double, c_dp, c_dp,
                                                ctypes.c_int]),
    "sssi_fwdTimeCpmlFor3dAw": (ctypes.c_int, [c_dp, c_dp, c_i64, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                                c_dp, c_dp, ctypes.c_int]),
    "sssi_fwdTimeCpmlFor3dAwPoint": (ctypes.c_int, [c_dp, c_i64, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_int,
                                                     ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                                     ctypes.c_double, ctypes.c_int, c_dp, c_dp, c_dp, c_dp, c_dp, c_dp,
                                                     ctypes.c_int]),
    "sssi_fwdTimeCpmlFor2dAwPoint": (ctypes.c_int, [c_dp, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_int,
                                                     ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                                     ctypes.c_int, c_dp, c_dp, c_dp, c_dp, c_dp, ctypes.c_int]),
    "sssi_fwdTimeCpmlFor2dAwNoAlloc": (ctypes.c_int, [c_dp, c_dp, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_int,
                                                       ctypes.c_double, ctypes.c_double, ctypes.c_double, c_dp, c_dp,
                                                       ctypes.c_int]),
    "sssi_fwdTimeSpongeFor2dAw": (ctypes.c_int, [c_dp, c_dp, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_double, c_dp, c_dp, ctypes.c_int]),
    "sssi_fwdTimeSpongeFor2dAwPoint": (ctypes.c_int, [c_dp, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_double,
                                                       ctypes.c_double, ctypes.c_double, ctypes.c_int, c_dp, c_dp,
                                                       c_dp, c_dp, c_dp, ctypes.c_int]),
    "sssi_rvsTimeSpongeFor2dAw": (ctypes.c_int, [c_dp, c_dp, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_double, c_dp, c_dp, ctypes.c_int]),
    "sssi_rtmTimeSpongeFor2dAw": (ctypes.c_int, [c_dp, c_dp, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_double, c_dp, c_i64, c_i64,
                                                  ctypes.c_double, ctypes.c_int, c_dp, c_dp, c_dp]),
    "sssi_fwdTimeSpmlFor2dEw": (ctypes.c_int, [c_dp, c_dp, c_dp, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_double, ctypes.c_double, ctypes.c_double, c_dp, c_dp, c_dp,
                                                c_dp, ctypes.c_int]),
    "sssi_fwdTimeSpmlFor2dEwPoint": (ctypes.c_int, [c_dp, c_dp, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_int,
                                                     ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                                     c_dp, c_dp, c_dp, c_dp, c_dp, c_dp, c_dp, ctypes.c_int]),
    "sssi_fwdTimeSpmlFor3dEw": (ctypes.c_int, [c_dp, c_dp, c_dp, c_dp, c_dp, c_i64, c_i64, c_i64, c_i64,
                                                ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                ctypes.c_double, ctypes.c_double, c_dp, c_dp, c_dp, c_dp, c_dp, c_dp,
                                                ctypes.c_int]),
    "sssi_fwdTimeSpmlFor3dEwPoint": (ctypes.c_int, [c_dp, c_dp, c_i64, c_i64, c_i64, c_i64, ctypes.c_int,
                                                     ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                                     ctypes.c_double, ctypes.c_int, c_dp, c_dp, c_dp, c_dp, c_dp,
                                                     c_dp, c_dp, c_dp, c_dp, c_dp, c_dp, ctypes.c_int]),
    "sssi_mat_write": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, c_dp, c_dp, c_dp, c_dp]),
    "sssi_mat_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, c_dp, c_i64, c_dp, c_dp]),
    "sssi_rtmTimeCpmlFor2dAw": (ctypes.c_int, [c_dp, c_dp, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_double, ctypes.c_double, ctypes.c_double, c_dp, c_i64,
                                                c_i64, ctypes.c_double, ctypes.c_int, ctypes.c_int, c_dp, c_dp,
                                                c_dp]),
}


class SSSIError(RuntimeError):
    """A libsssi_gb300 call returned a non-zero status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[sssi status {code}] {message}")
        self.code = code


def lib() -> ctypes.CDLL:
    """The loaded library (loads it on first use; raises if it is not built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not Path(LIB).exists():
                raise RuntimeError(f"{LIB} is not built: run `python -c 'import __graft_entry__ as g; g.build()'` "
                                   "(CUDA extension required, there is no CPU fallback)")
            L = ctypes.CDLL(str(LIB))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name, None)
                if fn is None:
                    continue
                fn.restype = res
                fn.argtypes = args
            _lib = L
        return _lib


def check(code: int) -> None:
    if code != 0:
        raise SSSIError(code, lib().sssi_last_error().decode(errors="replace"))


def launch_count() -> int:
    return int(lib().sssi_launch_count())
