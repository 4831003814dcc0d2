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

# name -> (restype, argtypes)
SIGNATURES = {
    "sssi_last_error": (ctypes.c_char_p, []),
    "sssi_version": (ctypes.c_int, []),
    "sssi_launch_count": (c_i64, []),
    "sssi_release_cache": (ctypes.c_int, []),
    "sssi_set_stream": (ctypes.c_int, [ctypes.c_void_p]),
    "sssi_enable_timing": (ctypes.c_int, [ctypes.c_int]),
    "sssi_last_timing": (ctypes.c_int, [c_dp, c_dp, ctypes.c_int, c_dp]),
    "sssi_dCoef": (ctypes.c_int, [ctypes.c_int, c_dp]),
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
