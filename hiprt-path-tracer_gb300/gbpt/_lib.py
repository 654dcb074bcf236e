"""ctypes binding of libgbpt.so (the C ABI declared in include/gbpt.h).

There is no fallback: if the library is missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_LIB = None

c_f = ctypes.POINTER(ctypes.c_float)
c_i32 = ctypes.POINTER(ctypes.c_int32)
c_u8 = ctypes.POINTER(ctypes.c_uint8)
c_u64 = ctypes.POINTER(ctypes.c_ulonglong)
c_vp = ctypes.c_void_p
i64 = ctypes.c_int64
i32 = ctypes.c_int32


class BvhParams(ctypes.Structure):
    _fields_ = [("sah_bins", i32), ("max_leaf_size", i32), ("num_threads", i32)]


class BvhStats(ctypes.Structure):
    _fields_ = [("n_triangles", i64), ("n_bvh_triangles", i64), ("n_nodes", i64), ("n_binary_nodes", i64),
                ("wide_depth", i32), ("node_bytes", i32), ("triangle_bytes", i32), ("reserved", i32),
                ("device_bytes", i64), ("build_seconds", ctypes.c_double), ("upload_seconds", ctypes.c_double)]


class TraceConfig(ctypes.Structure):
    _fields_ = [("kernel", i32), ("block", i32), ("refill_below", i32), ("postpone_below", i32),
                ("blocks_per_sm", i32), ("shared_stack", i32), ("triangle_test", i32), ("top_levels", i32),
                ("reserved", i32 * 4)]


class GbptError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"gbpt status {status}: {message}")
        self.status = status


# (name, restype, argtypes) of every exported entry point
SIGNATURES = [
    ("gbpt_status_string", ctypes.c_char_p, [ctypes.c_int]),
    ("gbpt_last_error", ctypes.c_char_p, []),
    ("gbpt_version", i32, []),
    ("gbpt_bvh_build", ctypes.c_int, [c_i32, c_f, i64, i64, ctypes.POINTER(BvhParams), ctypes.POINTER(c_vp)]),
    ("gbpt_bvh_get_stats", ctypes.c_int, [c_vp, ctypes.POINTER(BvhStats)]),
    ("gbpt_bvh_destroy", ctypes.c_int, [c_vp]),
    ("gbpt_trace_closest", ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, i64, c_vp, c_vp]),
    ("gbpt_trace_any", ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, i64, c_vp, c_vp]),
    ("gbpt_trace_closest_host", ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, i64, c_vp, c_vp]),
    ("gbpt_trace_any_host", ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, i64, c_vp, c_vp]),
    ("gbpt_trace_count", ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, i64, i32, c_vp, c_vp]),
    ("gbpt_bvh_set_trace_config", ctypes.c_int, [c_vp, i32, ctypes.POINTER(TraceConfig)]),
    ("gbpt_bvh_get_trace_config", ctypes.c_int, [c_vp, i32, ctypes.POINTER(TraceConfig)]),
    ("gbpt_trace_closest_cfg", ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, i64, c_vp, ctypes.POINTER(TraceConfig), c_vp]),
    ("gbpt_trace_any_cfg", ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, i64, c_vp, ctypes.POINTER(TraceConfig), c_vp]),
    ("gbpt_trace_autotune", ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, i64, i32, i32, ctypes.POINTER(TraceConfig),
                                           c_f, c_vp]),
]


def lib_path() -> str:
    return _build.LIB_PATH


def load() -> ctypes.CDLL:
    """Loads libgbpt.so (built in-tree by __graft_entry__.build()). Raises if it is missing."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"libgbpt.so is not built ({path}); run __graft_entry__.build() first")
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status: int) -> None:
    if status != 0:
        lib = load()
        raise GbptError(status, lib.gbpt_last_error().decode(errors="replace"))
