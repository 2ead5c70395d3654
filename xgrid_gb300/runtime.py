"""ctypes binding of libxgrid_gb300.so (include/xgrid_gb300.h).

The product path has no CPU fallback: when the library or a CUDA device is
missing, every call raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build

XG_MAX_DIM = 3
XG_MAX_LEVELS = 8
OVERSTEP = {"none": 0, "limit": 1, "wrap": 2}


class XGGrid(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int32),
                ("levels", ctypes.c_int32),
                ("shape", ctypes.c_int64 * XG_MAX_DIM),
                ("level", ctypes.c_void_p * XG_MAX_LEVELS),
                ("scratch", ctypes.c_void_p),
                ("mask", ctypes.c_void_p),
                ("aux", ctypes.c_void_p),
                ("aux_bytes", ctypes.c_int64)]


ENTRY_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(XGGrid), ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t,
                            ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p)

_lib = None

# exported symbol -> (restype, argtypes); every symbol declared in include/xgrid_gb300.h
SIGNATURES = {
    "xg_last_error": (ctypes.c_char_p, []),
    "xg_set_error": (None, [ctypes.c_char_p]),
    "xg_runtime_version": (ctypes.c_int, []),
    "xg_mask_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_void_p)]),
    "xg_mask_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "xg_mask_upload": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "xg_mask_version": (ctypes.c_uint64, [ctypes.c_void_p]),
    "xg_mask_device": (ctypes.c_void_p, [ctypes.c_void_p]),
    "xg_mask_cells": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p),
                                     ctypes.POINTER(ctypes.c_int64)]),
    "xg_mask_nonzero": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "xg_mask_tiles": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_int32,
                                     ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                     ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_int64)]),
    "xg_mask_tile_local": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_int32,
                                          ctypes.c_int, ctypes.POINTER(ctypes.c_int32), ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_int)]),
    "xg_mask_tile_reach": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_int32), ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "xg_mask_boxes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                                     ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                     ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_int64)]),
    "xg_mask_box_check": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
                                         ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                                         ctypes.c_int32, ctypes.c_int, ctypes.POINTER(ctypes.c_int32), ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                                         ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int)]),
    "xg_call": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(XGGrid), ctypes.c_int, ctypes.c_void_p,
                               ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int]),
    "xg_memcpy": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "xg_force_wide_index": (None, [ctypes.c_int]),
    "xg_wide_index_forced": (ctypes.c_int, []),
    "xg_graph_clear": (ctypes.c_int, [ctypes.c_void_p]),
    "xg_graph_count": (ctypes.c_int64, []),
    "xg_prof_enable": (None, [ctypes.c_int]),
    "xg_prof_enabled": (ctypes.c_int, []),
    "xg_prof_launch": (None, [ctypes.c_int, ctypes.c_void_p]),
    "xg_prof_end": (None, [ctypes.c_int, ctypes.c_void_p]),
    "xg_prof_launches": (ctypes.c_int64, []),
    "xg_prof_read": (ctypes.c_int, [ctypes.c_int64, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_float),
                                    ctypes.POINTER(ctypes.c_int64)]),
    "xg_prof_reset": (None, []),
}


def prof_records() -> list:
    """[(group id, ms)] of the launches recorded while profiling was on."""
    lib = load()
    count = ctypes.c_int64()
    check(lib.xg_prof_read(0, None, None, ctypes.byref(count)), "prof")
    n = count.value
    groups = (ctypes.c_int32 * max(n, 1))()
    ms = (ctypes.c_float * max(n, 1))()
    check(lib.xg_prof_read(n, groups, ms, ctypes.byref(count)), "prof")
    return [(groups[i], ms[i]) for i in range(n)]


def load(path: str | None = None):
    """Load (building if needed) the runtime library."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or build.ensure_runtime()
    if not os.path.exists(path):
        raise RuntimeError(f"xgrid runtime library missing: {path}")
    lib = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    msg = load().xg_last_error()
    return msg.decode() if msg else ""


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        raise Exception((f"{what}: " if what else "") + last_error())
