"""The C ABI: the runtime library loads and exports every function that
include/xgrid_gb300.h declares; errors come back through xg_last_error (no GPU)."""
import ctypes
import os
import re

import pytest

from xgrid_gb300 import build, runtime

HEADER = os.path.join(build.INCLUDE, "xgrid_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"#define[^\n]*(\\\n[^\n]*)*", "", text)
    names = re.findall(r"\b(xg_[a-z0-9_]+)\s*\(", text)
    return sorted(set(n for n in names if not n.startswith("xg_kernel")))


def test_header_declares_the_runtime_surface():
    names = declared_functions()
    for n in ("xg_last_error", "xg_mask_create", "xg_mask_upload", "xg_mask_tiles", "xg_call", "xg_prof_read"):
        assert n in names


def test_runtime_exports_every_declared_function():
    lib = runtime.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(declared_functions()) <= set(runtime.SIGNATURES)


def test_errors_come_back_as_messages():
    lib = runtime.load()
    out = ctypes.c_void_p()
    shape = (ctypes.c_int64 * 4)(2, 2, 2, 2)
    assert lib.xg_mask_create(4, shape, ctypes.byref(out)) != 0
    assert "1 to 3 dimensions" in runtime.last_error()
    shape = (ctypes.c_int64 * 2)(4, 0)
    assert lib.xg_mask_create(2, shape, ctypes.byref(out)) != 0
    assert "positive" in runtime.last_error()
    with pytest.raises(Exception, match="positive"):
        runtime.check(lib.xg_mask_create(2, shape, ctypes.byref(out)), "mask")


def test_mask_handle_without_device_memory():
    lib = runtime.load()
    out = ctypes.c_void_p()
    shape = (ctypes.c_int64 * 2)(8, 8)
    assert lib.xg_mask_create(2, shape, ctypes.byref(out)) == 0
    assert lib.xg_mask_version(out) == 0
    assert lib.xg_mask_destroy(out) == 0
