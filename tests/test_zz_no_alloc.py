"""No-alloc entry point vs the regular entry point (GPU, through the C ABI).

Some callers cannot call cudaMalloc: code under a fixed device-memory budget,
code that runs inside another framework's allocator, or a real-time loop where
an allocation may block.  For them a kernel declared with
``@xgrid.kernel(noalloc=True)`` exports ``xg_kernel_<name>_noalloc``, which takes
the scratch level of its in-place (two-phase) sweeps from a 64 MiB pool inside
the module instead of from the caller.  This file runs last so that a failure
here does not hide the other tests' results.
"""
import ctypes
import os

import numpy as np
import pytest

import xgrid
from xgrid_gb300 import device, runtime

pytestmark = pytest.mark.gpu


@xgrid.kernel(noalloc=True)
def relax(p: xgrid.grid[float, 2], f: xgrid.grid[float, 2], iters: int, h2: float) -> None:
    for _ in range(0, iters):
        p[0, 0] = 0.25 * (p[1, 0][0] + p[-1, 0][0] + p[0, 1][0] + p[0, -1][0] - h2 * f[0, 0][0])
        with xgrid.boundary(1):
            p[0, 0] = p[0, 1][0]
        with xgrid.boundary(2):
            p[0, 0] = 0.5


def _grids(n: int, seed: int):
    rng = np.random.default_rng(seed)
    p = xgrid.Grid((n, n), float)
    f = xgrid.Grid((n, n), float)
    p.now[...] = rng.random((n, n))
    f.now[...] = rng.random((n, n)) - 0.5
    b = p.boundary
    b[:, 0] = 1
    b[0, :] = b[-1, :] = b[:, -1] = 2
    return p, f


def _call_noalloc(p, f, iters: int, h2: float, kern=None) -> int:
    """Call the no-alloc entry point of ``kern`` (default ``relax``) on (p, f)."""
    return _call_grids(kern or relax, [p, f], [iters, h2])


def _call_grids(kern, grids, values) -> int:
    """Call ``xg_kernel_<name>_noalloc`` directly through the C ABI, checking that
    the caller's level pointers stay put and that free device memory does not
    change across the call."""
    import torch
    nk = kern.native
    fn = nk.lib.entry(f"xg_kernel_{nk.module.name}_noalloc")
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(runtime.XGGrid), ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t,
                   ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    for g in grids:
        g._op_invoke(nk.depth, True)
        g._sync_device(False)
    device.stream().synchronize()
    arr = (runtime.XGGrid * len(grids))(*[g.serialize() for g in grids])
    before = [[st.level[i] for i in range(st.levels)] for st in arr]
    packed = nk.pack(values)
    free0 = torch.cuda.mem_get_info()[0]
    rc = fn(arr, len(grids), ctypes.cast(ctypes.byref(packed), ctypes.c_void_p), ctypes.sizeof(packed), None, 0,
            device.stream_handle())
    device.stream().synchronize()
    assert torch.cuda.mem_get_info()[0] == free0, "the no-alloc call changed free device memory"
    if rc == 0:
        assert [[st.level[i] for i in range(st.levels)] for st in arr] == before, \
            "the caller's level pointers must not change"
        for g, st in zip(grids, arr):
            g._adopt(st)
    return rc


def _cache(tmp_path):
    """A fresh module cache per test, inside the tree."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    return os.path.join(root, ".xgrid_cache", "noalloc", tmp_path.name)


def test_noalloc_matches_regular_entry(tmp_path):
    xgrid.init(precision="double", cacheroot=_cache(tmp_path), opt_level=3)
    n = 96
    pa, fa = _grids(n, 11)
    pb, fb = _grids(n, 11)
    p0, f0 = pa.read(0), fa.read(0)
    # one regular call builds the mask tables of pb (the no-alloc call may not);
    # then the inputs are restored
    relax(pb, fb, 1, 0.01)
    pb.now[...] = p0
    fb.now[...] = f0
    for iters in (7, 4):  # two calls in a row; 7 leaves the result in the scratch level
        relax(pa, fa, iters, 0.01)
        assert _call_noalloc(pb, fb, iters, 0.01) == 0, runtime.last_error()
        assert pa.read(0).tobytes() == pb.read(0).tobytes()
        assert fa.read(0).tobytes() == fb.read(0).tobytes()


def test_noalloc_refuses_to_build_tables(tmp_path):
    xgrid.init(precision="double", cacheroot=_cache(tmp_path), opt_level=3)
    warm_p, warm_f = _grids(32, 1)
    relax(warm_p, warm_f, 1, 0.01)  # compiles the module
    p, f = _grids(40, 2)            # fresh masks: no tables yet
    rc = _call_noalloc(p, f, 2, 0.01)
    assert rc != 0
    assert "not built yet" in runtime.last_error()


def test_noalloc_rejects_grids_beyond_the_pool(tmp_path):
    xgrid.init(precision="double", cacheroot=_cache(tmp_path), opt_level=3)
    warm_p, warm_f = _grids(32, 1)
    relax(warm_p, warm_f, 1, 0.01)
    p, f = _grids(3000, 3)          # 72 MB of FP64 scratch > 64 MiB
    rc = _call_noalloc(p, f, 1, 0.01)
    assert rc != 0
    assert "more than the" in runtime.last_error()


@pytest.mark.parametrize("mode", ["persistent", "mixed"])
def test_noalloc_persistent_and_mixed_loops_match_regular_entry(tmp_path, mode):
    """The persistent loop launch and the mixed-precision loop: warmed up by one
    regular call with the same arguments, the no-alloc call gives the regular
    entry's bits (the mixed loop uses the grid's work area, which the caller
    provides like the levels)."""
    kw = {"persistent": True} if mode == "persistent" else {"mixed": "fp32"}
    xgrid.init(precision="double", cacheroot=_cache(tmp_path), opt_level=3, **kw)
    kern = xgrid.kernel(noalloc=True)(relax.func)
    n = 120
    pa, fa = _grids(n, 21)
    pb, fb = _grids(n, 21)
    p0, f0 = pa.read(0), fa.read(0)
    kern(pb, fb, 9, 0.01)
    pb.now[...] = p0
    fb.now[...] = f0
    for iters in (9, 9):
        kern(pa, fa, iters, 0.01)
        assert _call_noalloc(pb, fb, iters, 0.01, kern) == 0, runtime.last_error()
        assert pa.read(0).tobytes() == pb.read(0).tobytes()
