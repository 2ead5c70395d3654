"""Persistent loop launches (``xgrid.init(persistent=True)``): an
in-place loop whose body is one implicit main sweep and its boundary sweeps runs
as one cooperative launch in which each tile waits only for its neighbouring
tiles' previous iteration.  The results
are the same bits as one launch per iteration, for odd and even iteration
counts (the level/scratch exchange parity), 2-D and 3-D grids, extents that are
not multiples of the tile, and against the oracle.  A loop whose boundary cells
read cells of another tile falls back to one launch per iteration.  No tile
wait ever gives up (error word 0)."""
import numpy as np
import pytest

import xgrid
import workloads
from oracle import xgrid_oracle
from xgrid_gb300 import device, runtime
from xgrid_gb300.operator import Operator

pytestmark = pytest.mark.gpu

LOOP_SITE = 61   # profiling site of a persistent loop launch (group * 64 + 61)


def relax(p: xgrid.grid[float, 2], f: xgrid.grid[float, 2], iters: int, h2: float) -> None:
    for _ in range(0, iters):
        p[0, 0] = 0.25 * (p[1, 0][0] + p[-1, 0][0] + p[0, 1][0] + p[0, -1][0] - h2 * f[0, 0][0])
        with xgrid.boundary(1):
            p[0, 0] = p[0, 1][0]
        with xgrid.boundary(2):
            p[0, 0] = 0.5 * p[0, 0][0]


def relax3(p: xgrid.grid[float, 3], f: xgrid.grid[float, 3], iters: int) -> None:
    for _ in range(0, iters):
        p[0, 0, 0] = (p[1, 0, 0][0] + p[-1, 0, 0][0] + p[0, 1, 0][0] + p[0, -1, 0][0] +
                      p[0, 0, 1][0] + p[0, 0, -1][0]) / 6.0 - f[0, 0, 0][0]
        with xgrid.boundary(1):
            p[0, 0, 0] = 0.0


def _kernel(impl, fn, cacheroot, persistent, precision="double", overstep="none"):
    if impl is xgrid_oracle:
        impl.init(precision=precision, cacheroot=cacheroot, opt_level=3, overstep=overstep)
        return impl.kernel()(fn)
    impl.init(precision=precision, cacheroot=cacheroot, opt_level=3, overstep=overstep, persistent=persistent)
    return Operator(fn, "kernel", f"{fn.__name__}_{int(persistent)}_{precision}_{overstep}")


def _sites(k, call):
    """Profiling sites of the launches of one eager call."""
    from xgrid_gb300.native import NativeKernel
    if k.native is None:
        k.native = NativeKernel(k)
    lib = runtime.load()
    k.native.use_graph = False
    lib.xg_prof_reset()
    lib.xg_prof_enable(1)
    call()
    device.stream().synchronize()
    lib.xg_prof_enable(0)
    sites = [g % 64 for g, _ in runtime.prof_records()]
    lib.xg_prof_reset()
    k.native.use_graph = True
    return sites


def _relax_grids(impl, shape, seed, column=None):
    rng = np.random.default_rng(seed)
    p, f = impl.Grid(shape, float), impl.Grid(shape, float)
    p.now[...] = rng.random(shape)
    f.now[...] = rng.random(shape) - 0.5
    m = np.zeros(shape, np.int32)
    m[:, 0] = 1
    m[0, :] = m[-1, :] = m[:, -1] = 2
    if column is not None:
        m[5:-5, column] = 1     # boundary copy from column + 1
    p.boundary[...] = m
    return p, f


@pytest.mark.parametrize("iters", [1, 2, 3, 7, 50])
@pytest.mark.parametrize("shape", [(64, 64), (67, 131), (203, 45)])
def test_relax_loop_matches_per_launch_and_oracle(cacheroot, iters, shape):
    out = {}
    for name, impl, persistent in (("loop", xgrid, True), ("each", xgrid, False), ("oracle", xgrid_oracle, False)):
        k = _kernel(impl, relax, cacheroot, persistent)
        p, f = _relax_grids(impl, shape, 3)
        for _ in range(2):
            k(p, f, iters, 1e-3)
        out[name] = np.array(p.now).copy()
        if name == "loop":
            assert k.native.loop_error() == 0
            sites = _sites(k, lambda: k(p, f, iters, 1e-3))
            assert sites.count(LOOP_SITE) == 1, sites
    assert out["loop"].tobytes() == out["each"].tobytes()
    assert out["loop"].tobytes() == out["oracle"].tobytes()


@pytest.mark.parametrize("precision", ["double", "float"])
@pytest.mark.parametrize("overstep", ["none", "wrap"])
def test_3d_loop_matches_per_launch(cacheroot, precision, overstep):
    shape = (21, 37, 45)
    out = {}
    for persistent in (True, False):
        k = _kernel(xgrid, relax3, cacheroot, persistent, precision, overstep)
        rng = np.random.default_rng(5)
        p, f = xgrid.Grid(shape, float), xgrid.Grid(shape, float)
        p.now[...] = rng.random(shape)
        f.now[...] = 1e-3 * rng.random(shape)
        m = np.zeros(shape, np.int32)
        m[0], m[-1] = 1, 1
        p.boundary[...] = m
        k(p, f, 9)
        k(p, f, 4)
        out[persistent] = np.array(p.now).copy()
        if persistent:
            assert k.native.loop_error() == 0
    assert out[True].tobytes() == out[False].tobytes()


def test_cavity_loop_matches_per_launch(cacheroot):
    out = {}
    for persistent in (True, False):
        xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, persistent=persistent)
        k = Operator(workloads.cavity_kernel.func, "kernel", "cavity_kernel")
        grids, cfg = workloads.cavity_setup(257, 1e-4)
        args = (grids["b"], grids["p"], grids["u"], grids["v"], cfg)
        for _ in range(5):
            k(*args)
        out[persistent] = {g: grids[g].read(0).copy() for g in "bpuv"}
        if persistent:
            assert k.native.loop_error() == 0
            assert _sites(k, lambda: k(*args)).count(LOOP_SITE) == 1
    for g in "bpuv":
        assert out[True][g].tobytes() == out[False][g].tobytes(), g


def test_cross_tile_boundary_read_falls_back(cacheroot):
    """Boundary cells at column 31 copy column 32, which lies in the next tile of
    32-column tiles: the persistent launch does not apply."""
    out = {}
    for persistent in (True, False):
        k = _kernel(xgrid, relax, cacheroot, persistent)
        p, f = _relax_grids(xgrid, (96, 96), 4, column=31)
        k(p, f, 5, 1e-3)
        k(p, f, 5, 1e-3)
        out[persistent] = np.array(p.now).copy()
        if persistent:
            assert LOOP_SITE not in _sites(k, lambda: k(p, f, 5, 1e-3))
    assert out[True].tobytes() == out[False].tobytes()
