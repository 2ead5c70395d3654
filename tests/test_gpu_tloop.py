"""Several iterations of an in-place loop per launch (``loop_temporal``): the
pressure loop of the cavity program runs on shared-memory boxes with a halo of
``loop_temporal`` cells, recomputed every iteration.  Every level of every grid
equals the one-launch-per-iteration path bit for bit, for 2 to 4 iterations per
launch (50 iterations: launches of 2 and of a remainder), on seeded fields where
every cell is live, and the loop's launches are the box kernel's.  A loop whose
mask-0 cells read beyond the grid fails the box check and runs one launch per
iteration, with the same bits."""
import numpy as np
import pytest

import xgrid
import workloads
from xgrid_gb300 import device, runtime
from xgrid_gb300.operator import Operator

pytestmark = pytest.mark.gpu

TLOOP_SITE = 57


def _sites(k, call):
    """Profiling sites of the launches of one eager call."""
    lib = runtime.load()
    k.native.use_graph = False
    lib.xg_prof_reset()
    lib.xg_prof_enable(1)
    call()
    device.stream().synchronize()
    lib.xg_prof_enable(0)
    k.native.use_graph = True
    return [g for g, _ in runtime.prof_records()]


def _state(grids):
    return {g: (grids[g].read(0).tobytes(), grids[g].read(1).tobytes()) for g in "bpuv"}


@pytest.mark.parametrize("n,th,precision", [(257, 2, "double"), (257, 3, "double"), (257, 4, "double"),
                                             (1025, 2, "double"), (130, 3, "double"), (201, 3, "float")])
def test_boxes_give_the_bits_of_one_launch_per_iteration(cacheroot, n, th, precision):
    # the reference path: a module generated with one launch per iteration
    xgrid.init(precision=precision, cacheroot=cacheroot, opt_level=3, loop_temporal=0)
    single = Operator(workloads.cavity_kernel.func, "kernel", "cavity_kernel")
    gb, cfg = workloads.cavity_setup(n, 5e-6, seed=11)
    b = (gb["b"], gb["p"], gb["u"], gb["v"], cfg)
    single(*b)
    xgrid.init(precision=precision, cacheroot=cacheroot, opt_level=3, loop_temporal=th)
    boxed = Operator(workloads.cavity_kernel.func, "kernel", "cavity_kernel")
    ga, _ = workloads.cavity_setup(n, 5e-6, seed=11)
    a = (ga["b"], ga["p"], ga["u"], ga["v"], cfg)
    boxed(*a)
    sites = _sites(boxed, lambda: boxed(*a))
    single(*b)
    # 50 pressure iterations: ceil(50 / th) box launches of the pressure group
    assert sum(1 for s in sites if s % 64 == TLOOP_SITE) == -(-50 // th)
    for _ in range(3):
        boxed(*a)
        single(*b)
    assert _state(ga) == _state(gb)


def edge_read(p: xgrid.grid[float, 2], f: xgrid.grid[float, 2], iters: int) -> None:
    for _ in range(0, iters):
        p[0, 0] = 0.25 * (p[1, 0][0] + p[-1, 0][0] + p[0, 1][0] + p[0, -1][0]) - f[0, 0][0]
        with xgrid.boundary(1):
            p[0, 0] = 0.5 * p[1, 0][0]


def test_reads_beyond_the_grid_fall_back(cacheroot):
    """Mask-0 cells on the grid's faces read beyond it (zeros under overstep
    "none"): not provably exact on boxes, so one launch per iteration -- and the
    bits of that path."""
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, loop_temporal=2)
    shape = (70, 90)
    rng = np.random.default_rng(3)
    p0, f0 = rng.random(shape), rng.random(shape)
    m = np.zeros(shape, np.int32)
    m[30, 10:60] = 1
    out, sites = [], []
    for tl in (True, False):
        k = Operator(edge_read, "kernel", f"edge_read_{int(tl)}")
        p, f = xgrid.Grid(shape, float), xgrid.Grid(shape, float)
        p._extend_time(2)
        for lv in p._data:
            lv[...] = p0
        f.now[...] = f0
        p.boundary[...] = m
        k(p, f, 2)
        if not tl:
            k.native.set_tloop(False)
        sites.append(_sites(k, lambda: k(p, f, 9)))
        out.append(p.read(0))
    assert not any(s % 64 == TLOOP_SITE for s in sites[0])
    assert out[0].tobytes() == out[1].tobytes()


def plain_relax(p: xgrid.grid[float, 2], f: xgrid.grid[float, 2], iters: int) -> None:
    for _ in range(0, iters):
        p[0, 0] = 0.25 * (p[1, 0][0] + p[-1, 0][0] + p[0, 1][0] + p[0, -1][0]) - f[0, 0][0]


@pytest.mark.parametrize("iters", [7, 2, 1])
def test_loop_of_one_sweep_on_boxes(cacheroot, iters):
    """A loop of one Jacobi sweep (a frame of boundary cells that no sweep writes)
    runs on boxes too, with the bits of one launch per iteration, for iteration
    counts that leave remainders and for a single iteration (one plain launch)."""
    shape = (150, 211)
    rng = np.random.default_rng(8)
    p0, f0 = rng.random(shape), rng.random(shape)
    m = np.zeros(shape, np.int32)
    m[0, :] = m[-1, :] = m[:, 0] = m[:, -1] = 1
    out, sites = [], []
    for th in (3, 0):
        xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, loop_temporal=th)
        k = Operator(plain_relax, "kernel", "plain_relax")
        p, f = xgrid.Grid(shape, float), xgrid.Grid(shape, float)
        p._extend_time(2)
        for lv in p._data:
            lv[...] = p0
        f.now[...] = f0
        p.boundary[...] = m
        k(p, f, iters)
        sites.append(_sites(k, lambda: k(p, f, iters)))
        out.append(p.read(0))  # the kernel reads time level 0 only: one level
    boxed = sum(1 for s in sites[0] if s % 64 == TLOOP_SITE)
    assert boxed == (-(-iters // 3) if iters > 1 else 0)
    assert not any(s % 64 == TLOOP_SITE for s in sites[1])
    assert out[0].tobytes() == out[1].tobytes()
