"""Batched persistent execution of many independent problems of uneven size:
identical bits to one call per problem per step, and to the numpy oracle's
C-order semantics for non-square periodic grids."""
import numpy as np
import pytest

import xgrid
import workloads
from oracle import xgrid_oracle
from xgrid_gb300.operator import Operator

pytestmark = pytest.mark.gpu


def _problems(seed, count, lo, hi):
    return workloads.batch_setup(count, seed, lo, hi)


@pytest.mark.parametrize("steps", [1, 6, 7])
def test_batch_equals_sequential_calls(cacheroot, steps):
    xgrid.init(precision="float", cacheroot=cacheroot, opt_level=3, overstep="wrap")
    kb = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    ks = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    a = _problems(3, 12, 17, 150)
    b = _problems(3, 12, 17, 150)
    kb.batch(a, steps)
    for _ in range(steps):
        for args in b:
            ks(*args)
    for pa, pb in zip(a, b):
        assert pa[0].read(0).tobytes() == pb[0].read(0).tobytes()
        assert pa[0].read(1).tobytes() == pb[0].read(1).tobytes()


def test_batch_matches_oracle_nonsquare(cacheroot):
    xgrid.init(precision="float", cacheroot=cacheroot, opt_level=3, overstep="wrap")
    kb = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    probs = _problems(5, 6, 9, 70)
    init = [p[0].read(0) for p in probs]
    kb.batch(probs, 5)
    xgrid_oracle.init(precision="float", cacheroot=cacheroot, opt_level=3, overstep="wrap")
    ko = xgrid_oracle.kernel()(workloads.convdiff2d.func)
    for p, u0 in zip(probs, init):
        g = xgrid_oracle.Grid(u0.shape, float)
        g.now[...] = u0
        for _ in range(5):
            ko(g, *p[1:])
        assert p[0].read(0).tobytes() == g.now.tobytes()


def test_batch_graph_replay_across_calls(cacheroot):
    xgrid.init(precision="float", cacheroot=cacheroot, opt_level=3, overstep="wrap")
    kb = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    ks = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    a = _problems(8, 10, 30, 90)
    b = _problems(8, 10, 30, 90)
    for _ in range(4):  # eager, capture, replay, replay
        kb.batch(a, 3)
    for _ in range(12):
        for args in b:
            ks(*args)
    for pa, pb in zip(a, b):
        assert pa[0].read(0).tobytes() == pb[0].read(0).tobytes()


# ------------------------------------------------------ temporal blocking
def coupled2d(u: xgrid.grid[float, 2], v: xgrid.grid[float, 2], a: float, b: float) -> None:
    u[0, 0] = u[0, 0] + a * (v[0, 1] - v[0, -1]) + b * (v[1, 1] - u[0, 0])
    v[0, 0] = v[0, 0] + b * (u[1, 0] - u[-1, 0]) + a * (u[-1, -1] - v[0, 0])


def heat1d(u: xgrid.grid[float, 1], c: float) -> None:
    u[0] = u[0] + c * (u[-1] + u[1] - u[0] - u[0])


def _sequential(k, problems, steps):
    for _ in range(steps):
        for args in problems:
            k(*args)


def _same_levels(a, b, grids_per_problem=1):
    for pa, pb in zip(a, b):
        for i in range(grids_per_problem):
            for lvl in (0, 1):
                assert pa[i].read(lvl).tobytes() == pb[i].read(lvl).tobytes()


@pytest.mark.parametrize("temporal,steps", [((2, 8, 16), 2), ((3, 16, 40), 7), ((4, 32, 56), 9),
                                             ((8, 16, 48), 20), ((4, 32, 56), 1000 // 125)])
def test_temporal_blocking_equals_sequential_calls(cacheroot, temporal, steps):
    xgrid.init(precision="float", cacheroot=cacheroot, opt_level=3, overstep="wrap")
    kb = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    ks = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    a = _problems(11, 14, 9, 140)
    b = _problems(11, 14, 9, 140)
    kb.batch(a, steps, temporal=temporal)
    assert kb.native.temporal_supported()
    _sequential(ks, b, steps)
    _same_levels(a, b)


def test_temporal_blocking_replays_and_alternates(cacheroot):
    """Several calls in a row (eager, graph capture, replays) with odd and even
    step counts: the levels end where the ticks leave them every time."""
    xgrid.init(precision="float", cacheroot=cacheroot, opt_level=3, overstep="wrap")
    kb = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    ks = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    a = _problems(12, 9, 20, 100)
    b = _problems(12, 9, 20, 100)
    total = 0
    for steps in (5, 5, 6, 5, 5, 2):
        kb.batch(a, steps, temporal=(4, 16, 24))
        total += steps
    _sequential(ks, b, total)
    _same_levels(a, b)


def test_temporal_blocking_two_fields_and_one_dimension(cacheroot):
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, overstep="wrap")
    kb = Operator(coupled2d, "kernel", "coupled2d")
    ks = Operator(coupled2d, "kernel", "coupled2d")
    rng = np.random.default_rng(4)

    def make(rng):
        out = []
        for _ in range(5):
            ny, nx = (int(v) for v in rng.integers(12, 80, 2))
            u, v = xgrid.Grid((ny, nx), float), xgrid.Grid((ny, nx), float)
            u.now[...] = rng.random((ny, nx))
            v.now[...] = rng.random((ny, nx))
            out.append((u, v, float(rng.uniform(0.01, 0.1)), float(rng.uniform(0.01, 0.1))))
        return out
    a, b = make(np.random.default_rng(4)), make(np.random.default_rng(4))
    kb.batch(a, 11, temporal=(3, 16, 32))
    assert kb.native.temporal_supported()
    _sequential(ks, b, 11)
    _same_levels(a, b, 2)

    k1 = Operator(heat1d, "kernel", "heat1d")
    k2 = Operator(heat1d, "kernel", "heat1d")

    def make1(rng):
        out = []
        for _ in range(6):
            n = int(rng.integers(20, 3000))
            u = xgrid.Grid((n,), float)
            u.now[...] = rng.random(n)
            out.append((u, 0.2))
        return out
    a, b = make1(np.random.default_rng(5)), make1(np.random.default_rng(5))
    k1.batch(a, 13, temporal=(5, 1, 256))
    _sequential(k2, b, 13)
    _same_levels(a, b)


def test_temporal_blocking_falls_back_for_masks_and_small_extents(cacheroot):
    """A nonzero mask cell or a halo wider than a problem turns temporal blocking
    off for the call; the one-step-per-launch kernel gives the same bits."""
    xgrid.init(precision="float", cacheroot=cacheroot, opt_level=3, overstep="wrap")
    kb = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    ks = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    a = _problems(13, 4, 30, 60)
    b = _problems(13, 4, 30, 60)
    for p in (a[1], b[1]):
        p[0].boundary[3, 4] = 1
    kb.batch(a, 6, temporal=(4, 16, 32))
    _sequential(ks, b, 6)
    _same_levels(a, b)
    a = _problems(14, 3, 5, 12)
    b = _problems(14, 3, 5, 12)
    kb.batch(a, 9, temporal=(8, 8, 8))   # halo 8 > extents of 5..7
    _sequential(ks, b, 9)
    _same_levels(a, b)


def test_temporal_configurations_in_any_order(cacheroot):
    """Configurations of different shared-memory sizes, one after the other and
    each replayed from its CUDA graph: a larger tile after a smaller one (same
    depth and tile, other CTA shape) still launches and gives the same bits."""
    xgrid.init(precision="float", cacheroot=cacheroot, opt_level=3, overstep="wrap")
    kb = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    ks = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    a = _problems(15, 8, 70, 200)
    b = _problems(15, 8, 70, 200)
    total = 0
    for cfg in ((2, 32, 124, (32, 8, 1)), (2, 64, 60, (32, 8, 1)), (2, 32, 124, (64, 4, 1)),
                (2, 32, 124, (32, 8, 1))):
        for _ in range(3):  # eager, capture, replay
            kb.batch(a, 4, temporal=cfg)
            total += 4
    _sequential(ks, b, total)
    _same_levels(a, b)
