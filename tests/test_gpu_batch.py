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
