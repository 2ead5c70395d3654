"""Slab decomposition on the GPU with one rank: the kernel runs on the slab's
local grids (the grid's rows plus halo rows marked with ``HALO_MASK``), one
launch per sweep with the launch hook refreshing the halo rows (zeros at the
faces under overstep none, the opposite face under wrap), and gives the bits of
the one-grid path on every level of every grid.  Two or more ranks are
exercised on the CPU (tests/test_slab.py)."""
import numpy as np
import pytest

import xgrid
import workloads
from xgrid_gb300 import slab
from xgrid_gb300.operator import Operator

pytestmark = pytest.mark.gpu


def _grids(fields, plan=None):
    out = {}
    for name, (l0, l1, mask) in fields.items():
        g = xgrid.Grid(plan.local_shape if plan else l0.shape, float)
        g._extend_time(2)
        for lv, x in enumerate((l0, l1)):
            g._data[lv][...] = (plan.local_field(x) if plan else x).astype(g.numpy_dtype)
        g.boundary[...] = plan.local_mask(mask) if plan else mask
        out[name] = g
    return out


@pytest.mark.parametrize("case", ["cavity", "convdiff"])
def test_one_rank_slab_equals_the_whole_grid(cacheroot, case):
    if case == "cavity":
        n = 129
        st = workloads.cavity_state(n, 9)
        masks = workloads.cavity_masks(n)
        fields = {k: (st[k][0], st[k][1], masks[k]) for k in "bpuv"}
        cfg = workloads.Config(1.0, 0.1, 1e-5, 2.0 / (n - 1), 2.0 / (n - 1))
        fn, overstep, precision, steps = workloads.cavity_kernel.func, "none", "double", 4
        build = lambda g: (g["b"], g["p"], g["u"], g["v"], cfg)  # noqa: E731
    else:
        u0 = np.random.default_rng(3).random((40, 33))
        fields = {"u": (u0, np.zeros_like(u0), np.zeros(u0.shape, np.int32))}
        fn, overstep, precision, steps = workloads.convdiff2d.func, "wrap", "float", 6
        build = lambda g: (g["u"], 0.6, 0.09, 0.11, 0.1, 0.1)  # noqa: E731
    xgrid.init(precision=precision, cacheroot=cacheroot, opt_level=3, overstep=overstep)
    whole_k = Operator(fn, "kernel", f"{fn.__name__}_whole")
    whole = _grids(fields)
    for _ in range(steps):
        whole_k(*build(whole))
    shape = next(iter(fields.values()))[0].shape
    plan = slab.SlabPlan(shape, 1, 0, 1, overstep)
    sk = slab.SlabKernel(Operator(fn, "kernel", f"{fn.__name__}_slab"), plan)
    local = _grids(fields, plan)
    for _ in range(steps):
        sk(*build(local))
    for name in fields:
        for lv in range(2):
            got = local[name].read(lv)[plan.interior]
            assert got.tobytes() == whole[name].read(lv).tobytes(), f"{case}: {name} level {lv}"
