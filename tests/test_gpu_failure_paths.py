"""The device-side waits that can give up do so without a hang or a fault, and
report it.  Modules compiled with ``xgrid.init(fail_waits=True)`` make those
waits unable to succeed: the neighbour-tile wait of a persistent loop launch
polls once, and the TMA staging barrier of the temporally blocked mixed-precision
kernel expects more bytes than its copies deliver.  Each call must return,
its error word must read 1 (``loop_error`` / ``staging_error``), clearing must
reset it, and afterwards a regular module on the same context must still give
the oracle's bits."""
import numpy as np
import pytest

import xgrid
import workloads
from oracle import xgrid_oracle
from xgrid_gb300 import device
from xgrid_gb300.operator import Operator

pytestmark = pytest.mark.gpu


def relax(p: xgrid.grid[float, 2], f: xgrid.grid[float, 2], iters: int, h2: float) -> None:
    for _ in range(0, iters):
        p[0, 0] = 0.25 * (p[1, 0][0] + p[-1, 0][0] + p[0, 1][0] + p[0, -1][0] - h2 * f[0, 0][0])
        with xgrid.boundary(1):
            p[0, 0] = p[0, 1][0]
        with xgrid.boundary(2):
            p[0, 0] = 0.5 * p[0, 0][0]


def _grids(impl, n, seed):
    rng = np.random.default_rng(seed)
    p, f = impl.Grid((n, n), float), impl.Grid((n, n), float)
    p.now[...] = rng.random((n, n))
    f.now[...] = rng.random((n, n)) - 0.5
    m = np.zeros((n, n), np.int32)
    m[:, 0] = 1
    m[0, :] = m[-1, :] = m[:, -1] = 2
    p.boundary[...] = m
    return p, f


def _context_still_usable(cacheroot):
    """A regular module after the failed calls: same bits as the oracle."""
    out = []
    for impl in (xgrid, xgrid_oracle):
        impl.init(precision="double", cacheroot=cacheroot, opt_level=3)
        k = Operator(relax, "kernel", "relax_after_failure") if impl is xgrid else impl.kernel()(relax)
        p, f = _grids(impl, 96, 4)
        k(p, f, 6, 1e-3)
        out.append(np.array(p.now).copy())
    assert out[0].tobytes() == out[1].tobytes()


def test_tile_wait_gives_up_and_reports(cacheroot):
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, persistent=True, fail_waits=True)
    k = Operator(relax, "kernel", "relax_fail_tile_wait")
    p, f = _grids(xgrid, 512, 3)
    k(p, f, 20, 1e-3)          # returns: a CTA leaves at its first neighbour wait that does not succeed
    device.synchronize()
    assert k.native.loop_error() == 1
    assert k.native.loop_error(clear=True) == 1
    assert k.native.loop_error() == 0
    _context_still_usable(cacheroot)


def test_tma_staging_wait_gives_up_and_reports(cacheroot):
    """One cavity step at 257^2 with the FP32 defect loop: 13 temporally blocked
    launches, each CTA waiting about a second for the bytes that never come."""
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, mixed="fp32", mixed_temporal=4,
               fail_waits=True)
    k = Operator(workloads.cavity_kernel.func, "kernel", "cavity_fail_tma")
    grids, cfg = workloads.cavity_setup(257, 1e-5, seed=3)
    k(grids["b"], grids["p"], grids["u"], grids["v"], cfg)
    device.synchronize()
    assert k.native.staging_error(grids["p"]) == 1
    assert k.native.staging_error(grids["p"], clear=True) == 1
    assert k.native.staging_error(grids["p"]) == 0
    _context_still_usable(cacheroot)
