"""Mixed-precision (FP32 defect + FP64 residual/correction) lowering of the
cavity's pressure iterations: error bound vs the plain FP64 path, fallback to
FP64 when the fused conditions fail, non-affine loops left untouched."""
import numpy as np
import pytest

import xgrid
import workloads
from xgrid_gb300.operator import Operator

pytestmark = pytest.mark.gpu


def _cavity(cacheroot, n, steps, dt, mixed, every=0):
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, mixed=mixed, mixed_every=every)
    k = Operator(workloads.cavity_kernel.func, "kernel", "cavity_kernel")
    grids, cfg = workloads.cavity_setup(n, dt)
    for _ in range(steps):
        k(grids["b"], grids["p"], grids["u"], grids["v"], cfg)
    return {g: grids[g].read(0) for g in "puv"}, k


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("every", [0, 7])
def test_mixed_cavity_within_1e8_of_fp64(cacheroot, every):
    ref, _ = _cavity(cacheroot, 257, 60, 1e-5, None)
    out, k = _cavity(cacheroot, 257, 60, 1e-5, "fp32", every)
    assert k.native.module.aux_per_cell == {1: 14}
    for g in "puv":
        assert np.isfinite(out[g]).all()
        assert _rel(out[g], ref[g]) < 1e-8, g
    assert out["p"].tobytes() != ref["p"].tobytes()  # the FP32 path really ran


@xgrid.kernel()
def relax(p: xgrid.grid[float, 2], f: xgrid.grid[float, 2], iters: int) -> None:
    for _ in range(0, iters):
        p[0, 0] = 0.25 * (p[1, 0][0] + p[-1, 0][0] + p[0, 1][0] + p[0, -1][0]) - 0.01 * f[0, 0][0]
        with xgrid.boundary(1):
            p[0, 0] = p[0, 1][0]
        with xgrid.boundary(2):
            p[0, 0] = 0.0


@xgrid.kernel()
def relax_nonlinear(p: xgrid.grid[float, 2], iters: int) -> None:
    for _ in range(0, iters):
        p[0, 0] = 0.25 * (p[1, 0][0] + p[-1, 0][0]) * p[0, 1][0]
        with xgrid.boundary(2):
            p[0, 0] = 0.0


def _relax_run(cacheroot, mixed, column, nonlinear=False):
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, mixed=mixed)
    fn = relax_nonlinear.func if nonlinear else relax.func
    k = Operator(fn, "kernel", fn.__name__)
    n = 96
    rng = np.random.default_rng(3)
    p = xgrid.Grid((n, n), float)
    f = xgrid.Grid((n, n), float)
    p.now[...] = rng.random((n, n))
    f.now[...] = rng.random((n, n))
    b = p.boundary
    b[:, column] = 1
    b[0, :] = b[-1, :] = b[:, -1] = 2
    if nonlinear:
        k(p, 12)
    else:
        k(p, f, 12)
    return p.read(0), k


def test_mixed_falls_back_when_boundary_reads_cross_tiles(cacheroot):
    # mask-1 cells in column 31 read column 32, which belongs to the next 32-wide tile
    ref, _ = _relax_run(cacheroot, None, 31)
    out, k = _relax_run(cacheroot, "fp32", 31)
    assert k.native.module.aux_per_cell == {0: 14}
    assert out.tobytes() == ref.tobytes()


def test_mixed_relax_within_tolerance(cacheroot):
    """Random initial field: the first defects are O(1), so the interior carries
    FP32-level error; boundary cells follow their FP64 rule exactly."""
    ref, _ = _relax_run(cacheroot, None, 0)
    out, _ = _relax_run(cacheroot, "fp32", 0)
    assert _rel(out, ref) < 1e-6
    assert out.tobytes() != ref.tobytes()
    assert (out[0, :] == 0.0).all() and (out[-1, :] == 0.0).all() and (out[:, -1] == 0.0).all()
    assert (out[1:-1, 0] == out[1:-1, 1]).all()


def test_nonaffine_loop_stays_fp64(cacheroot):
    ref, _ = _relax_run(cacheroot, None, 0, nonlinear=True)
    out, k = _relax_run(cacheroot, "fp32", 0, nonlinear=True)
    assert k.native.module.aux_per_cell == {}
    assert out.tobytes() == ref.tobytes()
