"""Temporally blocked defect iterations of the mixed-precision pressure loop
(TMA-staged boxes, several iterations per launch).  With FP32 storage the
result has the same bits as one iteration per launch, for every depth and
box height (rows per warp), on square and non-square grids with odd extents; with 16-bit
storage (FP16 / BF16 and a power-of-two scale per field) the pressure stays
within the storage format's tolerance of the FP64 path.  The staging copies
never time out (error word of the work area stays 0)."""
import numpy as np
import pytest

import xgrid
import workloads
from xgrid_gb300 import device, mixed, runtime
from xgrid_gb300.operator import Operator

pytestmark = pytest.mark.gpu


def cavity_grids(ny, nx, dt):
    """Lid-driven cavity on ny x nx points (masks as in the cavity example)."""
    grids = {k: xgrid.Grid((ny, nx), float) for k in "bpuv"}
    m = {k: np.zeros((ny, nx), np.int32) for k in "bpuv"}
    m["u"][0, :] = 1
    m["u"][:, 0] = 1
    m["u"][:, -1] = 1
    m["u"][-1, :] = 2
    m["v"].fill(1)
    m["v"][1:-1, 1:-1] = 0
    m["p"][:, -1] = 1
    m["p"][0, :] = 2
    m["p"][:, 0] = 3
    m["p"][-1, :] = 4
    m["b"].fill(1)
    m["b"][1:-1, 1:-1] = 0
    for k in "bpuv":
        grids[k].boundary[...] = m[k]
    return grids, workloads.Config(1.0, 0.1, dt, 2.0 / (nx - 1), 2.0 / (ny - 1))


def kernel(cacheroot, mode):
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, mixed=mode)
    return Operator(workloads.cavity_kernel.func, "kernel", "cavity_kernel")


def run(k, shape, steps, temporal, rows=8, dt=1e-5):
    if k.native is None:
        from xgrid_gb300.native import NativeKernel
        k.native = NativeKernel(k)
    k.native.set_mixed_temporal(temporal, rows)
    grids, cfg = cavity_grids(*shape, dt)
    lib = runtime.load()
    lib.xg_prof_reset()
    for _ in range(steps):
        k(grids["b"], grids["p"], grids["u"], grids["v"], cfg)
    launches = lib.xg_prof_launches()
    out = {g: grids[g].read(0) for g in "puv"}
    device.stream().synchronize()
    word = int(grids["p"]._aux[mixed.aux_error_offset(grids["p"].shape):][:4].cpu().numpy().view(np.int32)[0])
    return out, launches, word


@pytest.mark.parametrize("shape", [(257, 257), (203, 333)])
@pytest.mark.parametrize("temporal,rows", [(4, 8), (3, 4), (1, 8), (6, 8), (8, 4), (8, 8)])
def test_fp32_temporal_equals_one_iteration_per_launch(cacheroot, shape, temporal, rows):
    k = kernel(cacheroot, "fp32")
    ref, n_ref, _ = run(k, shape, 6, 0)
    out, n_tb, word = run(k, shape, 6, temporal, rows)
    for g in "puv":
        bad = np.argwhere(out[g] != ref[g])
        assert bad.size == 0, (f"{g}: {len(bad)} cells differ, first {bad[:6].tolist()}, largest "
                               f"{np.abs(out[g] - ref[g]).max():.3e} (field max {np.abs(ref[g]).max():.3e}), "
                               f"staging error word {word}")
    assert word == 0
    # 49 defect launches per step become ceil(49 / temporal)
    assert n_tb < n_ref or temporal == 1


@pytest.mark.parametrize("mode,tol", [("fp16", 1e-5), ("bf16", 5e-5)])
def test_16bit_storage_within_tolerance_of_fp64(cacheroot, mode, tol):
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3)
    k64 = Operator(workloads.cavity_kernel.func, "kernel", "cavity_kernel")
    grids, cfg = cavity_grids(257, 257, 1e-5)
    for _ in range(30):
        k64(grids["b"], grids["p"], grids["u"], grids["v"], cfg)
    ref = {g: grids[g].read(0) for g in "puv"}
    k = kernel(cacheroot, mode)
    out, _, word = run(k, (257, 257), 30, 4)
    assert word == 0
    errs = {}
    for g in "puv":
        assert np.isfinite(out[g]).all(), g
        errs[g] = float(np.abs(out[g] - ref[g]).max() / np.abs(ref[g]).max())
    assert errs["p"] < tol, errs
    assert errs["u"] < tol and errs["v"] < tol, errs
    assert out["p"].tobytes() != ref["p"].tobytes()
    # boundary cells keep their FP64 rule exactly: copies of their neighbours, zero on the bottom row
    p = out["p"]
    assert (p[-1, :] == 0.0).all()
    assert (p[1:-1, -1] == p[1:-1, -2]).all() and (p[1:-1, 0] == p[1:-1, 1]).all()


@xgrid.kernel()
def relax_column(p: xgrid.grid[float, 2], f: xgrid.grid[float, 2], iters: int) -> None:
    for _ in range(0, iters):
        p[0, 0] = 0.25 * (p[1, 0][0] + p[-1, 0][0] + p[0, 1][0] + p[0, -1][0]) - 0.01 * f[0, 0][0]
        with xgrid.boundary(1):
            p[0, 0] = p[0, 1][0]
        with xgrid.boundary(2):
            p[0, 0] = 0.0


@pytest.mark.parametrize("column,temporal_used", [(60, True), (118, True), (122, False)])
def test_box_check_accepts_and_rejects(cacheroot, column, temporal_used):
    """A column of boundary cells that copies its right neighbour: deep inside a box
    (60), and at the last columns of the first tile (118: FP32 boxes are 128 columns
    with a halo of 4, tiles 120 wide) the temporal path runs; at column 122 (two
    columns from the first box's inner edge at 124) the copy would read a stale
    cell, the check refuses and the loop runs one iteration per launch.  Same bits
    either way."""
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, mixed="fp32")
    k = Operator(relax_column.func, "kernel", "relax_column")
    from xgrid_gb300.native import NativeKernel
    k.native = NativeKernel(k)
    lib = runtime.load()
    out, launches = {}, {}
    for T in (0, 4):
        k.native.set_mixed_temporal(T, 8)
        rng = np.random.default_rng(7)
        p, f = xgrid.Grid((300, 300), float), xgrid.Grid((300, 300), float)
        p.now[...] = rng.random((300, 300))
        f.now[...] = rng.random((300, 300))
        b = p.boundary
        b[1:-1, column] = 1
        b[0, :] = b[-1, :] = b[:, 0] = b[:, -1] = 2
        lib.xg_prof_reset()
        k(p, f, 30)
        launches[T] = lib.xg_prof_launches()
        out[T] = p.read(0)
    assert out[0].tobytes() == out[4].tobytes()
    assert (launches[4] < launches[0]) == temporal_used, launches
