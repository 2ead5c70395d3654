"""64-bit index kernels.  Every tile kernel is instantiated for 32-bit and
64-bit linear indices and the 64-bit one runs only for grids of 2^31 cells or
more, so (1) small grids are run through the 64-bit kernels as well (runtime
switch ``xg_force_wide_index``) and must give the same bits as the 32-bit ones —
explicit and implicit sweeps, fused boundary phases, edge tiles under every
overstep mode, the 3-D z-walk, the mixed-precision residual and correction —
and (2) one 2-D grid of 46341^2 > 2^31 cells runs three Jacobi iterations with
boundary phases, and its last rows (linear indices above 2^31) match the oracle
run on those rows."""
import numpy as np
import pytest

import xgrid
import workloads
from oracle import xgrid_oracle
from xgrid_gb300 import device, runtime
from xgrid_gb300.operator import Operator

pytestmark = pytest.mark.gpu


def relax(p: xgrid.grid[float, 2], f: xgrid.grid[float, 2], iters: int, h2: float) -> None:
    for _ in range(0, iters):
        p[0, 0] = 0.25 * (p[1, 0][0] + p[-1, 0][0] + p[0, 1][0] + p[0, -1][0] - h2 * f[0, 0][0])
        with xgrid.boundary(1):
            p[0, 0] = p[0, 1][0]
        with xgrid.boundary(2):
            p[0, 0] = 0.5 * p[0, 0][0]


def vardiff(u: xgrid.grid[float, 3], k: xgrid.grid[float, 3], dt: float) -> None:
    u[0, 0, 0] = u[0, 0, 0] + dt * ((k[0, 0, 0] + k[1, 0, 0]) * (u[1, 0, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[-1, 0, 0]) * (u[-1, 0, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, 1, 0]) * (u[0, 1, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, -1, 0]) * (u[0, -1, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, 0, 1]) * (u[0, 0, 1] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, 0, -1]) * (u[0, 0, -1] - u[0, 0, 0]))
    with xgrid.boundary(1):
        u[0, 0, 0] = 0.5 * u[0, 0, 0]


def _relax_run(cacheroot, shape, overstep):
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, overstep=overstep)
    k = Operator(relax, "kernel", f"relax_wide_{overstep}")
    rng = np.random.default_rng(1)
    p, f = xgrid.Grid(shape, float), xgrid.Grid(shape, float)
    p.now[...] = rng.random(shape)
    f.now[...] = rng.random(shape) - 0.5
    m = np.zeros(shape, np.int32)
    m[:, 0] = 1
    m[0, :] = m[-1, :] = m[:, -1] = 2
    p.boundary[...] = m
    for _ in range(3):
        k(p, f, 5, 1e-3)
    return [p.read(0)]


def _cavity_run(cacheroot, mode):
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, mixed=mode, mixed_temporal=0)
    k = Operator(workloads.cavity_kernel.func, "kernel", "cavity_kernel")
    grids, cfg = workloads.cavity_setup(129, 1e-4)
    for _ in range(4):
        k(grids["b"], grids["p"], grids["u"], grids["v"], cfg)
    return [grids[g].read(0) for g in "bpuv"]


def _vardiff_run(cacheroot, overstep, masked):
    xgrid.init(precision="float", cacheroot=cacheroot, opt_level=3, overstep=overstep)
    k = Operator(vardiff, "kernel", f"vardiff_wide_{overstep}")
    shape = (37, 29, 45)
    rng = np.random.default_rng(11)
    u, kk = xgrid.Grid(shape, float), xgrid.Grid(shape, float)
    u.now[...] = rng.random(shape)
    kk.now[...] = rng.uniform(0.01, 0.1, shape)
    if masked:
        u.boundary[5:9, 3:7, 10:12] = 1
    for _ in range(4):
        k(u, kk, 0.05)
    return [u.read(0)]


CASES = {
    "relax-none": lambda root: _relax_run(root, (67, 131), "none"),
    "relax-wrap": lambda root: _relax_run(root, (67, 131), "wrap"),
    "relax-limit": lambda root: _relax_run(root, (67, 131), "limit"),
    "cavity-plain": lambda root: _cavity_run(root, None),
    "cavity-mixed": lambda root: _cavity_run(root, "fp32"),
    "zwalk-wrap": lambda root: _vardiff_run(root, "wrap", False),
    "generic-3d-limit": lambda root: _vardiff_run(root, "limit", True),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_wide_index_kernels_give_the_same_bits(cacheroot, case):
    lib = runtime.load()
    out = {}
    try:
        for wide in (0, 1):
            lib.xg_force_wide_index(wide)
            lib.xg_graph_clear(None)
            out[wide] = CASES[case](cacheroot)
    finally:
        lib.xg_force_wide_index(0)
        lib.xg_graph_clear(None)
    for a, b in zip(out[0], out[1]):
        assert a.tobytes() == b.tobytes()


def test_grid_beyond_2_31_cells_matches_oracle_on_last_rows(cacheroot):
    """46341^2 FP32 cells (linear indices up to 2^31 + 4.6e6): three implicit
    Jacobi iterations with boundary phases; the oracle runs the last 16 rows (the
    three rows next to the cut see the cut, the other 13 are compared)."""
    import torch
    free, _ = torch.cuda.mem_get_info()
    if free < 80 * (1 << 30):
        pytest.skip("needs 80 GiB of free device memory")
    n = 46341
    assert n * n > 2 ** 31
    iters, rows = 3, 16
    xgrid.init(precision="float", cacheroot=cacheroot, opt_level=3)
    k = Operator(relax, "kernel", "relax_large")
    p, f = xgrid.Grid((n, n), float), xgrid.Grid((n, n), float)
    m = p.boundary
    m[:, 0] = 1
    m[0, :] = m[-1, :] = m[:, -1] = 2
    dev = torch.device("cuda")
    with torch.cuda.stream(device.stream()):
        y = torch.arange(n, device=dev, dtype=torch.float32)[:, None]
        x = torch.arange(n, device=dev, dtype=torch.float32)[None, :]
        p.tensor(0).copy_(torch.sin(y * 1e-3) * torch.cos(x * 7e-4))
        f.tensor(0).copy_(torch.cos(y * 3e-4 + x * 5e-4))
        del y, x
    device.stream().synchronize()
    p0 = p.tensor(0)[n - rows:].cpu().numpy().copy()
    f0 = f.tensor(0)[n - rows:].cpu().numpy().copy()
    mask_rows = np.ascontiguousarray(m[n - rows:])
    k(p, f, iters, 1e-3)
    device.stream().synchronize()
    got = p.tensor(0)[n - rows:].cpu().numpy()
    xgrid_oracle.init(precision="float", cacheroot=cacheroot, opt_level=3)
    ko = xgrid_oracle.kernel()(relax)
    po, fo = xgrid_oracle.Grid((rows, n), float), xgrid_oracle.Grid((rows, n), float)
    po.now[...] = p0
    fo.now[...] = f0
    po.boundary[...] = mask_rows
    ko(po, fo, iters, 1e-3)
    want = np.array(po.now)
    assert got[iters:].tobytes() == want[iters:].tobytes()
    del p, f
    torch.cuda.empty_cache()
