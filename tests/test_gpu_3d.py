"""3-D sweeps against the numpy oracle (C-order semantics), bit for bit: the
z-walk path of mask-free tiles, the generic loops of tiles that hold masked
cells (per-row wrapped or clamped coordinates in edge tiles), periodic and
clamped edges, extents that are not multiples of any tile, FP64 and FP32."""
import numpy as np
import pytest

import xgrid
from oracle import xgrid_oracle
from xgrid_gb300.operator import Operator

pytestmark = pytest.mark.gpu


def vardiff(u: xgrid.grid[float, 3], k: xgrid.grid[float, 3], dt: float) -> None:
    u[0, 0, 0] = u[0, 0, 0] + dt * ((k[0, 0, 0] + k[1, 0, 0]) * (u[1, 0, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[-1, 0, 0]) * (u[-1, 0, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, 1, 0]) * (u[0, 1, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, -1, 0]) * (u[0, -1, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, 0, 1]) * (u[0, 0, 1] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, 0, -1]) * (u[0, 0, -1] - u[0, 0, 0]))
    with xgrid.boundary(1):
        u[0, 0, 0] = 0.5 * u[0, 0, 0]


def run(impl, overstep, precision, shape, steps, masked):
    impl.init(precision=precision, cacheroot=_CACHE[0], opt_level=3, overstep=overstep)
    k = Operator(vardiff, "kernel", f"vardiff_{overstep}_{precision}") if impl is xgrid else \
        xgrid_oracle.kernel()(vardiff)
    rng = np.random.default_rng(11)
    u, kk = impl.Grid(shape, float), impl.Grid(shape, float)
    u.now[...] = rng.random(shape)
    kk.now[...] = rng.uniform(0.01, 0.1, shape)
    if masked:
        u.boundary[5:9, 3:7, 10:12] = 1   # a few masked cells: their tiles take the generic loops
    for _ in range(steps):
        k(u, kk, 0.05)
    return np.array(u.now)


_CACHE = [None]


@pytest.mark.parametrize("overstep", ["wrap", "limit"])
@pytest.mark.parametrize("precision", ["double", "float"])
@pytest.mark.parametrize("masked", [False, True])
def test_3d_sweeps_match_the_oracle(cacheroot, overstep, precision, masked):
    _CACHE[0] = cacheroot
    shape = (37, 29, 45)
    gpu = run(xgrid, overstep, precision, shape, 4, masked)
    ref = run(xgrid_oracle, overstep, precision, shape, 4, masked)
    assert gpu.dtype == ref.dtype
    assert gpu.tobytes() == ref.tobytes()


def vardiff_plain(u: xgrid.grid[float, 3], k: xgrid.grid[float, 3], dt: float) -> None:
    # one sweep (no boundary phase), so every call launches the single-sweep path
    u[0, 0, 0] = u[0, 0, 0] + dt * ((k[0, 0, 0] + k[1, 0, 0]) * (u[1, 0, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[-1, 0, 0]) * (u[-1, 0, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, 1, 0]) * (u[0, 1, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, -1, 0]) * (u[0, -1, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, 0, 1]) * (u[0, 0, 1] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, 0, -1]) * (u[0, 0, -1] - u[0, 0, 0]))


@pytest.mark.parametrize("overstep", ["wrap", "limit"])
@pytest.mark.parametrize("precision", ["double", "float"])
@pytest.mark.parametrize("shape", [(70, 35, 131), (41, 37, 132), (20, 19, 256)])
def test_staged_and_register_zwalk_agree(cacheroot, overstep, precision, shape):
    """Mask-free 3-D grids take the staged z-walk (planes streamed through shared
    memory); the register z-walk computes the same bits, and both equal the
    oracle.  Extents span several 8 x 128 column blocks and z chunks: rows of 131
    cells take element copies; rows of 132 take 16-byte copies in the full block
    and element copies in the partial one; rows of 256 are two full blocks whose
    halo columns wrap or clamp.  The module's count of staged launches shows which
    path ran."""
    xgrid.init(precision=precision, cacheroot=cacheroot, opt_level=3, overstep=overstep)
    rng = np.random.default_rng(5)
    u0, k0 = rng.random(shape), rng.uniform(0.01, 0.1, shape)
    out = []
    for staged in (True, False):
        k = Operator(vardiff_plain, "kernel", f"vardiff_zs_{overstep}_{precision}_{shape[2]}_{int(staged)}")
        u, kk = xgrid.Grid(shape, float), xgrid.Grid(shape, float)
        u.now[...] = u0
        kk._extend_time(2)
        for lv in kk._data:
            lv[...] = k0
        k(u, kk, 0.05)  # compiles
        k.native.set_zstage(staged)
        before = k.native.zstage_launches()
        for _ in range(3):
            k(u, kk, 0.05)
        assert (k.native.zstage_launches() > before) == staged
        out.append(u.read(0))
    xgrid_oracle.init(precision=precision, cacheroot=cacheroot, opt_level=3, overstep=overstep)
    ko = xgrid_oracle.kernel()(vardiff_plain)
    u, kk = xgrid_oracle.Grid(shape, float), xgrid_oracle.Grid(shape, float)
    u.now[...] = u0
    kk._extend_time(2)
    for lv in kk._data:
        lv[...] = k0
    for _ in range(4):
        ko(u, kk, 0.05)
    ref = np.array(u.now)
    assert out[0].tobytes() == out[1].tobytes()
    assert out[0].tobytes() == ref.tobytes()
