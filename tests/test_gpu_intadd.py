"""FP64 additions and subtractions that run on the integer pipe
(``xgrid.init(int_adds=n)``) return exactly the IEEE round-to-nearest result:
bit for bit against the GPU's FP64 unit and against numpy on the host, over
random bit patterns (every exponent, zeros, subnormals, infinities, NaN),
every exponent difference up to 70, near-total cancellation, exact ties, and
sums at the edges of the normal range.  A whole program (the cavity step)
gives the same bits with and without the integer-pipe additions."""
import numpy as np
import pytest

import xgrid
import workloads

pytestmark = pytest.mark.gpu


def _sum(q: xgrid.grid[float, 1], x: xgrid.grid[float, 1], y: xgrid.grid[float, 1]) -> None:
    q[0] = x[0][0] + y[0][0]


def _diff(q: xgrid.grid[float, 1], x: xgrid.grid[float, 1], y: xgrid.grid[float, 1]) -> None:
    q[0] = x[0][0] - y[0][0]


def _bits(rng, n):
    b = rng.integers(0, 2 ** 63, n, dtype=np.int64).view(np.uint64) | \
        (rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63))
    return b.view(np.float64)


def _sign(rng, n):
    return np.where(rng.random(n) < 0.5, -1.0, 1.0)


def pairs(rng, n):
    xs, ys = [_bits(rng, n)], [_bits(rng, n)]
    # every exponent difference 0..70, both signs, across the exponent range
    e = rng.integers(-1000, 1000, n)
    x = np.ldexp(rng.random(n) + 1.0, e) * _sign(rng, n)
    y = np.ldexp(rng.random(n) + 1.0, e - rng.integers(0, 71, n)) * _sign(rng, n)
    xs += [x, y]
    ys += [y, x]
    # near-total cancellation: y = -(x +- a few ulps)
    k = rng.integers(-6, 7, n)
    xs.append(x)
    ys.append(-(x.view(np.int64) + k).view(np.float64))
    # exact ties and near ties: y = m * 2^(E - 52 - j), E the exponent of x
    E = np.floor(np.log2(np.abs(x))).astype(np.int64)
    m = rng.integers(1, 8, n).astype(np.float64)
    j = rng.integers(1, 4, n)
    xs.append(x)
    ys.append(np.ldexp(m, E - 52 - j) * _sign(rng, n))
    # edges of the normal range: sums that overflow, differences that turn subnormal
    big = np.ldexp(rng.random(n) + 1.0, 1023) * _sign(rng, n)
    xs += [big, np.ldexp(rng.random(n) + 1.0, -1021)]
    ys += [big * (rng.random(n) * 0.5 + 0.5), -np.ldexp(rng.random(n) + 1.0, -1021 - rng.integers(0, 3, n))]
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                        -2.2250738585072014e-308, 1.7976931348623157e308, -1.7976931348623157e308, 1.0, -1.0])
    sx, sy = np.meshgrid(special, special)
    xs.append(sx.ravel())
    ys.append(sy.ravel())
    return np.concatenate(xs), np.concatenate(ys)


@pytest.mark.parametrize("seed", [0, 1])
def test_integer_pipe_addition_is_ieee(cacheroot, seed):
    rng = np.random.default_rng(seed)
    x, y = pairs(rng, 1 << 19)
    n = x.size
    outs = {}
    for every in (0, 1):
        xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, int_adds=every)
        res = []
        for fn in (_sum, _diff):
            k = xgrid.kernel(name=f"{fn.__name__.strip('_')}_{every}")(fn)
            q, xs, ys = (xgrid.Grid((n,), float) for _ in range(3))
            xs.now[...] = x
            ys.now[...] = y
            k(q, xs, ys)
            res.append(q.read(0).view(np.uint64).copy())
        outs[every] = res
        if every:
            assert "xg_dadd_i(" in k.native.module.source or "xg_dsub_i(" in k.native.module.source
    with np.errstate(all="ignore"):
        host = [(x + y).view(np.uint64), (x - y).view(np.uint64)]
    for op, soft, hard, ref in zip("+-", outs[1], outs[0], host):
        nan = np.isnan(soft.view(np.float64)) & np.isnan(hard.view(np.float64))
        bad = np.nonzero((soft != hard) & ~nan)[0]
        assert bad.size == 0, f"x {op} y: {bad.size} differ from the FP64 unit, first {x[bad[0]]!r}, {y[bad[0]]!r}"
        nan = np.isnan(soft.view(np.float64)) & np.isnan(ref.view(np.float64))
        bad = np.nonzero((soft != ref) & ~nan)[0]
        assert bad.size == 0, f"x {op} y: {bad.size} differ from numpy, first {x[bad[0]]!r}, {y[bad[0]]!r}"


@pytest.mark.parametrize("every", [1, 2, 3])
def test_cavity_bits_do_not_depend_on_the_pipe(cacheroot, every):
    out = {}
    for ia in (0, every):
        xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, int_adds=ia)
        k = xgrid.kernel(name=f"cavity_ia{ia}")(workloads.cavity_kernel.func)
        grids, cfg = workloads.cavity_setup(129, 1e-4)
        for _ in range(5):
            k(grids["b"], grids["p"], grids["u"], grids["v"], cfg)
        out[ia] = {g: grids[g].read(0).tobytes() for g in "bpuv"}
    assert out[0] == out[every]
