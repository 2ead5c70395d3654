"""Division by a launch-invariant divisor (precomputed reciprocal pair + one
Markstein correction; exponent arithmetic for a power of two) and
multiplication by a launch-invariant power of two return exactly the IEEE
result: checked bit for bit against the GPU's own ``/`` and ``*`` and against
numpy on the host, over random bit patterns (every exponent, zeros, subnormals,
infinities, NaN) and over values at the edges of the fast paths."""
import numpy as np
import pytest

import xgrid

pytestmark = pytest.mark.gpu


def _quotient(q: xgrid.grid[float, 1], x: xgrid.grid[float, 1], d: float) -> None:
    q[0] = x[0][0] / d


DIVISORS = [2.0 * (2.0 / 1024), 2.0 * ((2.0 / 1024) ** 2 + (2.0 / 1024) ** 2), 2.0 / 1024, 1e-5 / (2.0 / 1024),
            3.0, -7.25, 1.0, 0.1, np.nextafter(2.0, 3.0), np.nextafter(2.0, 1.0), 2.0 ** -1000, 2.0 ** 1000,
            -2.0 ** -1021, 1.7976931348623157e308, 5e-324, 0.0, np.inf]


def _inputs(rng, n):
    bits = rng.integers(0, 2 ** 63, n, dtype=np.int64).view(np.uint64) | \
        (rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63))
    raw = bits.view(np.float64)
    mant = rng.random(n) + 1.0
    exps = rng.integers(-1074, 1024, n)
    spread = np.ldexp(mant, exps) * np.where(rng.random(n) < 0.5, -1.0, 1.0)
    edges = []
    for d in DIVISORS:
        if d == 0 or not np.isfinite(d) or abs(d) < 2.0 ** -1022:
            continue
        ed = int(np.floor(np.log2(abs(d))))
        for e in (-900 + max(ed, 0), 1000 + ed, 1023):
            for k in (-2, -1, 0, 1):
                edges.append(np.ldexp(1.0 + rng.random(64), e + k))
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                        1.7976931348623157e308, 1.0, -1.0])
    x = np.concatenate([raw, spread, np.concatenate(edges), special])
    return x


@pytest.mark.parametrize("seed", [0, 1])
def test_divisor_path_equals_ieee_division(cacheroot, seed):
    rng = np.random.default_rng(seed)
    x = _inputs(rng, 1 << 21)
    n = x.size
    outs = {}
    for divisor in (True, False):
        xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, divisor=divisor)
        k = xgrid.kernel(name=f"quotient_{int(divisor)}")(_quotient)
        q = xgrid.Grid((n,), float)
        xs = xgrid.Grid((n,), float)
        xs.now[...] = x
        res = []
        for d in DIVISORS:
            k(q, xs, float(d))
            res.append(q.read(0).view(np.uint64).copy())
        outs[divisor] = res
    for d, a, b in zip(DIVISORS, outs[True], outs[False]):
        nan = np.isnan(a.view(np.float64)) & np.isnan(b.view(np.float64))
        bad = np.nonzero((a != b) & ~nan)[0]
        assert bad.size == 0, f"d={d!r}: {bad.size} mismatches, first x={x[bad[0]]!r}"
    # every quotient also equals numpy's IEEE division on the host (NaN payloads aside)
    for d, a in zip(DIVISORS, outs[True]):
        with np.errstate(all="ignore"):
            ref = (x / d).view(np.uint64)
        nan = np.isnan(a.view(np.float64)) & np.isnan(ref.view(np.float64))
        assert np.all((a == ref) | nan), f"d={d!r} differs from the host quotient"


def _product(q: xgrid.grid[float, 1], x: xgrid.grid[float, 1], m: float) -> None:
    q[0] = x[0][0] * m


MULTIPLIERS = [2.0 ** -18, 2.0 ** -20, -8.0, 1.0, -1.0, 2.0 ** 1000, 2.0 ** -1000, 2.0 ** -1022, 2.0 ** 1023,
               -2.0 ** -1022, 0.75, 3.0, 5e-324, 0.0, np.inf, np.nan, 2.0 ** 16]


def test_power_of_two_scaling_equals_ieee_product(cacheroot):
    """x * m with m = +-2^s is done by exponent arithmetic (FP64 multiply only at
    the edges of the normal range): bit-identical to the IEEE product for every
    input, including results that turn subnormal, overflow, zeros and NaN."""
    rng = np.random.default_rng(7)
    x = _inputs(rng, 1 << 20)
    edges = []
    for m in MULTIPLIERS:
        if m == 0 or not np.isfinite(m) or abs(m) < 2.0 ** -1022:
            continue
        s = int(np.floor(np.log2(abs(m))))
        for e in (-1075, -1074, -1023, -1022, -1021, 1022, 1023, 1024):
            for k in (-1, 0, 1):
                ex = e - s + k
                if -1074 <= ex <= 1023:
                    edges.append(np.ldexp(1.0 + rng.random(32), ex) * rng.choice([-1.0, 1.0], 32))
    x = np.concatenate([x, np.concatenate(edges)])
    n = x.size
    outs = {}
    for divisor in (True, False):
        xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, divisor=divisor)
        k = xgrid.kernel(name=f"product_{int(divisor)}")(_product)
        q = xgrid.Grid((n,), float)
        xs = xgrid.Grid((n,), float)
        xs.now[...] = x
        res = []
        for m in MULTIPLIERS:
            k(q, xs, float(m))
            res.append(q.read(0).view(np.uint64).copy())
        outs[divisor] = res
    for m, a, b in zip(MULTIPLIERS, outs[True], outs[False]):
        nan = np.isnan(a.view(np.float64)) & np.isnan(b.view(np.float64))
        bad = np.nonzero((a != b) & ~nan)[0]
        assert bad.size == 0, f"m={m!r}: {bad.size} mismatches, first x={x[bad[0]]!r}"
    # the scaled path must also agree with numpy's IEEE product (host reference)
    for m, a in zip(MULTIPLIERS, outs[True]):
        with np.errstate(all="ignore"):
            ref = (x * m).view(np.uint64)
        nan = np.isnan(a.view(np.float64)) & np.isnan(ref.view(np.float64))
        assert np.all((a == ref) | nan), f"m={m!r} differs from the host product"
