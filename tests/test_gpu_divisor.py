"""Division by a launch-invariant divisor (precomputed reciprocal pair + one
Markstein correction) returns exactly the IEEE quotient: checked bit for bit
against the GPU's own ``/`` over random bit patterns (every exponent, zeros,
subnormals, infinities, NaN) and over values at the edges of the fast window."""
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
        bad = np.nonzero(a != b)[0]
        assert bad.size == 0, f"d={d!r}: {bad.size} mismatches, first x={x[bad[0]]!r}"
