"""Small DSL programs run on three implementations of the ``xgrid`` API.

This module is executed with a global ``xgrid`` injected by the loader (see
``load_cases``): the reference package when ``make_golden.py`` records golden
vectors, the numpy oracle in the CPU tests, and the GPU backend in the GPU
tests.  ``CACHEROOT`` is injected the same way.  Every case returns a dict of
numpy arrays (grids as all their time levels stacked) and only uses inputs that
the reference handles correctly: square 2-D grids, 1-D grids, and reads that
stay inside the grid.
"""
import dataclasses
from typing import cast

import numpy as np

TEMP = 10
CASES = {}


def case(fn):
    CASES[fn.__name__] = fn
    return fn


def levels(g):
    return np.stack([np.array(x) for x in g._data])


# ------------------------------------------------------------- reference tests
@case
def int_const():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")

    @xgrid.kernel()
    def aux(a: xgrid.grid[int, 2]) -> None:
        a[0, 0] = 4

    g = xgrid.Grid((10, 10), int)
    aux(g)
    return {"a": levels(g)}


@case
def scalar_add():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")

    @xgrid.kernel()
    def aux(a: int, b: int) -> int:
        return a + b + TEMP

    pairs = [(0, 0), (3, 4), (999, 1), (-5, 2)]
    return {"r": np.array([aux(a, b) for a, b in pairs], dtype=np.int64)}


@dataclasses.dataclass
class Vector3i:
    x: int
    y: int
    z: int

    @xgrid.function(method=True)
    def dot(self, b: "Vector3i") -> int:
        return self.x * b.x + self.y * b.y + self.z * b.z


@case
def struct_dot():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")

    @xgrid.kernel()
    def aux(a: Vector3i, b: Vector3i) -> int:
        return a.dot(b)

    rng = np.random.default_rng(5)
    out = []
    for _ in range(4):
        a = Vector3i(*[int(v) for v in rng.integers(0, 1000, 3)])
        b = Vector3i(*[int(v) for v in rng.integers(0, 1000, 3)])
        out.append(aux(a, b))
    return {"r": np.array(out, dtype=np.int64)}


# ----------------------------------------------------------------- physics 1-D
def _step_1d(nx, dx):
    u0 = np.ones(nx)
    u0[int(.5 / dx):int(1 / dx + 1)] = 2
    return u0


@case
def convection_1d():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")
    nx, nt, dt, c = 41, 25, .025, 1.0
    dx = 2 / (nx - 1)
    u = xgrid.Grid((nx,), float)
    u.now[:] = _step_1d(nx, dx)
    u.boundary[0] = 1

    @xgrid.kernel()
    def conv(u: xgrid.grid[float, 1], c: float, dt: float, dx: float) -> None:
        u[0] = u[0] - c * dt / dx * (u[0] - u[-1])
        with xgrid.boundary(1):
            u[0] = 1.0

    for _ in range(nt):
        conv(u, c, dt, dx)
    return {"u": levels(u)}


@case
def convection_1d_nonlinear():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")
    nx, nt, dt = 41, 10, .025
    dx = 2 / (nx - 1)
    u = xgrid.Grid((nx,), float)
    u.now[:] = _step_1d(nx, dx)
    u.boundary[0] = 1

    @xgrid.kernel()
    def conv(u: xgrid.grid[float, 1], dt: float, dx: float) -> None:
        u[0] = u[0] - u[0] * dt / dx * (u[0] - u[-1])
        with xgrid.boundary(1):
            u[0] = 1.0

    for _ in range(nt):
        conv(u, dt, dx)
    return {"u": levels(u)}


@case
def diffusion_1d():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")
    nx, nt, dt, nu = 41, 20, .01, 0.01
    dx = 2 / (nx - 1)
    u = xgrid.Grid((nx,), float)
    u.now[:] = _step_1d(nx, dx)
    u.boundary[0] = 1
    u.boundary[-1] = 1

    @xgrid.kernel()
    def diff(u: xgrid.grid[float, 1], nu: float, dt: float, dx: float) -> None:
        u[0] = u[0] + nu * dt / dx ** 2.0 * (u[1] - 2.0 * u[0] + u[-1])
        with xgrid.boundary(1):
            u[0] = 1.0

    for _ in range(nt):
        diff(u, nu, dt, dx)
    return {"u": levels(u)}


@case
def convection_2d():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")
    n = 41
    dx = dy = 2 / (n - 1)
    c, sigma = 1.0, .5
    dt = sigma * (dx / c)
    u = xgrid.Grid((n, n), float)
    u0 = np.ones((n, n))
    u0[int(0.5 / dx):int(1 / dx) + 1, int(0.5 / dy):int(1 / dy) + 1] = 2
    u.now[...] = u0
    u.boundary[0, :] = 1
    u.boundary[:, 0] = 1

    @xgrid.kernel()
    def conv(u: xgrid.grid[float, 2], c: float, dt: float, dx: float, dy: float) -> None:
        cdx = c * dt / dx
        cdy = c * dt / dy
        u[0, 0] = u[0, 0] + cdx * (u[0, 0] - u[-1, 0]) - cdy * (u[0, 0] - u[0, -1])
        with xgrid.boundary(1):
            u[0, 0] = 1.0

    for _ in range(int(.7 / dt)):
        conv(u, c, dt, dx, dy)
    return {"u": levels(u)}


# ----------------------------------------------------------------- 2-D sweeps
@case
def diffusion_small():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")
    n = 64

    @xgrid.kernel()
    def heat(u: xgrid.grid[float, 2], c: float) -> None:
        u[0, 0] = u[0, 0] + c * (u[1, 0] + u[-1, 0] + u[0, 1] + u[0, -1] - 4.0 * u[0, 0])
        with xgrid.boundary(1):
            u[0, 0] = 0.0

    u = xgrid.Grid((n, n), float)
    u.now[...] = np.random.default_rng(0).random((n, n))
    b = u.boundary
    b[0, :] = b[-1, :] = b[:, 0] = b[:, -1] = 1
    for _ in range(20):
        heat(u, 0.2)
    return {"u": levels(u)}


@dataclasses.dataclass
class CavityConfig:
    rho: float
    nu: float
    dt: float
    dx: float
    dy: float


@case
def cavity_small():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")
    n = 33

    @xgrid.kernel()
    def cavity(b: xgrid.grid[float, 2], p: xgrid.grid[float, 2], u: xgrid.grid[float, 2],
               v: xgrid.grid[float, 2], cfg: CavityConfig) -> None:
        b[0, 0] = (cfg.rho * (1.0 / cfg.dt *
                              ((u[0, 1] - u[0, -1]) / (2.0 * cfg.dx) + (v[1, 0] - v[-1, 0]) / (2.0 * cfg.dy)) -
                              ((u[0, 1] - u[0, -1]) / (2.0 * cfg.dx)) ** 2.0 -
                              2.0 * ((u[1, 0] - u[-1, 0]) / (2.0 * cfg.dy) * (v[0, 1] - v[0, -1]) / (2.0 * cfg.dx)) -
                              ((v[1, 0] - v[-1, 0]) / (2.0 * cfg.dy)) ** 2.0))
        p[0, 0] = (((p[0, 1] + p[0, -1]) * cfg.dy ** 2.0 + (p[1, 0] + p[-1, 0]) * cfg.dx ** 2.0) /
                   (2.0 * (cfg.dx ** 2.0 + cfg.dy ** 2.0)) -
                   cfg.dx ** 2.0 * cfg.dy ** 2.0 / (2.0 * (cfg.dx ** 2.0 + cfg.dy ** 2.0)) * b[0, 0][0])
        with xgrid.boundary(1):
            p[0, 0] = p[0, -1][0]
        with xgrid.boundary(2):
            p[0, 0] = p[1, 0][0]
        with xgrid.boundary(3):
            p[0, 0] = p[0, 1][0]
        with xgrid.boundary(4):
            p[0, 0] = 0.0
        for _ in range(0, 50):
            p[0, 0] = (((p[0, 1][0] + p[0, -1][0]) * cfg.dy ** 2.0 + (p[1, 0][0] + p[-1, 0][0]) * cfg.dx ** 2.0) /
                       (2.0 * (cfg.dx ** 2.0 + cfg.dy ** 2.0)) -
                       cfg.dx ** 2.0 * cfg.dy ** 2.0 / (2.0 * (cfg.dx ** 2.0 + cfg.dy ** 2.0)) * b[0, 0][0])
            with xgrid.boundary(1):
                p[0, 0] = p[0, -1][0]
            with xgrid.boundary(2):
                p[0, 0] = p[1, 0][0]
            with xgrid.boundary(3):
                p[0, 0] = p[0, 1][0]
            with xgrid.boundary(4):
                p[0, 0] = 0.0
        u[0, 0] = (u[0, 0] -
                   u[0, 0] * cfg.dt / cfg.dx * (u[0, 0] - u[0, -1]) -
                   v[0, 0] * cfg.dt / cfg.dy * (u[0, 0] - u[-1, 0]) -
                   cfg.dt / (2.0 * cfg.rho * cfg.dx) * (p[0, 1][0] - p[0, -1][0]) +
                   cfg.nu * (cfg.dt / cfg.dx ** 2.0 * (u[0, 1] - 2.0 * u[0, 0] + u[0, -1]) +
                             cfg.dt / cfg.dy ** 2.0 * (u[1, 0] - 2.0 * u[0, 0] + u[-1, 0])))
        v[0, 0] = (v[0, 0] -
                   u[0, 0] * cfg.dt / cfg.dx * (v[0, 0] - v[0, -1]) -
                   v[0, 0] * cfg.dt / cfg.dy * (v[0, 0] - v[-1, 0]) -
                   cfg.dt / (2.0 * cfg.rho * cfg.dy) * (p[1, 0][0] - p[-1, 0][0]) +
                   cfg.nu * (cfg.dt / cfg.dx ** 2.0 * (v[0, 1] - 2.0 * v[0, 0] + v[0, -1]) +
                             cfg.dt / cfg.dy ** 2.0 * (v[1, 0] - 2.0 * v[0, 0] + v[-1, 0])))
        with xgrid.boundary(1):
            u[0, 0] = 0.0
            v[0, 0] = 0.0
        with xgrid.boundary(2):
            u[0, 0] = 1.0

    grids = {k: xgrid.Grid((n, n), float) for k in "bpuv"}
    u = grids["u"].boundary
    u[0, :] = u[:, 0] = u[:, -1] = 1
    u[-1, :] = 2
    vb = grids["v"].boundary
    vb.fill(1)
    vb[1:-1, 1:-1] = 0
    pb = grids["p"].boundary
    pb[:, -1] = 1
    pb[0, :] = 2
    pb[:, 0] = 3
    pb[-1, :] = 4
    bb = grids["b"].boundary
    bb.fill(1)
    bb[1:-1, 1:-1] = 0
    cfg = CavityConfig(1.0, 0.1, 1e-3, 2.0 / (n - 1), 2.0 / (n - 1))
    for _ in range(10):
        cavity(grids["b"], grids["p"], grids["u"], grids["v"], cfg)
    return {k: levels(g) for k, g in grids.items()}


@case
def wrap_2d():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double", overstep="wrap")
    n = 32

    @xgrid.kernel()
    def advect(u: xgrid.grid[float, 2], cx: float, cy: float, nu: float) -> None:
        u[0, 0] = (u[0, 0] - cx * (u[0, 1] - u[0, -1]) - cy * (u[1, 0] - u[-1, 0]) +
                   nu * (u[1, 0] + u[-1, 0] + u[0, 1] + u[0, -1] - 4.0 * u[0, 0]))

    u = xgrid.Grid((n, n), float)
    u.now[...] = np.random.default_rng(1).random((n, n))
    for _ in range(15):
        advect(u, 0.05, -0.03, 0.1)
    return {"u": levels(u)}


@case
def limit_2d():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double", overstep="limit")
    n = 24

    @xgrid.kernel()
    def smooth(u: xgrid.grid[float, 2]) -> None:
        u[0, 0] = (u[1, 1] + u[-1, -1] + u[1, -1] + u[-1, 1] + 2.0 * u[0, 0]) / 6.0

    u = xgrid.Grid((n, n), float)
    u.now[...] = np.random.default_rng(2).random((n, n))
    for _ in range(10):
        smooth(u)
    return {"u": levels(u)}


@case
def float_precision():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="float")
    n = 48

    @xgrid.kernel()
    def heat(u: xgrid.grid[float, 2], c: float) -> None:
        u[0, 0] = u[0, 0] + c * (u[1, 0] + u[-1, 0] + u[0, 1] + u[0, -1] - 4.0 * u[0, 0]) / 3.0
        with xgrid.boundary(1):
            u[0, 0] = 0.1

    u = xgrid.Grid((n, n), float)
    u.now[...] = np.random.default_rng(3).random((n, n)).astype(np.float32)
    b = u.boundary
    b[0, :] = b[-1, :] = b[:, 0] = b[:, -1] = 1
    for _ in range(20):
        heat(u, 0.6)
    return {"u": levels(u)}


@case
def time_levels():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")

    @xgrid.kernel()
    def lag(a: xgrid.grid[int, 1]) -> None:
        a[0] = a[0][-2] + 10

    g = xgrid.Grid((5,), int)
    out = []
    for _ in range(4):
        lag(g)
        out.append(levels(g)[:, 0].copy())
    return {"seq": np.stack(out)}


@xgrid.function()
def blend(a: float, b: float, w: float) -> float:
    if w > 1.0:
        w = 1.0
    return a * w + b * (1.0 - w)


@case
def control_flow():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")

    @xgrid.kernel()
    def prog(u: xgrid.grid[float, 2], v: xgrid.grid[float, 2], k: int, flag: bool) -> int:
        total = 0
        i = 0
        while i < k:
            i = i + 1
            if i % 2 == 0:
                continue
            total = total + i
        w = 0.25
        if flag:
            w = 0.75
        for j in range(0, k, 2):
            u[0, 0] = blend(u[0, 1], u[0, -1], w) if u[0, 0] > 0.5 else u[1, 0][-1] * 0.5 + v[0, 0]
            with xgrid.boundary(1):
                u[0, 0] = u[0, 0][-1] + 1.0 * cast(float, j)
        v[0, 0] = u[0, 0][0] - v[0, 0] if not (total > 100 and flag) else 2.0 * v[0, 0]
        return total * 3 - 7 / 2

    n = 20
    u = xgrid.Grid((n, n), float)
    v = xgrid.Grid((n, n), float)
    rng = np.random.default_rng(4)
    u.now[...] = rng.random((n, n))
    v.now[...] = rng.random((n, n))
    for g in (u, v):
        g.boundary[0, :] = g.boundary[-1, :] = g.boundary[:, 0] = g.boundary[:, -1] = 1
    rets = [prog(u, v, 7, True), prog(u, v, 4, False), prog(u, v, 30, True)]
    return {"u": levels(u), "v": levels(v), "ret": np.array(rets, dtype=np.int64)}


@case
def jacobi_small():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")
    n = 20

    @xgrid.kernel()
    def relax(p: xgrid.grid[float, 2], f: xgrid.grid[float, 2], iters: int, h2: float) -> None:
        for _ in range(0, iters):
            p[0, 0] = 0.25 * (p[1, 0][0] + p[-1, 0][0] + p[0, 1][0] + p[0, -1][0] - h2 * f[0, 0][0])
            with xgrid.boundary(1):
                p[0, 0] = p[0, 1][0]
            with xgrid.boundary(2):
                p[0, 0] = 0.5

    p = xgrid.Grid((n, n), float)
    f = xgrid.Grid((n, n), float)
    rng = np.random.default_rng(6)
    p.now[...] = rng.random((n, n))
    f.now[...] = rng.random((n, n)) - 0.5
    pb = p.boundary
    pb[:, 0] = 1
    pb[0, :] = 2
    pb[-1, :] = 2
    pb[:, -1] = 2
    for it in (3, 8):
        relax(p, f, it, 0.01)
    return {"p": levels(p), "f": levels(f)}


@case
def int_ops():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")
    n = 16

    @xgrid.kernel()
    def mix(a: xgrid.grid[int, 2], d: int) -> None:
        a[0, 0] = (a[0, 1] - a[1, 0]) / d + a[0, 0] % 7 - (-a[0, 0]) % 5
        with xgrid.boundary(1):
            a[0, 0] = a[0, 0] * 2 - 3

    a = xgrid.Grid((n, n), int)
    a.now[...] = np.random.default_rng(7).integers(-1000, 1000, (n, n))
    a.boundary[0, :] = a.boundary[-1, :] = a.boundary[:, 0] = a.boundary[:, -1] = 1
    for d in (3, -4, 7):
        mix(a, d)
    return {"a": levels(a)}


@case
def store_offset():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")
    n = 12

    @xgrid.kernel()
    def shift(u: xgrid.grid[float, 2]) -> None:
        u[1, 0] = u[0, 0] * 2.0 + 1.0

    u = xgrid.Grid((n, n), float)
    u.now[...] = np.random.default_rng(8).random((n, n))
    u.boundary[-1, :] = 1
    for _ in range(3):
        shift(u)
    return {"u": levels(u)}


@case
def depth3():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")
    n = 16

    @xgrid.kernel()
    def leap(u: xgrid.grid[float, 2], c: float) -> None:
        u[0, 0] = u[0, 0][-2] + c * (u[1, 0] + u[-1, 0] + u[0, 1] + u[0, -1] - 4.0 * u[0, 0])
        with xgrid.boundary(1):
            u[0, 0] = u[0, 0][-2]

    u = xgrid.Grid((n, n), float)
    u.now[...] = np.random.default_rng(9).random((n, n))
    u.boundary[0, :] = u.boundary[-1, :] = u.boundary[:, 0] = u.boundary[:, -1] = 1
    for _ in range(6):
        leap(u, 0.1)
    return {"u": levels(u)}


# --------------------------------------------- C interop inside grid sweeps
def _same_type(args):
    return args[0]


@xgrid.external(name="fabs", typecheck_override=_same_type)
def fabs(x: float) -> float:
    ...


@xgrid.external(name="XG_TWICE", typecheck_override=_same_type)
def twice(x: float) -> float:
    ...


@xgrid.function()
def smaller(a: float, b: float) -> float:
    r = 0.0
    with xgrid.c():
        "r = a < b ? a : b;"
    return r


@case
def c_interop():
    """Sweeps that call an external C function (``fabs`` from ``math.h``, included
    by ``import math``), a kernel macro used through an external name, and a
    helper whose body is inline C; inline C in the kernel body between sweeps."""
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")

    @xgrid.kernel(macro=["#define XG_TWICE(x) (2.0 * (x))"])
    def dev(u: xgrid.grid[float, 2], w: float) -> None:
        import math
        s = w
        with xgrid.c():
            "s = s * 0.5;"
        u[0, 0] = smaller(fabs(u[0, 1] - u[0, -1]), twice(u[1, 0])) + s * u[-1, 0]
        with xgrid.boundary(1):
            u[0, 0] = fabs(u[0, 0] - 0.5) * 0.5

    n = 18
    u = xgrid.Grid((n, n), float)
    u.now[...] = np.random.default_rng(12).random((n, n))
    u.boundary[0, :] = u.boundary[-1, :] = u.boundary[:, 0] = u.boundary[:, -1] = 1
    for w in (0.3, -0.7, 1.1):
        dev(u, w)
    return {"u": levels(u)}
