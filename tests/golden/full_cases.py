"""The benchmark programs at their full sizes, recorded as digests.

Executed like ``cases.py`` with a global ``xgrid`` injected by the loader: the
reference package when ``make_digests.py`` records the SHA-256 of every time
level of every grid, the oracle in the CPU tests.  Full-size outputs are too
large to commit (the cavity at 1025^2 holds 67 MB of levels), so the reference's
results are pinned by their digests: the 2-D diffusion program (512^2 FP64, u0
uniform in [0, 1) from seed 0, nu = 0.1, dx = 1/511, dt = 0.2 dx^2 / nu, zero
edges) for 500 steps, and the lid-driven cavity (1025^2 FP64, rho = 1,
nu = 0.1, dt = 1e-5, dx = dy = 2/1024, zero fields) for 5 steps (after 5 steps every
level of every grid is nonzero).  Two more cavity cases start from a seeded random
state in every cell of both levels of b, p, u and v (``cavity_state``), so that every
cell is live from the first step: 1025^2 at dt = 5e-6 for 20 steps (the benchmark's
size and time step) and 4097^2 at dt = 5e-7 for 3 steps.
"""
import dataclasses
import hashlib

import numpy as np

FULL = {}


def full(fn):
    FULL[fn.__name__] = fn
    return fn


def digests(g) -> list:
    return [hashlib.sha256(np.ascontiguousarray(np.array(x)).tobytes()).hexdigest() for x in g._data]


@full
def diffusion_512():
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")
    n = 512

    @xgrid.kernel()
    def heat(u: xgrid.grid[float, 2], c: float) -> None:
        u[0, 0] = u[0, 0] + c * (u[1, 0] + u[-1, 0] + u[0, 1] + u[0, -1] - 4.0 * u[0, 0])
        with xgrid.boundary(1):
            u[0, 0] = 0.0

    nu = 0.1
    dx = 1.0 / (n - 1)
    dt = 0.2 * dx * dx / nu
    c = nu * dt / (dx * dx)
    u = xgrid.Grid((n, n), float)
    u.now[...] = np.random.default_rng(0).random((n, n))
    b = u.boundary
    b[0, :] = b[-1, :] = b[:, 0] = b[:, -1] = 1
    for _ in range(500):
        heat(u, c)
    return {"u": digests(u), "c": repr(c)}


@dataclasses.dataclass
class CavityConfig:
    rho: float
    nu: float
    dt: float
    dx: float
    dy: float


def cavity_state(n: int, seed: int) -> dict:
    """Seeded initial levels of the cavity grids: U[0, 1) for level 0 then level 1
    of b, p, u and v, in that order, from one generator."""
    rng = np.random.default_rng(seed)
    return {k: [rng.random((n, n)) for _ in range(2)] for k in "bpuv"}


@full
def cavity_1025():
    return _cavity(1025, 1e-5, 5, None)


@full
def cavity_1025_seeded():
    return _cavity(1025, 5e-6, 20, 7)


@full
def cavity_4097_seeded():
    return _cavity(4097, 5e-7, 3, 8)


def _cavity(n: int, dt: float, steps: int, seed):
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="double")

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
    if seed is not None:
        for k, levels in cavity_state(n, seed).items():
            grids[k]._extend_time(2)
            for lv, x in enumerate(levels):
                grids[k]._data[lv][...] = x
    cfg = CavityConfig(1.0, 0.1, dt, 2.0 / (n - 1), 2.0 / (n - 1))
    for _ in range(steps):
        cavity(grids["b"], grids["p"], grids["u"], grids["v"], cfg)
    return {k: digests(g) for k, g in grids.items()}


@full
def convdiff_square():
    """Square periodic FP32 convection-diffusion problems (the batched program's
    stencil on grids the reference addresses correctly): 64^2, 257^2, 512^2,
    coefficients from seed 5, 200 steps each."""
    xgrid.init(cacheroot=CACHEROOT, opt_level=3, precision="float", overstep="wrap")

    @xgrid.kernel()
    def convdiff(u: xgrid.grid[float, 2], a0: float, axm: float, axp: float, aym: float, ayp: float) -> None:
        u[0, 0] = a0 * u[0, 0] + axm * u[0, -1] + axp * u[0, 1] + aym * u[-1, 0] + ayp * u[1, 0]

    rng = np.random.default_rng(5)
    out = {}
    for n in (64, 257, 512):
        cx, cy = (float(v) for v in rng.uniform(-1.0, 1.0, 2))
        nu = float(rng.uniform(0.01, 0.1))
        dx = 1.0 / n
        dt = 0.2 * dx * dx / nu
        gx, gy = 0.5 * cx * dt / dx, 0.5 * cy * dt / dx
        k = nu * dt / (dx * dx)
        u = xgrid.Grid((n, n), float)
        u.now[...] = rng.random((n, n)).astype(np.float32)
        for _ in range(200):
            convdiff(u, 1.0 - 4.0 * k, gx + k, k - gx, gy + k, k - gy)
        out[f"u{n}"] = digests(u)
    return out
