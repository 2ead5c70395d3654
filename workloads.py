"""DSL programs and seeded inputs of the benchmark configurations.

Each kernel is ordinary ``@xgrid.kernel`` user code.  The diffusion and cavity
bodies are written with the same expression trees, in the same order, as the
reference's diffusion test case and examples/cavity.py:74-143 (51 Jacobi sweeps
per step: one from the previous level, then 50 in place), because bit-for-bit
parity depends on the order of floating-point operations.  Inputs are synthetic
and seeded; they stand in for nothing external.
"""
import dataclasses

import numpy as np

import xgrid

float2d = xgrid.grid[float, 2]
float3d = xgrid.grid[float, 3]


# ----------------------------------------------------------------- diffusion
@xgrid.kernel()
def diffusion2d(u: float2d, c: float) -> None:
    # explicit FTCS 5-point heat step, Dirichlet zero on mask 1
    u[0, 0] = u[0, 0] + c * (u[1, 0] + u[-1, 0] + u[0, 1] + u[0, -1] - 4.0 * u[0, 0])
    with xgrid.boundary(1):
        u[0, 0] = 0.0


def diffusion_setup(n: int = 512, seed: int = 0):
    """512x512, u0 ~ U[0,1) from ``seed``, nu=0.1, dx=dy=1/(n-1), dt=0.2*dx^2/nu."""
    nu = 0.1
    dx = 1.0 / (n - 1)
    dt = 0.2 * dx * dx / nu
    c = nu * dt / (dx * dx)
    u = xgrid.Grid((n, n), float)
    u.now[...] = np.random.default_rng(seed).random((n, n))
    b = u.boundary
    b[0, :] = b[-1, :] = b[:, 0] = b[:, -1] = 1
    return u, c


# -------------------------------------------------------------------- cavity
@dataclasses.dataclass
class Config:
    rho: float
    nu: float
    dt: float
    dx: float
    dy: float


@xgrid.kernel()
def cavity_kernel(b: float2d, p: float2d, u: float2d, v: float2d, cfg: Config) -> None:
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


def cavity_masks(n: int) -> dict:
    """Boundary masks of the lid-driven cavity (same assignment order, hence the
    same corner values, as the reference example)."""
    m = {k: np.zeros((n, n), dtype=np.int32) for k in "bpuv"}
    u = m["u"]
    u[0, :] = 1
    u[:, 0] = 1
    u[:, -1] = 1
    u[-1, :] = 2
    m["v"].fill(1)
    m["v"][1:-1, 1:-1] = 0
    p = m["p"]
    p[:, -1] = 1
    p[0, :] = 2
    p[:, 0] = 3
    p[-1, :] = 4
    m["b"].fill(1)
    m["b"][1:-1, 1:-1] = 0
    return m


def cavity_state(n: int, seed: int) -> dict:
    """Seeded initial levels of the cavity grids: U[0, 1) for level 0 then level 1
    of b, p, u and v, in that order, from one generator (every cell live, the
    boundary cells of b included, which the program never writes)."""
    rng = np.random.default_rng(seed)
    return {k: [rng.random((n, n)) for _ in range(2)] for k in "bpuv"}


def cavity_setup(n: int = 1025, dt: float = 1e-5, seed=None):
    """u, v, p, b on [0,2]^2 with n x n points, rho=1, nu=0.1: zero fields, or
    both time levels from ``cavity_state(n, seed)``."""
    grids = {k: xgrid.Grid((n, n), float) for k in "bpuv"}
    for k, mask in cavity_masks(n).items():
        grids[k].boundary[...] = mask
    if seed is not None:
        for k, levels in cavity_state(n, seed).items():
            grids[k]._extend_time(2)
            for lv, x in enumerate(levels):
                grids[k]._data[lv][...] = x
    cfg = Config(1.0, 0.1, dt, 2.0 / (n - 1), 2.0 / (n - 1))
    return grids, cfg


# ---------------------------------------------------------- FP64 rate probe
@xgrid.kernel()
def fp64_probe(q: float2d, x: float2d, a: float) -> None:
    # 32 dependent FP64 additions per cell (no subtree is free of the load, so none
    # is hoisted): on an L2-resident grid the sweep measures the FP64 add rate
    q[0, 0] = x[0, 0] + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a + a


FP64_PROBE_ADDS = 32


# ----------------------------------------------------------- batched problems
@xgrid.kernel()
def convdiff2d(u: float2d, a0: float, axm: float, axp: float, aym: float, ayp: float) -> None:
    # linear convection-diffusion, central differences, written with coefficients
    # only: a Python float literal is a C double, which would promote an FP32
    # update to FP64 (periodic with overstep="wrap")
    u[0, 0] = a0 * u[0, 0] + axm * u[0, -1] + axp * u[0, 1] + aym * u[-1, 0] + ayp * u[1, 0]


def batch_params(count: int = 256, seed: int = 1, lo: int = 64, hi: int = 1024):
    """``count`` periodic FP32 problems: extents uniform in [lo, hi] per axis,
    velocities c ~ U[-1, 1], nu ~ U[0.01, 0.1], u0 ~ U[0, 1), dt from the CFL and
    diffusion limits; returns ``(u0, coefficients)`` per problem, the
    coefficients being the scalar arguments of ``convdiff2d``."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        ny, nx = (int(v) for v in rng.integers(lo, hi + 1, 2))
        cx, cy = (float(v) for v in rng.uniform(-1.0, 1.0, 2))
        nu = float(rng.uniform(0.01, 0.1))
        dx, dy = 1.0 / nx, 1.0 / ny
        dt = 0.2 * min(dx, dy) ** 2 / nu
        u0 = rng.random((ny, nx)).astype(np.float32)
        # per-step coefficients: central convection, explicit diffusion
        gx, gy = 0.5 * cx * dt / dx, 0.5 * cy * dt / dy
        kx, ky = nu * dt / (dx * dx), nu * dt / (dy * dy)
        out.append((u0, (1.0 - 2.0 * kx - 2.0 * ky, gx + kx, kx - gx, gy + ky, ky - gy)))
    return out


def batch_setup(count: int = 256, seed: int = 1, lo: int = 64, hi: int = 1024):
    """The problems of ``batch_params`` as argument tuples of ``convdiff2d``
    (one FP32 grid per problem, ``xgrid.init(precision="float")``)."""
    problems = []
    for u0, coeffs in batch_params(count, seed, lo, hi):
        u = xgrid.Grid(u0.shape, float)
        u.now[...] = u0.astype(u.numpy_dtype)
        problems.append((u, *coeffs))
    return problems


# ------------------------------------------------------------- differentiation
@xgrid.kernel()
def diffuse3d(u: float3d, k: float3d, dt: float) -> None:
    # variable-coefficient 7-point diffusion; face diffusivity (k_c + k_nb) / 2 with
    # the 1/2 and 1/h^2 folded into dt (periodic with overstep="wrap")
    u[0, 0, 0] = u[0, 0, 0] + dt * ((k[0, 0, 0] + k[1, 0, 0]) * (u[1, 0, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[-1, 0, 0]) * (u[-1, 0, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, 1, 0]) * (u[0, 1, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, -1, 0]) * (u[0, -1, 0] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, 0, 1]) * (u[0, 0, 1] - u[0, 0, 0]) +
                                    (k[0, 0, 0] + k[0, 0, -1]) * (u[0, 0, -1] - u[0, 0, 0]))


def adjoint_setup(n: int = 256, seed: int = 2):
    """u0 ~ U[0,1), kappa log-uniform in [0.01, 0.1], target ~ U[0,1) (seeded);
    dt at 0.8 of the explicit stability limit for kappa_max = 0.1."""
    rng = np.random.default_rng(seed)
    u0 = rng.random((n, n, n), dtype=np.float32)
    kappa = np.exp(rng.uniform(np.log(0.01), np.log(0.1), (n, n, n))).astype(np.float32)
    target = rng.random((n, n, n), dtype=np.float32)
    dt = 0.8 / (12.0 * 0.1)
    return u0, kappa, target, dt
