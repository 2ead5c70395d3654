"""Benchmark programs at their benchmark sizes: GPU path vs the C oracle
(bit-exact FP64 with multiply-add contraction disabled), fused vs unfused
launches, graph replay vs eager calls."""
import numpy as np
import pytest

import xgrid
import workloads
from oracle import native

pytestmark = pytest.mark.gpu


def _bits_equal(a, b):
    return np.asarray(a).tobytes() == np.asarray(b).tobytes()


def test_diffusion_512_500_steps(cacheroot):
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3)
    u, c = workloads.diffusion_setup(512, seed=0)
    for _ in range(500):
        workloads.diffusion2d(u, c)
    field, c2 = native.diffusion_field(512, seed=0)
    assert c == c2
    native.Oracle("port").diffusion(field, c2, 500)
    assert _bits_equal(u.read(0), field.levels[0])
    assert _bits_equal(u.read(1), field.levels[1])


@pytest.mark.parametrize("n,steps", [(1025, 3), (257, 20)])
def test_cavity_bitexact(cacheroot, n, steps):
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3)
    grids, cfg = workloads.cavity_setup(n, 1e-5)
    for _ in range(steps):
        workloads.cavity_kernel(grids["b"], grids["p"], grids["u"], grids["v"], cfg)
    f = native.cavity_fields(n)
    native.Oracle("port").cavity(f, (cfg.rho, cfg.nu, cfg.dt, cfg.dx, cfg.dy), steps)
    for k in "bpuv":
        for lv in range(2):
            assert _bits_equal(grids[k].read(lv), f[k].levels[lv]), f"{k} level {lv}"


@pytest.mark.parametrize("n,dt,steps,seed", [(1025, 5e-6, 20, 7), (4097, 5e-7, 3, 8)])
def test_cavity_seeded_every_cell_bitexact(cacheroot, n, dt, steps, seed):
    """Seeded random b, p, u, v in every cell of both levels (no cell compares zero
    with zero): 1025^2 at the benchmark's dt for 20 steps, 4097^2 for 3 steps.
    The C oracle reproduces the reference's own digests of these runs
    (tests/test_oracle_full.py), so this is GPU = reference, every level of every grid."""
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3)
    grids, cfg = workloads.cavity_setup(n, dt, seed=seed)
    for _ in range(steps):
        workloads.cavity_kernel(grids["b"], grids["p"], grids["u"], grids["v"], cfg)
    f = native.cavity_fields(n, seed)
    native.Oracle("port").cavity(f, (cfg.rho, cfg.nu, cfg.dt, cfg.dx, cfg.dy), steps)
    for k in "bpuv":
        for lv in range(2):
            got = grids[k].read(lv)
            assert np.isfinite(got).all(), f"{k} level {lv}"
            assert _bits_equal(got, f[k].levels[lv]), f"{k} level {lv}"


def test_cavity_unfused_and_eager_match(cacheroot):
    """Every launch strategy computes the same bits: fused groups + graphs,
    one launch per sweep, eager calls."""
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3)
    outs = []
    for fuse, graph in ((True, True), (False, True), (True, False)):
        grids, cfg = workloads.cavity_setup(129, 1e-4)
        k = workloads.cavity_kernel
        k(grids["b"], grids["p"], grids["u"], grids["v"], cfg)  # compile
        k.native.set_fuse(fuse)
        k.native.use_graph = graph
        for _ in range(6):
            k(grids["b"], grids["p"], grids["u"], grids["v"], cfg)
        outs.append({g: grids[g].read(0) for g in "bpuv"})
        k.native.set_fuse(True)
        k.native.use_graph = True
    for o in outs[1:]:
        for g in "bpuv":
            assert _bits_equal(o[g], outs[0][g]), g


def test_host_writes_between_calls_are_uploaded(cacheroot):
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3)
    u, c = workloads.diffusion_setup(64, seed=3)
    workloads.diffusion2d(u, c)
    u.now[10:20, 10:20] = 5.0  # host write after a call
    workloads.diffusion2d(u, c)
    field, _ = native.diffusion_field(64, seed=3)
    o = native.Oracle("port")
    o.diffusion(field, c, 1)
    field.levels[0][10:20, 10:20] = 5.0
    o.diffusion(field, c, 1)
    assert _bits_equal(u.read(0), field.levels[0])
