"""Generator, grouping and mixed-precision matching on the CPU (no GPU needed;
the generated CUDA is compiled by nvcc for sm_103a where nvcc is present)."""
import shutil

import pytest

import xgrid
import workloads
from xgrid_gb300 import mixed
from xgrid_gb300.codegen import CudaGenerator
from xgrid_gb300.config import get_config
from xgrid_gb300.operator import Operator


def _gen(op, **cfg):
    xgrid.init(precision="double", cacheroot="/tmp/xgcg", opt_level=3, **cfg)
    return CudaGenerator(Operator(op.func, "kernel", op.name), get_config()).generate()


def test_cavity_groups_and_launches():
    m = _gen(workloads.cavity_kernel)
    assert m.depth == 2
    assert m.groups == 3
    assert m.implicit_slots == [1]
    groups = {}
    for s in m.sweeps:
        groups.setdefault(s.group_index, []).append(s)
    # b + first p sweep + 4 boundaries | Jacobi + 4 boundaries | u + v + 3 walls
    assert [len(groups[i]) for i in sorted(groups)] == [6, 5, 5]
    jac = groups[1]
    assert jac[0].implicit and jac[0].write_version == 1
    assert all(s.mask != 0 for s in jac[1:])


def test_divisors_are_precomputed_and_deduplicated():
    m = _gen(workloads.cavity_kernel)
    assert "xg_divk(" in m.source
    # 2.0*cfg.dx, 2.0*cfg.dy, 2*(dx^2+dy^2), dx, dy: one parameter each per group
    assert m.source.count("xg_make_divisor((double)((2.0 * (cfg).dx)))") == 1
    m2 = _gen(workloads.cavity_kernel, divisor=False)
    assert "xg_divk(" not in m2.source.split("struct xga_")[1]


def test_mixed_matches_cavity_pressure_loop():
    m = _gen(workloads.cavity_kernel, mixed="fp32")
    assert m.aux_per_cell == {1: 14}
    assert "_mxd(" in m.source and "_mxc(" in m.source


def test_mixed_loop_has_temporal_tma_kernel():
    """2-D loops get the temporally blocked defect kernel: TMA box loads on an
    mbarrier, storage type per mode, the tile's boundary phases from box lists."""
    for mode, dt in (("fp32", "float"), ("fp16", "__half"), ("bf16", "__nv_bfloat16")):
        m = _gen(workloads.cavity_kernel, mixed=mode)
        assert "xgk_cavity_kernel_1_mxt" in m.source
        assert "xg_tma_load_2d(" in m.source and "xg_mbar_wait(" in m.source
        assert f"xgk_cavity_kernel_1_mxt<{dt}, RS>" in m.source
        assert m.source.count("xg_mask_boxes(") == 5  # box-zero flags + four boundary phases
    hdr = open(__import__("xgrid_gb300").build.CSRC + "/xgrid_gen.cuh").read()
    assert "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes" in hdr


def test_persistent_loop_kernel_for_in_place_loops():
    """The cavity pressure loop (implicit Jacobi sweep + four boundary sweeps) gets
    a persistent loop launch: a cooperative launch, each tile waiting for its
    neighbouring tiles' completion flags (zeroed by a memset before the launch),
    level and scratch alternating by iteration parity; a loop whose body uses the
    loop variable or writes two grids does not."""
    m = _gen(workloads.cavity_kernel, persistent=True)
    assert "xgk_cavity_kernel_1_loop" in m.source
    assert "cudaLaunchAttributeCooperative" in m.source
    assert "xg_tile_wait(p.flags, xg_tt" in m.source and "xg_tile_done(p.flags, xg_tt" in m.source
    assert "cudaMemsetAsync(p.flags, 0" in m.source and "xg_mask_tile_reach(" in m.source
    assert "(xg_it & 1) ? p.b1_0_1 : p.b1_0_0" in m.source
    assert m.source.count("_loop(xg_G, &xg_h, xg_K, xg_s)") == 1
    off = _gen(workloads.cavity_kernel)
    assert "_loop(" not in off.source
    nofuse = _gen(workloads.cavity_kernel, persistent=True, fuse=False)
    assert "_loop(" not in nofuse.source

    @xgrid.kernel()
    def uses_counter(p: xgrid.grid[float, 2], n: int) -> None:
        for i in range(0, n):
            p[0, 0] = 0.25 * (p[1, 0][0] + p[-1, 0][0] + p[0, 1][0] + p[0, -1][0]) if i > 2 else p[0, 1][0]

    @xgrid.kernel()
    def two_grids(p: xgrid.grid[float, 2], q: xgrid.grid[float, 2], n: int) -> None:
        for _ in range(0, n):
            p[0, 0] = 0.25 * (p[1, 0][0] + p[-1, 0][0] + p[0, 1][0] + p[0, -1][0])
            q[0, 0] = p[0, 0][0]

    for k in (uses_counter, two_grids):
        assert "_loop(xg_G" not in _gen(k, persistent=True).source


def test_affine_degree():
    xgrid.init(precision="double", cacheroot="/tmp/xgcg", opt_level=3)
    defn = Operator(workloads.cavity_kernel.func, "kernel", "cavity_kernel").ir
    loop = next(s for s in defn.body if s.__class__.__name__ == "For")
    assert mixed.degree(loop.body[0].value, "p") == 1
    assert all(mixed.degree(s.value, "p") in (0, 1) for s in loop.body[1:])
    assert mixed.degree(defn.body[0].value, "p") == 0  # the source term does not read p


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not available")
def test_generated_modules_compile(tmp_path):
    from xgrid_gb300.compiler import Compiler
    for kw in ({}, {"mixed": "fp32"}, {"mixed": "bf16"}, {"mixed": "fp16"}):
        m = _gen(workloads.cavity_kernel, **kw)
        Compiler(cacheroot=str(tmp_path)).compile(m.source, get_config().nvcc_flags)
    # batched (+ temporal blocking) and adjoint modules
    from xgrid_gb300.adjoint import AdjointGenerator
    xgrid.init(precision="float", cacheroot="/tmp/xgcg", opt_level=3, overstep="wrap")
    m = CudaGenerator(Operator(workloads.convdiff2d.func, "kernel", "convdiff2d"), get_config()).generate()
    Compiler(cacheroot=str(tmp_path)).compile(m.source, get_config().nvcc_flags)
    for fn, name in ((workloads.diffuse3d.func, "diffuse3d"), (workloads.convdiff2d.func, "convdiff2d")):
        gen = CudaGenerator(Operator(fn, "kernel", name), get_config())
        gen.generate()
        src, _ = AdjointGenerator(gen).source()
        Compiler(cacheroot=str(tmp_path)).compile(src, get_config().nvcc_flags)


def shadowing(u: xgrid.grid[float, 2], v: xgrid.grid[float, 2], a: float, s: float, G: float, p: float,
              h: float) -> None:
    # argument names that the generated C also uses internally
    u[0, 0] = a * u[0, 0] + s * u[0, 1] + G * v[-1, 0] + p * v[1, 0] + h
    v[0, 0] = v[0, 0] + a * (u[0, -1] - v[0, 0])


def returning(u: xgrid.grid[float, 2], ret: int, nret: int, r: float) -> int:
    total = 0
    i = 0
    while i < ret:
        i = i + 1
        if i % 2 == 0:
            continue
        total = total + i
    for j in range(0, nret):
        u[0, 0] = u[0, 1] * r + u[0, 0]
    return total * 3


def test_temporal_plan_and_power_of_two_scaling():
    m = _gen(workloads.cavity_kernel)
    # the Jacobi sweep multiplies by dx^2, dy^2 and a coefficient: scale parameters
    assert m.source.count("xg_make_scale(") >= 3 and "xg_mulk(" in m.source
    xgrid.init(precision="float", cacheroot="/tmp/xgcg", opt_level=3, overstep="wrap")
    mb = CudaGenerator(Operator(workloads.convdiff2d.func, "kernel", "convdiff2d"), get_config()).generate()
    assert mb.batch and "xgk_convdiff2d_tb" in mb.source
    xgrid.init(precision="float", cacheroot="/tmp/xgcg", opt_level=3, overstep="limit")
    mn = CudaGenerator(Operator(workloads.convdiff2d.func, "kernel", "convdiff2d"), get_config()).generate()
    assert mn.batch and "xgk_convdiff2d_tb" not in mn.source  # clamped edges do not block in time


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not available")
def test_argument_names_do_not_collide_with_generated_names(tmp_path):
    from xgrid_gb300.compiler import Compiler
    xgrid.init(precision="double", cacheroot="/tmp/xgcg", opt_level=3, overstep="wrap")
    m = CudaGenerator(Operator(shadowing, "kernel", "shadowing"), get_config()).generate()
    assert m.batch and "xgk_shadowing_tb" in m.source
    Compiler(cacheroot=str(tmp_path)).compile(m.source, get_config().nvcc_flags)
    m = CudaGenerator(Operator(returning, "kernel", "returning"), get_config()).generate()
    Compiler(cacheroot=str(tmp_path)).compile(m.source, get_config().nvcc_flags)


def noalloc_in_place(q: xgrid.grid[float, 2], r: xgrid.grid[float, 2]) -> None:
    q[0, 0] = 0.25 * (q[1, 0][0] + q[-1, 0][0] + q[0, 1][0] + q[0, -1][0])
    r[0, 0] = 0.5 * (r[0, 1][0] + q[0, 0][0])


def noalloc_explicit(u: xgrid.grid[float, 2], c: float) -> None:
    u[0, 0] = u[0, 0] + c * (u[0, 1] - u[0, 0])


def noalloc_scalar(a: int, b: int) -> int:
    return a * b + 1


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not available")
def test_noalloc_entry_is_exported_by_every_kind_of_kernel(tmp_path):
    """``noalloc=True`` always exports ``xg_kernel_<name>_noalloc``: with a scratch
    pool and the level-permutation undo when the kernel has in-place sweeps, as a
    plain table-build guard otherwise (also for kernels without grids)."""
    from xgrid_gb300.compiler import Compiler
    xgrid.init(precision="double", cacheroot="/tmp/xgcg", opt_level=3)
    for fn, pool in ((noalloc_in_place, True), (noalloc_explicit, False), (noalloc_scalar, False)):
        op = Operator(fn, "kernel", fn.__name__)
        op.noalloc = True
        m = CudaGenerator(op, get_config()).generate()
        assert f"xg_kernel_{fn.__name__}_noalloc(" in m.source
        assert (f"xg_noalloc_pool_{fn.__name__}[" in m.source) == pool
        assert "cudaMalloc" not in m.source.split(f"xg_kernel_{fn.__name__}_noalloc(")[1]
        lib = Compiler(cacheroot=str(tmp_path)).compile(m.source, get_config().nvcc_flags)
        out = __import__("subprocess").run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
        assert f"xg_kernel_{fn.__name__}_noalloc" in out


def wrap_relax(p: xgrid.grid[float, 2], f: xgrid.grid[float, 2], iters: int) -> None:
    for _ in range(0, iters):
        p[0, 0] = 0.25 * (p[1, 0][0] + p[-1, 0][0] + p[0, 1][0] + p[0, -1][0]) - f[0, 0][0]


def wide_relax(p: xgrid.grid[float, 2], f: xgrid.grid[float, 2], iters: int) -> None:
    for _ in range(0, iters):
        p[0, 0] = 0.25 * (p[2, 0][0] + p[-1, 0][0] + p[0, 1][0] + p[0, -1][0]) - f[0, 0][0]


def test_loop_iterations_per_launch_plan():
    """Several pressure iterations per launch: generated for the cavity's loop (main
    sweep reaching one cell, four boundary phases) and for a loop of one sweep when
    ``loop_temporal`` >= 2; not for reads reaching two cells, for periodic grids
    (overstep "wrap"), or with ``loop_temporal`` 0 -- there the launcher is a stub
    that declines."""
    def source(fn, name, **cfg):
        xgrid.init(precision="double", cacheroot="/tmp/xgcg", opt_level=3, **cfg)
        return CudaGenerator(Operator(fn, "kernel", name), get_config()).generate().source

    src = source(workloads.cavity_kernel.func, "cavity_kernel")
    assert "xgk_cavity_kernel_1_tl<" in src and "xgl_cavity_kernel_1_tloop(xg_G" in src
    assert "static const int32_t vals[] = {1, 2, 3, 4};" in src
    assert "constexpr int TH = 3" in src
    src = source(workloads.cavity_kernel.func, "cavity_kernel", loop_temporal=0)
    assert "_tl<" not in src and "return 0; }" in src
    for fn, cfg in ((wide_relax, {}), (wrap_relax, {"overstep": "wrap"})):
        src = source(fn, fn.__name__, **cfg)
        assert "_tl<" not in src, fn.__name__
    assert "_tl<" in source(wrap_relax, "wrap_relax")


def test_staged_geometry_fits_the_sm():
    """Staged z-walk shapes: whole 16-byte vectors per thread, whole rows per
    thread, shared memory that leaves at least one CTA per SM (three for FP32)."""
    from xgrid_gb300 import codegen
    for T in ("float", "double"):
        for nb in (1, 2, 3, 4):
            g = codegen.zstage_geometry(T, nb)
            assert g["NTX"] * g["V"] == g["TX"] and g["NTX"] * g["NTY"] == codegen.ZSTAGE_THREADS
            assert g["RY"] * g["NTY"] == g["TY"] and g["PX"] % g["V"] == 0
            assert g["R"] in (g["D"] + 3, g["D"] + 4) and g["blocks"] >= 1
            assert g["blocks"] * (g["smem"] + 1024) <= 228 * 1024
            if T == "float" and nb <= 3:
                assert g["blocks"] == 3
