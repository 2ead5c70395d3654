"""Slab decomposition on the CPU: two ``gloo`` ranks each run the oracle on
their slab of a grid (the slab's rows plus halo rows), refreshing halo rows
through ``xgrid_gb300.slab.exchange`` before every sweep that reads across the
cut, as the GPU module's launch hook does before every launch.  Gathered, the
slabs give the bits of the one-grid oracle for every level of every grid: the
lid-driven cavity (overstep none, boundary masks, in-place Jacobi sweeps),
periodic convection-diffusion on a non-square grid (wrap: the two ranks form a
ring), and clamped diffusion (limit)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case(name):
    """(kernel function, overstep, precision, {grid: (level 0, level 1, mask)}, argument builder, steps)."""
    import workloads
    rng = np.random.default_rng(17)
    if name == "cavity":
        n = 33
        st = workloads.cavity_state(n, 5)
        masks = workloads.cavity_masks(n)
        fields = {k: (st[k][0], st[k][1], masks[k]) for k in "bpuv"}
        cfg = workloads.Config(1.0, 0.1, 1e-4, 2.0 / (n - 1), 2.0 / (n - 1))
        return workloads.cavity_kernel.func, "none", "double", fields, lambda g: (g["b"], g["p"], g["u"], g["v"], cfg), 4
    if name == "convdiff":
        u0 = rng.random((22, 17))
        fields = {"u": (u0, np.zeros_like(u0), np.zeros(u0.shape, np.int32))}
        co = (0.6, 0.09, 0.11, 0.1, 0.1)
        return workloads.convdiff2d.func, "wrap", "float", fields, lambda g: (g["u"], *co), 6
    if name == "diffusion":
        u0 = rng.random((19, 13))
        m = np.zeros(u0.shape, np.int32)
        m[0, :] = 1
        fields = {"u": (u0, np.zeros_like(u0), m)}
        return workloads.diffusion2d.func, "limit", "double", fields, lambda g: (g["u"], 0.2), 5
    raise KeyError(name)


def _run(case, plan=None, exchange_rows=None):
    """Oracle run of a case on the whole grid, or on one slab with halo exchanges."""
    from oracle import xgrid_oracle
    from oracle.interp import Interpreter, depth_of
    from xgrid_gb300 import ir
    fn, overstep, precision, fields, build, steps = _case(case)
    xgrid_oracle.init(precision=precision, cacheroot="/tmp/xgslab", opt_level=3, overstep=overstep)
    k = xgrid_oracle.kernel()(fn)
    grids = {}
    for name, (l0, l1, mask) in fields.items():
        g = xgrid_oracle.Grid(plan.local_shape if plan else l0.shape, float)
        g._extend_time(2)
        for lv, x in enumerate((l0, l1)):
            g._data[lv][...] = plan.local_field(x) if plan else x
        g.boundary[...] = plan.local_mask(mask) if plan else mask
        grids[name] = g
    defn = k.ir
    depth = depth_of(defn)
    hook = None
    if plan is not None:
        def hook(stmt, env):
            done = []
            for st in ir.stencils(stmt.value):
                key = (st.variable.name, abs(st.time_offset))
                if st.space_offset[0] != 0 and key not in done:
                    done.append(key)
                    exchange_rows(env[key[0]].levels[key[1]])
    for _ in range(steps):
        args = build(grids)
        for a in args:
            if isinstance(a, xgrid_oracle.Grid):
                a._op_invoke(depth, True)
        Interpreter(defn, overstep, before_sweep=hook).run_kernel(list(args))
    return {name: [np.array(x) for x in g.levels] for name, g in grids.items()}


def _worker(rank, world, port, case, out):
    import sys
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    from xgrid_gb300 import slab
    dist.init_process_group("gloo", rank=rank, world_size=world, init_method=f"tcp://127.0.0.1:{port}")
    try:
        _, overstep, _, fields, _, _ = _case(case)
        shape = next(iter(fields.values()))[0].shape
        plan = slab.SlabPlan(shape, world, rank, 1, overstep)
        send_recv = slab.torch_send_recv()
        res = _run(case, plan, lambda arr: slab.exchange(plan, torch.from_numpy(arr), send_recv))
        # every rank's interior rows, gathered on rank 0
        parts = {k: [lv[plan.interior] for lv in v] for k, v in res.items()}
        gathered = [None] * world if rank == 0 else None
        dist.gather_object((plan.y0, plan.y1, parts), gathered, dst=0)
        if rank == 0:
            full = {}
            for y0, y1, p in gathered:
                for k, levels in p.items():
                    full.setdefault(k, [np.zeros((shape[0],) + lv.shape[1:], lv.dtype) for lv in levels])
                    for lv, x in zip(full[k], levels):
                        lv[y0:y1] = x
            np.savez(out, **{f"{k}_{i}": x for k, v in full.items() for i, x in enumerate(v)})
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("case", ["cavity", "convdiff", "diffusion"])
def test_two_rank_slabs_equal_the_whole_grid(tmp_path, case):
    out = str(tmp_path / "slabs.npz")
    ctx = mp.get_context("spawn")
    port = _port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, case, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(240)
        assert p.exitcode == 0
    slabs = np.load(out)
    whole = _run(case)
    for k, levels in whole.items():
        for i, x in enumerate(levels):
            assert slabs[f"{k}_{i}"].tobytes() == x.tobytes(), f"{case}: {k} level {i}"


def test_plan_partition_and_masks():
    from xgrid_gb300 import slab
    plans = [slab.SlabPlan((10, 7), 3, r) for r in range(3)]
    assert [(p.y0, p.y1) for p in plans] == [(0, 4), (4, 7), (7, 10)]
    assert plans[1].local_shape == (5, 7) and plans[1].interior == slice(1, 4)
    assert plans[0].neighbours() == (None, 1) and plans[2].neighbours() == (1, None)
    assert slab.SlabPlan((10, 7), 3, 0, overstep="wrap").neighbours() == (2, 1)
    m = np.arange(70, dtype=np.int32).reshape(10, 7)
    lm = plans[1].local_mask(m)
    assert (lm[0] == slab.HALO_MASK).all() and (lm[-1] == slab.HALO_MASK).all()
    assert (lm[1:4] == m[4:7]).all()
    f = np.arange(70.0).reshape(10, 7)
    assert (slab.SlabPlan((10, 7), 2, 0, overstep="wrap").local_field(f)[0] == f[9]).all()
    assert (slab.SlabPlan((10, 7), 2, 1, overstep="limit").local_field(f)[-1] == f[9]).all()
    assert (slab.SlabPlan((10, 7), 2, 1).local_field(f)[-1] == 0).all()
    with pytest.raises(ValueError):
        slab.SlabPlan((4, 4), 8, 0)
