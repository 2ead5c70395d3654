#!/usr/bin/env python
"""Benchmark of the stencil hot path on one GB300 (or N replicas).

Workload (default): the lid-driven cavity program on 1025 x 1025 FP64 grids,
dt = 5e-6 (see ``DT``), zero initial fields; one *step* is one call of the cavity kernel
(1 source sweep, 1 + 50 Jacobi sweeps of the pressure with four boundary passes
each, 2 momentum sweeps, velocity walls).  Metric: GLUP/s, counting one lattice
update per cell per full-grid sweep (54 per step; boundary passes excluded).

* ``value``: device time of K steps (CUDA events on the backend stream around
  each step, L2 flushed between steps by writing a 256 MiB buffer), grids
  resident in HBM.
* ``e2e``: the same steps through the public API with host buffers: every step
  reads ``u.now``, ``v.now``, ``p.now`` back (device→host) and the next call
  uploads them again (host→device, pinned), wall clock around the loop.
* ``roofline``: the dominant kernel (the fused Jacobi + boundary launch), its
  algorithmic bytes per launch over its mean duration inside the CUDA graphs the
  timed region replays (event-record nodes around every launch, L2 flushed
  between steps as in the timed region).
* ``cpu_baseline``: the reference's own generated C (compiled from
  ``oracle/_ref``) on all host cores for a bounded number of steps.

The same line carries one section per further configuration, each with its own
``roofline``, ``cpu_baseline`` and ``e2e``: ``diffusion`` (2-D FTCS 512^2 FP64,
500 steps), ``mixed`` (cavity 4097^2, FP32 / FP16 / BF16 defect correction vs
plain FP64), ``batched`` (256 periodic FP32 problems of uneven size, 1000
steps) and ``adjoint`` (3-D 256^3 FP32 rollout and gradient).

``--impl reference`` times that reference C path alone on the host cores.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SWEEPS_PER_STEP = 54  # b, 1 + 50 Jacobi, u, v
JIT_CACHE = os.path.join(ROOT, ".xgrid_cache", "bench")  # compiled kernel modules stay in the tree
# The configured dt = 1e-5 breaks the explicit-diffusion stability limit
# nu*dt*(1/dx^2 + 1/dy^2) <= 1/2 (0.52 at 1025^2, 8.4 at 4097^2) and the fields
# diverge after a few hundred steps; the benchmark uses the largest round dt
# below the limit.  The work per step does not depend on dt.
DT = {1025: 5e-6, 4097: 5e-7}


def workload_name(n: int) -> str:
    return f"lid-driven cavity {n}x{n} FP64 plain, dt={stable_dt(n):g}, 50+1 Jacobi sweeps/step"


def stable_dt(n: int) -> float:
    if n in DT:
        return DT[n]
    dx = 2.0 / (n - 1)
    return 0.2 * dx * dx / 0.1
METRIC = "GLUP/s & HBM-roofline % per stencil: mixed/batched vs plain FP64, same GB300"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1025)
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default tile shapes of the headline kernel")
    ap.add_argument("--cpu-sample", type=int, default=0, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-workload", default="cavity", help=argparse.SUPPRESS)
    ap.add_argument("--mixed-n", type=int, default=4097)
    ap.add_argument("--mixed-steps", type=int, default=500)
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--mixed-temporal", type=int, default=8,
                    help="defect iterations per launch of the mixed-precision loop (0: one per launch)")
    ap.add_argument("--batch-steps", type=int, default=1000)
    ap.add_argument("--adjoint-n", type=int, default=256)
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-diffusion", action="store_true")
    ap.add_argument("--persistent", type=int, default=0,
                    help="headline: run the pressure loop as one persistent launch per step (1) or one launch "
                         "per iteration (0)")
    ap.add_argument("--mixed", default=None, choices=[None, "fp32", "fp16", "bf16"],
                    help="kernels mode: precision lowering of the pressure loop")
    ap.add_argument("--workload", default="cavity", choices=["cavity", "batch", "adjoint"],
                    help="kernels mode: which workload to run")
    ap.add_argument("--temporal", default=None,
                    help="kernels mode, batch workload: steps per launch, or depth,ty,tx (1 = none)")
    ap.add_argument("--mode", default="bench", choices=["bench", "kernels"],
                    help="kernels: only run warm-up + steps (for profiler launch lists)")
    return ap.parse_args()


def kernels_only(args) -> None:
    """Set up the workload and run warm-up + steps, nothing else (profiling)."""
    import xgrid
    import workloads
    from xgrid_gb300 import device
    if args.workload == "batch":
        xgrid.init(precision="float", cacheroot=JIT_CACHE,
                   opt_level=3, overstep="wrap")
        probs = workloads.batch_setup(256, seed=1)
        temporal = None
        if args.temporal:
            parts = [int(x) for x in args.temporal.split(",")]
            temporal = parts[0] if len(parts) == 1 else tuple(parts)
        for _ in range(args.warmup + 1):
            workloads.convdiff2d.batch(probs, args.steps, temporal=temporal)
        device.synchronize()
        print(json.dumps({"mode": "kernels", "workload": "batch", "calls": args.warmup + 1}))
        return
    if args.workload == "adjoint":
        # 3-D variable-coefficient diffusion at n^3 FP32: forward rollout + gradient, checkpoints every 10
        import torch
        from xgrid_gb300 import adjoint
        from xgrid_gb300.operator import Operator
        xgrid.init(precision="float", cacheroot=JIT_CACHE,
                   opt_level=3, overstep="wrap")
        k = Operator(workloads.diffuse3d.func, "kernel", "diffuse3d")
        u0, kap, tgt, dt = workloads.adjoint_setup(args.n, 2)
        u0, kap, tgt = (torch.tensor(x, device="cuda") for x in (u0, kap, tgt))
        ro = adjoint.Rollout(k, args.steps, 10)
        for _ in range(args.warmup + 1):
            a, bb = u0.clone().requires_grad_(True), kap.clone().requires_grad_(True)
            ((ro(a, {"k": bb}, (dt,)) - tgt) ** 2).mean().backward()
        device.synchronize()
        print(json.dumps({"mode": "kernels", "workload": "adjoint", "n": args.n, "calls": args.warmup + 1}))
        return
    xgrid.init(precision="double", cacheroot=JIT_CACHE,
               opt_level=3, mixed=args.mixed, mixed_temporal=args.mixed_temporal, persistent=bool(args.persistent))
    grids, cfg = workloads.cavity_setup(args.n, stable_dt(args.n))
    args_ = (grids["b"], grids["p"], grids["u"], grids["v"], cfg)
    tilings = None
    if not args.no_tune and args.mixed is None:
        # the bench's tile choice (timed on these grids, cached on disk per shape)
        from xgrid_gb300 import autotune
        tilings = {str(g): list(t) for g, t in autotune.tune(workloads.cavity_kernel, *args_).items()}
    for _ in range(args.warmup + args.steps):
        workloads.cavity_kernel(*args_)
    device.synchronize()
    print(json.dumps({"mode": "kernels", "n": args.n, "calls": args.warmup + args.steps, "tilings": tilings}))


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_traffic(kernel_tag: str, n: int, key: str = "traffic_bytes_per_launch_", dims: int = 2):
    """DRAM bytes (read + write) per launch of a kernel, from the committed ncu
    summaries (``<key><n>: <bytes>`` lines in ``profiles/<kernel_tag>_*.md``).
    A capture at another size is scaled by the number of cells (n^dims; the
    kernel's traffic is proportional to its cells); None when no capture exists."""
    import glob
    found = {}
    for path in glob.glob(os.path.join(ROOT, "profiles", f"{kernel_tag}_*.md")):
        for line in open(path):
            if line.startswith(key):
                k, val = line.split(":", 1)
                found[int(k[len(key):])] = float(val)
    if n in found:
        return found[n], f"ncu capture at {n}^{dims}"
    if found:
        m = max(found)
        return found[m] * n ** dims / m ** dims, f"ncu capture at {m}^{dims} scaled by cells"
    return None, None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int) -> None:
        self.index = index
        self.proc = None
        self.path = tempfile.mktemp(prefix="xgclk", suffix=".csv")

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------- CPU side
def cpu_sample(workload: str, n: int, steps: int) -> dict:
    """Time ``steps`` steps of a workload on the host cores (run in a child process
    whose OpenMP / torch thread count is the core count): the reference's own
    generated C (``oracle/_ref``) where it exists, else the C restatement, and
    torch CPU autograd for the 3-D adjoint (the reference mis-indexes 3-D grids).
    Returns seconds and what ran."""
    import numpy as np

    from oracle import native
    if workload == "adjoint":
        import torch
        torch.set_num_threads(os.cpu_count() or 1)
        u0, kap, tgt, dt = workloads_mod().adjoint_setup(n, 2)
        u0, kap, tgt = (torch.tensor(x) for x in (u0, kap, tgt))
        torch_autograd_run(u0, kap, tgt, dt, 1)  # warm-up
        t0 = time.perf_counter()
        torch_autograd_run(u0, kap, tgt, dt, steps)
        return {"kind": "torch-cpu-autograd", "seconds": time.perf_counter() - t0, "steps": steps,
                "threads": torch.get_num_threads()}
    if workload == "convdiff":
        # equal-cell squares of the batched problems (the reference strides
        # non-square grids by the wrong extent): timing only, one call per problem
        run = native.convdiff_reference()
        fields = []
        for u0, coeffs in workloads_mod().batch_params(256, seed=1):
            side = int(round(float(np.sqrt(u0.size))))
            fields.append((native.Field32(np.resize(u0, (side, side))), tuple(np.float32(c) for c in coeffs)))
        for f, c in fields:
            run(f, c, 1)
        t0 = time.perf_counter()
        for _ in range(steps):
            for f, c in fields:
                run(f, c, 1)
        return {"kind": "reference", "seconds": time.perf_counter() - t0, "steps": steps,
                "cells": sum(int(f.levels[0].size) for f, _ in fields)}
    kind = "reference" if (native.ref_available() or native.ref_sources()) else "port"
    try:
        o = native.Oracle(kind, exact=False)
    except Exception:  # noqa: BLE001 - the reference sources are absent
        kind = "port"
        o = native.Oracle("port")
    if workload == "diffusion":
        field, c = native.diffusion_field(n, seed=0)
        o.diffusion(field, c, 1)
        t0 = time.perf_counter()
        o.diffusion(field, c, steps)
        return {"kind": kind, "seconds": time.perf_counter() - t0, "steps": steps}
    f = native.cavity_fields(n)
    cfg = (1.0, 0.1, stable_dt(n), 2.0 / (n - 1), 2.0 / (n - 1))
    o.cavity(f, cfg, 1)  # warm-up (page faults, thread team)
    t0 = time.perf_counter()
    o.cavity(f, cfg, steps)
    return {"kind": kind, "seconds": time.perf_counter() - t0, "steps": steps}


def workloads_mod():
    import workloads
    return workloads


def torch_autograd_run(u0, kap, tgt, dt: float, steps: int) -> float:
    """Forward rollout and gradient of the 3-D variable-coefficient diffusion
    through plain torch tensor ops (periodic shifts), on the tensors' device."""
    import torch
    a, bb = u0.clone().requires_grad_(True), kap.clone().requires_grad_(True)
    u = a
    for _ in range(steps):
        acc = None
        for d in range(3):
            for sh in (-1, 1):
                un, kn = torch.roll(u, -sh, d), torch.roll(bb, -sh, d)
                term = (bb + kn) * (un - u)
                acc = term if acc is None else acc + term
        u = u + dt * acc
    loss = ((u - tgt) ** 2).mean()
    loss.backward()
    return float(loss.detach())


def run_cpu(workload: str, n: int, steps: int) -> dict:
    cores = os.cpu_count() or 1
    env = dict(os.environ, OMP_NUM_THREADS=str(cores), OMP_PROC_BIND="close")
    cmd = [sys.executable, os.path.abspath(__file__), "--cpu-sample", str(steps), "--cpu-workload", workload,
           "--n", str(n)]
    out = subprocess.run(cmd, env=env, capture_output=True, text=True, check=True).stdout.strip().splitlines()[-1]
    r = json.loads(out)
    r["cores"] = r.get("threads", cores)
    return r


def bounded_steps(workload: str, n: int, seconds: float, cap: int) -> dict:
    """Run one step to calibrate, then as many steps as fit in ``seconds``."""
    probe = run_cpu(workload, n, 1)
    steps = max(1, min(cap, int(math.ceil(seconds / max(probe["seconds"], 1e-3)))))
    return run_cpu(workload, n, steps)


def cpu_baseline(n: int, seconds: float) -> dict:
    r = bounded_steps("cavity", n, seconds, 400)
    lups = SWEEPS_PER_STEP * n * n * r["steps"]
    return {"value": lups / r["seconds"] / 1e9, "unit": "GLUP/s", "cores": r["cores"], "kind": r["kind"],
            "sample": f"cavity {n}x{n} FP64, {r['steps']} steps ({r['seconds']:.1f} s), OpenMP on all host cores"}


# ---------------------------------------------------------------- GPU side
def replica_time(secs: float, world: int, device: str = "cuda") -> float:
    """Slowest rank's time (replicas only: ranks run independent copies of the
    workload and are synchronised by a barrier before and after timing)."""
    if world <= 1:
        return secs
    import torch
    t = torch.tensor([secs], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.barrier()
    return float(t.item())


def fp64_peak(n: int = 2048, calls: int = 10) -> float:
    """FP64 additions per second of the FP64 unit, measured with the DSL probe
    (32 chained additions per cell, fields resident in L2)."""
    import numpy as np
    import torch

    import xgrid
    import workloads
    from xgrid_gb300 import device
    from xgrid_gb300.operator import Operator
    xgrid.init(precision="double", cacheroot=JIT_CACHE,
               opt_level=3)
    k = Operator(workloads.fp64_probe.func, "kernel", "fp64_probe")
    q, x = xgrid.Grid((n, n), float), xgrid.Grid((n, n), float)
    x.now[...] = np.random.default_rng(0).random((n, n))
    for _ in range(3):
        k(q, x, 1e-3)
    s = device.stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.synchronize()
    e0.record(s)
    for _ in range(calls):
        k(q, x, 1e-3)
    e1.record(s)
    s.synchronize()
    return workloads.FP64_PROBE_ADDS * n * n * calls / (e0.elapsed_time(e1) * 1e-3)


def graph_launch_times(native_k, step, flush=None, rounds: int = 3):
    """({profiling site: [ms, ...]}, steps): the duration of every launch of ``step`` inside
    the CUDA graphs the timed region replays.  The kernel's graphs are captured
    again with profiling in graph-node mode (an event-record node before and after
    every launch); each replay records those events again.  A step may cycle
    through several graph keys (time levels and scratch buffers rotate), so the
    steps run until no new graph is captured, then ``rounds`` times that many
    replays, reading the events after each full cycle.  The kernel's graphs are
    dropped afterwards (the ones without event nodes are captured again)."""
    from xgrid_gb300 import device, runtime
    lib = runtime.load()
    lib.xg_graph_count.restype = ctypes.c_int64
    s = device.stream()
    lib.xg_graph_clear(ctypes.c_void_p(native_k.fn_ptr))
    lib.xg_prof_reset()
    lib.xg_prof_enable(2)
    counts, period = [], 0
    for _ in range(128):
        step()
        counts.append(int(lib.xg_graph_count()))
        grown = [i for i in range(1, len(counts)) if counts[i] > counts[i - 1]]
        if grown and counts[-1] == counts[-2] and len(grown) == counts[-1] - counts[0]:
            period = counts[-1] - counts[0]
            break
    s.synchronize()
    lib.xg_prof_enable(0)
    if period == 0:
        raise RuntimeError("the step's graphs did not settle into a cycle")
    for _ in range(period - 1):  # finish the cycle that the last call started
        step()
    by_site: dict = {}
    for _ in range(rounds):
        for _ in range(period):
            if flush is not None:
                flush()
            step()
        s.synchronize()
        for g, ms in runtime.prof_records():
            by_site.setdefault(g, []).append(ms)
    lib.xg_graph_clear(ctypes.c_void_p(native_k.fn_ptr))
    lib.xg_prof_reset()
    return by_site, rounds * period


def eager_launch_times(native_k, step, nsteps: int = 5):
    """({site: [ms]}, steps) from CUDA events around every launch of ``nsteps``
    eager (non-graph) calls: the fallback when event nodes cannot be timed."""
    from xgrid_gb300 import device, runtime
    lib = runtime.load()
    native_k.use_graph = False
    lib.xg_prof_reset()
    lib.xg_prof_enable(1)
    try:
        for _ in range(nsteps):
            step()
        device.stream().synchronize()
    finally:
        lib.xg_prof_enable(0)
        native_k.use_graph = True
    by_site: dict = {}
    for g, ms in runtime.prof_records():
        by_site.setdefault(g, []).append(ms)
    lib.xg_prof_reset()
    return by_site, nsteps


def launch_times(native_k, step, flush=None):
    """Launch durations inside the replayed graphs, else from eager calls; with the source."""
    try:
        by_site, steps = graph_launch_times(native_k, step, flush)
        return by_site, steps, "event nodes inside the replayed CUDA graphs"
    except Exception as e:  # noqa: BLE001 - report how the times were taken instead
        from xgrid_gb300 import device, runtime
        lib = runtime.load()
        lib.xg_prof_enable(0)
        device.stream().synchronize()
        lib.xg_graph_clear(ctypes.c_void_p(native_k.fn_ptr))
        lib.xg_prof_reset()
        by_site, steps = eager_launch_times(native_k, step)
        return by_site, steps, f"CUDA events around eager launches (graph event nodes failed: {e})"


# FP64 operations per cell of the cavity's Jacobi sweep after host hoisting: 3 additions and 1
# subtraction; the products by dx^2, dy^2 and the quotient by 2(dx^2+dy^2) are exact exponent
# arithmetic on the integer pipe when dx = dy = 2/(n-1) is a power of two (n = 2^k + 1).
JACOBI_FP64_OPS = 4
JACOBI_ITERS = 50     # pressure iterations of the loop in the cavity step
LOOP_SITE = 61        # profiling site (group * 64 + 61) of a persistent loop launch
TLOOP_SITE = 57       # profiling site (group * 64 + 57) of a launch of several loop iterations


def gpu_bench(args, rank: int, world: int):
    import torch

    import xgrid
    import workloads
    from xgrid_gb300 import device, runtime

    torch.cuda.set_device(rank % max(torch.cuda.device_count(), 1))
    cache = JIT_CACHE
    xgrid.init(precision="double", cacheroot=cache, opt_level=3, persistent=args.persistent)
    n = args.n
    grids, cfg = workloads.cavity_setup(n, stable_dt(n))
    kern = workloads.cavity_kernel
    b, p, u, v = grids["b"], grids["p"], grids["u"], grids["v"]

    def step():
        kern(b, p, u, v, cfg)

    tilings = None
    if not args.no_tune:
        # tile shape of every launch group picked by timing candidates on these grids
        # (their state is restored afterwards; the choice is cached on disk per shape)
        from xgrid_gb300 import autotune
        tilings = {str(g): list(t) for g, t in autotune.tune(kern, b, p, u, v, cfg).items()}
    for _ in range(args.warmup):
        step()
    s = device.stream()
    s.synchronize()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    lib = runtime.load()

    def timed(k: int):
        evs = []
        for _ in range(k):
            with torch.cuda.stream(s):
                flush.add_(1)  # L2 flush: 256 MiB read+write, outside the timed interval
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s)
            step()
            e1.record(s)
            evs.append((e0, e1))
        s.synchronize()
        return sum(a.elapsed_time(b_) for a, b_ in evs) / 1000.0

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk:
        secs = timed(args.steps)
    torch.cuda.synchronize()
    secs = replica_time(secs, world)
    lups_rank = SWEEPS_PER_STEP * n * n * args.steps

    # launch durations inside the timed region's CUDA graphs (event-record nodes)
    native_k = kern.native

    def flush_l2():
        with torch.cuda.stream(s):
            flush.add_(1)

    by_site, prof_steps, time_src = launch_times(native_k, step, flush_l2)
    launches_per_step = sum(len(v) for v in by_site.values()) / prof_steps
    dom_site, dom_ms = max(by_site.items(), key=lambda kv: sum(kv[1]))
    total_prof = sum(sum(x) for x in by_site.values())
    share = sum(dom_ms) / total_prof
    dom_per_step = len(dom_ms) / prof_steps
    # the dominant kernel's time per launch inside the timed region: the timed step times
    # its share of the launch time (event nodes add gaps between graph nodes, so their own
    # durations run longer than in the timed graphs)
    dom_avg_s = secs / args.steps * share / dom_per_step
    node_avg_s = statistics.mean(dom_ms) / 1000.0
    group = dom_site // 64
    # a persistent loop launch runs all 50 Jacobi iterations (+ boundary phases), a
    # temporal loop launch up to loop_temporal of them (50 / its launches per step)
    loop = dom_site % 64 == LOOP_SITE
    tl = dom_site % 64 == TLOOP_SITE
    iters = JACOBI_ITERS if loop else (JACOBI_ITERS / dom_per_step if tl else 1)
    bytes_per_cell = algorithmic_bytes(native_k.module, group)
    alg_bytes = bytes_per_cell * n * n * iters
    hbm_peak, peak_src = peaks()
    achieved = alg_bytes / dom_avg_s / 1e9
    traffic, traffic_src = profile_traffic("cavity_jacobi_loop_fp64" if loop else
                                           ("cavity_jacobi_tloop_fp64" if tl else "cavity_jacobi_fused_fp64"), n)
    pow2 = ((n - 1) & (n - 2)) == 0
    fp64 = None
    if pow2:
        peak64 = fp64_peak()
        rate64 = JACOBI_FP64_OPS * n * n * iters / dom_avg_s
        fp64 = {"bound": "fp64 pipe", "achieved_gops": rate64 / 1e9, "peak_gops": peak64 / 1e9,
                "frac": rate64 / peak64, "ops_per_cell": JACOBI_FP64_OPS,
                "peak_source": "32-addition FP64 probe sweep measured in this run (L2-resident 2048^2)"}
        xgrid.init(precision="double", cacheroot=cache, opt_level=3, persistent=args.persistent)

    # e2e through the public API with host buffers
    for g in (u, v, p):
        g.now  # noqa: B018 - host copies become current and authoritative
    torch.cuda.synchronize()
    e2e_steps = args.e2e_steps
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        step()
        for g in (u, v, p):
            g.now  # noqa: B018 - device→host read of the step's result
    s.synchronize()
    e2e_secs = time.perf_counter() - t0
    level_bytes = n * n * 8
    e2e = {"value": SWEEPS_PER_STEP * n * n * e2e_steps / e2e_secs / 1e9 * world, "unit": "GLUP/s",
           "h2d_bytes_per_step": 3 * level_bytes, "d2h_bytes_per_step": 3 * level_bytes,
           "steps": e2e_steps, "ms_per_step": e2e_secs / e2e_steps * 1e3}

    result = {
        "metric": METRIC,
        "value": lups_rank * world / secs / 1e9,
        "unit": "GLUP/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": secs / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic: zero initial fields, lid u=1 (deterministic)",
        "config": {"workload": workload_name(n), "parity": "bit-exact vs the reference's C",
                   "n": n, "sweeps_per_step": SWEEPS_PER_STEP, "l2": "flushed between steps (256 MiB write)",
                   "parallelism": f"replicas x{world}", "graph": True, "persistent_loop": bool(args.persistent),
                   "launches_per_step": launches_per_step,
                   "tilings": tilings},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic, "traffic_source": traffic_src,
                     "peak_source": peak_src,
                     "kernel": f"group {group} (site {dom_site}"
                               f"{', persistent loop: %d iterations per launch' % iters if loop else ''}"
                               f"{', %g iterations per launch on shared-memory boxes' % iters if tl else ''})",
                     "kernel_ms": dom_avg_s * 1e3,
                     "kernel_time": "ms_per_step x kernel_share / launches of the kernel per step",
                     "kernel_share": share, "share_source": time_src, "kernel_launches_per_step": dom_per_step,
                     "kernel_ms_event_nodes": node_avg_s * 1e3, "algorithmic_bytes_per_launch": alg_bytes,
                     "fp64": fp64},
        "e2e": e2e,
        "gpu_launches": int(round(launches_per_step * args.steps)),
        "clocks": clk.summary(),
    }
    return result


def diffusion_section(n: int = 512, steps: int = 500, runs: int = 3, cpu_seconds: float = 5.0) -> dict:
    """2-D FTCS diffusion, n^2 FP64, ``steps`` calls of the diffusion kernel per
    run (the reference's program, one call per time step).  ``value``: device
    time of a run (L2 flushed before each run; the 4 MB of levels then live in
    L2 for the run); ``roofline``: the fused sweep + boundary launch at 16
    algorithmic bytes per cell, its duration from event nodes inside the replayed
    graphs; ``e2e``: a run through the public API from a host array to a host
    array; ``parity``: SHA-256 of both levels after the first run of ``steps``
    steps from the seeded field against the reference's own digests; CPU
    baseline: the reference's generated C on all host cores."""
    import hashlib

    import numpy as np
    import torch

    import xgrid
    import workloads
    from xgrid_gb300 import device
    from xgrid_gb300.operator import Operator

    xgrid.init(precision="double", cacheroot=JIT_CACHE, opt_level=3)
    k = Operator(workloads.diffusion2d.func, "kernel", "diffusion2d")
    u, c = workloads.diffusion_setup(n, seed=0)
    u0 = u.read(0)
    for _ in range(steps):
        k(u, c)
    digests = [hashlib.sha256(u.read(lv).tobytes()).hexdigest() for lv in range(2)]
    # the tile shape picked by timing candidates on this grid (state restored afterwards), as for
    # the headline
    from xgrid_gb300 import autotune
    tilings = {str(g): list(t) for g, t in autotune.tune(k, u, c).items()}
    parity = None
    try:
        ref = json.load(open(os.path.join(ROOT, "tests", "golden", "full_digests.json")))["diffusion_512"]
        if n == 512 and steps == 500:
            parity = "bit-exact vs the reference's digests" if digests == ref["u"] else "MISMATCH"
    except (OSError, KeyError, ValueError):
        pass
    s = device.stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    evs = []
    for _ in range(runs):
        with torch.cuda.stream(s):
            flush.add_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(steps):
            k(u, c)
        e1.record(s)
        evs.append((e0, e1))
    s.synchronize()
    run_s = statistics.median(a.elapsed_time(b) for a, b in evs) / 1e3
    lups = n * n * steps
    by_site, nprof, time_src = launch_times(k.native, lambda: k(u, c))
    dom_site, dom_ms = max(by_site.items(), key=lambda kv: sum(kv[1]))
    share = sum(dom_ms) / sum(sum(v) for v in by_site.values())
    # the whole run of ``steps`` calls captured into one CUDA graph (the calls' launches,
    # level rotation included: an even number of steps returns every level to its buffer),
    # replayed: device time per step without the per-call host work
    k.native.use_graph = False
    whole = torch.cuda.CUDAGraph()
    with torch.cuda.graph(whole, stream=s, capture_error_mode="thread_local"):
        for _ in range(steps):
            k(u, c)
    k.native.use_graph = True
    s.synchronize()
    ev = []
    for _ in range(runs):
        with torch.cuda.stream(s):
            flush.add_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        with torch.cuda.stream(s):  # replay() launches on the current stream
            whole.replay()
        e1.record(s)
        ev.append((e0, e1))
    s.synchronize()
    graph_run_s = statistics.median(a.elapsed_time(b) for a, b in ev) / 1e3
    del whole
    kern_s = graph_run_s / steps * share / (len(dom_ms) / nprof)
    hbm, src = peaks()
    alg = 16.0 * n * n
    # end to end: host array in, ``steps`` calls, host array out
    e2e_t = []
    for _ in range(runs):
        t0 = time.perf_counter()
        u.now[...] = u0
        for _ in range(steps):
            k(u, c)
        np.asarray(u.now).sum()
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = statistics.median(e2e_t)
    cpu = bounded_steps("diffusion", n, cpu_seconds, steps)
    return {
        "config": f"2-D FTCS diffusion {n}x{n} FP64, u0 ~ U[0,1) seed 0, c = 0.2, zero edges, {steps} steps "
                  f"(one kernel call per step, graph replay per call)",
        "value": lups / run_s / 1e9, "unit": "GLUP/s", "ms_per_run": run_s * 1e3, "steps_per_run": steps,
        "parity": parity, "tilings": tilings,
        "whole_run_graph": {"value": lups / graph_run_s / 1e9, "unit": "GLUP/s", "ms_per_run": graph_run_s * 1e3,
                            "what": f"the {steps} calls captured into one CUDA graph and replayed (no per-call "
                                    f"host work)"},
        "roofline": {"bound": "hbm", "achieved": alg / kern_s / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": alg / kern_s / 1e9 / hbm, "peak_source": src, "kernel_ms": kern_s * 1e3,
                     "kernel_time": "whole-run graph: ms per step x kernel_share / launches per step",
                     "kernel_share": share, "share_source": time_src,
                     "kernel_ms_event_nodes": statistics.mean(dom_ms),
                     "algorithmic_bytes_per_launch": alg,
                     "note": "levels (4 MB) are L2-resident during a run: bound by launch latency, "
                             "not by HBM"},
        "e2e": {"value": lups / e2e_s / 1e9, "unit": "GLUP/s", "h2d_bytes_per_step": n * n * 8,
                "d2h_bytes_per_step": n * n * 8, "ms_per_run": e2e_s * 1e3,
                "step": f"one run of {steps} time steps from a host array to a host array"},
        "cpu_baseline": {"value": n * n * cpu["steps"] / cpu["seconds"] / 1e9, "unit": "GLUP/s",
                         "cores": cpu["cores"], "kind": cpu["kind"],
                         "sample": f"diffusion {n}x{n} FP64, {cpu['steps']} steps ({cpu['seconds']:.2f} s), "
                                   f"OpenMP on all host cores"},
    }


def mixed_section(n: int, steps: int, temporal: int = 4) -> dict:
    """Cavity at n^2 for ``steps`` steps: plain FP64 vs defect iterations with
    FP64 residual/correction (``mixed`` = "fp32", "fp16", "bf16": storage of the
    defect between launches, FP32 arithmetic, ``temporal`` iterations per
    launch), same initial state; steps/s of each (CUDA events over the second
    half of the run; fields exceed L2) and the error of p, u, v against the FP64
    run."""
    import numpy as np
    import torch

    import xgrid
    import workloads
    from xgrid_gb300 import device
    from xgrid_gb300.operator import Operator

    dt = stable_dt(n)
    out, fields, kernels, tuned = {}, {}, {}, {}
    for mode in (None, "fp32", "fp16", "bf16"):
        xgrid.init(precision="double", cacheroot=JIT_CACHE,
                   opt_level=3, mixed=mode, mixed_temporal=temporal)
        k = Operator(workloads.cavity_kernel.func, "kernel", "cavity_kernel")
        grids, cfg = workloads.cavity_setup(n, dt)
        args = (grids["b"], grids["p"], grids["u"], grids["v"], cfg)
        kernels[mode] = (k, args, grids)
        # tile shapes of the launch groups timed on these grids (state restored afterwards)
        from xgrid_gb300 import autotune
        tuned[mode or "fp64"] = {str(g): list(t) for g, t in autotune.tune(k, *args).items()}
        half = steps // 2
        for _ in range(steps - half):
            k(*args)
        s = device.stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(half):
            k(*args)
        e1.record(s)
        s.synchronize()
        ms = e0.elapsed_time(e1) / half
        fields[mode] = {g: grids[g].read(0) for g in "puv"}
        out["fp64" if mode is None else mode] = {"ms_per_step": ms, "steps_per_s": 1e3 / ms,
                                                 "value": SWEEPS_PER_STEP * n * n / (ms * 1e-3) / 1e9,
                                                 "unit": "GLUP/s", "tilings": tuned[mode or "fp64"]}
    # algorithmic bytes per cell and step.  "sweep" counts every pressure iteration as one
    # sweep without temporal reuse (50 FP64 Jacobi sweeps, or residual + 49 defect iterations +
    # correction); "launch" counts what the launches of the mixed path must move at least: the
    # residual, ceil(49 / temporal) defect launches (the first reads r32 and writes d (and the
    # 16-bit r), the others read r and d and write d) and the correction (p in, d in, p out).
    # The FP64 groups of the step (source b with the first p sweep; u, v) come from the module.
    hbm, _ = peaks()
    xgrid.init(precision="double", cacheroot=JIT_CACHE, opt_level=3)
    kp = Operator(workloads.cavity_kernel.func, "kernel", "cavity_kernel")
    from xgrid_gb300.native import NativeKernel
    kp.native = NativeKernel(kp)
    mod = kp.native.module
    outer = algorithmic_bytes(mod, 0) + algorithmic_bytes(mod, 2)
    jac = algorithmic_bytes(mod, 1)
    iters = 49
    nl = -(-iters // max(1, temporal))
    for mode in ("fp64", "fp32", "fp16", "bf16"):
        o = out[mode]
        if mode == "fp64":
            sweep = launch = outer + 50 * jac
        else:
            es = 4 if mode == "fp32" else 2
            sweep = outer + (jac + 4) + iters * 3 * es + (16 + es)
            first = 4 + es + (es if es == 2 else 0)
            launch = outer + (jac + 4) + first + (nl - 1) * 3 * es + (16 + es)
        o["bytes_per_cell_step"] = {"sweep": sweep, "launch": launch}
        o["sweep_gbs"] = sweep * n * n / (o["ms_per_step"] * 1e-3) / 1e9
        o["launch_gbs"] = launch * n * n / (o["ms_per_step"] * 1e-3) / 1e9
        o["launch_hbm_frac"] = o["launch_gbs"] / hbm
    for mode in ("fp32", "fp16", "bf16"):
        err = {}
        for g in "puv":
            a, ref = fields[mode][g], fields[None][g]
            err[g] = {"max_rel": float(np.abs(a - ref).max() / np.abs(ref).max()),
                      "l2_rel": float(np.linalg.norm(a - ref) / np.linalg.norm(ref))}
        out[mode]["error_vs_fp64"] = err
        out[mode]["speedup_vs_fp64"] = out["fp64"]["ms_per_step"] / out[mode]["ms_per_step"]
    # dominant kernels inside the replayed graphs: the plain FP64 Jacobi launch and the
    # temporally blocked FP32 defect launch (12 algorithmic bytes per cell: d and r in, d out)
    hbm_peak, src = peaks()
    rl = {}
    # sites: group 1 (the pressure loop) fused Jacobi launch = 64 + 63, temporal defect launch = 64 + 59
    for mode, tag, bpc, site in ((None, "fp64_jacobi", 24.0, 127), ("fp32", "fp32_defect", 12.0, 123)):
        k, args, _ = kernels[mode]
        by_site, nsteps, time_src = launch_times(k.native, lambda: k(*args))
        if mode is None and 64 + TLOOP_SITE in by_site:
            site = 64 + TLOOP_SITE  # several Jacobi iterations per launch
        if site not in by_site:
            continue
        ms = by_site[site]
        total = sum(sum(v) for v in by_site.values())
        share = sum(ms) / total
        per_step = len(ms) / nsteps
        if site == 64 + TLOOP_SITE:
            bpc = bpc * JACOBI_ITERS / per_step
        ks = out["fp64" if mode is None else mode]["ms_per_step"] * 1e-3 * share / per_step
        rl[tag] = {"bound": "hbm", "achieved": bpc * n * n / ks / 1e9, "peak": hbm_peak, "unit": "GB/s",
                   "frac": bpc * n * n / ks / 1e9 / hbm_peak, "peak_source": src, "kernel_ms": ks * 1e3,
                   "kernel_time": "ms_per_step x kernel_share / launches per step", "site": site,
                   "launches_per_step": per_step, "kernel_share": share, "share_source": time_src,
                   "kernel_ms_event_nodes": statistics.mean(ms), "algorithmic_bytes_per_launch": bpc * n * n,
                   "shares": {str(g): sum(v) / total for g, v in by_site.items()}}
    out["roofline"] = rl
    # end to end through the public API, FP32 mode: u, v, p read back to the host every
    # step and uploaded again by the next call
    k, args, grids = kernels["fp32"]
    for g in "puv":
        grids[g].now  # noqa: B018 - host copies current and authoritative
    e2e_steps = 10
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        k(*args)
        for g in "puv":
            grids[g].now  # noqa: B018
    device.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    lb = n * n * 8
    out["e2e"] = {"value": SWEEPS_PER_STEP * n * n / e2e_s / 1e9, "unit": "GLUP/s", "mode": "fp32",
                  "h2d_bytes_per_step": 3 * lb, "d2h_bytes_per_step": 3 * lb, "ms_per_step": e2e_s * 1e3,
                  "steps": e2e_steps}
    cpu = bounded_steps("cavity", n, 8.0, 3)
    out["cpu_baseline"] = {"value": SWEEPS_PER_STEP * n * n * cpu["steps"] / cpu["seconds"] / 1e9, "unit": "GLUP/s",
                           "steps_per_s": cpu["steps"] / cpu["seconds"], "cores": cpu["cores"], "kind": cpu["kind"],
                           "sample": f"cavity {n}x{n} FP64, {cpu['steps']} steps ({cpu['seconds']:.1f} s) of the "
                                     f"{steps}-step run, extrapolated; OpenMP on all host cores"}
    out["config"] = (f"cavity {n}x{n}, dt={dt:g}, {steps} steps from zero fields; defect iterations in FP32 "
                     f"arithmetic ({temporal} per launch, TMA-staged tiles; fp16/bf16: 16-bit storage with a "
                     f"power-of-two scale per field), FP64 source, residual, correction and projection; one "
                     f"correction per 50-iteration loop")
    return out


def batch_section(count: int, steps: int, seq_steps: int) -> dict:
    """256 periodic FP32 convection-diffusion problems of uneven size: one
    persistent work-queue launch per step (graph over all steps) vs one call per
    problem per step; GLUP/s and GB/s at 8 algorithmic bytes per update."""
    import numpy as np
    import torch

    import xgrid
    import workloads
    from xgrid_gb300 import device
    from xgrid_gb300.operator import Operator

    xgrid.init(precision="float", cacheroot=JIT_CACHE,
               opt_level=3, overstep="wrap")
    k = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    probs = workloads.batch_setup(count, seed=1)
    cells = sum(int(np.prod(p[0].shape)) for p in probs)
    s = device.stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(temporal):
        k.batch(probs, steps, temporal=temporal)  # eager (descriptors, tables)
        k.batch(probs, steps, temporal=temporal)  # capture
        s.synchronize()
        e0.record(s)
        k.batch(probs, steps, temporal=temporal)
        e1.record(s)
        s.synchronize()
        return e0.elapsed_time(e1)

    ms_1 = timed(1)
    t0 = time.perf_counter()
    temporal = k.native.tuned_temporal(probs)
    tune_s = time.perf_counter() - t0
    ms_b = timed(temporal)
    for _ in range(2):
        for args in probs:
            k(*args)
    s.synchronize()
    e0.record(s)
    for _ in range(seq_steps):
        for args in probs:
            k(*args)
    e1.record(s)
    s.synchronize()
    ms_s = e0.elapsed_time(e1) * steps / seq_steps
    hbm, src = peaks()
    out = {"problems": count, "cells": cells, "steps": steps,
           "batched": {"ms": ms_b, "value": cells * steps / (ms_b * 1e-3) / 1e9, "unit": "GLUP/s",
                       "gbs": 8.0 * cells * steps / (ms_b * 1e-3) / 1e9,
                       "temporal": {"depth": temporal[0], "tile": [temporal[1], temporal[2]],
                                    "block": list(temporal[3]), "tuned_in_s": tune_s}},
           "one_step_per_launch": {"ms": ms_1, "value": cells * steps / (ms_1 * 1e-3) / 1e9, "unit": "GLUP/s",
                                   "gbs": 8.0 * cells * steps / (ms_1 * 1e-3) / 1e9},
           "per_problem_calls": {"ms": ms_s, "value": cells * steps / (ms_s * 1e-3) / 1e9, "unit": "GLUP/s",
                                 "timed_steps": seq_steps}}
    out["batched"]["hbm_frac"] = out["batched"]["gbs"] / hbm
    out["one_step_per_launch"]["hbm_frac"] = out["one_step_per_launch"]["gbs"] / hbm
    out["speedup_vs_per_problem"] = ms_s / ms_b
    # the batched kernel: one launch advances every tile ``depth`` steps; algorithmic bytes
    # count 8 per cell and step (read and write one FP32 level), no temporal reuse
    out["roofline"] = {"bound": "hbm", "achieved": out["batched"]["gbs"], "peak": hbm, "unit": "GB/s",
                       "frac": out["batched"]["hbm_frac"], "peak_source": src,
                       "kernel_ms": ms_b / (steps / temporal[0]),
                       "algorithmic_bytes_per_launch": 8.0 * cells * temporal[0],
                       "note": f"whole call = {steps // temporal[0]} launches in one CUDA graph"}
    # end to end: every problem's field from a host array, ``steps`` steps, back to the host
    host0 = [np.array(p[0].read(0)) for p in probs]
    t0 = time.perf_counter()
    for p, h in zip(probs, host0):
        p[0].now[...] = h
    k.batch(probs, steps, temporal=temporal)
    total = 0.0
    for p in probs:
        total += float(np.asarray(p[0].now)[0, 0])
    e2e_s = time.perf_counter() - t0
    out["e2e"] = {"value": cells * steps / e2e_s / 1e9, "unit": "GLUP/s", "h2d_bytes_per_step": 4 * cells,
                  "d2h_bytes_per_step": 4 * cells, "ms": e2e_s * 1e3,
                  "step": f"one call of {steps} steps from host arrays to host arrays"}
    cpu = bounded_steps("convdiff", 0, 10.0, 50)
    out["cpu_baseline"] = {"value": cpu["cells"] * cpu["steps"] / cpu["seconds"] / 1e9, "unit": "GLUP/s",
                           "cores": cpu["cores"], "kind": cpu["kind"],
                           "sample": f"reference C, one call per problem per step, {count} squares of the problems' "
                                     f"cell counts ({cpu['cells']} cells), {cpu['steps']} steps "
                                     f"({cpu['seconds']:.1f} s); timing only (the reference mis-indexes non-square "
                                     f"grids), OpenMP on all host cores"}
    out["config"] = (f"{count} problems, extents U[64,1024] per axis (seed 1), FP32, periodic, convection-diffusion "
                     f"5-point, {steps} steps in one CUDA graph of persistent launches")
    return out


def adjoint_section(n: int, steps: int, every: int, torch_n: int, cpu_n: int = 64) -> dict:
    """3-D variable-coefficient diffusion, FP32, periodic: forward rollout and its
    gradient w.r.t. the initial field and the diffusivity (adjoint kernels; the
    forward pass keeps every state when ``every`` is 1, else a checkpoint every
    ``every`` steps, and the checkpointed variant is timed beside it).  Compared with PyTorch autograd through
    the same stencil on tensors: on the GPU at ``torch_n``^3, and on all host
    cores at ``cpu_n``^3 (the CPU baseline; the reference mis-indexes 3-D grids).
    ``e2e``: host arrays in, loss gradient arrays out."""
    import numpy as np
    import torch

    import xgrid
    import workloads
    from xgrid_gb300 import adjoint, device
    from xgrid_gb300.operator import Operator

    xgrid.init(precision="float", cacheroot=JIT_CACHE,
               opt_level=3, overstep="wrap")
    k = Operator(workloads.diffuse3d.func, "kernel", "diffuse3d")

    def run_ours(m, nsteps, host=False, interval=every):
        u0, kap, tgt, dt = workloads.adjoint_setup(m, 2)
        dev = [torch.tensor(x, device="cuda") for x in (u0, kap, tgt)]
        ro = adjoint.Rollout(k, nsteps, interval)
        a, bb = dev[0].clone().requires_grad_(True), dev[1].clone().requires_grad_(True)
        s = device.stream()
        # warm-up (compile, tables)
        ((ro(a, {"k": bb}, (dt,)) - dev[2]) ** 2).mean().backward()
        torch.cuda.synchronize()
        s.synchronize()
        t0 = time.perf_counter()
        if host:  # from host arrays: upload, rollout, gradient, gradients back to the host
            a = torch.from_numpy(u0).cuda().requires_grad_(True)
            bb = torch.from_numpy(kap).cuda().requires_grad_(True)
            tg = torch.from_numpy(tgt).cuda()
        else:
            a.grad = None
            bb.grad = None
            tg = dev[2]
        uT = ro(a, {"k": bb}, (dt,))
        s.synchronize()
        t1 = time.perf_counter()
        loss = ((uT - tg) ** 2).mean()
        loss.backward()
        if host:
            ga, gk = a.grad.cpu().numpy(), bb.grad.cpu().numpy()
            float(ga[0, 0, 0] + gk[0, 0, 0])
        torch.cuda.synchronize()
        s.synchronize()
        t2 = time.perf_counter()
        return t1 - t0, t2 - t1, float(loss.detach())

    f, bwd, loss = run_ours(n, steps)
    cells = n ** 3
    hbm, src = peaks()
    kept = "every state kept (state pool in HBM)" if every == 1 else f"checkpoint every {every}"
    recomputed = 0 if every == 1 else steps - (steps + every - 1) // every
    out = {"config": f"{n}^3 FP32 periodic, {steps} steps, {kept}, loss MSE to a random target",
           "forward_s": f, "backward_s": bwd, "loss": loss,
           "forward_glups": cells * steps / f / 1e9, "forward_gbs": 12.0 * cells * steps / f / 1e9,
           "backward_glups": cells * steps / bwd / 1e9,
           "state_pool_bytes": steps * 4 * cells if every == 1 else 0,
           "backward_note": f"backward = {recomputed} recomputed forward steps + {steps} adjoint steps "
                            "(24 B/update: read lam, u, k and the gradient of k, write lam and the gradient)"}
    tf, tf_src = profile_traffic("diffuse3d_zstage_fp32", n, dims=3)
    out["roofline"] = {"bound": "hbm", "achieved": out["forward_gbs"], "peak": hbm, "unit": "GB/s",
                       "frac": out["forward_gbs"] / hbm, "peak_source": src, "traffic": tf, "traffic_source": tf_src,
                       "kernel_ms": f / steps * 1e3, "algorithmic_bytes_per_launch": 12.0 * cells,
                       "note": "forward staged z-walk kernel, one launch per step (read u, k; write u)"}
    if every == 1:
        ab = 24.0 * cells * steps / bwd / 1e9
        ta, ta_src = profile_traffic("diffuse3d_zstage_fp32", n, key="adjoint_traffic_bytes_per_launch_", dims=3)
        out["adjoint_roofline"] = {"bound": "hbm", "achieved": ab, "peak": hbm, "unit": "GB/s", "frac": ab / hbm,
                                   "peak_source": src, "kernel_ms": bwd / steps * 1e3, "traffic": ta,
                                   "traffic_source": ta_src, "algorithmic_bytes_per_launch": 24.0 * cells,
                                   "note": "adjoint step kernel; backward time / steps (the backward pass is the "
                                           "adjoint launches only)"}
        cf, cb, _ = run_ours(n, steps, interval=20)
        out["checkpointed"] = {"every": 20, "forward_s": cf, "backward_s": cb,
                               "note": f"{steps - (steps + 19) // 20} recomputed forward steps in the backward pass"}
    fh, bh, _ = run_ours(n, steps, host=True)
    out["e2e"] = {"value": cells * steps / (fh + bh) / 1e9, "unit": "GLUP/s (forward steps / forward+backward time)",
                  "h2d_bytes_per_step": 3 * 4 * cells, "d2h_bytes_per_step": 2 * 4 * cells,
                  "s": fh + bh, "step": f"one rollout of {steps} steps and its gradient, host arrays in and out"}
    # PyTorch autograd through the same stencil on the GPU, smaller grid
    fs, bs, _ = run_ours(torch_n, steps)
    u0, kap, tgt, dt = workloads.adjoint_setup(torch_n, 2)
    u0, kap, tgt = (torch.tensor(x, device="cuda") for x in (u0, kap, tgt))
    torch_autograd_run(u0, kap, tgt, dt, steps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    torch_autograd_run(u0, kap, tgt, dt, steps)
    torch.cuda.synchronize()
    tt = time.perf_counter() - t0
    out["torch_autograd_gpu"] = {"n": torch_n, "fwd_bwd_s": tt, "ours_fwd_bwd_s": fs + bs,
                                 "speedup": tt / (fs + bs)}
    # CPU baseline: torch autograd on all host cores at cpu_n^3, ours at the same size
    fc, bc, _ = run_ours(cpu_n, steps)
    cpu = bounded_steps("adjoint", cpu_n, 10.0, steps)
    per_step_cpu = cpu["seconds"] / cpu["steps"]
    out["cpu_baseline"] = {"value": cpu_n ** 3 / per_step_cpu / 1e9, "unit": "GLUP/s (forward steps / fwd+bwd time)",
                           "cores": cpu["cores"], "kind": cpu["kind"],
                           "sample": f"torch CPU autograd through the same stencil, {cpu_n}^3 FP32, {cpu['steps']} "
                                     f"steps forward + backward ({cpu['seconds']:.1f} s), {cpu['cores']} threads",
                           "ours_same_size_value": cpu_n ** 3 * steps / (fc + bc) / 1e9}
    return out


def algorithmic_bytes(module, group: int) -> float:
    """Bytes per cell of one launch of ``group``: distinct buffers read (not
    produced earlier in the launch) plus distinct buffers written, main sweeps
    only (boundary passes touch O(N) cells)."""
    elem = {i: gt.element.nbytes for i, (_, gt) in enumerate(module.grid_args)}
    read, written = [], []
    for s in module.sweeps:
        if s.group_index != group or not s.is_main:
            continue
        for _, ld in s.loads:
            key = (ld.slot, ld.level, ld.version)
            if key not in written and key not in read:
                read.append(key)
        w = (s.slot, s.level, s.write_version)
        if w not in written:
            written.append(w)
    return float(sum(elem[k[0]] for k in read) + sum(elem[k[0]] for k in written))


def reference_arm(args, rank: int, world: int):
    if rank != 0:
        return None
    n = args.n
    probe = run_cpu("cavity", n, 1)
    per_step = max(1, int(math.ceil(args.cpu_seconds / 10 / max(probe["seconds"], 1e-3))))
    per_step = min(per_step, 5)
    run_cpu("cavity", n, max(1, args.warmup))
    r = run_cpu("cavity", n, args.steps * per_step if args.steps * per_step * probe["seconds"] < 240 else
                max(1, int(240 / max(probe["seconds"], 1e-3))))
    lups = SWEEPS_PER_STEP * n * n * r["steps"]
    val = lups / r["seconds"] / 1e9
    return {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "GLUP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["seconds"] / r["steps"] * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: zero initial fields, lid u=1 (deterministic)",
        "config": {"workload": workload_name(n), "n": n, "sweeps_per_step": SWEEPS_PER_STEP},
        "cpu_baseline": {"value": val, "unit": "GLUP/s", "cores": r["cores"], "kind": r["kind"],
                         "sample": f"cavity {n}x{n} FP64, {r['steps']} steps ({r['seconds']:.1f} s)"},
        "e2e": {"value": val, "unit": "GLUP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse_args()
    if args.cpu_sample:
        print(json.dumps(cpu_sample(args.cpu_workload, args.n, args.cpu_sample)))
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.mode == "kernels":
        kernels_only(args)
        return
    if args.impl == "reference":
        out = reference_arm(args, rank, world)
        if out is not None:
            print(json.dumps(out))
        return
    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    out = gpu_bench(args, rank, world)
    if rank == 0 and not args.no_diffusion:
        out["diffusion"] = diffusion_section(512, 500)
    if rank == 0 and not args.no_mixed:
        out["mixed"] = mixed_section(args.mixed_n, args.mixed_steps, args.mixed_temporal)
    if rank == 0 and not args.no_batch:
        out["batched"] = batch_section(256, args.batch_steps, max(5, args.batch_steps // 50))
    if rank == 0 and not args.no_adjoint:
        out["adjoint"] = adjoint_section(args.adjoint_n, 200, 1, 128)
    if rank == 0:
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(args.n, args.cpu_seconds)
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
