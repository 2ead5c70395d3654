"""Autotuner: tile shape and temporal-block depth per stencil, shape and dtype.

The reference has no tuner (its generated C is one OpenMP loop per sweep,
xgrid/lang/generator.py:289-361); on the GPU the tile shape of a sweep group and
the number of steps a batched launch advances (temporal blocking) decide the
speed, and the best choice depends on the stencil, the grid shapes and the
element type.  Both tuners time candidates on the caller's own data and leave
it untouched:

* the grids' time levels (device copies and the level order) are saved before
  the first candidate and restored after the last, so a tuned call gives the
  same bits as an untuned one;
* every candidate is timed with CUDA events on the backend stream, after a
  warm-up call that also captures its CUDA graph; the best of a few repetitions
  counts;
* results are cached in ``<cacheroot>/autotune.json`` under a key made of the
  compiled module (its md5-named file: stencil, dtype and compiler flags), the
  device name and the grid shapes, so a later process reuses them without timing.

``tune_batch`` picks ``(depth, ty, tx, block)`` of the batched path
(``kernel.batch``); ``tune`` picks ``(tz, ty, tx, block)`` of every launch group
of a kernel called once per step.
"""
from __future__ import annotations

import hashlib
import json
import os

from . import device
from .log import Logger

logger = Logger("autotune")

CACHE_FILE = "autotune.json"
TUNE_STEPS = 24        # steps per timed batched call: divisible by every candidate depth
REPEATS = 2


# ------------------------------------------------------------------ cache
def _cache_path(cacheroot: str) -> str:
    return os.path.join(cacheroot, CACHE_FILE)


def _load(cacheroot: str) -> dict:
    try:
        with open(_cache_path(cacheroot)) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def _store(cacheroot: str, key: str, value) -> None:
    os.makedirs(cacheroot, exist_ok=True)
    data = _load(cacheroot)
    data[key] = value
    tmp = _cache_path(cacheroot) + f".{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, _cache_path(cacheroot))


def _key(native, kind: str, shapes) -> str:
    t = device.torch()
    name = t.cuda.get_device_name() if t.cuda.is_available() else "nodevice"
    h = hashlib.md5(repr(sorted(shapes)).encode()).hexdigest()
    return f"{kind}:{os.path.basename(native.path)}:{name}:{h}"


# --------------------------------------------------------------- snapshot
class Snapshot:
    """Device copies and level order of some grids, restorable."""

    def __init__(self, grids) -> None:
        t = device.torch()
        self.saved = []
        with t.cuda.stream(device.stream()):
            for g in grids:
                levels = list(g._levels)
                copies = [(lv, lv.dev.clone() if lv.dev is not None else None, lv.auth) for lv in levels]
                self.saved.append((g, levels, copies))

    def restore(self) -> None:
        t = device.torch()
        with t.cuda.stream(device.stream()):
            for g, levels, copies in self.saved:
                g._levels[:] = levels
                for lv, copy, auth in copies:
                    if copy is not None:
                        lv.dev.copy_(copy)
                        lv.auth = auth
                    elif lv.dev is not None and auth == "zero":
                        # a level that had no device buffer and was zero: the timed calls
                        # allocated and wrote one; zero it and let it stand for the level
                        lv.dev.zero_()
                        lv.auth = "dev"
                    else:
                        lv.auth = auth  # "host": the host copy is uploaded at the next call
        device.stream().synchronize()


def _time(fn) -> float:
    """Best of ``REPEATS`` timed calls (ms) after one warm-up call."""
    t = device.torch()
    s = device.stream()
    fn()
    best = float("inf")
    for _ in range(REPEATS):
        e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
        s.synchronize()
        e0.record(s)
        fn()
        e1.record(s)
        s.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


# ---------------------------------------------------------------- batched
def batch_candidates(one_dim: bool) -> list:
    """(depth, ty, tx, block) candidates of the batched path (depth 1: one step per launch)."""
    if one_dim:
        out = [(1, 1, 256, (256, 1, 1))]
        for d in (2, 4, 6, 8, 12):
            for tx in (512, 1024, 2048):
                out.append((d, 1, tx - 2 * d, (256, 1, 1)))
        return out
    out = [(1, 32, 64, (32, 8, 1))]
    for d in (2, 3, 4, 6, 8):
        for ty, tx, block in ((16, 64, (32, 8, 1)), (32, 64, (32, 8, 1)), (32, 128, (32, 8, 1)),
                              (64, 64, (32, 8, 1)), (32, 128, (64, 4, 1)), (64, 128, (32, 8, 1))):
            out.append((d, ty, tx - 2 * d, block))
    return out


def tune_batch(native, problems, candidates=None) -> tuple:
    """Time the candidates on ``problems`` and return the fastest configuration
    (cached per module, device and problem shapes)."""
    from .config import get_config
    cfg = get_config()
    grids = []
    shapes = []
    for args in problems:
        gs, _ = native.split(tuple(args))
        grids.extend(gs)
        shapes.append(tuple(g.shape for g in gs))
    key = _key(native, "batch", shapes)
    hit = _load(cfg.cacheroot).get(key)
    if hit is not None:
        return (int(hit[0]), int(hit[1]), int(hit[2]), tuple(int(b) for b in hit[3]))
    one_dim = all(len(s[0]) == 1 for s in shapes)
    cands = candidates if candidates is not None else batch_candidates(one_dim)
    snap = Snapshot(grids)
    results = []
    try:
        for c in cands:
            try:
                ms = _time(lambda: native.batch(problems, TUNE_STEPS, temporal=c))
            except Exception as err:  # a candidate the device cannot run (shared memory) is skipped
                logger.info(f"candidate {c} skipped: {err}")
                continue
            results.append((ms, c))
    finally:
        snap.restore()
    if not results:
        logger.dead("autotune: no batched candidate ran")
    ms, best = min(results, key=lambda r: r[0])
    logger.info(f"batched {native.module.name}: depth {best[0]}, tile {best[1]}x{best[2]}, block {best[3]} "
                f"({ms / TUNE_STEPS * 1e3:.1f} us/step)")
    _store(cfg.cacheroot, key, [best[0], best[1], best[2], list(best[3]),
                                {"us_per_step": ms / TUNE_STEPS * 1e3}])
    return best


# ------------------------------------------------------------ single calls
def balanced_candidates(shape, sms: int) -> list:
    """2-D tilings whose tile count is a whole number of waves, k x SMs x (3, 4 or 6
    resident CTAs per SM, the tile kernels' occupancies), with tiles of equal work:
    x tiles of 32 to 256 columns (the last one absorbs the remainder, a column or
    two on 2^n + 1 grids) and a tile count along y given directly (a negative ty),
    y being split evenly.  Power-of-two tiles of a 2^n + 1 grid give 2^m tiles,
    which never fill 152 x 4 slots (1025^2 with 64 x 32 tiles: 512 tiles, 84 % of
    one wave)."""
    if len(shape) != 2 or sms <= 0:
        return []
    Y, X = shape
    out = []
    for per_sm in (3, 4, 6):
        for tx in (32, 64, 128, 256):
            nx = X // tx
            if nx < 1:
                continue
            for k in (1, 2):
                target = k * sms * per_sm
                if target % nx or not 1 <= target // nx <= Y:
                    continue
                for block in ((32, 8, 1), (64, 4, 1)):
                    if block[0] > tx:
                        continue
                    c = (1, -(target // nx), tx, *block)
                    if c not in out:
                        out.append(c)
    return out


def group_candidates(ndim: int) -> list:
    """(tz, ty, tx, block.x, block.y, block.z) candidates of a launch group."""
    if ndim == 1:
        return [(1, 1, tx, b, 1, 1) for tx in (256, 512, 1024, 2048, 4096) for b in (128, 256) if tx >= b]
    if ndim == 2:
        out = [(1, ty, tx, 32, 8, 1) for tx in (32, 64, 128) for ty in (8, 16, 32, 64)]
        out += [(1, ty, tx, 64, 4, 1) for tx in (64, 128) for ty in (16, 32, 64)]
        return out
    # 3-D: tall tiles for the z-walk of mask-free 7-point sweeps, flat ones for the generic loop
    out = [(tz, ty, tx, 32, 8, 1) for tz, ty, tx in
           ((1, 8, 32), (1, 16, 32), (2, 16, 32), (4, 8, 32), (32, 8, 32), (64, 8, 32))]
    out += [(tz, 4, 64, 64, 4, 1) for tz in (16, 32, 64, 128)]
    return out


def tune(op, *args, calls: int = 2) -> dict:
    """Pick the tile shape of every launch group of kernel ``op`` for these
    arguments (one group at a time, the others at their current tiling) and
    apply it; returns {group: tiling}."""
    from .config import get_config
    from .native import NativeKernel
    cfg = get_config()
    if op.native is None:
        op.native = NativeKernel(op)
    nk = op.native
    grids, _ = nk.split(args)
    key = _key(nk, "groups", [tuple(g.shape for g in grids)])
    hit = _load(cfg.cacheroot).get(key)
    groups = list(range(nk.module.groups))
    if hit is not None:
        chosen = {int(g): tuple(t) for g, t in hit.items()}
        for g, t in chosen.items():
            nk.set_tiling(g, t)
        return chosen
    ndim = max(len(g.shape) for g in grids)
    t = device.torch()
    sms = t.cuda.get_device_properties(t.cuda.current_device()).multi_processor_count
    cands = group_candidates(ndim)
    if ndim == 2:
        cands += [c for c in balanced_candidates(max((g.shape for g in grids), key=lambda s: s[0] * s[1]), sms)
                  if c not in cands]
    snap = Snapshot(grids)
    chosen = {}

    def run():
        for _ in range(calls):
            op(*args)
    try:
        for g in groups:
            base = nk._tiling_key(g)
            results = []
            for c in [base] + [c for c in cands if c != base]:
                nk.set_tiling(g, c)
                try:
                    results.append((_time(run), c))
                except Exception as err:
                    logger.info(f"group {g} tiling {c} skipped: {err}")
            ms, best = min(results, key=lambda r: r[0])
            nk.set_tiling(g, best)
            chosen[g] = tuple(best)
    finally:
        snap.restore()
    _store(cfg.cacheroot, key, {str(g): list(t) for g, t in chosen.items()})
    logger.info(f"{nk.module.name}: tilings {chosen}")
    return chosen
