"""Tile autotuner on the GPU: tuning a kernel's launch groups on the caller's
grids leaves their state (every level, the level order) as it found it, picks
one of the candidates for every group, changes no result bit (the tiling only
moves work between CTAs), and a second tuning of the same module, device and
shapes comes from the on-disk cache without timing anything."""
import pytest

import xgrid
import workloads
from xgrid_gb300 import autotune
from xgrid_gb300.codegen import DEFAULT_TILING
from xgrid_gb300.operator import Operator

pytestmark = pytest.mark.gpu


def _state(grids):
    return {g: (grids[g].read(0).tobytes(), grids[g].read(1).tobytes()) for g in "bpuv"}


def test_tune_keeps_state_and_bits(cacheroot, monkeypatch):
    n = 193
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3)
    tuned = Operator(workloads.cavity_kernel.func, "kernel", "cavity_kernel")
    plain = Operator(workloads.cavity_kernel.func, "kernel", "cavity_kernel")
    ga, cfg = workloads.cavity_setup(n, 1e-4)
    gb, _ = workloads.cavity_setup(n, 1e-4)
    a = (ga["b"], ga["p"], ga["u"], ga["v"], cfg)
    b = (gb["b"], gb["p"], gb["u"], gb["v"], cfg)
    for _ in range(2):
        tuned(*a)
        plain(*b)
    before = _state(ga)
    # a key no earlier run has stored: this shape and a fresh cache file
    monkeypatch.setattr(autotune, "CACHE_FILE", "autotune_test.json")
    import os
    path = os.path.join(cacheroot, "autotune_test.json")
    if os.path.exists(path):
        os.remove(path)
    timed = []
    real = autotune._time
    monkeypatch.setattr(autotune, "_time", lambda fn: timed.append(1) or real(fn))
    chosen = autotune.tune(tuned, *a)
    assert timed, "the first tuning timed no candidate"
    assert _state(ga) == before
    groups = tuned.native.module.groups
    assert sorted(chosen) == list(range(groups))
    allowed = set(autotune.group_candidates(2)) | {tuple(DEFAULT_TILING[2])}
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    allowed |= set(autotune.balanced_candidates((n, n), sms))
    for g, t in chosen.items():
        assert tuple(t) in allowed, (g, t)
    for _ in range(3):
        tuned(*a)
        plain(*b)
    for g in "bpuv":
        assert ga[g].read(0).tobytes() == gb[g].read(0).tobytes(), g
    # cached: same choice, nothing timed
    timed.clear()
    again = autotune.tune(tuned, *a)
    assert again == chosen and not timed


def test_tuned_batch_equals_default_batch(cacheroot):
    """The batched path's tuned (depth, tile) against one step per launch: same bits."""
    xgrid.init(precision="float", cacheroot=cacheroot, opt_level=3, overstep="wrap")
    k1 = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    k2 = Operator(workloads.convdiff2d.func, "kernel", "convdiff2d")
    a = workloads.batch_setup(16, 9, 40, 200)
    b = workloads.batch_setup(16, 9, 40, 200)
    k1.batch(a, 1)                      # builds the module
    cfg = autotune.tune_batch(k1.native, a)
    assert cfg in autotune.batch_candidates(False)
    k1.batch(a, 24, temporal=cfg)
    k2.batch(b, 1)
    k2.batch(b, 24, temporal=1)
    for pa, pb in zip(a, b):
        assert pa[0].read(0).tobytes() == pb[0].read(0).tobytes()


@pytest.mark.parametrize("persistent", [False, True])
@pytest.mark.parametrize("tiling", [(1, -76, 128, 32, 8, 1), (1, -7, 64, 64, 4, 1), (1, -257, 32, 32, 8, 1),
                                    (1, 27, 64, 32, 8, 1)])
def test_even_tile_rows_keep_the_bits(cacheroot, tiling, persistent):
    """A tiling moves work between CTAs only: rows of tiles split evenly (given as a
    count, e.g. 76 rows of 3 or 4 cells on 257 rows, or as a least height) and
    columns of tx cells give the default tiling's bits in every level, for fused
    groups and for persistent loop launches."""
    n = 257
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3, persistent=persistent)
    tiled = Operator(workloads.cavity_kernel.func, "kernel", "cavity_kernel")
    plain = Operator(workloads.cavity_kernel.func, "kernel", "cavity_kernel")
    ga, cfg = workloads.cavity_setup(n, 1e-5, seed=3)
    gb, _ = workloads.cavity_setup(n, 1e-5, seed=3)
    a = (ga["b"], ga["p"], ga["u"], ga["v"], cfg)
    b = (gb["b"], gb["p"], gb["u"], gb["v"], cfg)
    tiled(*a)
    plain(*b)
    for g in range(tiled.native.module.groups):
        tiled.native.set_tiling(g, tiling)
    for _ in range(4):
        tiled(*a)
        plain(*b)
    assert _state(ga) == _state(gb)


def test_tuning_fresh_grids_keeps_their_state(cacheroot, monkeypatch):
    """Tuning before the first call (levels not yet on the device, zero or written
    on the host) leaves the grids as a first call finds them: the run that follows
    gives the bits of an untuned run."""
    import os
    n = 129
    xgrid.init(precision="double", cacheroot=cacheroot, opt_level=3)
    monkeypatch.setattr(autotune, "CACHE_FILE", "autotune_fresh.json")
    path = os.path.join(cacheroot, "autotune_fresh.json")
    if os.path.exists(path):
        os.remove(path)
    out = []
    for tune in (True, False):
        k = Operator(workloads.cavity_kernel.func, "kernel", "cavity_kernel")
        grids, cfg = workloads.cavity_setup(n, 1e-4)
        grids["u"].now[5:9, 5:9] = 0.25  # a host-written level next to zero ones
        a = (grids["b"], grids["p"], grids["u"], grids["v"], cfg)
        if tune:
            autotune.tune(k, *a)
        for _ in range(3):
            k(*a)
        out.append(_state(grids))
    assert out[0] == out[1]
