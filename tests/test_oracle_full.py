"""The C oracle at the benchmark programs' full sizes against the reference's
own results, pinned as SHA-256 digests of every time level (recorded by
``tests/golden/make_digests.py`` from the reference package): diffusion 512^2
FP64 for 500 steps, the lid-driven cavity 1025^2 FP64 for 5 steps from zero
fields, and the cavity from a seeded random state in every cell of both levels
(1025^2 at the benchmark's dt = 5e-6 for 20 steps, 4097^2 at dt = 5e-7 for 3
steps).  The GPU
tests compare the GPU path with this oracle at the same sizes, so the chain GPU
= oracle = reference holds at full size, not only on the small golden cases."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import native

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DIGESTS = json.load(open(os.path.join(HERE, "full_digests.json")))


def _digests(levels):
    return [hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest() for x in levels]


def test_diffusion_512_500_steps_matches_reference_digests():
    ref = DIGESTS["diffusion_512"]
    field, c = native.diffusion_field(512, seed=0)
    assert repr(c) == ref["c"]
    native.Oracle("port").diffusion(field, c, 500)
    assert _digests(field.levels) == ref["u"]


def test_cavity_1025_5_steps_matches_reference_digests():
    ref = DIGESTS["cavity_1025"]
    n = 1025
    f = native.cavity_fields(n)
    native.Oracle("port").cavity(f, (1.0, 0.1, 1e-5, 2.0 / (n - 1), 2.0 / (n - 1)), 5)
    for k in "bpuv":
        assert _digests(f[k].levels) == ref[k], k


@pytest.mark.parametrize("case,n,dt,steps,seed", [("cavity_1025_seeded", 1025, 5e-6, 20, 7),
                                                   ("cavity_4097_seeded", 4097, 5e-7, 3, 8)])
def test_cavity_seeded_matches_reference_digests(case, n, dt, steps, seed):
    ref = DIGESTS[case]
    f = native.cavity_fields(n, seed)
    before = {k: f[k].levels[0].copy() for k in "puv"}
    native.Oracle("port").cavity(f, (1.0, 0.1, dt, 2.0 / (n - 1), 2.0 / (n - 1)), steps)
    for k in "bpuv":
        assert _digests(f[k].levels) == ref[k], k
    for k in "puv":  # every level finite, and the run changed the interior
        assert all(np.isfinite(x).all() for x in f[k].levels), k
        assert not np.array_equal(f[k].levels[0][1:-1, 1:-1], before[k][1:-1, 1:-1]), k


def test_numpy_oracle_square_periodic_fp32_matches_reference_digests(tmp_path):
    """The batched program's stencil on square periodic FP32 grids (64^2, 257^2,
    512^2 for 200 steps): the numpy oracle runs the same program text as the
    reference did."""
    import sys
    sys.path.insert(0, HERE)
    from loader import load_cases
    from oracle import xgrid_oracle
    mod = load_cases(xgrid_oracle, str(tmp_path), "oracle", "full_cases.py")
    assert mod.FULL["convdiff_square"]() == DIGESTS["convdiff_square"]
