"""The C restatement of the benchmark programs agrees with the numpy oracle
and with the reference's own generated C (when it has been generated here)."""
import os

import numpy as np
import pytest

from oracle import native

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_c_oracle_cavity_matches_golden():
    g = np.load(os.path.join(HERE, "cavity_small.npz"))
    f = native.cavity_fields(33)
    native.Oracle("port").cavity(f, (1.0, 0.1, 1e-3, 2 / 32, 2 / 32), 10)
    for k in "bpuv":
        assert np.stack(f[k].levels).tobytes() == g[k].tobytes()


def test_c_oracle_diffusion_matches_golden():
    g = np.load(os.path.join(HERE, "diffusion_small.npz"))["u"]
    u0 = np.random.default_rng(0).random((64, 64))
    mask = np.zeros((64, 64), dtype=np.int32)
    mask[0, :] = mask[-1, :] = mask[:, 0] = mask[:, -1] = 1
    field = native.Field(u0, mask)
    native.Oracle("port").diffusion(field, 0.2, 20)
    assert np.stack(field.levels).tobytes() == g.tobytes()


@pytest.mark.skipif(not (native.ref_available() or native.ref_sources()),
                    reason="the reference's generated C is not present (oracle/make_ref.py writes it)")
@pytest.mark.parametrize("n,steps", [(65, 4), (129, 2)])
def test_c_oracle_matches_reference_generated_c(n, steps):
    out = []
    for kind in ("port", "reference"):
        f = native.cavity_fields(n)
        native.Oracle(kind).cavity(f, (1.0, 0.1, 1e-4, 2 / (n - 1), 2 / (n - 1)), steps)
        out.append(f)
    for k in "bpuv":
        assert out[0][k].levels[0].tobytes() == out[1][k].levels[0].tobytes()


@pytest.mark.skipif(not (native.ref_available() or native.ref_sources()),
                    reason="the reference's generated C is not present (oracle/make_ref.py writes it)")
def test_reference_generated_convdiff_matches_reference_digests():
    """The batched program's reference C (the CPU baseline of the batched workload)
    reproduces the reference package's own digests on square periodic FP32 grids."""
    import hashlib
    import json
    dig = json.load(open(os.path.join(HERE, "full_digests.json")))["convdiff_square"]
    rng = np.random.default_rng(5)
    run = native.convdiff_reference(exact=True)
    for n in (64, 257, 512):
        cx, cy = (float(v) for v in rng.uniform(-1.0, 1.0, 2))
        nu = float(rng.uniform(0.01, 0.1))
        dx = 1.0 / n
        dt = 0.2 * dx * dx / nu
        gx, gy = 0.5 * cx * dt / dx, 0.5 * cy * dt / dx
        k = nu * dt / (dx * dx)
        f = native.Field32(rng.random((n, n)).astype(np.float32))
        run(f, (1.0 - 4.0 * k, gx + k, k - gx, gy + k, k - gy), 200)
        assert [hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest() for x in f.levels] == dig[f"u{n}"]
