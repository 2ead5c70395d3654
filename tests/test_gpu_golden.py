"""GPU path vs the reference's golden vectors: bit-exact for every case
(integer grids and FP64/FP32 with multiply-add contraction disabled)."""
import json
import os

import numpy as np
import pytest

import xgrid
from loader import load_cases

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
INDEX = json.load(open(os.path.join(HERE, "golden_index.json")))

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cases(cacheroot):
    return load_cases(xgrid, cacheroot, "gpu")


@pytest.mark.parametrize("name", sorted(INDEX))
def test_gpu_matches_reference(cases, name):
    out = cases.CASES[name]()
    ref = np.load(os.path.join(HERE, f"{name}.npz"))
    assert sorted(ref.files) == sorted(out)
    for k in ref.files:
        a, b = ref[k], np.asarray(out[k]).astype(ref[k].dtype)
        assert a.shape == b.shape, f"{name}:{k} shape {a.shape} vs {b.shape}"
        if a.tobytes() != b.tobytes():
            diff = np.abs(a.astype(float) - b.astype(float))
            idx = np.unravel_index(np.argmax(diff), diff.shape)
            pytest.fail(f"{name}:{k} differs at {idx}: ref {a[idx]!r} gpu {b[idx]!r} (max |diff| {diff.max():.3e}, "
                        f"{int((diff > 0).sum())} cells)")
