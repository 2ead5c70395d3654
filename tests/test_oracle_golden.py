"""The numpy oracle reproduces the reference's outputs (golden vectors recorded
from the reference by tests/golden/make_golden.py) bit for bit."""
import json
import os

import numpy as np
import pytest

from loader import load_cases
from oracle import xgrid_oracle

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
INDEX = json.load(open(os.path.join(HERE, "golden_index.json")))
# cases that run C the numpy oracle does not interpret (inline C, C externals,
# macros): the GPU tests compare those with the reference's recording directly
REFERENCE_ONLY = {"c_interop"}


def same_bits(a: np.ndarray, b: np.ndarray) -> bool:
    b = np.asarray(b)
    if a.shape != b.shape:
        return False
    b = b.astype(a.dtype)
    return a.tobytes() == b.tobytes()


@pytest.fixture(scope="module")
def cases(tmp_path_factory):
    return load_cases(xgrid_oracle, str(tmp_path_factory.mktemp("oracle")), "oracle")


@pytest.mark.parametrize("name", sorted(set(INDEX) - REFERENCE_ONLY))
def test_oracle_matches_reference(cases, name):
    assert INDEX[name] == "ok"
    out = cases.CASES[name]()
    ref = np.load(os.path.join(HERE, f"{name}.npz"))
    assert sorted(ref.files) == sorted(out)
    for k in ref.files:
        assert same_bits(ref[k], out[k]), f"{name}:{k}"


def test_time_level_rotation_sequence():
    """a[0] = a[0][-2] + 10 evolves [10,0,0] -> [10,10,0] -> [20,10,10] -> [20,20,10]."""
    seq = np.load(os.path.join(HERE, "time_levels.npz"))["seq"]
    assert seq.tolist() == [[10, 0, 0], [10, 10, 0], [20, 10, 10], [20, 20, 10]]
