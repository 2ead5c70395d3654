"""Autotuner logic on the CPU: candidate lists are valid launch shapes, the
wave-balanced 2-D candidates fill whole waves of resident CTAs, and the on-disk
cache round-trips (written atomically, merged with earlier keys, unreadable files
ignored)."""
import json
import os

import pytest

from xgrid_gb300 import autotune


@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_group_candidates_are_valid_launches(ndim):
    for tz, ty, tx, bx, by, bz in autotune.group_candidates(ndim):
        assert bx * by * bz <= 256 and bx % 32 == 0
        assert min(tz, ty, tx) >= 1
        if ndim < 3:
            assert tz == 1
        if ndim == 1:
            assert ty == 1


@pytest.mark.parametrize("shape", [(1025, 1025), (2049, 2049), (513, 1537), (4097, 4097)])
@pytest.mark.parametrize("sms", [152, 148, 132])
def test_balanced_candidates_fill_whole_waves(shape, sms):
    """Every candidate's tile count (rows of tiles given as a count, columns of tx
    cells) is exactly k waves of 3, 4 or 6 resident CTAs per SM."""
    Y, X = shape
    cands = autotune.balanced_candidates(shape, sms)
    assert cands, "no balanced candidate"
    for tz, ty, tx, bx, by, bz in cands:
        assert tz == 1 and bz == 1 and (bx, by) in ((32, 8), (64, 4)) and ty < 0 and tx >= bx
        count = (-ty) * (X // tx)
        assert count in {k * sms * per for per in (3, 4, 6) for k in (1, 2)}, (ty, tx, count)


def test_balanced_candidates_for_1025_fill_152_sms():
    # the 1025^2 cavity on 152 SMs x 4 CTAs: 76 rows of 128-column tiles = 608 tiles
    assert (1, -76, 128, 32, 8, 1) in autotune.balanced_candidates((1025, 1025), 152)
    assert autotune.balanced_candidates((1025, 1025, 3), 152) == []
    assert autotune.balanced_candidates((64, 64), 152) == []


def test_batch_candidates_depths_divide_the_tuning_steps():
    for one_dim in (True, False):
        for depth, ty, tx, block in autotune.batch_candidates(one_dim):
            assert autotune.TUNE_STEPS % depth == 0
            assert block[0] * block[1] * block[2] <= 256
            assert tx >= 1 and ty >= 1


def test_cache_round_trip(tmp_path):
    root = str(tmp_path)
    assert autotune._load(root) == {}
    autotune._store(root, "a", [1, 2, 3])
    autotune._store(root, "b", {"0": [1, 64, 32, 32, 8, 1]})
    data = autotune._load(root)
    assert data == {"a": [1, 2, 3], "b": {"0": [1, 64, 32, 32, 8, 1]}}
    assert not [f for f in os.listdir(root) if f.endswith(".tmp")]
    with open(os.path.join(root, autotune.CACHE_FILE), "w") as f:
        f.write("{ not json")
    assert autotune._load(root) == {}
    with open(os.path.join(root, autotune.CACHE_FILE), "w") as f:
        json.dump([1, 2], f)
    assert autotune._load(root) == {}
