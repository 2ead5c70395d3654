import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the generated CUDA kernels")


@pytest.fixture(scope="session")
def cacheroot():
    """Cache root of the kernel modules the tests compile: inside the tree, so the
    loaded modules are the repository's own (md5-named, safe to share between runs)."""
    path = os.path.join(ROOT, ".xgrid_cache", "tests")
    os.makedirs(path, exist_ok=True)
    return path
