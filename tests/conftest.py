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
def cacheroot(tmp_path_factory):
    return str(tmp_path_factory.mktemp("xgcache"))
