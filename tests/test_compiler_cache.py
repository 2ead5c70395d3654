"""JIT compiler and on-disk module cache (the reference's ``ffi.Compiler`` test,
test.py:80-110, on nvcc): the cache root is created, a source compiles once and
is reused from the md5-named cache (also by a second process), and a source
with a syntax error raises ``Exception`` with the compiler's message."""
import os
import shutil
import subprocess
import sys

import pytest

from xgrid_gb300.compiler import Compiler

pytestmark = pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not available")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SIMPLE = ('#include "xgrid_gen.cuh"\n'
          'extern "C" float universe(float a, float b) { return a + b; }\n'
          '__global__ void branch(int* a) { if (*a) *a = 2; }\n')


def test_cacheroot_created_and_module_reused(tmp_path):
    root = str(tmp_path / "cache")
    cc = Compiler(cacheroot=root)
    assert os.path.isdir(root)
    lib = cc.compile(SIMPLE, ["-O2"])
    stamp = os.path.getmtime(lib)
    assert cc.compile(SIMPLE, ["-O2"]) == lib          # same source and flags: cached
    assert os.path.getmtime(lib) == stamp
    assert cc.compile(SIMPLE, ["-O3"]) != lib          # flags are part of the key
    # a second process finds the same library without compiling
    code = (f"import sys, os; sys.path.insert(0, {ROOT!r}); from xgrid_gb300.compiler import Compiler; "
            f"print(Compiler(cacheroot={root!r}).compile({SIMPLE!r}, ['-O2']))")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, check=True).stdout
    assert out.strip().splitlines()[-1] == lib
    assert os.path.getmtime(lib) == stamp
    import ctypes
    f = ctypes.CDLL(lib).universe
    f.restype, f.argtypes = ctypes.c_float, [ctypes.c_float, ctypes.c_float]
    assert f(1.5, 2.25) == 3.75


def test_syntax_error_raises(tmp_path):
    cc = Compiler(cacheroot=str(tmp_path))
    with pytest.raises(Exception, match="failed to compile"):
        cc.compile("innt main() {}", ["-O2"])
