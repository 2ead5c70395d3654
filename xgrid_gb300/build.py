"""Build of the native runtime (libxgrid_gb300.so) with nvcc for sm_103a.

The runtime is compiled in-tree into ``xgrid_gb300/lib/``; generated kernel
modules link against it.  ``ensure_runtime`` rebuilds when a source is newer than
the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "lib")
RUNTIME = os.path.join(LIBDIR, "libxgrid_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
RUNTIME_SOURCES = [os.path.join(CSRC, "xgrid_runtime.cu")]
RUNTIME_DEPS = RUNTIME_SOURCES + [os.path.join(INCLUDE, "xgrid_gb300.h"), os.path.join(CSRC, "xgrid_internal.h")]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build the GB300 backend")
    return path


def _stale(target: str, deps: list) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_runtime(force: bool = False, verbose: bool = False) -> str:
    """Compile libxgrid_gb300.so (C++ host runtime, cudart static)."""
    if not force and not _stale(RUNTIME, RUNTIME_DEPS):
        return RUNTIME
    os.makedirs(LIBDIR, exist_ok=True)
    tmp = RUNTIME + f".{os.getpid()}.tmp"
    cmd = [nvcc(), "-shared", "-Xcompiler", "-fPIC", *ARCH, "-O3", "-lineinfo", "-std=c++17",
           "-I", INCLUDE, "-I", CSRC, *RUNTIME_SOURCES, "-o", tmp]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("failed to build the runtime:\n" + proc.stderr)
    os.replace(tmp, RUNTIME)
    return RUNTIME


def ensure_runtime() -> str:
    return build_runtime(force=False)
