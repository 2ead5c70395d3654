"""nvcc driver with an md5-keyed cache, and the ctypes loader of kernel modules.

Mirrors the reference's ``Compiler``/``Library`` (xgrid/util/ffi.py:13-94):
the command line is written as the first line of ``<cacheroot>/<md5>.cu``, the
library ``<md5>.cu.so`` is reused when the cached source matches exactly, and a
failed compile raises with the compiler's stderr.  The compiler is nvcc for
sm_103a and the module links against the runtime library.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
import threading

from . import build
from .log import Logger

_lock = threading.Lock()


def _header_digest() -> str:
    h = hashlib.md5()
    for p in (os.path.join(build.CSRC, "xgrid_gen.cuh"), os.path.join(build.CSRC, "xgrid_internal.h"),
              os.path.join(build.INCLUDE, "xgrid_gb300.h")):
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


class Compiler:
    """Compiles generated CUDA sources into shared objects under ``cacheroot``."""

    def __init__(self, *, cacheroot: str) -> None:
        self.logger = Logger(self)
        self.cacheroot = os.path.join(".", cacheroot) if not os.path.isabs(cacheroot) else cacheroot
        os.makedirs(self.cacheroot, exist_ok=True)
        self.nvcc = build.nvcc()

    def command(self, flags: list) -> list:
        runtime_dir = build.LIBDIR
        return [self.nvcc, "-shared", "-Xcompiler", "-fPIC", *build.ARCH, "-lineinfo", "-std=c++17",
                "-w", "-I", build.INCLUDE, "-I", build.CSRC, *flags,
                "-L", runtime_dir, "-lxgrid_gb300", "-Xlinker", f"-rpath,{runtime_dir}"]

    def compile(self, source: str, flags: list) -> str:
        build.ensure_runtime()
        args = self.command(flags)
        text = f"// {' '.join(args)}\n// headers {_header_digest()}\n" + source
        name = os.path.join(self.cacheroot, hashlib.md5(text.encode()).hexdigest() + ".cu")
        lib = name + ".so"
        with _lock:
            cached = False
            if os.path.exists(name) and os.path.exists(lib):
                with open(name) as f:
                    cached = f.read() == text
            if not cached:
                with open(name, "w") as f:
                    f.write(text)
                tmp = lib + f".{os.getpid()}.tmp"
                proc = subprocess.run(args + [name, "-o", tmp], capture_output=True, text=True)
                if proc.returncode != 0:
                    self.logger.dead(f"failed to compile '{name}' due to:", proc.stderr)
                os.replace(tmp, lib)
        self.logger.info(f"jit compiled '{name}' {'with' if cached else 'without'} cache to '{lib}'")
        return lib


class Library:
    """A loaded kernel module."""

    def __init__(self, path: str) -> None:
        self.logger = Logger(self)
        from . import runtime
        runtime.load()  # the module links against the runtime library
        self.path = path
        self.dylib = ctypes.CDLL(path)

    def entry(self, symbol: str):
        fn = getattr(self.dylib, symbol, None)
        if fn is None:
            self.logger.dead(f"failed to get function '{symbol}'")
        return fn
