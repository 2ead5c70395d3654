"""Build and drive the compiled oracles (test infrastructure only).

* ``libxg_oracle.so`` from ``oracle/c/xg_oracle.c`` (gcc, OpenMP,
  ``-ffp-contract=off``): the C restatement of the benchmark programs.
* ``oracle/_ref/<kernel>.c`` (written by ``make_ref.py`` from the reference's own
  generator) compiled twice with gcc: ``<kernel>.so`` with the reference's flags
  (``-shared -fpic -lm -fopenmp -O3``, xgrid/util/ffi.py:64-70 and
  xgrid/util/init.py:23-32) for timing, and ``<kernel>.exact.so`` with
  ``-ffp-contract=off`` for bit parity on hosts whose gcc contracts
  multiply-adds by default (aarch64).

Drivers rotate time levels before every call exactly as the reference's
``Grid._op_invoke`` (xgrid/xgrid/__init__.py:49-54): the last level moves to the
front and becomes the level that is written.
"""
from __future__ import annotations

import ctypes
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD, "libxg_oracle.so")


def _gcc(src: str, out: str, flags: list) -> None:
    tmp = out + f".{os.getpid()}.tmp"
    cmd = ["gcc", "-shared", "-fpic", *flags, src, "-o", tmp, "-lm"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"gcc failed for {src}:\n{proc.stderr}")
    os.replace(tmp, out)


def build_oracle() -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "c", "xg_oracle.c")
    if not os.path.exists(ORACLE_SO) or os.path.getmtime(src) > os.path.getmtime(ORACLE_SO):
        _gcc(src, ORACLE_SO, ["-O3", "-fopenmp", "-ffp-contract=off"])
    return ORACLE_SO


def build_ref() -> list:
    """Compile the reference's generated C (generating it first when the
    sources are missing and ``XGRID_REFERENCE`` names the reference checkout)."""
    sources = sorted(glob.glob(os.path.join(REF, "*.c")))
    if not sources:
        from . import make_ref
        checkout = make_ref.reference_checkout()
        if checkout:
            sources = make_ref.generate(checkout)
    built = []
    for src in sources:
        base = src[:-2]
        for out, extra in ((base + ".so", []), (base + ".exact.so", ["-ffp-contract=off"])):
            if not os.path.exists(out) or os.path.getmtime(src) > os.path.getmtime(out):
                _gcc(src, out, ["-O3", "-fopenmp", *extra])
            built.append(out)
    return built


def build_all() -> None:
    build_oracle()
    build_ref()


def ref_sources() -> list:
    """The reference's generated C sources written by ``make_ref.py``."""
    return sorted(glob.glob(os.path.join(REF, "*.c")))


def ref_available() -> bool:
    return all(os.path.exists(os.path.join(REF, k + ".so")) for k in ("diffusion2d", "cavity_kernel", "convdiff2d"))


# ------------------------------------------------------------------ drivers
class CavityConfig(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("rho", "nu", "dt", "dx", "dy")]


class RefGrid2d(ctypes.Structure):
    """``struct __Grid2d_d`` of the reference's generated C (generator.py:158-165)."""

    _fields_ = [("time", ctypes.c_int32), ("shape", ctypes.c_int32 * 2),
                ("data", ctypes.POINTER(ctypes.POINTER(ctypes.c_double))),
                ("boundary_mask", ctypes.POINTER(ctypes.c_int32))]


class RefGrid2dF(ctypes.Structure):
    """``struct __Grid2d_f`` of the reference's generated C (FP32 levels)."""

    _fields_ = [("time", ctypes.c_int32), ("shape", ctypes.c_int32 * 2),
                ("data", ctypes.POINTER(ctypes.POINTER(ctypes.c_float))),
                ("boundary_mask", ctypes.POINTER(ctypes.c_int32))]


_DP = ctypes.POINTER(ctypes.c_double)
_FP = ctypes.POINTER(ctypes.c_float)
_IP = ctypes.POINTER(ctypes.c_int32)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def _ip(a: np.ndarray):
    return a.ctypes.data_as(_IP)


class Field:
    """Two time levels and a mask, rotated like the reference's Grid."""

    def __init__(self, level0: np.ndarray, mask: np.ndarray, level1=None) -> None:
        self.levels = [np.ascontiguousarray(level0, dtype=np.float64).copy(),
                       np.zeros_like(level0, dtype=np.float64) if level1 is None
                       else np.ascontiguousarray(level1, dtype=np.float64).copy()]
        self.mask = np.ascontiguousarray(mask, dtype=np.int32)
        self._ptrs = None

    def tick(self) -> None:
        self.levels.insert(0, self.levels.pop())

    def ref_struct(self) -> RefGrid2d:
        g = RefGrid2d()
        g.time = len(self.levels)
        g.shape[0], g.shape[1] = self.levels[0].shape
        self._ptrs = (_DP * len(self.levels))(*[_dp(x) for x in self.levels])
        g.data = ctypes.cast(self._ptrs, ctypes.POINTER(_DP))
        g.boundary_mask = _ip(self.mask)
        return g


class Field32:
    """Two FP32 time levels and a mask (the batched program), rotated like Field."""

    def __init__(self, level0: np.ndarray, mask=None) -> None:
        level0 = np.ascontiguousarray(level0, dtype=np.float32)
        self.levels = [level0.copy(), np.zeros_like(level0)]
        self.mask = np.zeros(level0.shape, np.int32) if mask is None else np.ascontiguousarray(mask, np.int32)
        self._ptrs = None

    def tick(self) -> None:
        self.levels.insert(0, self.levels.pop())

    def ref_struct(self) -> RefGrid2dF:
        g = RefGrid2dF()
        g.time = len(self.levels)
        g.shape[0], g.shape[1] = self.levels[0].shape
        self._ptrs = (_FP * len(self.levels))(*[x.ctypes.data_as(_FP) for x in self.levels])
        g.data = ctypes.cast(self._ptrs, ctypes.POINTER(_FP))
        g.boundary_mask = _ip(self.mask)
        return g


def convdiff_reference(exact: bool = False):
    """The reference's generated C of the batched program (FP32, periodic):
    ``fn(Field32, (a0, axm, axp, aym, ayp), steps)``.  Square grids only: the
    reference strides non-square grids by the wrong extent."""
    path = os.path.join(REF, "convdiff2d" + (".exact.so" if exact else ".so"))
    if not os.path.exists(path):
        build_ref()
    lib = ctypes.CDLL(path)
    lib.convdiff2d.argtypes = [RefGrid2dF] + [ctypes.c_float] * 5
    lib.convdiff2d.restype = None

    def run(field: Field32, coeffs, steps: int) -> None:
        for _ in range(steps):
            field.tick()
            lib.convdiff2d(field.ref_struct(), *coeffs)
    return run


class Oracle:
    """C restatement (``kind='port'``) or the reference's generated C
    (``kind='reference'``, ``exact`` selects the no-contraction build)."""

    def __init__(self, kind: str = "port", exact: bool = True) -> None:
        self.kind = kind
        if kind == "port":
            self.lib = ctypes.CDLL(build_oracle())
            self.lib.xo_diffusion_step.argtypes = [_DP, _DP, _IP, ctypes.c_int, ctypes.c_double]
            self.lib.xo_diffusion_step.restype = None
            self.lib.xo_cavity_step.argtypes = [_DP, _DP, _DP, _DP, _DP, _DP, _DP, _IP, _IP, _IP, _IP, ctypes.c_int,
                                                CavityConfig, _DP]
            self.lib.xo_cavity_step.restype = None
        elif kind == "reference":
            if not ref_available():
                build_ref()
            suffix = ".exact.so" if exact else ".so"
            self.diff = ctypes.CDLL(os.path.join(REF, "diffusion2d" + suffix))
            self.diff.diffusion2d.argtypes = [RefGrid2d, ctypes.c_double]
            self.diff.diffusion2d.restype = None
            self.cav = ctypes.CDLL(os.path.join(REF, "cavity_kernel" + suffix))
            self.cav.cavity_kernel.argtypes = [RefGrid2d, RefGrid2d, RefGrid2d, RefGrid2d, CavityConfig]
            self.cav.cavity_kernel.restype = None
        else:
            raise ValueError(kind)
        self._scratch = None

    def diffusion(self, u: Field, c: float, steps: int) -> None:
        n = u.levels[0].shape[0]
        for _ in range(steps):
            u.tick()
            if self.kind == "port":
                self.lib.xo_diffusion_step(_dp(u.levels[0]), _dp(u.levels[1]), _ip(u.mask), n, c)
            else:
                self.diff.diffusion2d(u.ref_struct(), c)

    def cavity(self, f: dict, cfg: tuple, steps: int) -> None:
        n = f["u"].levels[0].shape[0]
        g = CavityConfig(*cfg)
        if self._scratch is None or self._scratch.shape != (n, n):
            self._scratch = np.zeros((n, n))
        for _ in range(steps):
            for k in "bpuv":
                f[k].tick()
            if self.kind == "port":
                self.lib.xo_cavity_step(_dp(f["b"].levels[0]), _dp(f["p"].levels[0]), _dp(f["p"].levels[1]),
                                        _dp(f["u"].levels[0]), _dp(f["u"].levels[1]), _dp(f["v"].levels[0]),
                                        _dp(f["v"].levels[1]), _ip(f["b"].mask), _ip(f["p"].mask), _ip(f["u"].mask),
                                        _ip(f["v"].mask), n, g, _dp(self._scratch))
            else:
                self.cav.cavity_kernel(f["b"].ref_struct(), f["p"].ref_struct(), f["u"].ref_struct(),
                                       f["v"].ref_struct(), g)


def cavity_fields(n: int, seed=None) -> dict:
    """Cavity grids with the benchmark's masks: zero fields, or both levels from
    ``workloads.cavity_state(n, seed)``."""
    import workloads
    masks = workloads.cavity_masks(n)
    if seed is None:
        return {k: Field(np.zeros((n, n)), masks[k]) for k in "bpuv"}
    state = workloads.cavity_state(n, seed)
    return {k: Field(state[k][0], masks[k], state[k][1]) for k in "bpuv"}


def diffusion_field(n: int = 512, seed: int = 0) -> tuple:
    mask = np.zeros((n, n), dtype=np.int32)
    mask[0, :] = mask[-1, :] = mask[:, 0] = mask[:, -1] = 1
    nu = 0.1
    dx = 1.0 / (n - 1)
    dt = 0.2 * dx * dx / nu
    c = nu * dt / (dx * dx)
    return Field(np.random.default_rng(seed).random((n, n)), mask), c
