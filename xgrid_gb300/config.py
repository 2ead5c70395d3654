"""Global configuration set by ``xgrid.init``.

Keyword signature and defaults follow xgrid/util/init.py:48-66 (``parallel``, ``cc``,
``cacheroot``, ``comment``, ``overstep``, ``opt_level``, ``precision``).  The GPU
backend keeps their meaning where one exists:

* ``precision`` decides the width of ``float`` at parse time (4 or 8 bytes), as in
  the reference (xgrid/util/init.py:34-36, xgrid/util/typing/annotation.py:41-42).
* ``overstep`` selects neighbour addressing at the domain edge: ``none`` (row-major
  flattened offset, reads outside the allocation return 0), ``limit`` (clamp) or
  ``wrap`` (periodic).
* ``opt_level`` maps to ``nvcc -O``; ``cacheroot`` holds the md5-keyed ``.cu``/``.so``.
* ``parallel`` and ``cc`` are accepted and ignored: every sweep runs on the GPU.

Backend options (new keywords, all optional):

* ``exact``: ``True`` compiles device code with ``--fmad=false`` and host code with
  ``-ffp-contract=off`` so FP64 results are bit-identical to the reference's C
  backend; ``False`` lets the compilers contract multiply-adds (results within
  1e-12 relative of the exact path).
* ``mixed``: ``None`` (plain), ``"fp32"``, ``"fp16"`` or ``"bf16"``: run the
  iterations of affine in-place (Jacobi) loops on a defect field with FP32
  arithmetic and FP64 residual and correction passes (see ``xgrid_gb300.mixed``).
  ``"fp16"`` and ``"bf16"`` store the defect and the residual between launches
  in 16 bits with a power-of-two scale per field.
* ``mixed_temporal``: defect iterations per launch of the temporally blocked
  defect kernel (TMA-staged tile + halo in shared memory; default 8, the fastest
  of 4/6/8 measured on a GB300 at 4097^2); 0 runs one iteration per launch
  without shared-memory staging (FP32 storage).
* ``mixed_rows``: rows per warp of that kernel (4 or 8; the box is 128 columns
  by eight times this many rows, halo included).
* ``int_adds``: every n-th FP64 addition or subtraction of a sweep runs as an
  exact round-to-nearest integer-pipe routine instead of the FP64 unit (0: none,
  1: all); the results are the same bits, only the pipe balance changes.
* ``persistent``: run an in-place loop whose body is one launch group (an
  implicit main sweep of a grid and its boundary sweeps, e.g. Jacobi iterations)
  as one cooperative launch in which each tile waits only for its neighbouring
  tiles' previous iteration (per-tile completion flags), instead of one launch
  per iteration; same arithmetic, same bits.  Calls of one module with this
  option must not overlap on the GPU (the flags are a module-wide array).
* ``loop_temporal``: iterations per launch of an in-place loop of that kind on
  2-D grids under overstep "none" whose level fits in a quarter of L2 (boxes of
  the grid staged in shared memory with a halo of that many cells, recomputed per
  iteration; ``xgrid_gb300.tloop``; default 3, the fastest of 2/3/4 measured on a
  GB300 for the 1025^2 cavity); 0 or 1: one launch per iteration.  Same arithmetic per cell, same bits; applies
  only when the box check proves every read exact, else one launch per
  iteration.
* ``fail_waits``: for testing only.  Compile modules whose give-up waits cannot
  succeed (the neighbour-tile wait of a persistent loop polls once; a TMA
  staging barrier expects more bytes than its copies deliver), so that those waits run
  out: the kernel sets its error word and returns, after draining its copies.
  Results of such modules are invalid by construction.
* ``graph``: capture each distinct kernel call into a CUDA graph and replay it.
* ``fuse``: fuse consecutive sweeps into one launch where the masks allow it.
* ``divisor``: precompute loop-invariant divisors on the host and divide with a
  correctly rounded multiply/FMA sequence (checked per divisor).
* ``autotune``: pick the batched path's temporal-block depth and tile shape by
  timing candidates on the first call for a set of problem shapes (cached on disk
  in ``cacheroot``; see ``xgrid_gb300.autotune``).
"""
from __future__ import annotations

import dataclasses
import sys
from typing import Literal, Optional

from .log import Logger

logger = Logger("xgrid")

_OVERSTEP = ("none", "limit", "wrap")
_PRECISION = ("float", "double")
_MIXED = (None, "fp32", "fp16", "bf16")
MIXED_ROWS = (4, 8)


@dataclasses.dataclass
class Configuration:
    parallel: bool
    cc: list
    cacheroot: str
    comment: bool
    overstep: Literal["none", "limit", "wrap"]
    opt_level: Literal[0, 1, 2, 3]
    precision: Literal["float", "double"]
    exact: bool = True
    mixed: Optional[str] = None
    graph: bool = True
    fuse: bool = True
    divisor: bool = True
    mixed_every: int = 0
    autotune: bool = True
    mixed_temporal: int = 8
    mixed_rows: int = 8
    int_adds: int = 0
    persistent: bool = False
    fail_waits: bool = False
    loop_temporal: int = 3

    def __repr__(self) -> str:
        return repr(dataclasses.asdict(self))

    @property
    def fsize(self) -> int:
        return 4 if self.precision == "float" else 8

    @property
    def nvcc_flags(self) -> list[str]:
        flags = [f"-O{self.opt_level}"]
        if self.exact:
            flags += ["--fmad=false", "-Xcompiler", "-ffp-contract=off"]
        if self.fail_waits:
            flags.append("-DXG_FAIL_WAITS")
        return flags


_config: Configuration | None = None


def get_config() -> Configuration:
    if _config is None:
        logger.dead("Please call init first to initialize")
    return _config


def init(*, parallel: bool = True, cc: list = ["gcc", "clang"], cacheroot: str = ".xgrid",
         comment: bool = False, overstep: Literal["none", "limit", "wrap"] = "none",
         opt_level: Literal[0, 1, 2, 3] = 2, precision: Literal["float", "double"] = "float",
         exact: bool = True, mixed: Optional[str] = None, graph: bool = True,
         fuse: bool = True, divisor: bool = True, mixed_every: int = 0, autotune: bool = True,
         mixed_temporal: int = 8, mixed_rows: int = 8, int_adds: int = 0, persistent: bool = False,
         fail_waits: bool = False, loop_temporal: int = 3) -> None:
    """Set the global configuration (same keywords as the reference plus GPU options)."""
    global _config
    if sys.version_info < (3, 10):
        logger.fail(f"Minimum Python 3.10 is required, current version is {sys.version_info}")
    if overstep not in _OVERSTEP:
        logger.dead(f"Invalid overstep '{overstep}', expected one of {_OVERSTEP}")
    if precision not in _PRECISION:
        logger.dead(f"Invalid precision '{precision}', expected one of {_PRECISION}")
    if mixed not in _MIXED:
        logger.dead(f"Invalid mixed precision '{mixed}', expected one of {_MIXED}")
    if opt_level not in (0, 1, 2, 3):
        logger.dead(f"Invalid opt_level '{opt_level}'")
    if not 0 <= int(mixed_temporal) <= 16:
        logger.dead(f"Invalid mixed_temporal {mixed_temporal}: 0 (off) to 16 iterations per launch")
    if int(int_adds) < 0:
        logger.dead(f"Invalid int_adds {int_adds}: 0 (off) or every n-th addition")
    if not 0 <= int(loop_temporal) <= 8:
        logger.dead(f"Invalid loop_temporal {loop_temporal}: 0 (off) to 8 iterations per launch")
    if int(mixed_rows) not in MIXED_ROWS:
        logger.dead(f"Invalid mixed_rows {mixed_rows}, expected one of {MIXED_ROWS}")
    _config = Configuration(parallel, list(cc), cacheroot, comment, overstep, opt_level,
                            precision, exact, mixed, graph, fuse, divisor, int(mixed_every), bool(autotune),
                            int(mixed_temporal), int(mixed_rows), int(int_adds), bool(persistent),
                            bool(fail_waits), int(loop_temporal))
    logger.info(f"initialized with configuration: {_config}")
