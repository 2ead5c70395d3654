"""CPU ``xgrid`` API backed by the numpy oracle (test infrastructure only).

Same names and call protocol as the reference package (xgrid/__init__.py:1-53,
xgrid/lang/operator.py:29-41, xgrid/xgrid/__init__.py:21-86): kernels tick every
grid argument to their depth in argument order and then run; grids keep a list
of numpy time levels and an int32 boundary mask.  Parsing and typing reuse the
package's front end, so that a program written for ``xgrid`` runs unchanged on
the reference, on this oracle and on the GPU backend.
"""
from __future__ import annotations

import numpy as np

import xgrid_gb300 as _gb
from xgrid_gb300.config import get_config
from xgrid_gb300.log import Logger
from xgrid_gb300.operator import Operator
from xgrid_gb300.types import GridType, Value, numpy_dtype, parse_annotation

from .interp import Interpreter, depth_of

init = _gb.init
grid = _gb.grid
ptr = _gb.ptr
boundary = _gb.boundary
c = _gb.c
function = _gb.function
external = _gb.external
shape = _gb.shape
dimension = _gb.dimension
tick = _gb.tick


class Grid:
    """Reference grid semantics on numpy levels."""

    def __init__(self, shape: tuple, dtype: type) -> None:
        self.logger = Logger(self)
        element = parse_annotation(dtype)
        if not isinstance(element, Value):
            self.logger.dead(f"Grid element should be value instead of '{element}'")
        if isinstance(shape, int):
            shape = (shape,)
        self.element = element
        self.shape = tuple(int(s) for s in shape)
        self.numpy_dtype = numpy_dtype(element)
        self.typing = GridType(element, len(self.shape))
        self.levels = [np.zeros(self.shape, dtype=self.numpy_dtype)]
        self.boundary = np.zeros(self.shape, dtype=np.int32)

    @property
    def dimension(self) -> int:
        return len(self.shape)

    @property
    def now(self) -> np.ndarray:
        return self.levels[0]

    @property
    def _data(self) -> list:
        return self.levels

    def fill(self, data: np.ndarray, time: int = 0) -> None:
        level = abs(time)
        if level >= len(self.levels):
            self._extend_time(level + 1)
        self.levels[level] = np.array(data, dtype=self.numpy_dtype)

    def read(self, level: int = 0) -> np.ndarray:
        return self.levels[level].copy()

    def _extend_time(self, depth: int) -> None:
        while len(self.levels) < depth:
            self.levels.append(np.zeros(self.shape, dtype=self.numpy_dtype))
        del self.levels[depth:]

    def _op_invoke(self, depth: int, tick: bool) -> None:
        self._extend_time(depth)
        if tick:
            self.levels.insert(0, self.levels.pop())

    def __getitem__(self, index):
        return self.now[index]

    def __setitem__(self, index, value) -> None:
        self.now[index] = value


class OracleKernel(Operator):
    def __call__(self, *args):
        if self.mode != "kernel":
            return super().__call__(*args)
        defn = self.ir
        if len(args) != len(defn.signature.arguments):
            raise TypeError(f"this function takes {len(defn.signature.arguments)} argument ({len(args)} given)")
        depth = depth_of(defn)
        for a in args:
            if isinstance(a, Grid):
                a._op_invoke(depth, self.tick)
        return Interpreter(defn, get_config().overstep).run_kernel(list(args))


def kernel(*, name: str | None = None, includes: list | None = None, tick: bool = True, macro: list | None = None):
    def aux(func):
        return OracleKernel(func, "kernel", name, includes, tick=tick, macro=macro)
    return aux
