"""GB300-native backend of the xgrid stencil DSL.

Public API as in xgrid/__init__.py:1-53: ``init, kernel, function, external, ptr,
grid, boundary, c, Grid, shape, dimension, tick``.  ``@kernel`` bodies are lowered
to CUDA sweeps for sm_103a (``codegen``), compiled by nvcc into a module that is
called through a C ABI (``include/xgrid_gb300.h``), and grids live in device
memory with pointer-swapped time levels (``grid``).
"""
from __future__ import annotations

import struct
from typing import Any

from .config import Configuration, get_config, init
from .grid import Grid
from .lang import boundary, c
from .operator import Operator, external, function, kernel
from .types import BaseType, GridType, Integer, Void, grid, ptr


def _dimension_typecheck(args: list) -> BaseType:
    if not isinstance(args[0], GridType):
        raise Exception(f"Incompatible dimension to type '{args[0]}'")
    return Integer(struct.calcsize("i"))


def _shape_typecheck(args: list) -> BaseType:
    if not isinstance(args[0], GridType):
        raise Exception(f"Incompatible shape to type '{args[0]}'")
    if not isinstance(args[1], Integer):
        raise Exception(f"Incompatible shape dimension '{args[1]}'")
    return Integer(struct.calcsize("i"))


def _tick_typecheck(args: list) -> BaseType:
    if not isinstance(args[0], GridType):
        raise Exception(f"Incompatible tick to type '{args[0]}'")
    return Void()


@external(typecheck_override=_dimension_typecheck)
def dimension(grid: Any) -> int:
    ...


@external(typecheck_override=_shape_typecheck)
def shape(grid: Any, dimension: int) -> int:
    ...


@external(typecheck_override=_tick_typecheck)
def tick(grid: Any) -> None:
    ...


__all__ = ["kernel", "function", "init", "ptr", "grid", "boundary", "c", "external", "Grid", "shape",
           "dimension", "tick"]
