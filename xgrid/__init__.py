"""Drop-in name for the GB300 backend: ``import xgrid`` gives the same API as the
reference package (xgrid/__init__.py:1-53), implemented by ``xgrid_gb300``, so
existing kernels such as the lid-driven cavity example run unchanged."""
import sys as _sys

from xgrid_gb300 import (Grid, boundary, c, dimension, external, function, grid, init, kernel, ptr,
                         shape, tick)
from xgrid_gb300 import log as _log
from xgrid_gb300 import types as _types

# module paths some user code imports from the reference package
_sys.modules.setdefault("xgrid.util.logging", _log)
_sys.modules.setdefault("xgrid.util.typing.value", _types)
_sys.modules.setdefault("xgrid.util.typing", _types)

__all__ = ["kernel", "function", "init", "ptr", "grid", "boundary", "c", "external", "Grid", "shape",
           "dimension", "tick"]
