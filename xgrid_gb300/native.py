"""A compiled ``@xgrid.kernel``: generate → nvcc → load → call.

Replaces ``Generator(op).result`` plus ``Library.function`` of the reference
(xgrid/lang/generator.py:106-108, 228-237; xgrid/util/ffi.py:13-35).  Calling
checks the argument count (``TypeError`` as in ffi.py:31-33), ticks the grids
(operator.py:36-39), uploads host-modified levels and masks, packs the
non-grid arguments into the module's argument struct and calls the entry
point through the runtime's graph cache.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import device, runtime
from .codegen import CudaGenerator
from .compiler import Compiler, Library
from .config import get_config
from .grid import Grid
from .log import Logger
from .types import Structure, Void


class NativeKernel:
    def __init__(self, operator) -> None:
        self.logger = Logger(self)
        self.op = operator
        self.config = get_config()
        self.module = CudaGenerator(operator, self.config).generate()
        self.depth = self.module.depth
        flags = self.config.nvcc_flags
        self.path = Compiler(cacheroot=self.config.cacheroot).compile(self.module.source, flags)
        self.lib = Library(self.path)
        self.fn = self.lib.entry(self.module.entry)
        self.fn_ptr = ctypes.cast(self.fn, ctypes.c_void_p).value
        self.config_fn = self.lib.entry(f"xg_config_{self.module.name}")
        self.config_fn.restype = ctypes.c_int
        self.config_fn.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int32), ctypes.c_int]
        fields = [(n, t.ctype) for n, t in self.module.value_args]
        self.args_type = type(f"xga_{self.module.name}", (ctypes.Structure,), {"_fields_": fields})
        rt = self.module.return_type
        self.ret_type = None if isinstance(rt, Void) else rt
        self.scratch_slots = set(self.module.implicit_slots)
        self.nargs = len(self.module.arg_order)
        self.use_graph = self.config.graph and not self.module.device_only
        self.mixed_fn = getattr(self.lib.dylib, f"xg_mixed_{self.module.name}", None)
        if self.mixed_fn is not None:
            self.mixed_fn.argtypes = [ctypes.c_int64]
            self.mixed_fn.restype = ctypes.c_int

    def set_mixed_every(self, every: int) -> None:
        """Iterations between FP64 corrections of mixed-precision loops (0 = once per loop)."""
        self.mixed_fn(int(every))
        runtime.load().xg_graph_clear(self.fn_ptr)

    # ---------------------------------------------------------------- tuning
    def set_tiling(self, group: int, tiling: tuple) -> None:
        """(tz, ty, tx, block.x, block.y, block.z) for one launch group."""
        arr = (ctypes.c_int32 * 6)(*tiling)
        self.config_fn(group, arr, -1)
        runtime.load().xg_graph_clear(self.fn_ptr)

    def set_fuse(self, fuse: bool) -> None:
        self.config_fn(-1, None, 1 if fuse else 0)
        runtime.load().xg_graph_clear(self.fn_ptr)

    # ------------------------------------------------------------------ call
    def __call__(self, *args):
        if len(args) != self.nargs:
            raise TypeError(f"this function takes {self.nargs} argument ({len(args)} given)")
        grids, values = [], []
        for (kind, idx), a in zip(self.module.arg_order, args):
            if kind == "grid":
                if not isinstance(a, Grid):
                    self.logger.dead(f"argument '{self.module.grid_args[idx][0]}' expects an xgrid.Grid")
                gt = self.module.grid_args[idx][1]
                if a.element != gt.element or a.dimension != gt.dimension:
                    self.logger.dead(f"argument '{self.module.grid_args[idx][0]}' expects {gt!r}, "
                                     f"got {a.typing!r}")
                grids.append(a)
            else:
                values.append(a)
        if len({id(g) for g in grids}) != len(grids):
            self.logger.dead("the same Grid is passed twice to one kernel call")
        device.require_cuda()
        # tick in argument order, as the reference does
        for g in grids:
            g._op_invoke(self.depth, self.op.tick)
        uploaded = False
        for i, g in enumerate(grids):
            aux = self.module.aux_per_cell.get(i, 0) * int(np.prod(g.shape))
            uploaded |= g._sync_device(i in self.scratch_slots, aux)
        if uploaded:
            device.stream().synchronize()
        packed = self.pack(values)
        arr = (runtime.XGGrid * max(len(grids), 1))(*[g.serialize() for g in grids])
        ret = self.ret_type.ctype() if self.ret_type is not None else None
        rc = runtime.load().xg_call(self.fn_ptr, arr, len(grids),
                                    ctypes.cast(ctypes.byref(packed), ctypes.c_void_p) if values else None,
                                    ctypes.sizeof(packed) if values else 0,
                                    ctypes.cast(ctypes.byref(ret), ctypes.c_void_p) if ret is not None else None,
                                    ctypes.sizeof(ret) if ret is not None else 0,
                                    device.stream_handle(), 1 if self.use_graph else 0)
        if rc != 0:
            self.logger.dead(f"kernel '{self.module.name}' failed: {runtime.last_error()}")
        for g, st in zip(grids, arr):
            g._adopt(st)
        if ret is None:
            return None
        if isinstance(self.ret_type, Structure):
            return self.ret_type.deserialize(ret)
        return self.ret_type.deserialize(ret.value)

    def pack(self, values: list):
        packed = self.args_type()
        for (name, t), v in zip(self.module.value_args, values):
            setattr(packed, name, t.serialize(v))
        return packed
