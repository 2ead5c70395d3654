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

from . import device, mixed, runtime
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

    def set_mixed_temporal(self, depth: int, rows: int | None = None) -> None:
        """Defect iterations per launch of mixed-precision loops (0: one FP32
        iteration per launch, no shared-memory staging) and rows per warp of
        the temporally blocked kernel (4 or 8)."""
        fn = getattr(self.lib.dylib, f"xg_mixed_tb_{self.module.name}", None)
        if fn is None:
            self.logger.dead(f"kernel '{self.module.name}' has no temporally blocked mixed-precision loop")
        fn.restype = ctypes.c_int
        if fn(ctypes.c_int(int(depth)), ctypes.c_int(int(rows) if rows is not None else -1)) != 0:
            self.logger.dead(runtime.last_error())
        runtime.load().xg_graph_clear(self.fn_ptr)

    def set_zstage(self, on: bool) -> None:
        """Staged z-walk of mask-free 3-D sweeps (planes streamed through shared
        memory, the default) or the register z-walk (horizontal neighbours through L1)."""
        fn = getattr(self.lib.dylib, f"xg_zstage_set_{self.module.name}")
        fn.restype = ctypes.c_int
        fn(ctypes.c_int(1 if on else 0))
        runtime.load().xg_graph_clear(self.fn_ptr)

    def set_tloop(self, on: bool) -> None:
        """Several iterations of an in-place loop per launch where the box check
        allows it (the default, ``loop_temporal`` iterations), or one launch per
        iteration."""
        fn = getattr(self.lib.dylib, f"xg_tloop_set_{self.module.name}")
        fn.restype = ctypes.c_int
        fn(ctypes.c_int(1 if on else 0))
        runtime.load().xg_graph_clear(self.fn_ptr)

    def zstage_launches(self) -> int:
        """Staged z-walk launches this module's host code has issued (graph
        replays re-run captured launches without counting)."""
        fn = getattr(self.lib.dylib, f"xg_zstage_launches_get_{self.module.name}")
        fn.restype = ctypes.c_longlong
        return int(fn())

    def set_mixed_every(self, every: int) -> None:
        """Iterations between FP64 corrections of mixed-precision loops (0 = once per loop)."""
        self.mixed_fn(int(every))
        runtime.load().xg_graph_clear(self.fn_ptr)

    def loop_error(self, clear: bool = False) -> int:
        """1 when a neighbour-tile wait of a persistent loop launch gave up (the
        results of that call are invalid), else 0; ``clear`` resets the word.
        Synchronises with the device."""
        fn = getattr(self.lib.dylib, f"xg_loop_error_{self.module.name}")
        fn.restype = ctypes.c_int
        fn.argtypes = [ctypes.c_int]
        rc = fn(1 if clear else 0)
        if rc < 0:
            self.logger.dead("reading the persistent-loop error word failed")
        return rc

    def staging_error(self, grid, clear: bool = False) -> int:
        """1 when a TMA staging copy of a mixed-precision loop on ``grid`` did not
        complete in time (the results of that call are invalid), else 0; ``clear``
        resets the word.  Synchronises with the device."""
        aux = getattr(grid, "_aux", None)
        if aux is None:
            return 0
        off = mixed.aux_error_offset(grid.shape)
        device.stream().synchronize()
        word = aux[off:off + 4]
        err = int(np.frombuffer(word.cpu().numpy().tobytes(), dtype=np.int32)[0])
        if clear and err:
            with device.torch().cuda.stream(device.stream()):
                word.zero_()
            device.stream().synchronize()
        return 1 if err else 0

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
    def split(self, args):
        """(grids, values) of one call's arguments, type-checked."""
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
        return grids, values

    def __call__(self, *args):
        grids, values = self.split(args)
        if len({id(g) for g in grids}) != len(grids):
            self.logger.dead("the same Grid is passed twice to one kernel call")
        device.require_cuda()
        # tick in argument order, as the reference does
        for g in grids:
            g._op_invoke(self.depth, self.op.tick)
        uploaded = False
        for i, g in enumerate(grids):
            aux = mixed.aux_bytes(g.shape) if i in self.module.aux_per_cell else 0
            uploaded |= g._sync_device(i in self.scratch_slots, aux)
        copied = None
        if uploaded:
            # the launch follows the uploads on the stream; the host arrays may be
            # modified again once the copies (not the launch) are done
            copied = self._upload_event()
            copied.record(device.stream())
        packed = self.pack(values)
        arr = (runtime.XGGrid * max(len(grids), 1))(*[g.serialize() for g in grids])
        ret = self.ret_type.ctype() if self.ret_type is not None else None
        rc = runtime.load().xg_call(self.fn_ptr, arr, len(grids),
                                    ctypes.cast(ctypes.byref(packed), ctypes.c_void_p) if values else None,
                                    ctypes.sizeof(packed) if values else 0,
                                    ctypes.cast(ctypes.byref(ret), ctypes.c_void_p) if ret is not None else None,
                                    ctypes.sizeof(ret) if ret is not None else 0,
                                    device.stream_handle(), 1 if self.use_graph else 0)
        if copied is not None:
            copied.synchronize()
        if rc != 0:
            self.logger.dead(f"kernel '{self.module.name}' failed: {runtime.last_error()}")
        for g, st in zip(grids, arr):
            g._adopt(st)
        if ret is None:
            return None
        if isinstance(self.ret_type, Structure):
            return self.ret_type.deserialize(ret)
        return self.ret_type.deserialize(ret.value)

    def _upload_event(self):
        ev = getattr(self, "_uploaded", None)
        if ev is None:
            ev = self._uploaded = device.torch().cuda.Event()
        return ev

    def pack(self, values: list):
        packed = self.args_type()
        for (name, t), v in zip(self.module.value_args, values):
            setattr(packed, name, t.serialize(v))
        return packed

    # --------------------------------------------------------------- batched
    def set_temporal(self, depth: int, ty: int = 32, tx: int = 64, block: tuple = (32, 8, 1)) -> None:
        """Temporal blocking of the batched path: ``depth`` steps per launch (1 turns
        it off) on tiles of ``ty`` x ``tx`` cells, CTAs of ``block`` threads."""
        if depth < 1 or ty < 1 or tx < 1:
            self.logger.dead("temporal blocking: depth, ty and tx must be positive")
        self._temporal = (int(depth), int(ty), int(tx), tuple(int(b) for b in block))

    def temporal_supported(self) -> bool:
        return self.module.batch and hasattr(self.lib.dylib, f"xg_batch_tb_{self.module.name}")

    def batch(self, problems, steps: int = 1, temporal=None) -> None:
        """Batched execution (see ``xgrid_gb300.batch``).  ``temporal`` overrides
        the kernel's temporal-blocking setting for this call: a ``(depth, ty, tx)``
        tuple, or 1 to run one step per launch."""
        if not self.module.batch:
            self.logger.dead(f"kernel '{self.module.name}' cannot run batched: its body must be one run of "
                             f"explicit mask-0 grid assignments")
        steps = int(steps)
        if steps <= 0 or not problems:
            return
        device.require_cuda()
        lib = self.lib.dylib
        if not hasattr(self, "_batch"):
            info = getattr(lib, f"xg_batch_info_{self.module.name}")
            depth, dsize, group = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32()
            info(ctypes.byref(depth), ctypes.byref(dsize), ctypes.byref(group))
            prep = getattr(lib, f"xg_batch_prepare_{self.module.name}")
            prep.restype = ctypes.c_int
            blocks_fn = getattr(lib, f"xg_batch_blocks_{self.module.name}")
            blocks_fn.restype = ctypes.c_int
            fn = getattr(lib, f"xg_batch_{self.module.name}")
            self._batch = {"depth": depth.value, "dsize": dsize.value, "group": group.value, "prep": prep,
                           "blocks": blocks_fn, "fn": ctypes.cast(fn, ctypes.c_void_p).value, "desc": {},
                           "counters": None, "nblocks": {}}
        B = self._batch
        if (temporal is None and getattr(self, "_temporal", None) is None and self.config.autotune
                and steps >= 2 and self.temporal_supported()):
            temporal = self.tuned_temporal(problems)
        tb = self._temporal_for(temporal, steps)
        all_grids, all_values = [], []
        for args in problems:
            grids, values = self.split(tuple(args))
            all_grids.extend(grids)
            all_values.append(values)
        if len({id(g) for g in all_grids}) != len(all_grids):
            self.logger.dead("batched problems must not share grids")
        uploaded = False
        for g in all_grids:
            g._extend_time(B["depth"])
            uploaded |= g._sync_device(tb is not None)
        if uploaded:
            device.stream().synchronize()
        nprob = len(problems)
        ng = len(self.module.grid_args)
        arr = (runtime.XGGrid * (nprob * ng))(*[g.serialize() for g in all_grids])
        packed = b"".join(bytes(self.pack(v)) for v in all_values)
        stride = ctypes.sizeof(self.args_type) if self.module.value_args else 0
        tiling = self._tiling_key(B["group"])
        key = (tuple((st.level[k] or 0) for st in arr for k in range(B["depth"])),
               tuple((st.scratch or 0) if tb else 0 for st in arr),
               tuple(st.mask or 0 for st in arr), tuple(runtime.load().xg_mask_version(st.mask) for st in arr),
               packed, tiling, tb[:3] if tb else None)
        entry = B["desc"].get(key)
        if entry is None:
            host = ctypes.create_string_buffer(nprob * (B["dsize"] + 16))
            total, maxc, total_tb = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(-1)
            args_buf = ctypes.create_string_buffer(packed, max(len(packed), 1))
            tbcfg = (ctypes.c_int32 * 3)(*tb[:3]) if tb else None
            rc = B["prep"](arr, ctypes.c_int(nprob), args_buf, ctypes.c_size_t(stride), host,
                           ctypes.c_size_t(len(host)), ctypes.byref(total), ctypes.byref(maxc), tbcfg,
                           ctypes.byref(total_tb))
            if rc != 0:
                self.logger.dead(f"batch preparation failed: {runtime.last_error()}")
            if tb and total_tb.value < 0:
                self.logger.info(f"temporal blocking not used: {runtime.last_error()}")
            t = device.torch()
            dev = device.alloc_bytes(len(host))
            with t.cuda.stream(device.stream()):
                dev[: len(host)].copy_(t.frombuffer(bytearray(host.raw), dtype=t.uint8), non_blocking=False)
            if len(B["desc"]) > 16:
                B["desc"].clear()
            entry = B["desc"][key] = (dev, total.value, maxc.value, total_tb.value)
        dev, total, maxc, total_tb = entry
        if tb and total_tb >= 0:
            self._batch_temporal(B, tb, dev, total_tb, steps, nprob, maxc)
            self._after_batch(all_grids, steps, B["depth"])
            return
        if B["counters"] is None or B["counters"].numel() < steps * 8:
            B["counters"] = device.alloc_bytes(steps * 8)
        block = tiling[3:6]
        threads = block[0] * block[1] * block[2]
        if threads not in B["nblocks"]:
            nb = ctypes.c_int()
            if B["blocks"](ctypes.c_int(threads), ctypes.byref(nb)) != 0:
                self.logger.dead(runtime.last_error())
            B["nblocks"][threads] = nb.value
        ba = BatchArgs(dev.data_ptr(), total, steps, 0, B["counters"].data_ptr(), nprob, 1 if self.op.tick else 0,
                       1 if maxc < (1 << 31) - 1 else 0, B["nblocks"][threads], (ctypes.c_int32 * 3)(*block))
        rc = runtime.load().xg_call(B["fn"], None, 0, ctypes.cast(ctypes.byref(ba), ctypes.c_void_p),
                                    ctypes.sizeof(ba), None, 0, device.stream_handle(), 1 if self.use_graph else 0)
        if rc != 0:
            self.logger.dead(f"batched kernel '{self.module.name}' failed: {runtime.last_error()}")
        self._after_batch(all_grids, steps, B["depth"])

    def tuned_temporal(self, problems) -> tuple:
        """The autotuner's (depth, ty, tx, block) for these problems' shapes."""
        shapes = tuple(tuple(a.shape for a in args if isinstance(a, Grid)) for args in problems)
        memo = self.__dict__.setdefault("_tuned", {})
        if shapes not in memo:
            from . import autotune
            memo[shapes] = autotune.tune_batch(self, problems)
        return memo[shapes]

    def _after_batch(self, grids, steps: int, depth: int) -> None:
        for g in grids:
            if self.op.tick:
                for _ in range(steps % depth):
                    g._levels.insert(0, g._levels.pop())
            for lv in g._levels:
                lv.auth = "dev"

    def _temporal_for(self, temporal, steps: int):
        """(depth, ty, tx, block) of this call's temporal blocking, or None."""
        if steps < 2 or not self.temporal_supported():
            return None
        if temporal is None:
            cfg = getattr(self, "_temporal", None)
            if cfg is None:
                cfg = DEFAULT_TEMPORAL
        elif isinstance(temporal, int):
            cfg = (temporal, 32, 64, (32, 8, 1))
        else:
            t = tuple(temporal)
            cfg = t + ((32, 8, 1),) if len(t) == 3 else t
        if cfg[0] <= 1:
            return None
        return (int(cfg[0]), int(cfg[1]), int(cfg[2]), tuple(int(b) for b in cfg[3]))

    def _batch_temporal(self, B, tb, dev, total_tb: int, steps: int, nprob: int, maxc: int) -> None:
        depth, ty, tx, block = tb
        threads = block[0] * block[1] * block[2]
        ck = (threads,) + tb[:3]
        if ck not in B["nblocks"]:
            fn = getattr(self.lib.dylib, f"xg_batch_tb_blocks_{self.module.name}")
            fn.restype = ctypes.c_int
            smem, nb = ctypes.c_int(), ctypes.c_int()
            if fn(ctypes.c_int(threads), ctypes.c_int(depth), ctypes.c_int(ty), ctypes.c_int(tx),
                  ctypes.byref(smem), ctypes.byref(nb)) != 0:
                self.logger.dead(runtime.last_error())
            B["nblocks"][ck] = (smem.value, nb.value)
        smem, nb = B["nblocks"][ck]
        if B["counters"] is None or B["counters"].numel() < steps * 8:
            B["counters"] = device.alloc_bytes(steps * 8)
        fn = ctypes.cast(getattr(self.lib.dylib, f"xg_batch_tb_{self.module.name}"), ctypes.c_void_p).value
        ba = BatchTemporalArgs(dev.data_ptr(), total_tb, steps, B["counters"].data_ptr(), nprob,
                               1 if maxc < (1 << 31) - 1 else 0, nb, depth, ty, tx, smem,
                               (ctypes.c_int32 * 3)(*block))
        rc = runtime.load().xg_call(fn, None, 0, ctypes.cast(ctypes.byref(ba), ctypes.c_void_p),
                                    ctypes.sizeof(ba), None, 0, device.stream_handle(), 1 if self.use_graph else 0)
        if rc != 0:
            self.logger.dead(f"batched kernel '{self.module.name}' failed: {runtime.last_error()}")

    def _tiling_key(self, group: int) -> tuple:
        arr = (ctypes.c_int32 * 6)()
        getter = getattr(self.lib.dylib, f"xg_get_tiling_{self.module.name}")
        getter(ctypes.c_int(group), arr)
        return tuple(arr)


# steps per launch, tile rows, tile columns, CTA shape of the temporally blocked batched path
DEFAULT_TEMPORAL = (4, 32, 56, (32, 8, 1))


class BatchTemporalArgs(ctypes.Structure):
    _fields_ = [("desc", ctypes.c_void_p), ("total", ctypes.c_int64), ("steps", ctypes.c_int64),
                ("counters", ctypes.c_void_p), ("nprob", ctypes.c_int32), ("small", ctypes.c_int32),
                ("blocks", ctypes.c_int32), ("T", ctypes.c_int32), ("ty", ctypes.c_int32), ("tx", ctypes.c_int32),
                ("smem", ctypes.c_int32), ("block", ctypes.c_int32 * 3)]


class BatchArgs(ctypes.Structure):
    _fields_ = [("desc", ctypes.c_void_p), ("total", ctypes.c_int64), ("steps", ctypes.c_int64),
                ("step0", ctypes.c_int64), ("counters", ctypes.c_void_p), ("nprob", ctypes.c_int32),
                ("tick", ctypes.c_int32), ("small", ctypes.c_int32), ("blocks", ctypes.c_int32),
                ("block", ctypes.c_int32 * 3)]
