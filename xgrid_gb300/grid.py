"""``xgrid.Grid``: device-resident time levels with host mirrors.

Interface and semantics follow xgrid/xgrid/__init__.py:21-86: ``Grid(shape,
dtype)``; ``now`` is level 0; ``boundary`` is an int32 array of the grid's shape;
before each kernel call the level list is resized to the kernel's depth (new
levels are zero, surplus levels are dropped) and rotated so that the oldest level
becomes level 0 (``_op_invoke``, :43-54).  Here a level is a device buffer and the
rotation moves buffer handles, never data.

Host mirrors: ``now``, ``_data``, ``[]`` and ``fill`` hand out numpy arrays that the
caller may modify, so each access downloads the level if the device copy is newer
and marks the host copy authoritative; the next kernel call uploads it.  Reading
the ``boundary`` property marks the mask possibly modified; the next call
compares it with the uploaded copy and recompiles the mask tables when it
changed.  ``read(level)`` returns a copy without dirtying anything.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import device, runtime
from .log import Logger
from .types import GridType, Value, numpy_dtype, parse_annotation


class _Level:
    """One time level: ``auth`` says which copy is current ('zero', 'host', 'dev')."""

    __slots__ = ("host", "dev", "auth")

    def __init__(self) -> None:
        self.host = None
        self.dev = None
        self.auth = "zero"


class Grid:
    def __init__(self, shape: tuple, dtype: type) -> None:
        self.logger = Logger(self)
        element = parse_annotation(dtype)
        if not isinstance(element, Value):
            self.logger.dead(f"Grid element should be value instead of '{element}'")
        if isinstance(shape, int):
            shape = (shape,)
        self.element = element
        self.shape = tuple(int(s) for s in shape)
        if not 1 <= len(self.shape) <= 3:
            self.logger.dead(f"Grid of {len(self.shape)} dimensions is not supported (1 to 3)")
        if any(s <= 0 for s in self.shape):
            self.logger.dead(f"Grid extents must be positive, got {self.shape}")
        self.numpy_dtype = numpy_dtype(element)
        self.typing = GridType(element, len(self.shape))
        self._levels = [_Level()]
        self._boundary = np.zeros(self.shape, dtype=np.int32)
        self._mask_dirty = True
        self._mask_uploaded = None
        self._mask = None
        self._scratch = None
        self._aux = None
        self._nbytes = int(np.prod(self.shape)) * self.numpy_dtype.itemsize

    # ------------------------------------------------------------ reference API
    @property
    def dimension(self) -> int:
        return len(self.shape)

    @property
    def boundary(self) -> np.ndarray:
        self._mask_dirty = True
        return self._boundary

    @boundary.setter
    def boundary(self, value) -> None:
        arr = np.asarray(value, dtype=np.int32)
        if arr.shape != self.shape:
            self.logger.dead(f"Boundary of shape {arr.shape} does not match grid shape {self.shape}")
        self._boundary = np.ascontiguousarray(arr).copy()
        self._mask_dirty = True

    @property
    def now(self) -> np.ndarray:
        return self._host(0, dirty=True)

    @property
    def _data(self) -> list:
        return [self._host(i, dirty=True) for i in range(len(self._levels))]

    def fill(self, data: np.ndarray, time: int = 0) -> None:
        """Set level ``|time|`` (extending the level list if needed)."""
        data = np.asarray(data)
        if data.shape != self.shape or data.dtype != self.numpy_dtype:
            self.logger.dead("Unable to fill grid with incompatible shape or data type")
        level = abs(time)
        if level >= len(self._levels):
            self._extend_time(level + 1)
        self._host(level, dirty=True)[...] = data

    def __getitem__(self, index):
        return self.now[index]

    def __setitem__(self, index, value) -> None:
        self.now[index] = value

    def _extend_time(self, depth: int) -> None:
        while len(self._levels) < depth:
            self._levels.append(_Level())
        del self._levels[depth:]

    def _op_invoke(self, depth: int, tick: bool) -> None:
        self._extend_time(depth)
        if tick:
            self._levels.insert(0, self._levels.pop())

    # --------------------------------------------------------------- backend
    @property
    def time(self) -> int:
        return len(self._levels)

    def read(self, level: int = 0) -> np.ndarray:
        """Copy of a level (no dirty marking)."""
        return self._host(level, dirty=False).copy()

    def tensor(self, level: int = 0):
        """Device view of a level as a torch tensor of the grid's shape."""
        if self._sync_device(False):
            device.stream().synchronize()  # uploads done before any stream uses the view
        dt = device.torch_dtype(self.numpy_dtype)
        if dt is None:
            self.logger.dead("tensor() is only available for numeric grids")
        lv = self._levels[level]
        lv.auth = "dev"  # the caller may write through the view
        return lv.dev.view(dt)[: int(np.prod(self.shape))].view(self.shape)

    def _host(self, level: int, dirty: bool) -> np.ndarray:
        lv = self._levels[level]
        if lv.host is None:
            lv.host = device.host_array(self.shape, self.numpy_dtype, zero=(lv.auth != "dev"))
            if lv.auth == "zero":
                lv.auth = "host"
        if lv.auth == "dev":
            device.copy_async(lv.host.ctypes.data, lv.dev.data_ptr(), self._nbytes)
            device.stream().synchronize()
            lv.auth = "both"
        if dirty:
            lv.auth = "host"
        return lv.host

    def _sync_device(self, need_scratch: bool, aux_bytes: int = 0) -> bool:
        """Allocate and upload what the device lacks; True when host data was
        uploaded (the caller then waits for the copies before returning, so the
        host arrays handed out earlier can be modified again safely)."""
        device.require_cuda()
        uploaded = False
        for lv in self._levels:
            if lv.dev is None:
                lv.dev = device.alloc_bytes(self._nbytes, zero=(lv.auth == "zero"))
                if lv.auth == "zero":
                    lv.auth = "dev"
            if lv.auth == "host":
                if not lv.host.flags.c_contiguous:
                    lv.host = np.ascontiguousarray(lv.host)
                device.copy_async(lv.dev.data_ptr(), lv.host.ctypes.data, self._nbytes)
                lv.auth = "both"
                uploaded = True
        if need_scratch and self._scratch is None:
            self._scratch = device.alloc_bytes(self._nbytes)
        if aux_bytes and (self._aux is None or self._aux.numel() < aux_bytes):
            # zeroed: the work area ends with an error word that kernels only ever set
            self._aux = device.alloc_bytes(aux_bytes, zero=True)
        if self._mask_dirty or self._mask is None:
            self._upload_mask()
        return uploaded

    def _upload_mask(self) -> None:
        lib = runtime.load()
        if self._mask is None:
            handle = ctypes.c_void_p()
            shape = (ctypes.c_int64 * 3)(*self.shape)
            runtime.check(lib.xg_mask_create(len(self.shape), shape, ctypes.byref(handle)), "mask")
            self._mask = handle.value
            self._mask_lib = lib
        mask = np.ascontiguousarray(self._boundary, dtype=np.int32)
        if self._mask_uploaded is None or not np.array_equal(mask, self._mask_uploaded):
            runtime.check(lib.xg_mask_upload(self._mask, mask.ctypes.data), "mask upload")
            self._mask_uploaded = mask.copy()
        self._mask_dirty = False

    def serialize(self) -> runtime.XGGrid:
        """C-ABI view (device pointers) of this grid, cf. xgrid/xgrid/__init__.py:60-68."""
        g = runtime.XGGrid()
        g.ndim = len(self.shape)
        g.levels = len(self._levels)
        for i, n in enumerate(self.shape):
            g.shape[i] = n
        for i, lv in enumerate(self._levels[: runtime.XG_MAX_LEVELS]):
            g.level[i] = lv.dev.data_ptr()
        g.scratch = self._scratch.data_ptr() if self._scratch is not None else None
        g.mask = self._mask
        g.aux = self._aux.data_ptr() if self._aux is not None else None
        g.aux_bytes = self._aux.numel() if self._aux is not None else 0
        return g

    def _adopt(self, g: runtime.XGGrid) -> None:
        """Take back the level/scratch exchange that a call made, and mark every
        level as device-current."""
        if len(self._levels) > runtime.XG_MAX_LEVELS:
            self.logger.dead(f"at most {runtime.XG_MAX_LEVELS} time levels are supported")
        bufs = {lv.dev.data_ptr(): lv.dev for lv in self._levels}
        if self._scratch is not None:
            bufs[self._scratch.data_ptr()] = self._scratch
        new_levels = [bufs[g.level[i]] for i in range(len(self._levels))]
        used = {b.data_ptr() for b in new_levels}
        if self._scratch is not None:
            self._scratch = bufs[g.scratch] if g.scratch else None
            if self._scratch is not None and self._scratch.data_ptr() in used:
                self.logger.dead("internal error: scratch buffer aliases a level")
        for lv, buf in zip(self._levels, new_levels):
            lv.dev = buf  # the host mirror stays attached to the level as staging memory
            lv.auth = "dev"

    def __del__(self) -> None:
        mask = getattr(self, "_mask", None)
        lib = getattr(self, "_mask_lib", None)
        if mask is not None and lib is not None:
            try:
                lib.xg_mask_destroy(mask)
            except Exception:  # noqa: BLE001 - interpreter shutdown
                pass
