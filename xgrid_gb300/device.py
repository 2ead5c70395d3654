"""CUDA device and stream plumbing (PyTorch provides allocation and streams).

All backend work — uploads, kernel launches, downloads — is ordered on one
dedicated stream.  There is no CPU fallback: without a CUDA device every call
into the product path raises.
"""
from __future__ import annotations

import numpy as np

_stream = None
_handle = None
_cuda_ok = False


def torch():
    import torch as _torch
    return _torch


def require_cuda() -> None:
    global _cuda_ok
    if _cuda_ok:
        return
    t = torch()
    if t.cuda.is_available():
        _cuda_ok = True  # a device that was visible stays visible for the process
    else:
        raise Exception("xgrid: no CUDA device is visible; the GB300 backend runs every sweep on the GPU "
                        "and has no CPU fallback")


def stream():
    """The backend's stream (created on first use)."""
    global _stream
    require_cuda()
    if _stream is None:
        _stream = torch().cuda.Stream()
    return _stream


def stream_handle() -> int:
    global _handle
    if _handle is None:
        _handle = stream().cuda_stream
    return _handle


def copy_async(dst: int, src: int, nbytes: int) -> None:
    """Asynchronous copy on the backend stream between device memory and
    page-locked host memory (addresses as integers)."""
    from . import runtime
    runtime.check(runtime.load().xg_memcpy(dst, src, nbytes, stream_handle()), "copy")


def synchronize() -> None:
    if _stream is not None:
        _stream.synchronize()


_TORCH_DTYPES = {
    np.dtype(np.float64): "float64", np.dtype(np.float32): "float32", np.dtype(np.int64): "int64",
    np.dtype(np.int32): "int32", np.dtype(np.int16): "int16", np.dtype(np.int8): "int8",
    np.dtype(np.bool_): "bool",
}


def torch_dtype(np_dtype):
    name = _TORCH_DTYPES.get(np.dtype(np_dtype))
    return getattr(torch(), name) if name else None


def alloc_bytes(nbytes: int, zero: bool = False):
    """Device byte buffer allocated on the backend stream (so the caching
    allocator orders its reuse after our launches)."""
    t = torch()
    with t.cuda.stream(stream()):
        buf = t.empty(max(nbytes, 16), dtype=t.uint8, device="cuda")
        if zero:
            buf.zero_()
    return buf


def host_array(shape, np_dtype, zero: bool = True) -> np.ndarray:
    """Host array, page-locked when a CUDA device is present (faster copies)."""
    dt = np.dtype(np_dtype)
    t = torch()
    n = int(np.prod(shape)) if len(shape) else 1
    if t.cuda.is_available():
        # the array's base chain holds the pinned tensor alive
        buf = t.empty(n * dt.itemsize, dtype=t.uint8, pin_memory=True)
        arr = buf.numpy().view(dt).reshape(shape)
        if zero:
            arr[...] = np.zeros((), dtype=dt)
        return arr
    return np.zeros(shape, dtype=dt) if zero else np.empty(shape, dtype=dt)
