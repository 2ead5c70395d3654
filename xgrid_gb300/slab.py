"""Slab decomposition of one grid across ranks (one GPU per process).

The reference runs one grid in one process (its only parallelism is OpenMP
over one shared array, xgrid/lang/generator.py:354-356).  For grids beyond
one GPU's memory, a grid is cut along its slowest axis (the first DSL index)
into slabs of consecutive rows, one per rank.  Each rank holds its slab plus
``halo`` rows on either side in ordinary ``Grid``s and runs the unchanged
kernel on them; before every launch that reads a buffer at a nonzero offset
along the cut axis, the halo rows of that buffer are refreshed from the
neighbouring ranks (their rows next to the cut), a point-to-point exchange
into each rank's own halo rows -- no collective.

* Halo rows carry the mask value ``HALO_MASK``, which no sweep selects, so no
  kernel writes them and every level keeps them like any other unselected cell.
* At the grid's outer faces the halo rows stand in for what the one-grid kernel
  reads beyond the face: zeros under ``overstep="none"`` (reads outside the
  allocation read zero), a copy of the face row under ``"limit"``, the rows of
  the opposite face under ``"wrap"`` (the ranks form a ring).
* The exchange runs in the module's launch hook (``xg_set_hook_<name>``), before
  each single-sweep launch, on the kernel's stream; the module runs with fused
  launches and CUDA graphs off, and without persistent or mixed-precision loops.
* Reads along the cut axis must not reach further than ``halo`` rows.

The same ``SlabPlan`` and ``exchange`` drive the CPU oracle in the tests
(``torch.distributed`` with gloo on CPU tensors); on GPUs the transport is
``torch.distributed`` point-to-point on device tensors (NCCL).
"""
from __future__ import annotations

import ctypes
import dataclasses

import numpy as np

HALO_MASK = -(2 ** 31)


@dataclasses.dataclass
class SlabPlan:
    """Rows ``[y0, y1)`` of a grid of ``shape`` owned by ``rank`` of ``world``,
    stored with ``halo`` rows on either side."""

    shape: tuple
    world: int
    rank: int
    halo: int = 1
    overstep: str = "none"

    def __post_init__(self) -> None:
        self.shape = tuple(int(s) for s in self.shape)
        n = self.shape[0]
        if not 0 <= self.rank < self.world:
            raise ValueError(f"rank {self.rank} outside a world of {self.world}")
        if self.halo < 1:
            raise ValueError("a slab needs at least one halo row per side")
        base, extra = divmod(n, self.world)
        if base < self.halo:
            raise ValueError(f"{n} rows over {self.world} ranks leave slabs thinner than the halo of {self.halo}")
        self.y0 = self.rank * base + min(self.rank, extra)
        self.y1 = self.y0 + base + (1 if self.rank < extra else 0)

    @property
    def rows(self) -> int:
        return self.y1 - self.y0

    @property
    def local_shape(self) -> tuple:
        return (self.rows + 2 * self.halo,) + self.shape[1:]

    @property
    def interior(self) -> slice:
        return slice(self.halo, self.halo + self.rows)

    def neighbours(self) -> tuple:
        """(rank above, rank below): None at an outer face unless the grid wraps."""
        up, down = self.rank - 1, self.rank + 1
        if self.overstep == "wrap":
            return up % self.world, down % self.world
        return (up if up >= 0 else None), (down if down < self.world else None)

    def global_rows(self) -> np.ndarray:
        """Global row of every local row (halo rows beyond a face lie outside 0..n-1)."""
        return np.arange(self.y0 - self.halo, self.y1 + self.halo)

    def local_mask(self, mask: np.ndarray) -> np.ndarray:
        """The slab's rows of the global mask, halo rows set to ``HALO_MASK``."""
        out = np.full(self.local_shape, HALO_MASK, dtype=np.int32)
        out[self.interior] = np.asarray(mask, dtype=np.int32)[self.y0:self.y1]
        return out

    def local_field(self, field: np.ndarray) -> np.ndarray:
        """The slab's rows of a global field with halo rows filled as an exchange
        would fill them (the initial state)."""
        field = np.asarray(field)
        out = np.zeros(self.local_shape, dtype=field.dtype)
        n = self.shape[0]
        for i, g in enumerate(self.global_rows()):
            if 0 <= g < n:
                out[i] = field[g]
            elif self.overstep == "wrap":
                out[i] = field[g % n]
            elif self.overstep == "limit":
                out[i] = field[min(max(g, 0), n - 1)]
        return out


def exchange(plan: SlabPlan, buf, send_recv) -> None:
    """Refresh the halo rows of one local buffer (a tensor of ``plan.local_shape``).

    ``send_recv(ops)`` runs a list of ``("send" | "recv", tensor, peer)``
    point-to-point operations together; between two ranks, sends and receives
    pair up in the order they are listed.  A rank sends its last ``halo`` rows
    down and its first ``halo`` rows up, then receives its top halo from above
    and its bottom halo from below -- in that order on every rank, so that with
    two ranks in a ring (each the other's upper and lower neighbour) the rows
    sent down arrive in the top halo.  At an outer face without a neighbour the
    halo is zeros (``none``) or a copy of the face row (``limit``); a single
    rank that wraps copies its own rows."""
    h, r = plan.halo, plan.rows
    up, down = plan.neighbours()
    top, bottom = buf[0:h], buf[h + r:h + r + h]
    first, last = buf[h:2 * h], buf[r:h + r]
    if up is not None and up == plan.rank:      # one rank, periodic: the ring closes on itself
        top.copy_(last)
        bottom.copy_(first)
        return
    ops = []
    if down is not None:
        ops.append(("send", last, down))
    if up is not None:
        ops.append(("send", first, up))
    if up is not None:
        ops.append(("recv", top, up))
    elif plan.overstep == "limit":
        top.copy_(first[0:1].expand_as(top))
    if down is not None:
        ops.append(("recv", bottom, down))
    elif plan.overstep == "limit":
        bottom.copy_(last[h - 1:h].expand_as(bottom))
    if ops:
        send_recv(ops)


def torch_send_recv(group=None):
    """Point-to-point transport over ``torch.distributed`` (NCCL for device
    tensors, gloo for CPU tensors): all operations of one exchange are batched."""
    import torch.distributed as dist

    def run(ops):
        p2p = []
        for kind, t, peer in ops:
            if not t.is_contiguous():  # rows of a C-order buffer along its first axis always are
                raise Exception("slab exchange: halo rows must be contiguous")
            p2p.append(dist.P2POp(dist.isend if kind == "send" else dist.irecv, t, peer, group))
        for work in dist.batch_isend_irecv(p2p):
            work.wait()
    return run


def halo_reads(sweeps, axis: int) -> dict:
    """{launch site: [(grid slot, level)]}: the buffers each single-sweep launch
    reads at a nonzero offset along the cut axis (``axis`` in z, y, x order)."""
    out, position = {}, {}
    for s in sweeps:
        j = position[s.group_index] = position.get(s.group_index, -1) + 1  # index within its launch group
        seen = []
        for _, ld in s.loads:
            key = (ld.slot, ld.level)
            if ld.offset[axis] != 0 and key not in seen:
                seen.append(key)
        out[s.group_index * 64 + j] = seen
    return out


class SlabKernel:
    """Run a compiled ``@xgrid.kernel`` on this rank's slab grids, refreshing
    halo rows before every launch that reads across the cut.

    ``kernel``: the operator; ``plan``: this rank's ``SlabPlan`` (its ``overstep``
    must be the configuration's); ``send_recv``: the transport (default
    ``torch_send_recv()``).  Call it with the kernel's arguments, the grid
    arguments being this rank's local grids (``plan.local_shape``, masks from
    ``plan.local_mask``, fields from ``plan.local_field``)."""

    def __init__(self, kernel, plan: SlabPlan, send_recv=None) -> None:
        from . import runtime
        from .native import NativeKernel
        if kernel.native is None:
            kernel.native = NativeKernel(kernel)
        self.kernel = kernel
        self.plan = plan
        self.send_recv = send_recv or torch_send_recv()
        nk = kernel.native
        cfg = nk.config
        if cfg.mixed is not None or cfg.persistent:
            raise Exception("slab decomposition runs plain single-sweep launches: initialise without mixed "
                            "precision and persistent loops")
        if cfg.overstep != plan.overstep:
            raise Exception(f"slab plan overstep '{plan.overstep}' differs from the configuration's "
                            f"'{cfg.overstep}'")
        nk.set_fuse(False)
        nk.use_graph = False
        dim = nk.module.grid_args[0][1].dimension
        axis = 3 - dim  # the first DSL index in (z, y, x) order
        for s in nk.module.sweeps:
            for _, ld in s.loads:
                if abs(ld.offset[axis]) > plan.halo:
                    raise Exception(f"a sweep reads {abs(ld.offset[axis])} rows across the cut, more than the "
                                    f"halo of {plan.halo}")
        self.reads = halo_reads(nk.module.sweeps, axis)
        self._buffers = {}
        self._error = None
        hook_type = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(runtime.XGGrid),
                                     ctypes.c_int, ctypes.c_void_p)
        self._hook = hook_type(self._on_launch)  # kept alive as long as the module may call it
        setter = nk.lib.entry(f"xg_set_hook_{nk.module.name}")
        setter.restype = ctypes.c_int
        setter.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        setter(ctypes.cast(self._hook, ctypes.c_void_p), None)

    def _on_launch(self, ctx, site, grids, ngrids, stream) -> int:
        try:
            for slot, level in self.reads.get(site, ()):
                ptr = grids[slot].level[level]
                buf = self._buffers.get(ptr)
                if buf is None:
                    raise Exception(f"slab exchange: unknown buffer at 0x{ptr:x}")
                exchange(self.plan, buf, self.send_recv)
            return 0
        except Exception as e:  # noqa: BLE001 - reported through the kernel's error path
            self._error = e
            return -1

    def __call__(self, *args):
        import torch

        from . import device
        nk = self.kernel.native
        grids, _ = nk.split(args)
        for g in grids:
            if g.shape != self.plan.local_shape:
                raise Exception(f"slab grid of shape {g.shape}, the plan's local shape is {self.plan.local_shape}")
        self._error = None
        # every buffer the call may read (all levels at the kernel's depth, scratch levels),
        # allocated and current now, viewed as tensors by address for the exchange
        uploaded = False
        for i, g in enumerate(grids):
            g._extend_time(nk.depth)
            uploaded |= g._sync_device(i in nk.scratch_slots)
        if uploaded:
            device.stream().synchronize()
        self._buffers = {}
        for g in grids:
            dt = device.torch_dtype(g.numpy_dtype)
            bufs = [lv.dev for lv in g._levels] + ([g._scratch] if g._scratch is not None else [])
            for b in bufs:
                self._buffers[b.data_ptr()] = b.view(dt)[: int(np.prod(g.shape))].view(g.shape)
        with torch.cuda.stream(device.stream()):
            try:
                return self.kernel(*args)
            except Exception:
                if self._error is not None:
                    raise Exception(f"slab exchange failed: {self._error}") from self._error
                raise
