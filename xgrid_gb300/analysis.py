"""Sweep classification and launch grouping.

A grid assignment ``g[o] = expr`` inside an ``@xgrid.kernel`` is a *sweep*: the
reference lowers it to a loop nest over the whole grid filtered by
``boundary_mask == k`` (xgrid/lang/generator.py:285-364).  ``StencilParser``
(xgrid/lang/generator.py:50-76) tags each sweep with its target, its mask ``k``
and whether it is *implicit* (the right-hand side reads the target at time 0
under mask 0), which the reference runs as a two-phase loop through a scratch
array (generator.py:312-352).  This module computes the same tags plus what the
GPU launcher needs: the distinct loads of every sweep, and a partition of
consecutive sweeps into *groups* that one kernel launch may execute.

Group rules (a group is a run of mask-0 "main" sweeps followed by mask-k
"boundary" sweeps, executed tile by tile with ``__syncthreads`` between phases):

* buffers are versioned: an implicit sweep on ``P`` reads ``(P, 0, v)`` and
  writes ``(P, 0, v+1)`` (the scratch buffer that replaces level 0);
* a main sweep may read a buffer at a nonzero offset only if no sweep of the
  group writes that buffer version (another tile may not have written it yet);
* a sweep that stores at a nonzero offset runs alone;
* boundary sweeps that read a buffer written in the group at a nonzero offset
  need every such read to stay inside the reading cell's tile — checked at run
  time on the mask (``xg_mask_tile_local``); when it fails the group runs as one
  launch per sweep.
"""
from __future__ import annotations

import dataclasses

from . import ir
from .log import Logger
from .types import GridType


def pad3(offset: tuple) -> tuple:
    """DSL offset (one entry per dimension) → (z, y, x)."""
    return (0,) * (3 - len(offset)) + tuple(offset)


@dataclasses.dataclass(frozen=True)
class Load:
    slot: int        # grid argument index
    level: int       # |time offset|
    version: int     # buffer version within the group (implicit sweeps bump it)
    offset: tuple    # (z, y, x)


@dataclasses.dataclass(eq=False)
class Sweep:
    stmt: ir.Assignment
    slot: int
    mask: int
    implicit: bool
    level: int           # level written (|time offset| of the store)
    store_offset: tuple  # (z, y, x)
    loads: list = dataclasses.field(default_factory=list)   # list[(ir.Stencil, Load)]
    write_version: int = 0
    read_version_of_target: int = 0
    group_index: int = -1

    @property
    def is_main(self) -> bool:
        return self.mask == 0

    def distinct_loads(self) -> list:
        seen = []
        for _, ld in self.loads:
            if ld not in seen:
                seen.append(ld)
        return seen


@dataclasses.dataclass(eq=False)
class Group:
    sweeps: list
    index: int = 0
    # (phase index, offsets needing the tile-locality check)
    local_checks: list = dataclasses.field(default_factory=list)

    @property
    def mains(self) -> list:
        return [s for s in self.sweeps if s.is_main]

    @property
    def bnds(self) -> list:
        return [s for s in self.sweeps if not s.is_main]

    @property
    def fusable(self) -> bool:
        return len(self.sweeps) > 1 and len(self.mains) > 0


def classify(stmt: ir.Assignment, slots: dict, logger: Logger) -> Sweep:
    """Tag one grid assignment (xgrid/lang/generator.py:57-76)."""
    target = stmt.terminal
    assert isinstance(target, ir.Stencil)
    if target.context != "store":
        # g[o][t] = ... : the time subscript makes the grid access a load
        # (xgrid/lang/parser.py:509-518), which the reference rejects as a target
        # (xgrid/lang/generator.py:62-65); every sweep writes level 0
        logger.dead(f"Unable to perform load operation to grid '{target.variable.name}' without stencil context")
    sweep = Sweep(stmt, slots[target.variable.name], target.boundary_mask, False,
                  abs(target.time_offset), pad3(target.space_offset))
    for node in ir.walk(stmt.value):
        if isinstance(node, ir.Stencil):
            if node.context == "store":
                logger.dead(f"Unable to store to grid '{node.variable.name}' inside an expression")
            if node.time_offset == 0 and node.variable.name == target.variable.name and node.boundary_mask == 0:
                sweep.implicit = True
    return sweep


def check_loads(body: list, logger: Logger) -> None:
    """Grid loads are only legal on the right-hand side of a grid assignment
    (xgrid/lang/generator.py:62-65)."""
    for stmt in body:
        if isinstance(stmt, ir.Assignment) and isinstance(stmt.terminal, ir.Stencil):
            continue
        if isinstance(stmt, (ir.If, ir.While)):
            parts = [stmt.condition]
            nested = [stmt.body] + ([stmt.orelse] if isinstance(stmt, ir.If) else [])
        elif isinstance(stmt, ir.For):
            parts, nested = [stmt.start, stmt.end, stmt.step], [stmt.body]
        else:
            parts, nested = [stmt], []
        for part in parts:
            for node in ir.walk(part):
                if isinstance(node, ir.Stencil):
                    logger.dead(f"Unable to perform load operation to grid '{node.variable.name}' without stencil context")
        for block in nested:
            check_loads(block, logger)


def build_groups(sweeps: list, counter: list, fuse: bool) -> list:
    """Partition a run of consecutive sweeps into launch groups (rules above)."""
    groups: list[Group] = []
    current: list[Sweep] = []
    versions: dict = {}
    writes: set = set()
    main_reads: set = set()   # (slot, level, version) read at a nonzero offset by a main sweep

    def close():
        nonlocal current, versions, writes, main_reads
        if current:
            for member in current:
                member.group_index = counter[0]
            groups.append(Group(current, counter[0]))
            counter[0] += 1
        current, versions, writes, main_reads = [], {}, set(), set()

    def annotate(s: Sweep, vers: dict) -> tuple:
        loads = []
        for st, _ in s.loads:
            lv = abs(st.time_offset)
            slot = s._slots[st.variable.name]
            loads.append((st, Load(slot, lv, vers.get((slot, lv), 0), pad3(st.space_offset))))
        tgt = (s.slot, s.level)
        s.read_version_of_target = vers.get(tgt, 0)
        s.write_version = s.read_version_of_target + (1 if s.implicit else 0)
        return loads

    for s in sweeps:
        if not fuse or any(s.store_offset):
            close()
            s.loads = annotate(s, {})
            current = [s]
            close()
            continue
        for attempt in range(2):
            if s.is_main and any(not c.is_main for c in current):
                close()
            loads = annotate(s, versions)
            wkey = (s.slot, s.level, s.write_version)
            conflict = False
            if s.is_main:
                for _, ld in loads:
                    if any(ld.offset) and (ld.slot, ld.level, ld.version) in writes:
                        conflict = True
                if s.implicit and (s.slot, s.level, s.read_version_of_target) in writes:
                    conflict = True
            if wkey in main_reads:
                conflict = True
            if conflict and current and attempt == 0:
                close()
                continue
            break
        s.loads = loads
        current.append(s)
        writes.add((s.slot, s.level, s.write_version))
        if s.is_main:
            for _, ld in loads:
                if any(ld.offset):
                    main_reads.add((ld.slot, ld.level, ld.version))
        if s.implicit:
            versions[(s.slot, s.level)] = s.write_version
    close()

    for g in groups:
        if not g.fusable:
            continue
        written = {(s.slot, s.level, s.write_version) for s in g.sweeps}
        for j, s in enumerate(g.sweeps):
            if s.is_main:
                continue
            offs = sorted({ld.offset for _, ld in s.loads
                           if any(ld.offset) and (ld.slot, ld.level, ld.version) in written})
            if offs:
                g.local_checks.append((j, offs))
    return groups


def collect_sweep(stmt: ir.Assignment, slots: dict, logger: Logger) -> Sweep:
    s = classify(stmt, slots, logger)
    s._slots = slots
    s.loads = [(st, None) for st in ir.stencils(stmt.value)]
    return s


def grid_slots(defn: ir.Definition) -> dict:
    slots = {}
    for name, t in defn.signature.arguments:
        if isinstance(t, GridType):
            slots[name] = len(slots)
    return slots
