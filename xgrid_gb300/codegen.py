"""IR → CUDA (sm_103a) source for one ``@xgrid.kernel``.

Replaces the reference's C/OpenMP generator (xgrid/lang/generator.py:79-442).
The emitted module has

* the user's dataclasses as C structs and every reachable ``@xgrid.function`` as
  a ``__host__ __device__`` function (generator.py:144-165, 184-226, 405-419);
* per launch group (see ``analysis``) one fused kernel plus one kernel per
  sweep, built from three templates:
    - main sweep: tiles of (tz, ty, tx) cells, one CTA per tile, each thread
      walking the tile's cells; tiles whose cells all have mask 0 skip the mask
      read, tiles whose neighbourhood lies inside the grid use unchecked
      addressing; an implicit sweep writes the grid's scratch buffer (and copies
      the cells it does not update) and the launcher exchanges scratch and
      level 0 — the two-phase semantics of generator.py:312-352 without a
      per-call malloc;
    - boundary sweep: one thread per cell of the mask value's cell list instead
      of a full-grid mask scan (generator.py:353-361);
    - fused group: the main phase, then each boundary phase on the tile's own
      boundary cells, separated by ``__syncthreads``;
* a host entry ``xg_kernel_<name>`` that runs the body's control flow on the
  CPU, evaluates every loop-invariant scalar subtree of a sweep once on the
  host (the values the reference recomputes per cell; same IEEE operations, so
  the results are identical) and launches the groups in program order;
* kernels without grid arguments run their body in one device thread.

Expressions keep the reference's C spelling and evaluation order: literals are
C doubles (``repr(v).lower()``, generator.py:393-394), ``x ** 2.0`` becomes one
multiplication (gcc folds ``pow(x, 2.0)`` that way; generator.py:377-383), other
powers call ``pow``/``powf``.
"""
from __future__ import annotations

import dataclasses
import hashlib
import math

from . import analysis, ir
from .config import Configuration
from .log import Logger
from .types import (Boolean, Floating, GridType, Ignore, Integer, Pointer, Structure,
                    Void)

OVERSTEP = {"none": "XG_OVERSTEP_NONE", "limit": "XG_OVERSTEP_LIMIT", "wrap": "XG_OVERSTEP_WRAP"}

# z-walk of 3-D sweeps: planes whose loads are issued together, resident 256-thread CTAs per SM
ZWALK_PLANES = 4
ZWALK_BLOCKS = 4

# staged z-walk of mask-free 3-D sweeps: (y, x) column block of a CTA, thread rows, planes
# prefetched beyond the next one (chunk lengths along z: xg_zstage_chunks)
ZSTAGE_TILE = (8, 128)
ZSTAGE_THREADS = 256
ZSTAGE_AHEAD = 1
ZSTAGE_AHEAD_WIDE = 1  # with three or more staged buffers (three CTAs per SM still fit)
ZSTAGE_MAX_BLOCKS = 3
ZSTAGE_ONE_BARRIER = True

# (tz, ty, tx, block.x, block.y, block.z) per grid dimensionality
DEFAULT_TILING = {1: (1, 1, 1024, 256, 1, 1), 2: (1, 64, 32, 32, 8, 1), 3: (64, 4, 64, 64, 4, 1)}

# tile prologue and cell loop shared by the tile kernels (32-bit coordinates,
# 64-bit linear index per row)
TILE_PROLOGUE = ["  const xg_tile T = xg_tile_of(p.Z, p.Y, p.X, p.tz, p.ty, p.tx, p.nty, p.ntx, p.ntz);",
                 "  const int64_t t = T.t;",
                 "  const int z0 = T.z0, z1 = T.z1, y0 = T.y0, y1 = T.y1, x0 = T.x0, x1 = T.x1;",
                 "  const I sy = (I)p.X, sz = (I)(p.X * p.Y);",
                 "  (void)sy; (void)sz; (void)t;"]
# I is the kernel's index type: int when the grid has fewer than 2^31 cells
CELL_LOOP = ["  for (int z = z0; z < z1; ++z)",
             "  for (int y = y0 + (int)threadIdx.y; y < y1; y += (int)blockDim.y) {",
             "    const I row_ = (I)z * sz + (I)y * sy;",
             "    for (int x = x0 + (int)threadIdx.x; x < x1; x += (int)blockDim.x) {",
             "    const I c = row_ + (I)x;"]

_INT_RANK = {"bool": 0, "int8_t": 1, "int16_t": 2, "int": 3, "int32_t": 3, "int64_t": 4}


def c_type(t) -> str:
    if isinstance(t, Void):
        return "void"
    if isinstance(t, Boolean):
        return "bool"
    if isinstance(t, Integer):
        return f"int{t.width_bits}_t"
    if isinstance(t, Floating):
        return "float" if t.width_bytes == 4 else "double"
    if isinstance(t, Structure):
        return f"struct {t.name}"
    if isinstance(t, Pointer):
        return c_type(t.element) + "*"
    raise TypeError(f"type {t!r} has no C spelling")


def arith(a: str, b: str) -> str:
    """C usual arithmetic conversions for the types the DSL produces."""
    if "double" in (a, b):
        return "double"
    if "float" in (a, b):
        return "float"
    ra, rb = _INT_RANK.get(a, 3), _INT_RANK.get(b, 3)
    r = max(ra, rb, 3)
    return "int64_t" if r == 4 else "int"


def literal(value) -> str:
    if isinstance(value, bool):
        return "true" if value else "false"
    if isinstance(value, float):
        if math.isnan(value):
            return "(0.0/0.0)"
        if math.isinf(value):
            return "(1.0/0.0)" if value > 0 else "(-1.0/0.0)"
    return repr(value).lower()


def pow_exponent(expr: ir.Expression):
    """Exponent folded by gcc (2, 1, 0, -1), else None."""
    if isinstance(expr, ir.Constant) and not isinstance(expr.value, bool) and expr.value in (2, 1, 0, -1):
        return float(expr.value)
    if isinstance(expr, ir.Unary) and expr.operator is ir.UnaryOperator.Neg and isinstance(expr.right, ir.Constant) \
            and not isinstance(expr.right.value, bool) and expr.right.value == 1:
        return -1.0
    return None


@dataclasses.dataclass
class Module:
    """What the Python side needs to call a generated module."""

    source: str
    name: str
    entry: str
    depth: int
    grid_args: list          # [(name, GridType)]
    value_args: list         # [(name, type)] in declaration order
    arg_order: list          # ("grid"|"value", index) per declared argument
    return_type: object
    implicit_slots: list     # grid slots that need a scratch buffer
    aux_per_cell: dict       # grid slot -> bytes per cell of the mixed-precision work area
    batch: bool              # the module exports the batched entry points
    groups: int
    device_only: bool        # kernel has no grid arguments (body runs on the device)
    sweeps: list             # analysis.Sweep per grid assignment (for the oracle and tests)


class CudaGenerator:
    def __init__(self, operator, config: Configuration) -> None:
        self.logger = Logger(self)
        self.op = operator
        self.cfg = config
        self.defn: ir.Definition = operator.ir
        self.structs: dict[str, Structure] = {}
        self.functions: dict = {}       # id(func) -> (Operator, mangled)
        self.function_order: list = []
        self.device_chunks: list[str] = []
        self.host_chunks: list[str] = []
        self.depth = 0
        self.group_counter = [0]
        self.group_tiling: dict = {}
        self.sweeps: list = []
        self.mixed_slots: dict = {}   # grid slot -> aux bytes per cell of mixed-precision loops
        self.group_emitters: list = []
        self._plans: dict = {}
        self.loop_groups: list = []   # groups with a persistent loop launch
        self.slots = analysis.grid_slots(self.defn)
        self.grid_names = {name: i for name, i in self.slots.items()}
        self.mode = OVERSTEP[config.overstep]

    # ================================================================ types
    def use_type(self, t) -> str:
        if isinstance(t, Structure):
            if t.name not in self.structs:
                for _, et in t.elements:
                    self.use_type(et)
                self.structs[t.name] = t
        elif isinstance(t, Pointer):
            self.use_type(t.element)
        return c_type(t)

    def ctype(self, e: ir.Expression) -> str:
        """C type of an expression as gcc would type the reference's C."""
        if isinstance(e, ir.Constant):
            if isinstance(e.value, bool):
                return "int"
            return "int" if isinstance(e.value, int) else "double"
        if isinstance(e, (ir.Identifier, ir.Stencil, ir.Access, ir.Call, ir.Cast)):
            return self.use_type(e.type)
        if isinstance(e, ir.GridInfo):
            return "int"
        if isinstance(e, ir.Unary):
            if e.operator is ir.UnaryOperator.Not:
                return "int"
            return arith(self.ctype(e.right), "int")
        if isinstance(e, ir.Condition):
            a, b = self.ctype(e.body), self.ctype(e.orelse)
            return a if a == b else arith(a, b)
        if isinstance(e, ir.Binary):
            if e.operator.is_compare() or e.operator.is_logic():
                return "int"
            if e.operator is ir.BinaryOperator.Pow:
                return "double" if (isinstance(e.type, Floating) and e.type.width_bits == 64) else "float"
            return arith(self.ctype(e.left), self.ctype(e.right))
        raise TypeError(f"cannot type {type(e).__name__}")

    # ========================================================== expressions
    def expr(self, e: ir.Expression, env) -> str:
        """C source of an expression.  ``env`` resolves stencils, hoisted subtrees
        and grid info (host or device context)."""
        sub = env.substitute(e)
        if sub is not None:
            return sub
        div = getattr(env, "div_map", {}).get(id(e))
        if div is not None:
            return f"xg_divk((double)({self.expr(e.left, env)}), p.h.{div.name})"
        mul = getattr(env, "mul_map", {}).get(id(e))
        if mul is not None:
            h, other = mul
            return f"xg_mulk((double)({self.expr(other, env)}), p.h.{h.name})"
        if isinstance(e, ir.Constant):
            return literal(e.value)
        if isinstance(e, ir.Identifier):
            if isinstance(e.variable.type, Pointer):
                return f"(*{e.variable.name})"
            return e.variable.name
        if isinstance(e, ir.Stencil):
            return env.stencil(e)
        if isinstance(e, ir.Access):
            return f"({self.expr(e.value, env)}).{e.attribute}"
        if isinstance(e, ir.Unary):
            return f"({e.operator.value} {self.expr(e.right, env)})"
        if isinstance(e, ir.Condition):
            return f"({self.expr(e.condition, env)} ? {self.expr(e.body, env)} : {self.expr(e.orelse, env)})"
        if isinstance(e, ir.Cast):
            return f"(({self.use_type(e.type)})({self.expr(e.value, env)}))"
        if isinstance(e, ir.GridInfo):
            return env.grid_info(e, self)
        if isinstance(e, ir.Binary):
            if e.operator is ir.BinaryOperator.Pow:
                double = isinstance(e.type, Floating) and e.type.width_bits == 64
                k = pow_exponent(e.right)
                base = self.expr(e.left, env)
                t = "double" if double else "float"
                if k == 2.0:
                    return f"xg_sq_{'d' if double else 'f'}(({t})({base}))"
                if k == 1.0:
                    return f"(({t})({base}))"
                if k == 0.0:
                    return f"(({t})1)"
                if k == -1.0:
                    return f"(({t})1 / ({t})({base}))"
                return f"{'pow' if double else 'powf'}({base}, {self.expr(e.right, env)})"
            if e.operator is ir.BinaryOperator.Mod and "int" not in self.ctype(e):
                self.logger.dead("Operator '%' requires integer operands in C")
            every = getattr(env, "int_adds", 0)
            if every and e.operator in (ir.BinaryOperator.Add, ir.BinaryOperator.Sub) and self.ctype(e) == "double":
                # every n-th distinct FP64 addition of a sweep runs on the integer pipe (same IEEE
                # result); repeated subexpressions keep one choice so the compiler can still merge them
                lc, rc = self.expr(e.left, env), self.expr(e.right, env)
                key = (e.operator.value, lc, rc)
                soft = env.add_memo.get(key)
                if soft is None:
                    env.add_count += 1
                    soft = env.add_memo[key] = env.add_count % every == 0
                if soft:
                    fn = "xg_dadd_i" if e.operator is ir.BinaryOperator.Add else "xg_dsub_i"
                    return f"{fn}((double)({lc}), (double)({rc}))"
                return f"({lc} {e.operator.value} {rc})"
            return f"({self.expr(e.left, env)} {e.operator.value} {self.expr(e.right, env)})"
        if isinstance(e, ir.Call):
            return self.call(e, env)
        raise TypeError(f"cannot emit {type(e).__name__}")

    def call(self, e: ir.Call, env) -> str:
        from .operator import Operator
        args = []
        for i, a in enumerate(e.arguments):
            code = self.expr(a, env)
            at = e.operator.signature.arguments[i][1]
            if isinstance(at, Pointer) and a.type == at.element:
                code = f"&{code}"
            args.append(code)
        if isinstance(e.operator, ir.Constructor):
            self.use_type(e.operator.type)
            return f"xg_make_{e.operator.type.name}({', '.join(args)})"
        op: Operator = e.operator
        if op.mode == "external":
            # an external names a C function or macro that the kernel's includes, macros or
            # the CUDA headers provide; inside a sweep it runs on the device, so it must be
            # device-callable there (CUDA's math functions are, and so is a macro)
            if op.name in ("tick",):
                self.logger.dead(f"External operator '{op.name}' has no implementation")
            return f"{op.name}({', '.join(args)})"
        return f"{self.function(op)}({', '.join(args)})"

    def function(self, op) -> str:
        key = (op.func, op.self_type.name if op.self_type is not None else None, op.name)
        if key in self.functions:
            return self.functions[key][1]
        mangled = f"xgf_{op.self_type.name}_{op.name}" if op.self_type is not None else f"xgf_{op.name}"
        used = {v[1] for v in self.functions.values()}
        base, n = mangled, 1
        while mangled in used:
            mangled = f"{base}_{n}"
            n += 1
        self.functions[key] = (op, mangled)
        self.function_order.append(key)
        defn = op.ir
        for name, t in defn.signature.arguments:
            if isinstance(t, GridType):
                self.logger.dead(f"Function '{op.name}' takes a grid argument; only kernels may sweep grids")
        return mangled

    # ============================================================ statements
    def block(self, stmts: list, env, indent: str, out: list, ret_mode: str) -> None:
        """Emit a statement list (host entry or device function body)."""
        i = 0
        while i < len(stmts):
            s = stmts[i]
            if isinstance(s, ir.Assignment) and isinstance(s.terminal, ir.Stencil):
                run = []
                while i < len(stmts) and isinstance(stmts[i], ir.Assignment) and isinstance(stmts[i].terminal, ir.Stencil):
                    run.append(stmts[i])
                    i += 1
                if env.device:
                    self.logger.dead("Grid sweeps are only allowed in kernels")
                self.emit_run(run, env, indent, out)
                continue
            i += 1
            if self.cfg.comment:
                out.append(f'#line {s.location.line} "{s.location.file}"')
            if isinstance(s, ir.Assignment):
                out.append(f"{indent}{self.expr(s.terminal, env)} = {self.expr(s.value, env)};")
            elif isinstance(s, ir.Return):
                out.extend(env.ret(self, s, indent))
            elif isinstance(s, ir.Break):
                out.append(f"{indent}break;")
            elif isinstance(s, ir.Continue):
                out.append(f"{indent}continue;")
            elif isinstance(s, ir.Evaluation):
                out.append(f"{indent}{self.expr(s.value, env)};")
            elif isinstance(s, ir.Inline):
                out.append(s.source)
            elif isinstance(s, ir.If):
                out.append(f"{indent}if ({self.expr(s.condition, env)}) {{")
                self.block(s.body, env, indent + "  ", out, ret_mode)
                if s.orelse:
                    out.append(f"{indent}}} else {{")
                    self.block(s.orelse, env, indent + "  ", out, ret_mode)
                out.append(f"{indent}}}")
            elif isinstance(s, ir.While):
                out.append(f"{indent}while ({self.expr(s.condition, env)}) {{")
                self.block(s.body, env, indent + "  ", out, ret_mode)
                out.append(f"{indent}}}")
            elif isinstance(s, ir.For) and self.mixed_plan(s) is not None:
                from . import mixed
                from .mixed import MixedLoopEmitter
                plan = self.mixed_plan(s)
                for sw in plan.group.sweeps:
                    for st, _ in sw.loads:
                        self.depth = max(self.depth, abs(st.time_offset))
                    self.depth = max(self.depth, sw.level)
                self.sweeps.extend(plan.group.sweeps)
                self.mixed_slots[plan.slot] = mixed.AUX_BYTES_PER_CELL
                MixedLoopEmitter(self, plan).emit(env, indent, out)
            elif isinstance(s, ir.For) and self.loop_plan(s) is not None:
                self.emit_loop(s, env, indent, out)
            elif isinstance(s, ir.For):
                v = s.variable.name
                out.append(f"{indent}for ({v} = {self.expr(s.start, env)}; {v} < {self.expr(s.end, env)}; "
                           f"{v} += {self.expr(s.step, env)}) {{")
                self.block(s.body, env, indent + "  ", out, ret_mode)
                out.append(f"{indent}}}")
            else:
                raise TypeError(f"cannot emit statement {type(s).__name__}")

    def mixed_plan(self, loop: ir.For):
        if self.cfg.mixed is None:
            return None
        if id(loop) not in self._plans:
            from . import mixed
            plan = mixed.match(self, loop)
            if plan is not None and not all(mixed.coefficients_stencil_free(sw.stmt.value, plan.target)
                                            for sw in plan.group.sweeps):
                plan = None
            self._plans[id(loop)] = plan
        return self._plans[id(loop)]

    def loop_plan(self, loop: ir.For):
        """The launch group of an in-place loop that runs as one persistent launch, or None.

        The loop qualifies when its body is one implicit main sweep of a grid
        followed by boundary sweeps of that grid (all at the cell itself, level
        0), nothing in it depends on the loop variable, the sweeps form one
        fusable launch group and every load of the rewritten grid reads level 0:
        each iteration is then the same launch with the level and the scratch
        buffer exchanged."""
        if not ((self.cfg.persistent or self.cfg.loop_temporal >= 2) and self.cfg.fuse) or not loop.body:
            return None
        key = ("loop", id(loop))
        if key in self._plans:
            return self._plans[key]
        self._plans[key] = None
        body = loop.body
        if not all(isinstance(s, ir.Assignment) and isinstance(s.terminal, ir.Stencil) for s in body):
            return None
        names = {s.terminal.variable.name for s in body}
        if len(names) != 1:
            return None
        target = names.pop()
        uses = lambda node: any(isinstance(x, ir.Identifier) and x.variable.name == loop.variable.name
                                for x in ir.walk(node))
        for i, st in enumerate(body):
            t = st.terminal
            if t.time_offset != 0 or any(t.space_offset) or (i == 0) != (t.boundary_mask == 0) or uses(st.value):
                return None
        sweeps = [analysis.collect_sweep(st, self.slots, self.logger) for st in body]
        if not sweeps[0].implicit or any(sw.implicit for sw in sweeps[1:]):
            return None
        slot = self.slots[target]
        for sw in sweeps:
            if any(st.variable.name == target and st.time_offset != 0 for st, _ in sw.loads):
                return None
        counter = [self.group_counter[0]]
        groups = analysis.build_groups(sweeps, counter, True)
        # a persistent loop runs the fused kernel; several iterations per launch also take a
        # loop of one sweep
        single = len(groups) == 1 and len(groups[0].sweeps) == 1 and not self.cfg.persistent
        if len(groups) != 1 or not (groups[0].fusable or single) or groups[0].sweeps[0] is not sweeps[0]:
            return None
        if any(sw.write_version != 1 for sw in sweeps) or sweeps[0].read_version_of_target != 0:
            return None
        self._plans[key] = (slot, groups[0])
        return self._plans[key]

    def emit_loop(self, loop: ir.For, env, indent: str, out: list) -> None:
        """Host block of a persistent loop: count the iterations as the loop
        would (leaving the loop variable at its final value), run them in one
        launch, else (launch not applicable) one group launch per iteration."""
        slot, group = self.loop_plan(loop)
        for sw in group.sweeps:
            for st, _ in sw.loads:
                self.depth = max(self.depth, abs(st.time_offset))
            self.depth = max(self.depth, sw.level)
        self.sweeps.extend(group.sweeps)
        gid = group.index
        self.group_counter[0] = gid + 1
        em = SweepGroupEmitter(self, group)
        dim = self.defn.signature.arguments[em.arg_index(slot)][1].dimension
        self.group_tiling[gid] = DEFAULT_TILING[dim]
        em.prepare()
        n, v = self.op.name, loop.variable.name
        out.append(f"{indent}{{")
        out.extend(em.host_hoists(env, indent + "  "))
        out.append(f"{indent}  int64_t xg_K = 0;")
        out.append(f"{indent}  for ({v} = {self.expr(loop.start, env)}; {v} < {self.expr(loop.end, env)}; "
                   f"{v} += {self.expr(loop.step, env)}) ++xg_K;")
        out.append(f"{indent}  if (xg_K > 0) {{")
        # a persistent loop when asked for, else several iterations per launch, else one
        if self.cfg.persistent:
            out.append(f"{indent}    int xg_r = xg_fuse_{n} ? xgl_{n}_{gid}_loop(xg_G, &xg_h, xg_K, xg_s) : 0;")
            out.append(f"{indent}    if (xg_r == 0 && xg_fuse_{n}) xg_r = xgl_{n}_{gid}_tloop(xg_G, &xg_h, xg_K, xg_s);")
        else:
            out.append(f"{indent}    int xg_r = xg_fuse_{n} ? xgl_{n}_{gid}_tloop(xg_G, &xg_h, xg_K, xg_s) : 0;")
        out.append(f"{indent}    if (xg_r < 0) return xg_r;")
        out.append(f"{indent}    if (xg_r == 0) for (int64_t xg_i = 0; xg_i < xg_K; ++xg_i) "
                   f"XG_TRY(xgl_{n}_{gid}(xg_G, &xg_h, xg_s));")
        out.append(f"{indent}  }}")
        out.append(f"{indent}}}")
        em.emit_kernels()
        from . import tloop
        tloop.emit(em, self.cfg.loop_temporal)
        self.group_emitters.append(em)
        if self.cfg.persistent:
            em.emit_loop()
            self.loop_groups.append(gid)

    # ================================================================ sweeps
    def emit_run(self, run: list, env, indent: str, out: list) -> None:
        sweeps = [analysis.collect_sweep(s, self.slots, self.logger) for s in run]
        for s in sweeps:
            for st, _ in s.loads:
                self.depth = max(self.depth, abs(st.time_offset))
            self.depth = max(self.depth, s.level)
        self.sweeps.extend(sweeps)
        groups = analysis.build_groups(sweeps, self.group_counter, self.cfg.fuse)
        for g in groups:
            em = SweepGroupEmitter(self, g)
            dim = self.defn.signature.arguments[em.arg_index(g.sweeps[0].slot)][1].dimension
            self.group_tiling[g.index] = DEFAULT_TILING[dim]
            em.emit(env, indent, out)
            self.group_emitters.append(em)

    # ================================================================ module
    def generate(self) -> Module:
        d = self.defn
        analysis.check_loads(d.body, self.logger)
        grid_args, value_args, order = [], [], []
        for name, t in d.signature.arguments:
            if isinstance(t, GridType):
                if d.signature.arguments and t.dimension not in (1, 2, 3):
                    self.logger.dead(f"Grid '{name}' has {t.dimension} dimensions; 1 to 3 are supported")
                self.use_type(t.element)
                order.append(("grid", len(grid_args)))
                grid_args.append((name, t))
            else:
                if isinstance(t, Ignore):
                    self.logger.dead(f"Argument '{name}' of a kernel needs a concrete type")
                self.use_type(t)
                order.append(("value", len(value_args)))
                value_args.append((name, t))
        rtype = d.signature.return_type
        self.use_type(rtype)
        device_only = not grid_args
        name = self.op.name
        entry = f"xg_kernel_{name}"

        body: list[str] = []
        if device_only:
            env = DeviceScalarEnv(self)
            body_lines: list[str] = []
            self.block(d.body, env, "  ", body_lines, "device")
            self.device_chunks.append(self.scalar_kernel(name, value_args, rtype, d, body_lines))
            body.extend(self.scalar_entry(name, entry, value_args, rtype))
        else:
            env = HostEnv(self)
            lines: list[str] = []
            self.block(d.body, env, "  ", lines, "host")
            body.extend(self.host_entry(name, entry, value_args, rtype, d, lines))

        src: list[str] = ['#include "xgrid_gen.cuh"']
        for inc in self.op.includes:
            src.append(f'#include "{inc}"')
        # preprocessor lines of the kernel's macros also precede the device code, so
        # that sweeps (externals named after a macro) see them; every macro line is
        # still emitted at the top of the entry's body, where the reference puts it
        # (xgrid/lang/generator.py:223-224)
        for m in self.op.macro:
            if m.lstrip().startswith("#"):
                src.append(m)
        src.append("")
        fn_protos, fn_defs = self.function_defs()
        src.extend(self.struct_defs())
        src.extend(fn_protos)
        src.extend(fn_defs)
        src.append(f"static const int xg_overstep = {self.mode};")
        src.append(f"struct xga_{name} {{")
        for an, at in value_args:
            src.append(f"  {c_type(at)} {an};")
        if not value_args:
            src.append("  char xg_empty;")
        src.append("};")
        src.append(f"static int xg_fuse_{name} = {1 if self.cfg.fuse else 0};")
        src.append(f"static int xg_zstage_{name} = 1;  // staged z-walk of mask-free 3-D sweeps (0: register z-walk)")
        src.append(f"static long long xg_zstage_launches_{name} = 0;  // staged z-walk launches issued by the host")
        src.append(f"static int xg_tloop_{name} = 1;  // several loop iterations per launch where possible (0: one)")
        # launch hook (slab decomposition): called before every single-sweep launch with the
        # launch's site (group * 64 + sweep), so that a caller can refresh halo rows first
        src.append(f"static xg_launch_hook_fn xg_hook_{name} = NULL;")
        src.append(f"static void* xg_hook_ctx_{name} = NULL;")
        src.append(f"static int64_t xg_mixed_every_{name} = {int(self.cfg.mixed_every)};")
        src.append(f"static int32_t xg_tiling_{name}[{max(self.group_counter[0], 1)}][6] = {{")
        for gi in range(max(self.group_counter[0], 1)):
            src.append("  {" + ", ".join(str(v) for v in self.group_tiling.get(gi, DEFAULT_TILING[2])) + "},")
        src.append("};")
        batch_host = None
        from . import batch as batch_mod
        if (not device_only and batch_mod.qualifies(self) and len(self.group_emitters) == 1
                and batch_mod.BatchEmitter.usable(self.group_emitters[0].g)):
            em = self.group_emitters[0]
            dev, batch_host = batch_mod.BatchEmitter(self, em.g, em).emit(value_args)
            self.device_chunks.extend(dev)
        src.extend(self.device_chunks)
        src.extend(self.host_chunks)
        src.extend(body)
        if batch_host:
            src.append(batch_host)
        src.append(f'extern "C" int xg_config_{name}(int group, const int32_t* cfg, int fuse) {{')
        src.append(f"  if (fuse >= 0) xg_fuse_{name} = fuse;")
        src.append(f"  if (group < 0 || group >= {self.group_counter[0]} || !cfg) return 0;")
        src.append(f"  for (int i = 0; i < 6; ++i) xg_tiling_{name}[group][i] = cfg[i];")
        src.append("  return 0;")
        src.append("}")
        src.append(f'extern "C" int xg_groups_{name}(void) {{ return {self.group_counter[0]}; }}')
        src.append(f'extern "C" int xg_zstage_set_{name}(int on) {{ xg_zstage_{name} = on; return 0; }}')
        src.append(f'extern "C" long long xg_zstage_launches_get_{name}(void) {{ return xg_zstage_launches_{name}; }}')
        src.append(f'extern "C" int xg_tloop_set_{name}(int on) {{ xg_tloop_{name} = on; return 0; }}')
        src.append(f'extern "C" int xg_set_hook_{name}(xg_launch_hook_fn fn, void* ctx) {{')
        src.append(f"  xg_hook_{name} = fn;")
        src.append(f"  xg_hook_ctx_{name} = ctx;")
        src.append("  return 0;")
        src.append("}")
        src.append(f'extern "C" int xg_get_tiling_{name}(int group, int32_t* cfg) {{')
        src.append(f"  if (group < 0 || group >= {max(self.group_counter[0], 1)}) return -1;")
        src.append(f"  for (int i = 0; i < 6; ++i) cfg[i] = xg_tiling_{name}[group][i];")
        src.append("  return 0;")
        src.append("}")
        src.append(f'extern "C" int xg_mixed_{name}(int64_t every) {{ xg_mixed_every_{name} = every; return 0; }}')
        # error word of the persistent loops (1: a neighbour-tile wait gave up, the results
        # of that call are invalid); clear = 1 resets it
        src.append(f'extern "C" int xg_loop_error_{name}(int clear) {{')
        src.append("  int e = 0;")
        for gid in self.loop_groups:
            src += ["  {", "    unsigned w[2] = {0u, 0u};",
                    f"    if (cudaMemcpyFromSymbol(w, xg_sync_{name}_{gid}, sizeof w) != cudaSuccess) return -1;",
                    "    if (w[1]) e = 1;",
                    "    if (clear && w[1]) {", "      const unsigned z[2] = {0u, 0u};",
                    f"      if (cudaMemcpyToSymbol(xg_sync_{name}_{gid}, z, sizeof z) != cudaSuccess) return -1;",
                    "    }", "  }"]
        src.append("  (void)clear;")
        src.append("  return e;")
        src.append("}")
        implicit = sorted({s.slot for s in self.sweeps if s.implicit})
        if getattr(self.op, "noalloc", False):
            src.extend(self.noalloc_entry(name, entry, grid_args, implicit))
        return Module("\n".join(src) + "\n", name, entry, self.depth + 1, grid_args, value_args, order, rtype,
                      implicit, dict(self.mixed_slots), batch_host is not None, self.group_counter[0], device_only,
                      self.sweeps)

    def noalloc_entry(self, name, entry, grid_args, implicit) -> list[str]:
        """``<entry>_noalloc``: same computation as ``<entry>``, for callers that
        cannot allocate device memory.  The scratch level of every grid that an
        in-place (two-phase) sweep needs is carved out of one file-scope device
        array.  The call exchanges level and scratch buffers as the regular entry
        does, which leaves each such grid's levels permuted among the caller's
        buffers and the array; afterwards device copies put every level's result
        back into the caller's buffer of that level (the buffer left holding no
        level serves as the spare that breaks cycles), so the caller's level
        pointers never change.  Kernels without in-place sweeps get a wrapper
        that only forbids table builds (they need no scratch)."""
        head = [f'extern "C" int {entry}_noalloc(xg_grid* G, int ngrids, const void* args, size_t nargs, void* ret, '
                f'size_t nret, void* stream) {{']
        if not implicit:
            return head + [
                "  // no in-place sweep: no scratch; a missing mask table is an error, not an allocation",
                "  xg_internal_noalloc_scope(1);",
                f"  const int rc = {entry}(G, ngrids, args, nargs, ret, nret, stream);",
                "  xg_internal_noalloc_scope(0);",
                "  return rc;",
                "}"]
        elems = ", ".join(f"sizeof({c_type(grid_args[s][1].element)})" for s in implicit)
        slots = ", ".join(str(s) for s in implicit)
        k = len(implicit)
        pool = f"xg_noalloc_pool_{name}"
        return [
            "// Scratch of the no-alloc variant: a fixed pool in device memory, held by every",
            "// GPU that loads this module until the process exits.  All calls share it.",
            "#define XG_NOALLOC_POOL_BYTES ((size_t)64 << 20)",
            "#define XG_NOALLOC_MAX_DEVICES 64",
            f"static __device__ __align__(256) unsigned char {pool}[XG_NOALLOC_POOL_BYTES];",
            f"static void* {pool}_addr[XG_NOALLOC_MAX_DEVICES];",
        ] + head + [
            "  cudaStream_t s = (cudaStream_t)stream;",
            f"  if (ngrids != {len(grid_args)}) XG_FAIL(\"{name}_noalloc: expected {len(grid_args)} grids, got %d\", "
            f"ngrids);",
            "  int dev = 0;",
            "  XG_CUDA(cudaGetDevice(&dev));",
            "  if (dev < 0 || dev >= XG_NOALLOC_MAX_DEVICES) XG_FAIL(\"no-alloc entry: device %d out of range\", dev);",
            f"  if (!{pool}_addr[dev]) {{  // once per device, with that device current",
            "    void* p = NULL;",
            f"    XG_CUDA(cudaGetSymbolAddress(&p, {pool}));",
            f"    {pool}_addr[dev] = p;",
            "  }",
            f"  unsigned char* base = (unsigned char*){pool}_addr[dev];",
            f"  xg_grid L[{len(grid_args)}];",
            "  memcpy(L, G, sizeof L);",
            f"  const int slots[{k}] = {{{slots}}};",
            f"  const size_t elem[{k}] = {{{elems}}};",
            f"  size_t bytes[{k}], off = 0;",
            f"  for (int i = 0; i < {k}; ++i) {{",
            "    xg_ext e = xg_extent(&L[slots[i]]);",
            "    bytes[i] = elem[i] * (size_t)(e.z * e.y * e.x);",
            "    if (off + bytes[i] > XG_NOALLOC_POOL_BYTES)",
            f"      XG_FAIL(\"{name}_noalloc: grids need %zu bytes of scratch, more than the %zu-byte pool of the "
            f"no-alloc entry point\", off + bytes[i], (size_t)XG_NOALLOC_POOL_BYTES);",
            "    L[slots[i]].scratch = base + off;",
            "    off += (bytes[i] + 255) & ~(size_t)255;",
            "  }",
            "  xg_internal_noalloc_scope(1);",
            f"  int rc = {entry}(L, ngrids, args, nargs, ret, nret, stream);",
            "  xg_internal_noalloc_scope(0);",
            "  if (rc != 0) return rc;",
            "  // undo the level permutation: the level whose caller buffer is the spare moves",
            "  // there (its old buffer becomes the spare); when none does, the rest are cycles",
            "  // among the caller's buffers and one of them moves to the spare (the pool) first",
            f"  for (int i = 0; i < {k}; ++i) {{",
            "    const int g = slots[i];",
            "    const int nl = L[g].levels < XG_MAX_LEVELS ? L[g].levels : XG_MAX_LEVELS;",
            "    void* spare = L[g].scratch;",
            "    for (int round = 0; round < 2 * XG_MAX_LEVELS + 2; ++round) {",
            "      int pending = -1, moved = 0;",
            "      for (int lv = 0; lv < nl; ++lv) {",
            "        if (L[g].level[lv] == G[g].level[lv]) continue;",
            "        pending = lv;",
            "        if (G[g].level[lv] == spare) {",
            "          XG_CUDA(cudaMemcpyAsync(G[g].level[lv], L[g].level[lv], bytes[i], cudaMemcpyDeviceToDevice, s));",
            "          spare = L[g].level[lv];",
            "          L[g].level[lv] = G[g].level[lv];",
            "          moved = 1;",
            "        }",
            "      }",
            "      if (pending < 0) break;",
            "      if (!moved) {",
            "        XG_CUDA(cudaMemcpyAsync(spare, L[g].level[pending], bytes[i], cudaMemcpyDeviceToDevice, s));",
            "        void* t_ = L[g].level[pending];",
            "        L[g].level[pending] = spare;",
            "        spare = t_;",
            "      }",
            "    }",
            "    for (int lv = 0; lv < nl; ++lv)",
            "      if (L[g].level[lv] != G[g].level[lv])",
            f"        XG_FAIL(\"{name}_noalloc: internal error, level %d of grid %d not restored\", lv, g);",
            "  }",
            "  return 0;",
            "}",
        ]

    def struct_defs(self) -> list[str]:
        out = []
        for s in self.structs.values():
            out.append(f"struct {s.name} {{")
            for n, t in s.elements:
                out.append(f"  {c_type(t)} {n};")
            out.append("};")
            params = ", ".join(f"{c_type(t)} {n}" for n, t in s.elements)
            fields = "; ".join(f"v.{n} = {n}" for n, _ in s.elements)
            out.append(f"XG_HD struct {s.name} xg_make_{s.name}({params}) {{ struct {s.name} v; {fields}; return v; }}")
        return out

    def function_defs(self):
        protos, defs = [], []
        done = 0
        while done < len(self.function_order):
            key = self.function_order[done]
            done += 1
            op, mangled = self.functions[key]
            d = op.ir
            rt = self.use_type(d.signature.return_type)
            params = ", ".join(f"{self.use_type(t)} {n}" for n, t in d.signature.arguments)
            proto = f"static __host__ __device__ {rt} {mangled}({params})"
            protos.append(proto + ";")
            lines = [proto + " {"]
            for vn, var in d.scope.items():
                if vn not in d.signature.argnames_map:
                    lines.append(f"  {self.use_type(var.type)} {vn};")
            for m in op.macro:
                lines.append(m)
            env = FunctionEnv(self)
            self.block(d.body, env, "  ", lines, "function")
            lines.append("}")
            defs.extend(lines)
        # struct definitions may have grown while emitting functions; they are
        # written before the prototypes, so nothing else to do here.
        return protos, defs

    def scalar_kernel(self, name, value_args, rtype, d, body_lines) -> str:
        rt = c_type(rtype)
        out = []
        if not isinstance(rtype, Void):
            out.append(f"static __device__ {rt} xg_ret_{name};")
        out.append(f"__global__ void xgk_{name}_scalar(struct xga_{name} xg_a) {{")
        for an, at in value_args:
            out.append(f"  {c_type(at)} {an} = xg_a.{an};")
        for vn, var in d.scope.items():
            if vn not in d.signature.argnames_map:
                out.append(f"  {self.use_type(var.type)} {vn};")
        for m in self.op.macro:
            out.append(m)
        out.extend(body_lines)
        out.append("}")
        return "\n".join(out)

    def scalar_entry(self, name, entry, value_args, rtype) -> list[str]:
        rt = c_type(rtype)
        out = [f'extern "C" int {entry}(xg_grid* G, int ngrids, const void* args, size_t nargs, void* ret, '
               f'size_t nret, void* stream) {{',
               "  (void)G; (void)ngrids;",
               "  cudaStream_t s = (cudaStream_t)stream;",
               f"  struct xga_{name} a;",
               f"  if (nargs != {'sizeof(a)' if value_args else '0'}) XG_FAIL(\"{name}: argument block has %zu bytes, "
               f"expected %zu\", nargs, (size_t){'sizeof(a)' if value_args else '0'});",
               "  memset(&a, 0, sizeof a);",
               "  if (nargs) memcpy(&a, args, nargs);",
               "  xg_prof_launch(-1, s);",
               f"  xgk_{name}_scalar<<<1, 1, 0, s>>>(a);",
               "  XG_CUDA(cudaGetLastError());",
               "  xg_prof_end(-1, s);"]
        if not isinstance(rtype, Void):
            out += [f"  if (!ret || nret != sizeof({rt})) XG_FAIL(\"{name}: return buffer has %zu bytes\", nret);",
                    f"  XG_CUDA(cudaMemcpyFromSymbolAsync(ret, xg_ret_{name}, sizeof({rt}), 0, "
                    f"cudaMemcpyDeviceToHost, s));",
                    "  XG_CUDA(cudaStreamSynchronize(s));"]
        out += ["  return 0;", "}"]
        return out

    def host_entry(self, name, entry, value_args, rtype, d, lines) -> list[str]:
        # generated names in the entry's scope start with xg_ (reserved), so kernel
        # arguments and locals keep their own names, as inline C expects
        out = [f'extern "C" int {entry}(xg_grid* xg_G, int xg_ngrids, const void* xg_args, size_t xg_nargs, '
               f'void* xg_ret, size_t xg_nret, void* xg_stream) {{',
               "  cudaStream_t xg_s = (cudaStream_t)xg_stream;",
               f"  if (xg_ngrids != {len(self.slots)}) XG_FAIL(\"{name}: expected {len(self.slots)} grids, got %d\", "
               f"xg_ngrids);",
               f"  struct xga_{name} xg_a;",
               f"  if (xg_nargs != {'sizeof(xg_a)' if value_args else '0'}) XG_FAIL(\"{name}: argument block has %zu "
               f"bytes, expected %zu\", xg_nargs, (size_t){'sizeof(xg_a)' if value_args else '0'});",
               "  memset(&xg_a, 0, sizeof xg_a);",
               "  if (xg_nargs) memcpy(&xg_a, xg_args, xg_nargs);",
               "  (void)xg_ret; (void)xg_nret; (void)xg_s;"]
        for an, at in value_args:
            out.append(f"  {c_type(at)} {an} = xg_a.{an};")
        for vn, var in d.scope.items():
            if vn not in d.signature.argnames_map:
                out.append(f"  {self.use_type(var.type)} {vn};")
        for m in self.op.macro:
            out.append(m)
        out.extend(lines)
        out += ["  return 0;", "}"]
        return out


# ==================================================================== envs
class HostEnv:
    device = False

    def __init__(self, gen: CudaGenerator) -> None:
        self.gen = gen

    def substitute(self, e):
        return None

    def stencil(self, e):
        self.gen.logger.dead(f"Unable to perform load operation to grid '{e.variable.name}' without stencil context")

    def grid_info(self, e: ir.GridInfo, gen) -> str:
        slot = gen.slots[e.variable.name]
        if e.info == "dimension":
            return str(e.variable.type.dimension)
        return f"((int32_t)xg_G[{slot}].shape[{gen.expr(e.dimension, self)}])"

    def ret(self, gen, s: ir.Return, indent: str) -> list[str]:
        if s.value is None:
            return [f"{indent}return 0;"]
        t = c_type(s.value.type)
        return [f"{indent}{{ {t} xg_r = {gen.expr(s.value, self)};",
                f"{indent}  if (xg_ret && xg_nret == sizeof xg_r) memcpy(xg_ret, &xg_r, sizeof xg_r);",
                f"{indent}  return 0; }}"]


class FunctionEnv(HostEnv):
    device = False

    def ret(self, gen, s, indent):
        if s.value is None:
            return [f"{indent}return;"]
        return [f"{indent}return {gen.expr(s.value, self)};"]

    def grid_info(self, e, gen):
        gen.logger.dead("shape/dimension need a grid argument of a kernel")


class DeviceScalarEnv(FunctionEnv):
    """Body of a kernel without grids, run by one device thread."""

    device = True

    def ret(self, gen, s, indent):
        if s.value is None:
            return [f"{indent}return;"]
        return [f"{indent}{{ xg_ret_{gen.op.name} = {gen.expr(s.value, self)}; return; }}"]


@dataclasses.dataclass
class Hoisted:
    name: str
    ctype: str
    expr: ir.Expression
    divisor: bool = False  # an xg_divisor built from ``expr`` on the host
    scale: bool = False    # an xg_scale (multiplier) built from ``expr`` on the host


class SweepEnv:
    """Device context of one sweep: stencils → preloaded locals, hoisted subtrees
    → kernel parameters."""

    device = True

    def __init__(self, gen, hoisted: dict, loadnames: dict, div_map: dict | None = None,
                 mul_map: dict | None = None) -> None:
        self.gen = gen
        self.hoisted = hoisted
        self.loadnames = loadnames
        self.div_map = div_map or {}
        self.mul_map = mul_map or {}
        self.int_adds = int(getattr(gen.cfg, "int_adds", 0))
        self.add_count = 0
        self.add_memo: dict = {}

    def substitute(self, e):
        h = self.hoisted.get(id(e))
        return f"p.h.{h.name}" if h is not None else None

    def stencil(self, e):
        return self.loadnames[id(e)]

    def grid_info(self, e, gen):
        raise AssertionError("grid info is always hoisted")


def has_stencil(e) -> bool:
    return any(isinstance(n, ir.Stencil) for n in ir.walk(e))


def unsafe_int_div(e) -> bool:
    return any(isinstance(n, ir.Binary) and n.operator in (ir.BinaryOperator.Div, ir.BinaryOperator.Mod)
               and isinstance(n.type, Integer) for n in ir.walk(e))


def zstage_geometry(T: str, nb: int) -> dict:
    """Shape of a staged z-walk CTA for element type ``T`` and ``nb`` staged
    buffers: V cells per 16-byte vector, NTX x NTY threads, RY rows per thread,
    plane rows of PX = TX + 2V elements (cell x0 at column V, halo at V - 1 and
    V + TX), D planes beyond the next one in flight (one when three or more
    buffers share the ring, so that three CTAs fit on an SM)."""
    ty, tx = ZSTAGE_TILE
    size = 8 if T == "double" else 4
    v = 16 // size
    ntx = tx // v
    nty = ZSTAGE_THREADS // ntx
    assert nty >= 1 and ty % nty == 0, "staged tile rows must be a multiple of the thread rows"
    d = ZSTAGE_AHEAD if nb <= 2 else ZSTAGE_AHEAD_WIDE
    px = tx + 2 * v
    plane = nb * (ty + 2) * px * size

    def fit(slots):
        # CTAs per SM that the shared memory allows (228 KiB per SM, 1 KiB reserved per CTA), at
        # most ZSTAGE_MAX_BLOCKS: the register budget ptxas gets follows from it
        return max(1, min(ZSTAGE_MAX_BLOCKS, (228 * 1024) // (slots * plane + 1024)))
    # D + 3 slots: planes z - 1, z, z + 1 and D in flight, a second barrier per plane before a
    # slot is refilled; one slot more lets the plane's first barrier cover the refill
    slots = d + 4 if ZSTAGE_ONE_BARRIER and fit(d + 4) == fit(d + 3) else d + 3
    return {"V": v, "NTX": ntx, "NTY": nty, "RY": ty // nty, "D": d, "PX": px, "TY": ty, "TX": tx,
            "R": slots, "smem": slots * plane, "size": size, "blocks": fit(slots)}


def zstage_frame(kname: str, ptype: str, T: str, srcs: list, loads: list, outs: list) -> str:
    """A staged z-walk kernel.  Each CTA owns a (TY, TX) column block of a chunk
    of ``zlen`` planes (a launch argument) and streams the planes z0-1 .. z1 of
    every source buffer, block plus a one-cell halo (wrapped or clamped), through
    a ring of shared-memory slots with cp.async, D planes beyond the next one in
    flight; 16-byte copies where the block's rows and halo lie inside the grid
    and ``vec`` says the rows are 16-byte aligned, element copies otherwise.
    Every thread owns a 16-byte vector of V consecutive cells in RY rows: per
    plane it reads each needed row of each buffer as one vector from shared
    memory, plus the single cells left and right of it, and computes its V cells
    one by one with the scalar expression (same arithmetic per cell as the
    other paths); results leave as one 16-byte store per row when ``vec``.

    ``loads``: (variable, source index, (oz, oy, ox)), offsets within one cell;
    ``outs``: (destination pointer, value, guard or None, accumulate) -- the cell
    value (an expression of the load variables) is stored, or added to the
    destination's value when ``accumulate``; a guard skips the output when it
    is null.  The parameter struct has Z, Y, X."""
    g = zstage_geometry(T, len(srcs))
    V, NTX, NTY, RY, D, PX, TY, TX, R = (g[k] for k in ("V", "NTX", "NTY", "RY", "D", "PX", "TY", "TX", "R"))

    VT = "double2" if T == "double" else "float4"
    nb = len(srcs)
    comp = "xyzw"
    K = [f"template <typename I> __global__ void __launch_bounds__({ZSTAGE_THREADS}, {g['blocks']}) "
         f"{kname}(const __grid_constant__ {ptype} p, const int zlen, const int vec) {{",
         f"  constexpr int TY = {TY}, TX = {TX}, V = {V}, NTX = {NTX}, NT = {ZSTAGE_THREADS}, D = {D};",
         f"  constexpr int PX = {PX}, PY = TY + 2, PL = PY * PX, R = {R}, NB = {nb};",
         "  constexpr int CR = TX / V + 2, KC = (PY * CR + NT - 1) / NT;  // copies per row and per thread",
         "  extern __shared__ __align__(16) unsigned char xg_zs_raw[];",
         f"  {T}* const ring = ({T}*)xg_zs_raw;  // [R][NB][PY][PX]",
         "  const int tid = threadIdx.x;",
         "  const int ntx = (int)((p.X + TX - 1) / TX), nty = (int)((p.Y + TY - 1) / TY);",
         "  const int ix = blockIdx.x % ntx, iy = (blockIdx.x / ntx) % nty, iz = blockIdx.x / (ntx * nty);",
         "  const int x0 = ix * TX, y0 = iy * TY, z0 = iz * zlen;",
         "  const int z1 = z0 + zlen < (int)p.Z ? z0 + zlen : (int)p.Z;",
         "  const I sy = (I)p.X, sz = (I)(p.X * p.Y);",
         "  // a full block of 16-byte aligned rows: each staged row is TX / V 16-byte copies of the",
         "  // block's cells and two element copies of its halo cells (wrapped or clamped)",
         "  const bool vst = vec && x0 + TX <= (int)p.X;",
         "  I goff[KC];",
         "  int soff[KC];  // ring offset of a 16-byte copy, or -2 - offset of an element copy, -1: none",
         "#pragma unroll",
         "  for (int k = 0; k < KC; ++k) {",
         "    const int e = tid + k * NT, r = e / CR, j = e % CR;",
         "    soff[k] = -1;",
         "    goff[k] = 0;",
         "    if (vst && r < PY) {",
         "      const I row = (I)xg_axis(xg_overstep, y0 - 1 + r, (int)p.Y) * sy;",
         "      if (j < TX / V) {",
         "        soff[k] = r * PX + V + j * V;",
         "        goff[k] = row + x0 + j * V;",
         "      } else {",
         "        const int left = j == TX / V;",
         "        soff[k] = -2 - (r * PX + (left ? V - 1 : V + TX));",
         "        goff[k] = row + (I)xg_axis(xg_overstep, left ? x0 - 1 : x0 + TX, (int)p.X);",
         "      }",
         "    }",
         "  }",
         f"  const {T}* const src[NB] = {{{', '.join(srcs)}}};",
         "  auto stage = [&](int q) {  // plane q into its ring slot (no copies for q beyond the chunk)",
         "    if (q <= z1) {",
         "      const I zb = (I)xg_axis(xg_overstep, q, (int)p.Z) * sz;",
         f"      {T}* const slot = ring + ((q - z0 + 1) % R) * NB * PL;",
         "      if (vst) {",
         "#pragma unroll",
         "        for (int b = 0; b < NB; ++b)",
         "#pragma unroll",
         "          for (int k = 0; k < KC; ++k) {",
         "            if (soff[k] >= 0) xg_cp_async16(slot + b * PL + soff[k], src[b] + zb + goff[k]);",
         "            else if (soff[k] < -1) xg_cp_async(slot + b * PL + (-2 - soff[k]), src[b] + zb + goff[k]);",
         "          }",
         "      } else {  // element copies of columns V - 1 .. V + TX of every row",
         "        for (int e = tid; e < PY * (TX + 2); e += NT) {",
         "          const int r = e / (TX + 2), c = e % (TX + 2);",
         "          const I off = (I)xg_axis(xg_overstep, y0 - 1 + r, (int)p.Y) * sy + "
         "(I)xg_axis(xg_overstep, x0 - 1 + c, (int)p.X);",
         "#pragma unroll",
         "          for (int b = 0; b < NB; ++b) xg_cp_async(slot + b * PL + r * PX + V - 1 + c, src[b] + zb + off);",
         "        }",
         "      }",
         "    }",
         "    xg_cp_async_commit();",
         "  };",
         "#pragma unroll",
         "  for (int q = 0; q < D + 2; ++q) stage(z0 - 1 + q);  // planes z0 - 1 .. z0 + D",
         "  const int tx_t = tid % NTX, ty_t = tid / NTX;",
         "  const int c0 = V + V * tx_t, x = x0 + V * tx_t;  // the thread's first cell: ring column, grid x",
         "  XG_ZSTAGE_WINDOW",
         "  for (int z = z0; z < z1; ++z) {",
         "    stage(z + D + 1);  // into the slot of plane z + D + 2 - R, read for the last time before the",
         "                       // previous plane's first barrier (R = D + 4) or its second (R = D + 3)",
         "    xg_cp_async_wait_group<D>();  // planes up to z + 1 have landed",
         "    __syncthreads();",
         f"    const {T}* const pl_m = ring + ((z - z0) % R) * NB * PL;      // plane z - 1",
         f"    const {T}* const pl_c = ring + ((z - z0 + 1) % R) * NB * PL;  // plane z",
         f"    const {T}* const pl_p = ring + ((z - z0 + 2) % R) * NB * PL;  // plane z + 1",
         "    (void)pl_m; (void)pl_p;",
         "#pragma unroll",
         f"    for (int i = 0; i < {RY}; ++i) {{",
         f"      const int r = ty_t + i * {NTY} + 1, y = y0 + r - 1;",
         "      if (y < (int)p.Y) {  // the same for every lane of a warp that covers whole rows",
         "        const I gb = (I)z * sz + (I)y * sy + (I)x;"]
    # rows of the ring this thread reads: (buffer, oz, oy) -> which of x-1 / x+V it needs too
    rows = {}
    for _, b, (oz, oy, ox) in loads:
        need = rows.setdefault((b, oz, oy), set())
        need.add(ox)
    plane = {-1: "pl_m", 0: "pl_c", 1: "pl_p"}
    zw = sorted({b for (b, oz, oy) in rows if oz == 1 and oy == 0})
    if zw:
        K.append("        if (z == z0) {  // the window's first planes")
        for b in zw:
            for nm, pl in (("m", "pl_m"), ("c", "pl_c")):
                K.append(f"          zw{b}_{nm}[i] = *reinterpret_cast<const {VT}*>(&{pl}[{b} * PL + r * PX + c0]);")
        K.append("        }")

    def rn(b, oz, oy):
        return f"w{b}_{'m' if oz < 0 else ('p' if oz > 0 else 'c')}{'m' if oy < 0 else ('p' if oy > 0 else 'c')}"
    # buffers read at the next plane's centre row keep their centre rows of planes z - 1
    # and z in registers (a window shifted by one plane per step)
    zwin = sorted({b for (b, oz, oy) in rows if oz == 1 and oy == 0})
    for (b, oz, oy), oxs in rows.items():
        base = f"{plane[oz]}[{b} * PL + (r + ({oy})) * PX + c0"
        w = rn(b, oz, oy)
        if b in zwin and oy == 0 and oz <= 0:
            K.append(f"        const {VT} {w} = zw{b}_{'m' if oz < 0 else 'c'}[i];")
        else:
            K.append(f"        const {VT} {w} = *reinterpret_cast<const {VT}*>(&{base}]);")
        if -1 in oxs:
            K.append(f"        const {T} {w}_l = {base} - 1];")
        if 1 in oxs:
            K.append(f"        const {T} {w}_r = {base} + V];")
    for o, _ in enumerate(outs):
        K.append(f"        {T} o{o}[V];")
    for j in range(V):
        K.append("        {")
        for vn, b, (oz, oy, ox) in loads:
            w = rn(b, oz, oy)
            jj = j + ox
            val = f"{w}_l" if jj < 0 else (f"{w}_r" if jj >= V else f"{w}.{comp[jj]}")
            K.append(f"          const {T} {vn} = {val};")
        K.append(f"          const I gi = gb + {j};")
        K.append("          (void)gi;")
        for o, (_, value, _, _) in enumerate(outs):
            K.append(f"          o{o}[{j}] = {value};")
        K.append("        }")
    K.append("        if (x < (int)p.X) {")
    K.append("        if (vec) {  // one 16-byte store per output")
    for o, (dst, _, guard, acc) in enumerate(outs):
        ind = "          "
        if guard:
            K.append(f"{ind}if ({guard}) {{")
            ind += "  "
        vals = ", ".join(f"o{o}[{j}]" for j in range(V))
        if acc:
            K.append(f"{ind}{VT} a = *reinterpret_cast<const {VT}*>(&{dst}[gb]);")
            vals = ", ".join(f"a.{comp[j]} + (o{o}[{j}])" for j in range(V))
        K.append(f"{ind}*reinterpret_cast<{VT}*>(&{dst}[gb]) = make_{VT}({vals});")
        if guard:
            K.append("          }")
    K.append("        } else {")
    K.append("#pragma unroll")
    K.append("          for (int j = 0; j < V; ++j)")
    K.append("            if (x + j < (int)p.X) {")
    for o, (dst, _, guard, acc) in enumerate(outs):
        pre = f"if ({guard}) " if guard else ""
        if acc:
            K.append(f"              {pre}{dst}[gb + j] = {dst}[gb + j] + (o{o}[j]);")
        else:
            K.append(f"              {pre}{dst}[gb + j] = o{o}[j];")
    K += ["            }",
          "        }",
          "        }"]
    for b in zw:
        K += [f"        zw{b}_m[i] = zw{b}_c[i];", f"        zw{b}_c[i] = {rn(b, 1, 0)};"]
    K += ["      }",
          "    }"]
    if R == D + 3:
        K.append("    __syncthreads();  // the slot of plane z - 1 is refilled at the next plane")
    K += ["  }",
          "  xg_cp_async_wait_all();",
          "}"]
    decl = " ".join(f"{VT} zw{b}_m[{RY}], zw{b}_c[{RY}];" for b in zw)
    K = [line.replace("  XG_ZSTAGE_WINDOW", f"  {decl}" if decl else "") for line in K]
    return "\n".join(line for line in K if line)


def zstage_launch(kname: str, T: str, nb: int, ind: str, aligned: list, before: list, after: list) -> list:
    """Host lines launching ``kname`` (a ``zstage_frame`` kernel) with parameters
    ``p`` on stream ``s`` when its shared memory fits; ``aligned``: the pointers
    (sources and destinations) that must be 16-byte aligned for 16-byte copies;
    ``before`` / ``after`` run around the launch, which ends with ``return 0``.
    Falls through otherwise."""
    g = zstage_geometry(T, nb)
    ty, tx = ZSTAGE_TILE
    al = " && ".join(f"((uintptr_t)({a}) & 15) == 0" for a in aligned) or "1"
    L = ["{",
         f"  const size_t smem = {g['smem']};",
         "  static int avail32 = -1, avail64 = -1;",
         "  const bool small = xg_small_index(p.Z, p.Y, p.X);",
         f"  if (small && avail32 < 0) XG_TRY(xg_smem_optin({kname}<int>, &avail32));",
         f"  if (!small && avail64 < 0) XG_TRY(xg_smem_optin({kname}<int64_t>, &avail64));",
         "  int zlen = 0;",
         "  int64_t nt = 0;",
         f"  XG_TRY(xg_zstage_chunks(p.Z, p.Y, p.X, {ty}, {tx}, &zlen, &nt));",
         f"  const int vec = (p.X % {g['V']}) == 0 && {al};",
         "  if (smem <= (size_t)(small ? avail32 : avail64) && nt <= 0x7fffffffLL) {"]
    L += ["    " + b for b in before]
    L += [f"    if (small) {kname}<int><<<(unsigned)nt, {ZSTAGE_THREADS}, smem, s>>>(p, zlen, vec);",
          f"    else {kname}<int64_t><<<(unsigned)nt, {ZSTAGE_THREADS}, smem, s>>>(p, zlen, vec);",
          "    XG_CUDA(cudaGetLastError());"]
    L += ["    " + a for a in after]
    L += ["    return 0;", "  }", "}"]
    return [ind + line for line in L]


class SweepGroupEmitter:
    """Kernels and launchers of one launch group."""

    def __init__(self, gen: CudaGenerator, group: analysis.Group) -> None:
        self.gen = gen
        self.g = group
        self.name = gen.op.name
        self.gid = group.index
        self.hoisted: list[Hoisted] = []
        self.hoist_map: dict = {}
        self.div_map: dict = {}
        self.mul_map: dict = {}
        self.by_text: dict = {}  # (kind, host C text) -> Hoisted: equal subtrees share one parameter

    def _param(self, e: ir.Expression, divisor: bool, scale: bool = False) -> "Hoisted":
        text = self.gen.expr(e, HostEnv(self.gen))
        key = ("k" if divisor else ("s" if scale else "v"), text)
        h = self.by_text.get(key)
        if h is None:
            name = f"{key[0]}{len(self.hoisted)}"
            ctype = "xg_divisor" if divisor else ("xg_scale" if scale else self.gen.ctype(e))
            h = Hoisted(name, ctype, e, divisor, scale)
            self.hoisted.append(h)
            self.by_text[key] = h
        return h

    # ---------------------------------------------------------- hoisting
    def hoist(self, e: ir.Expression, conditional: bool = False) -> None:
        """Hoist maximal stencil-free subtrees (not bare constants)."""
        if not has_stencil(e):
            if isinstance(e, ir.Constant):
                return
            if conditional and unsafe_int_div(e):
                pass  # an integer division guarded by a condition stays per cell
            else:
                self.hoist_map[id(e)] = self._param(e, False)
                return
        if isinstance(e, ir.Binary):
            if (e.operator is ir.BinaryOperator.Div and self.gen.cfg.divisor and self.gen.ctype(e) == "double"
                    and not has_stencil(e.right)):
                # x / d with d fixed for the launch: precomputed reciprocal pair on the host
                self.div_map[id(e)] = self._param(e.right, True)
                self.hoist(e.left, conditional)
                return
            if (e.operator is ir.BinaryOperator.Mul and self.gen.cfg.divisor and self.gen.ctype(e) == "double"
                    and has_stencil(e.left) != has_stencil(e.right)):
                # x * m with m fixed for the launch: exponent arithmetic when m is +-2^s
                inv, other = (e.right, e.left) if has_stencil(e.left) else (e.left, e.right)
                self.mul_map[id(e)] = (self._param(inv, False, True), other)
                self.hoist(other, conditional)
                return
            cond = conditional or e.operator.is_logic()
            self.hoist(e.left, conditional)
            self.hoist(e.right, cond)
        elif isinstance(e, ir.Unary):
            self.hoist(e.right, conditional)
        elif isinstance(e, ir.Condition):
            self.hoist(e.condition, conditional)
            self.hoist(e.body, True)
            self.hoist(e.orelse, True)
        elif isinstance(e, ir.Cast):
            self.hoist(e.value, conditional)
        elif isinstance(e, ir.Access):
            self.hoist(e.value, conditional)
        elif isinstance(e, ir.Call):
            for a in e.arguments:
                self.hoist(a, conditional)

    # ----------------------------------------------------------- emission
    def emit(self, env: HostEnv, indent: str, out: list) -> None:
        self.prepare()
        out.append(f"{indent}{{")
        out.extend(self.host_hoists(env, indent + "  "))
        out.append(f"{indent}  XG_TRY(xgl_{self.name}_{self.gid}(xg_G, &xg_h, xg_s));")
        out.append(f"{indent}}}")
        self.emit_kernels()

    def prepare(self) -> None:
        for s in self.g.sweeps:
            self.hoist(s.stmt.value)

    def host_hoists(self, env, indent: str) -> list:
        """Host lines declaring ``xg_h`` and evaluating every hoisted subtree."""
        gen, n, gid = self.gen, self.name, self.gid
        out = [f"{indent}struct xgh_{n}_{gid} xg_h;", f"{indent}memset(&xg_h, 0, sizeof xg_h);"]
        for h in self.hoisted:
            if h.divisor:
                out.append(f"{indent}xg_h.{h.name} = xg_make_divisor((double)({gen.expr(h.expr, env)}));")
            elif h.scale:
                out.append(f"{indent}xg_h.{h.name} = xg_make_scale((double)({gen.expr(h.expr, env)}));")
            else:
                out.append(f"{indent}xg_h.{h.name} = {gen.expr(h.expr, env)};")
        return out

    def emit_kernels(self) -> None:
        gen, n, gid = self.gen, self.name, self.gid
        hs = [f"struct xgh_{n}_{gid} {{"]
        for h in self.hoisted:
            hs.append(f"  {h.ctype} {h.name};")
        if not self.hoisted:
            hs.append("  char xg_empty;")
        hs.append("};")
        gen.device_chunks.append("\n".join(hs))
        if self.g.fusable:
            self.emit_fused()
        for j, s in enumerate(self.g.sweeps):
            if s.is_main:
                self.emit_main_single(j, s)
            else:
                self.emit_bnd_single(j, s)
        lines = [f"static int xgl_{n}_{gid}(xg_grid* G, const struct xgh_{n}_{gid}* h, cudaStream_t s) {{"]
        if self.g.fusable:
            lines += [f"  if (xg_fuse_{n}) {{",
                      f"    int r = xgl_{n}_{gid}_fused(G, h, s);",
                      "    if (r < 0) return r;",
                      "    if (r > 0) return 0;",
                      "  }"]
        for j, _ in enumerate(self.g.sweeps):
            lines.append(f"  XG_TRY(xgl_{n}_{gid}_s{j}(G, h, s));")
        lines += ["  return 0;", "}"]
        gen.host_chunks.append("\n".join(lines))

    # ------------------------------------------------------------ helpers
    def elem(self, slot: int) -> str:
        return c_type(self.gen.defn.signature.arguments[self.arg_index(slot)][1].element)

    def arg_index(self, slot: int) -> int:
        k = -1
        for i, (_, t) in enumerate(self.gen.defn.signature.arguments):
            if isinstance(t, GridType):
                k += 1
                if k == slot:
                    return i
        raise IndexError(slot)

    def buffers(self, sweeps) -> list:
        """Distinct (slot, level, version) buffers read or written by ``sweeps``."""
        bufs = []
        for s in sweeps:
            for _, ld in s.loads:
                b = (ld.slot, ld.level, ld.version)
                if b not in bufs:
                    bufs.append(b)
            for b in [(s.slot, s.level, s.read_version_of_target), (s.slot, s.level, s.write_version)]:
                if b not in bufs:
                    bufs.append(b)
        return bufs

    @staticmethod
    def bname(b) -> str:
        return f"b{b[0]}_{b[1]}_{b[2]}"

    def buffer_ptr_host(self, b, single) -> str:
        """Host expression of a buffer pointer before this launch's exchanges.

        Fused launch: version 0 is the level pointer, version 1 the scratch buffer
        that an implicit sweep of the group writes.  Single-sweep launch (``single``
        is that sweep): every earlier exchange has already happened, so every
        buffer is the current level pointer except the write of an implicit sweep.
        """
        slot, level, version = b
        if single is not None:
            if single.implicit and b == (single.slot, single.level, single.write_version):
                return f"G[{slot}].scratch"
            return f"G[{slot}].level[{level}]"
        if version == 0:
            return f"G[{slot}].level[{level}]"
        return f"G[{slot}].scratch"

    def slots_used(self, sweeps) -> list:
        out = []
        for b in self.buffers(sweeps):
            if b[0] not in out:
                out.append(b[0])
        return out

    def min_blocks(self) -> int:
        """Resident 256-thread CTAs per SM asked of ptxas: FP64 sweeps are bound by
        the FP64 pipe and keep registers for ILP; FP32/integer sweeps are memory
        bound and want occupancy."""
        wide = any(self.elem(b[0]) == "double" for b in self.buffers(self.g.sweeps))
        return 4 if wide else 6

    def restrict_locals(self, sweeps) -> list:
        """Kernel-local __restrict__ copies of the buffer pointers: distinct buffer
        names never alias (a grid is passed once; levels and scratch are separate
        allocations), which lets the compiler issue the loads of several cells
        before their stores."""
        return [f"  {self.elem(b[0])}* __restrict__ {self.bname(b)} = p.{self.bname(b)};"
                for b in self.buffers(sweeps)]

    def params_struct(self, tag: str, sweeps, extra: list) -> str:
        n, gid = self.name, self.gid
        lines = [f"struct xgp_{n}_{gid}_{tag} {{", f"  struct xgh_{n}_{gid} h;",
                 "  int64_t Z, Y, X;", "  int32_t tz, ty, tx;", "  int64_t ntz, nty, ntx;", "  int same;"]
        for b in self.buffers(sweeps):
            lines.append(f"  {self.elem(b[0])}* {self.bname(b)};")
        for slot in self.slots_used(sweeps):
            lines.append(f"  int64_t e{slot}[3];")
        lines.extend(f"  {x};" for x in extra)
        lines.append("};")
        return "\n".join(lines)

    @staticmethod
    def axis_name(axis: str, o: int) -> str:
        return axis if o == 0 else f"w{axis}_{'m' if o < 0 else 'p'}{abs(o)}"

    def axis_decls(self, sweeps, indent: str) -> list:
        """Edge-tile coordinates (wrap/limit) for every axis offset the loads use."""
        if self.gen.cfg.overstep == "none":
            return []
        used = set()
        for s in sweeps:
            for _, ld in s.loads:
                for axis, o in zip("zyx", ld.offset):
                    if o:
                        used.add((axis, o))
        ext = {"z": "p.Z", "y": "p.Y", "x": "p.X"}
        return [f"{indent}const int {self.axis_name(a, o)} = xg_axis(xg_overstep, {a} + ({o}), (int){ext[a]});"
                for a, o in sorted(used)]

    def load_code(self, sweep, ld: analysis.Load, fast) -> str:
        """Load of one stencil: ``fast`` (True) unchecked interior addressing,
        "edge" per-axis edge coordinates (all grids of the domain's extent),
        False generic per-grid addressing."""
        b = self.bname((ld.slot, ld.level, ld.version))
        oz, oy, ox = ld.offset
        if fast == "flat":
            # overstep "none" with every grid of the launch in one shape: the reference's
            # flattened neighbour ((z+oz)*Y + (y+oy))*X + (x+ox) is c plus a constant
            e = f"p.e{sweep.slot}"
            off = f"({oz}) * ({e}[1] * {e}[2]) + ({oy}) * {e}[2] + ({ox})"
            return f"xg_ldc({b}, xg_flat((int64_t)c + {off}, {e}[0] * {e}[1] * {e}[2]))"
        if fast == "edge_row":
            return f"{b}[{self._row_base(oz, oy)} + (I){self.axis_name('x', ox)}]"
        if fast == "edge":
            if self.gen.cfg.overstep == "none":
                off = f"({oz}) * (int64_t)sz + ({oy}) * (int64_t)sy + ({ox})"
                return f"xg_ldc({b}, xg_flat((int64_t)c + {off}, (int64_t)sz * p.Z))"
            return (f"{b}[(I){self.axis_name('z', oz)} * sz + (I){self.axis_name('y', oy)} * sy + "
                    f"(I){self.axis_name('x', ox)}]")
        if fast:
            off = []
            if oz:
                off.append(f"({oz}) * sz")
            if oy:
                off.append(f"({oy}) * sy")
            if ox:
                off.append(f"({ox})")
            idx = "c" + "".join(f" + {o}" for o in off)
            return f"{b}[{idx}]"
        e = f"p.e{ld.slot}"
        return (f"xg_ldc({b}, xg_addr(xg_overstep, z, y, x, {oz}, {oy}, {ox}, {e}[0], {e}[1], {e}[2]))")

    def value_code(self, sweep, fast: bool, indent: str) -> tuple[list, str]:
        """Preload lines and the value expression of a sweep at cell (z,y,x)=c."""
        lines, names = [], {}
        local = {}
        for st, ld in sweep.loads:
            if ld not in local:
                vn = f"l{len(local)}"
                local[ld] = vn
                lines.append(f"{indent}const {self.elem(ld.slot)} {vn} = {self.load_code(sweep, ld, fast)};")
            names[id(st)] = local[ld]
        env = SweepEnv(self.gen, self.hoist_map, names, self.div_map, self.mul_map)
        return lines, self.gen.expr(sweep.stmt.value, env)

    @staticmethod
    def _row_base(oz: int, oy: int) -> str:
        def part(a, o):
            return f"{a}{'m' if o < 0 else 'p'}{abs(o)}" if o else f"{a}0"
        return f"rb_{part('z', oz)}_{part('y', oy)}"

    def zmarch_ok(self, mains: list, bnd_phases: list) -> bool:
        """3-D single-sweep launch whose loads at a z offset have no y/x offset
        (7-point style) and whose edges wrap or clamp: mask-free tiles walk z."""
        if bnd_phases or len(mains) != 1 or self.gen.cfg.overstep == "none":
            return False
        s = self.g.sweeps[mains[0]]
        if any(s.store_offset):
            return False
        for slot in self.slots_used([s]):
            t = self.gen.defn.signature.arguments[self.arg_index(slot)][1]
            if t.dimension != 3:
                return False
        for _, ld in s.loads:
            oz, oy, ox = ld.offset
            if abs(oz) > 1 or (oz and (oy or ox)):
                return False
        return True

    def zmarch_body(self, j: int, mask_var: str) -> list:
        """Mask-free tiles: every thread owns one (y, x) column of the tile and walks
        it through z.  Loads at z +- 1 come from a three-value register window per
        buffer, loads at y/x offsets from memory at the current plane through
        per-column offsets that are wrapped (or clamped) once per thread.  Same
        arithmetic per cell as the other paths."""
        s = self.g.sweeps[j]
        dst = self.bname((s.slot, s.level, s.write_version))
        hor = sorted({(ld.offset[1], ld.offset[2]) for _, ld in s.loads if ld.offset[0] == 0})
        if (0, 0) not in hor:
            hor.append((0, 0))
        vert = {}  # buffer -> set of z offsets
        for _, ld in s.loads:
            if ld.offset[1] == 0 and ld.offset[2] == 0:
                vert.setdefault(self.bname((ld.slot, ld.level, ld.version)), set()).add(ld.offset[0])
        win = {b: zs for b, zs in vert.items() if zs & {-1, 1}}
        ys = sorted({oy for oy, _ in hor if oy})
        xs = sorted({ox for _, ox in hor if ox})

        def off(oy, ox):
            return f"o_{'m' if oy < 0 else 'p'}{abs(oy)}_{'m' if ox < 0 else 'p'}{abs(ox)}"
        L = [f"  if ({mask_var} && p.same) {{",
             "    for (int y = y0 + (int)threadIdx.y; y < y1; y += (int)blockDim.y)",
             "    for (int x = x0 + (int)threadIdx.x; x < x1; x += (int)blockDim.x) {"]
        L += [f"      const int {self.axis_name('y', o)} = xg_axis(xg_overstep, y + ({o}), (int)p.Y);" for o in ys]
        L += [f"      const int {self.axis_name('x', o)} = xg_axis(xg_overstep, x + ({o}), (int)p.X);" for o in xs]
        L += [f"      const I {off(oy, ox)} = (I){self.axis_name('y', oy)} * sy + (I){self.axis_name('x', ox)};"
              for oy, ox in hor]
        c0 = off(0, 0)
        if any(-1 in zs for zs in win.values()):
            L.append("      const int zlo = xg_axis(xg_overstep, z0 - 1, (int)p.Z);")
        for b, zs in win.items():
            t = self.elem(int(b[1:].split("_")[0]))
            L.append(f"      {t} w{b}_m = {b}[(I){'zlo' if -1 in zs else 'z0'} * sz + {c0}];")
            L.append(f"      {t} w{b}_c = {b}[(I)z0 * sz + {c0}];")
        def plane(ind, zb, names_of, tag):
            """Loads and store of one plane: zb its base, names_of(buffer, oz) the window values."""
            out, names, local = [], {}, {}
            for st, ld in s.loads:
                b = self.bname((ld.slot, ld.level, ld.version))
                oz, oy, ox = ld.offset
                if b in win and oy == 0 and ox == 0:
                    names[id(st)] = names_of(b, oz)
                    continue
                if ld not in local:
                    vn = f"h{tag}_{len(local)}"
                    local[ld] = vn
                    out.append(f"{ind}const {self.elem(ld.slot)} {vn} = {b}[{zb} + {off(oy, ox)}];")
                names[id(st)] = local[ld]
            env = SweepEnv(self.gen, self.hoist_map, names, self.div_map, self.mul_map)
            return out, f"{ind}{dst}[{zb} + {c0}] = {self.gen.expr(s.stmt.value, env)};"

        U = ZWALK_PLANES  # planes per step: the loads of U planes are in flight together
        L += ["      int z = z0;",
              f"      for (; z + {U} <= z1; z += {U}) {{",
              "        const I zb0 = (I)z * sz;"]
        L += [f"        const I zb{k} = zb{k - 1} + sz;" for k in range(1, U)]
        if any(1 in zs for zs in win.values()):
            L.append(f"        const int zn = xg_axis(xg_overstep, z + {U}, (int)p.Z);")
        for b, zs in win.items():
            t = self.elem(int(b[1:].split("_")[0]))
            for k in range(U - 1):
                L.append(f"        const {t} w{b}_{k + 1} = {b}[zb{k + 1} + {c0}];")
            L.append(f"        const {t} w{b}_{U} = {b}[(I){'zn' if 1 in zs else f'(z + {U - 1})'} * sz + {c0}];")

        def wname(k):
            def names_of(b, oz):
                idx = k + oz  # plane index relative to z: -1 -> w_m, 0 -> w_c, j >= 1 -> w_j
                return f"w{b}_m" if idx == -1 else (f"w{b}_c" if idx == 0 else f"w{b}_{idx}")
            return names_of
        stores = []
        for k in range(U):
            loads, store = plane("        ", f"zb{k}", wname(k), str(k))
            L += loads
            stores.append(store)
        L += stores
        for b in win:
            L += [f"        w{b}_m = {f'w{b}_c' if U == 1 else f'w{b}_{U - 1}'};", f"        w{b}_c = w{b}_{U};"]
        L += ["      }",
              "      for (; z < z1; ++z) {",
              "        const I zb = (I)z * sz;"]
        if any(1 in zs for zs in win.values()):
            L.append("        const int zn = xg_axis(xg_overstep, z + 1, (int)p.Z);")
        for b, zs in win.items():
            t = self.elem(int(b[1:].split("_")[0]))
            L.append(f"        const {t} w{b}_p = {b}[(I){'zn' if 1 in zs else 'z'} * sz + {c0}];")
        loads, store = plane("        ", "zb", lambda b, oz: f"w{b}_{'m' if oz < 0 else ('p' if oz > 0 else 'c')}", "r")
        L += loads + [store]
        for b in win:
            L += [f"        w{b}_m = w{b}_c;", f"        w{b}_c = w{b}_p;"]
        L.append("      }")
        L += ["    }", "  }"]
        return L

    def edge_row_loop(self, mains: list, indent: str) -> list:
        """Cell loop of edge tiles under wrap/limit: the wrapped (or clamped) z and
        y coordinates and the row base of every (z, y) offset pair are computed
        once per row, only the x coordinates once per cell."""
        sweeps = [self.g.sweeps[j] for j in mains]
        pairs = sorted({(ld.offset[0], ld.offset[1]) for s in sweeps for _, ld in s.loads})
        zs = sorted({oz for oz, _ in pairs if oz})
        ys = sorted({oy for _, oy in pairs if oy})
        out = [f"{indent}for (int z = z0; z < z1; ++z)",
               f"{indent}for (int y = y0 + (int)threadIdx.y; y < y1; y += (int)blockDim.y) {{",
               f"{indent}  const I row_ = (I)z * sz + (I)y * sy;"]
        out += [f"{indent}  const int {self.axis_name('z', o)} = xg_axis(xg_overstep, z + ({o}), (int)p.Z);"
                for o in zs]
        out += [f"{indent}  const int {self.axis_name('y', o)} = xg_axis(xg_overstep, y + ({o}), (int)p.Y);"
                for o in ys]
        out += [f"{indent}  const I {self._row_base(oz, oy)} = (I){self.axis_name('z', oz)} * sz + "
                f"(I){self.axis_name('y', oy)} * sy;" for oz, oy in pairs]
        out += [f"{indent}  for (int x = x0 + (int)threadIdx.x; x < x1; x += (int)blockDim.x) {{",
                f"{indent}  const I c = row_ + (I)x;"]
        return out

    def main_body(self, sweeps_idx: list, fast, indent: str, mask_vars: dict) -> list:
        lines = []
        if fast == "edge":
            lines += self.axis_decls([self.g.sweeps[j] for j in sweeps_idx], indent)
        elif fast == "edge_row":
            xs = sorted({ld.offset[2] for j in sweeps_idx for _, ld in self.g.sweeps[j].loads if ld.offset[2]})
            lines += [f"{indent}const int {self.axis_name('x', o)} = xg_axis(xg_overstep, x + ({o}), (int)p.X);"
                      for o in xs]
        for j in sweeps_idx:
            s = self.g.sweeps[j]
            dst = self.bname((s.slot, s.level, s.write_version))
            src = self.bname((s.slot, s.level, s.read_version_of_target))
            pre, val = self.value_code(s, fast, indent + "  ")
            cond = f"{mask_vars[j]} || p.m{j}[c] == 0"
            lines.append(f"{indent}if ({cond}) {{")
            lines.extend(pre)
            if any(s.store_offset):
                oz, oy, ox = s.store_offset
                e = f"p.e{s.slot}"
                lines.append(f"{indent}  xg_stc({dst}, xg_addr(xg_overstep, z, y, x, {oz}, {oy}, {ox}, "
                             f"{e}[0], {e}[1], {e}[2]), ({self.elem(s.slot)})({val}));")
            else:
                lines.append(f"{indent}  {dst}[c] = {val};")
            if s.implicit and not any(s.store_offset):
                lines.append(f"{indent}}} else {{")
                lines.append(f"{indent}  {dst}[c] = {src}[c];")
            lines.append(f"{indent}}}")
        return lines

    def rows_for(self, mains: list) -> int:
        """Rows per thread and iteration of the two-phase path (0: not used): as
        many as the registers allow for the sweep's distinct loads."""
        if len(mains) != 1:
            return 0
        s = self.g.sweeps[mains[0]]
        if any(s.store_offset):
            return 0
        numeric = ("float", "double", "int8_t", "int16_t", "int32_t", "int64_t")
        if not all(self.elem(b[0]) in numeric for b in self.buffers([s])):
            return 0
        nl = len(s.distinct_loads()) + (1 if s.implicit else 0)
        return 4 if nl <= 6 else (2 if nl <= 12 else 0)

    def rows_loop(self, j: int, mask_var: str, indent: str = "  ", mode: str = "fast", R: int = 4) -> list:
        """Cell loop that walks ``R`` rows per thread and iteration in two phases:
        every load of the rows first (predicated on the row being in the tile),
        then the stores, so that loads of several rows are in flight together (a
        latency-bound streaming sweep needs that to reach HBM bandwidth).
        ``mode`` "fast": unchecked offsets (interior tiles); "edge": wrapped or
        clamped coordinates computed per row and axis offset (edge tiles whose
        grids share the domain's extent)."""
        s = self.g.sweeps[j]
        dst = self.bname((s.slot, s.level, s.write_version))
        src = self.bname((s.slot, s.level, s.read_version_of_target))
        none = self.gen.cfg.overstep == "none"
        out = [f"{indent}for (int z = z0; z < z1; ++z)",
               f"{indent}for (int yb = y0 + (int)threadIdx.y; yb < y1; yb += {R} * (int)blockDim.y)",
               f"{indent}for (int x = x0 + (int)threadIdx.x; x < x1; x += (int)blockDim.x) {{"]
        if mode == "edge" and not none:
            zs = sorted({ld.offset[0] for ld in s.distinct_loads() if ld.offset[0]})
            xs = sorted({ld.offset[2] for ld in s.distinct_loads() if ld.offset[2]})
            out += [f"{indent}  const int {self.axis_name('z', o)} = xg_axis(xg_overstep, z + ({o}), (int)p.Z);"
                    for o in zs]
            out += [f"{indent}  const int {self.axis_name('x', o)} = xg_axis(xg_overstep, x + ({o}), (int)p.X);"
                    for o in xs]
        exprs = []
        for r in range(R):
            out.append(f"{indent}  const int y_{r} = yb + {r} * (int)blockDim.y;")
            out.append(f"{indent}  const bool ok_{r} = {'true' if r == 0 else f'y_{r} < y1'};")
            out.append(f"{indent}  const I c_{r} = (I)z * sz + (I)y_{r} * sy + (I)x;")
            if mode == "edge" and not none:
                ys = sorted({ld.offset[1] for ld in s.distinct_loads() if ld.offset[1]})
                out += [f"{indent}  const int wy{r}_{'m' if o < 0 else 'p'}{abs(o)} = "
                        f"xg_axis(xg_overstep, y_{r} + ({o}), (int)p.Y);" for o in ys]
            names, local = {}, {}
            for st, ld in s.loads:
                if ld not in local:
                    vn = f"l{len(local)}_{r}"
                    local[ld] = vn
                    b = self.bname((ld.slot, ld.level, ld.version))
                    oz, oy, ox = ld.offset
                    t = self.elem(ld.slot)
                    if mode == "fast":
                        off = "".join(f" + ({o}) * {m}" for o, m in ((oz, "sz"), (oy, "sy")) if o) + \
                            (f" + ({ox})" if ox else "")
                        ref = f"{b}[c_{r}{off}]"
                    elif none:
                        off = f"({oz}) * (int64_t)sz + ({oy}) * (int64_t)sy + ({ox})"
                        ref = f"xg_ldc({b}, xg_flat((int64_t)c_{r} + {off}, (int64_t)sz * p.Z))"
                    else:
                        wy = f"wy{r}_{'m' if oy < 0 else 'p'}{abs(oy)}" if oy else f"y_{r}"
                        ref = f"{b}[(I){self.axis_name('z', oz)} * sz + (I){wy} * sy + (I){self.axis_name('x', ox)}]"
                    out.append(f"{indent}  const {t} {vn} = ok_{r} ? {ref} : ({t})0;")
                names[id(st)] = local[ld]
            if s.implicit:
                t = self.elem(s.slot)
                out.append(f"{indent}  const {t} s_{r} = ok_{r} ? {src}[c_{r}] : ({t})0;")
            env = SweepEnv(self.gen, self.hoist_map, names, self.div_map, self.mul_map)
            exprs.append(self.gen.expr(s.stmt.value, env))
        for r in range(R):
            out.append(f"{indent}  if (ok_{r}) {{")
            out.append(f"{indent}    if ({mask_var} || p.m{j}[c_{r}] == 0) {dst}[c_{r}] = {exprs[r]};")
            if s.implicit:
                out.append(f"{indent}    else {dst}[c_{r}] = s_{r};")
            out.append(f"{indent}  }}")
        out.append(f"{indent}}}")
        return out

    def loop_locals(self, sweeps) -> list:
        """Buffer pointers of the persistent loop kernel: the level and the scratch
        buffer of the implicit sweep change roles every iteration (plain pointers,
        no __restrict__, so no load takes the read-only path); the others are
        read-only for the whole launch."""
        out = []
        for b in self.buffers(sweeps):
            if b[0] == self.g.sweeps[0].slot and b[1] == self.g.sweeps[0].level:
                other = (b[0], b[1], 1 - b[2])
                out.append(f"  {self.elem(b[0])}* {self.bname(b)} = (xg_it & 1) ? p.{self.bname(other)} : "
                           f"p.{self.bname(b)};")
            else:
                out.append(f"  {self.elem(b[0])}* __restrict__ {self.bname(b)} = p.{self.bname(b)};")
        return out

    def main_kernel(self, tag: str, mains: list, bnd_phases: list, final=None, loop: bool = False) -> str:
        """Tile kernel: main sweeps ``mains`` (indices into the group) then the
        boundary phases ``bnd_phases`` on the tile's own cells.  ``loop``: the
        persistent variant, p.K iterations of the group in one cooperative launch
        (tiles strided over the CTAs, each tile waiting for its neighbouring tiles'
        previous iteration)."""
        n, gid = self.name, self.gid
        sweeps = [self.g.sweeps[j] for j in mains]
        # neighbourhood of the main loads, for the unchecked fast path
        lo = [0, 0, 0]
        hi = [0, 0, 0]
        for s in sweeps:
            for _, ld in s.loads:
                for a in range(3):
                    lo[a] = min(lo[a], ld.offset[a])
                    hi[a] = max(hi[a], ld.offset[a])
        zm = self.zmarch_ok(mains, bnd_phases)
        blocks = ZWALK_BLOCKS if zm else self.min_blocks()  # the z walk keeps several planes in registers
        lines = [f"template <typename I> __global__ void __launch_bounds__(256, {blocks}) xgk_{n}_{gid}_{tag}("
                 f"const __grid_constant__ struct xgp_{n}_{gid}_{tag} p) {{"]
        members = [self.g.sweeps[j] for j in list(mains) + list(bnd_phases)]
        if loop:
            lines += ["  for (int xg_it = 0; xg_it < (int)p.K; ++xg_it) {",
                      "  for (int xg_tt = blockIdx.x; xg_tt < (int)(p.ntz * p.nty * p.ntx); xg_tt += gridDim.x) {",
                      "  if (xg_it > 0 && !xg_tile_wait(p.flags, xg_tt, p.ntz, p.nty, p.ntx, p.wrap, (unsigned)xg_it, "
                      "p.err)) return;",
                      "  const xg_tile T = xg_tile_at(xg_tt, p.Z, p.Y, p.X, p.tz, p.ty, p.tx, p.nty, p.ntx, p.ntz);"]
            lines += TILE_PROLOGUE[1:] + self.loop_locals(members)
        else:
            lines += TILE_PROLOGUE + self.restrict_locals(members)
        lines += [
                 f"  const bool fast = p.same && z0 + ({lo[0]}) >= 0 && z1 - 1 + ({hi[0]}) < p.Z && "
                 f"y0 + ({lo[1]}) >= 0 && y1 - 1 + ({hi[1]}) < p.Y && x0 + ({lo[2]}) >= 0 && x1 - 1 + ({hi[2]}) < p.X;"]
        mask_vars = {}
        for j in mains:
            mask_vars[j] = f"mz{j}"
            lines.append(f"  const bool mz{j} = p.tzero{j}[t] != 0;")
        R = self.rows_for(mains)
        if zm:
            lines += self.zmarch_body(mains[0], mask_vars[mains[0]])
            lines.append("  else if (fast) {")
        else:
            lines.append("  if (fast) {")
        if R:
            lines += self.rows_loop(mains[0], mask_vars[mains[0]], "    ", "fast", R)
        else:
            lines += ["  " + l for l in CELL_LOOP]
            lines += self.main_body(mains, True, "      ", mask_vars)
            lines.append("    }}")
        lines.append("  } else if (p.same) {")
        if R:
            lines += self.rows_loop(mains[0], mask_vars[mains[0]], "    ", "edge", R)
        elif self.gen.cfg.overstep != "none":
            lines += self.edge_row_loop(mains, "    ")
            lines += self.main_body(mains, "edge_row", "      ", mask_vars)
            lines.append("    }}")
        else:
            lines += ["  " + l for l in CELL_LOOP]
            lines += self.main_body(mains, "edge", "      ", mask_vars)
            lines.append("    }}")
        lines.append("  } else {")
        lines += ["  " + l for l in CELL_LOOP]
        lines += self.main_body(mains, False, "      ", mask_vars)
        lines.append("    }}")
        lines.append("  }")
        for j in bnd_phases:
            s = self.g.sweeps[j]
            dst = self.bname((s.slot, s.level, s.write_version))
            pre, val = self.value_code(s, False, "    ")
            lines += ["  __syncthreads();",
                      "  {",
                      "    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);",
                      "    const int nthr = blockDim.x * blockDim.y * blockDim.z;",
                      f"    for (int64_t e = p.bo{j}[t] + tid; e < p.bo{j}[t + 1]; e += nthr) {{",
                      f"    const int64_t c = p.bc{j}[e];"]
            decode = [f"    const int64_t x = c % p.e{s.slot}[2], y = (c / p.e{s.slot}[2]) % p.e{s.slot}[1], "
                      f"z = c / (p.e{s.slot}[2] * p.e{s.slot}[1]);",
                      "    (void)x; (void)y; (void)z;"]
            if self.gen.cfg.overstep == "none":
                # no coordinates needed when every grid has the launch's shape
                fpre, fval = self.value_code(s, "flat", "      ")
                lines += ["    if (p.same) {"] + fpre + [f"      {dst}[c] = {fval};", "    } else {"]
                lines += ["  " + l for l in decode + pre] + [f"      {dst}[c] = {val};", "    }"]
            else:
                lines += decode + pre + [f"    {dst}[c] = {val};"]
            lines += ["    }", "  }"]
        if final:
            # a list of per-cell lines, or (lines before the cell loop, per-cell lines, lines after it)
            pre, body, post = final if isinstance(final, tuple) else ([], final, [])
            lines += ["  __syncthreads();"] + ["  " + l for l in pre] + CELL_LOOP
            lines += ["    " + l for l in body]
            lines.append("  }}")
            lines += ["  " + l for l in post]
        if loop:
            lines += ["  xg_tile_done(p.flags, xg_tt, (unsigned)(xg_it + 1));",
                      "  }",
                      "  }"]
        lines.append("}")
        return "\n".join(lines)

    def fill_params(self, tag: str, sweeps, dom_slot: int, single=None, indent: str = "  ") -> list:
        n, gid = self.name, self.gid
        lines = [f"{indent}struct xgp_{n}_{gid}_{tag} p;",
                 f"{indent}memset(&p, 0, sizeof p);",
                 f"{indent}p.h = *h;",
                 f"{indent}const int32_t* tl = xg_tiling_{n}[{gid}];",
                 f"{indent}xg_ext dom = xg_extent(&G[{dom_slot}]);",
                 f"{indent}p.Z = dom.z; p.Y = dom.y; p.X = dom.x;",
                 f"{indent}p.tz = tl[0]; p.ty = tl[1]; p.tx = tl[2];",
                 f"{indent}p.ntz = xg_tiles_along(p.Z, p.tz); p.nty = xg_tiles_along(p.Y, p.ty); "
                 f"p.ntx = xg_tiles_along(p.X, p.tx);",
                 f"{indent}p.same = 1;"]
        for slot in self.slots_used(sweeps):
            lines += [f"{indent}{{ xg_ext e = xg_extent(&G[{slot}]); p.e{slot}[0] = e.z; p.e{slot}[1] = e.y; "
                      f"p.e{slot}[2] = e.x; if (!xg_same_ext(e, dom)) p.same = 0; }}"]
        for b in self.buffers(sweeps):
            lines.append(f"{indent}p.{self.bname(b)} = ({self.elem(b[0])}*){self.buffer_ptr_host(b, single)};")
        return lines

    def check_levels(self, sweeps, single=None, indent="  ") -> list:
        lines = []
        for b in self.buffers(sweeps):
            slot, level, version = b
            lines.append(f"{indent}if (G[{slot}].levels <= {level}) XG_FAIL(\"{self.name}: grid argument {slot} "
                         f"has %d time levels, level {level} is read\", G[{slot}].levels);")
            if "scratch" in self.buffer_ptr_host(b, single):
                lines.append(f"{indent}if (!G[{slot}].scratch) XG_FAIL(\"{self.name}: grid argument {slot} "
                             f"has no scratch buffer\");")
        return lines

    def zstage_buffers(self, j: int):
        """Buffers a staged z-walk of sweep ``j`` streams through shared memory, or
        None when the sweep does not qualify: a z-walk sweep (7-point style, edges
        wrapped or clamped), explicit, every load within one cell in y and x, every
        loaded buffer of one element type."""
        s = self.g.sweeps[j]
        if s.implicit or not self.zmarch_ok([j], []):
            return None
        bufs = []
        for _, ld in s.loads:
            if abs(ld.offset[1]) > 1 or abs(ld.offset[2]) > 1:
                return None
            b = (ld.slot, ld.level, ld.version)
            if b not in bufs:
                bufs.append(b)
        if len({self.elem(b[0]) for b in bufs}) != 1 or self.elem(bufs[0][0]) not in ("float", "double"):
            return None
        return bufs

    def zstage_kernel(self, tag: str, j: int, bufs: list) -> str:
        """Staged z-walk of sweep ``j`` (``zstage_frame``): same arithmetic per
        cell as the other paths."""
        n, gid = self.name, self.gid
        s = self.g.sweeps[j]
        T = self.elem(bufs[0][0])
        dst = self.bname((s.slot, s.level, s.write_version))
        names, local = {}, {}
        loads = []
        for st, ld in s.loads:
            if ld not in local:
                local[ld] = f"l{len(local)}"
                loads.append((local[ld], bufs.index((ld.slot, ld.level, ld.version)), ld.offset))
            names[id(st)] = local[ld]
        env = SweepEnv(self.gen, self.hoist_map, names, self.div_map, self.mul_map)
        val = self.gen.expr(s.stmt.value, env)
        return zstage_frame(f"xgk_{n}_{gid}_{tag}_zs", f"struct xgp_{n}_{gid}_{tag}", T,
                            [f"p.{self.bname(b)}" for b in bufs], loads, [(f"p.{dst}", val, None, False)])

    def emit_main_single(self, j: int, s) -> None:
        n, gid = self.name, self.gid
        tag = f"s{j}"
        sweeps = [s]
        extra = [f"const int32_t* m{j}", f"const uint8_t* tzero{j}"]
        self.gen.device_chunks.append(self.params_struct(tag, sweeps, extra))
        implicit_scatter = s.implicit and any(s.store_offset)
        self.gen.device_chunks.append(self.main_kernel(tag, [j], []))
        zbufs = self.zstage_buffers(j)
        if zbufs:
            self.gen.device_chunks.append(self.zstage_kernel(tag, j, zbufs))
        L = [f"static int xgl_{n}_{gid}_{tag}(xg_grid* G, const struct xgh_{n}_{gid}* h, cudaStream_t s) {{"]
        L += self.check_levels(sweeps, s)
        L += self.fill_params(tag, sweeps, s.slot, s)
        L += [f"  p.m{j} = xg_mask_device(G[{s.slot}].mask);",
              "  int64_t ntiles = 0;",
              f"  XG_TRY(xg_mask_tiles(G[{s.slot}].mask, tl, 0, &p.tzero{j}, NULL, NULL, &ntiles));",
              "  if (ntiles != p.ntz * p.nty * p.ntx) XG_FAIL(\"tile table mismatch\");"]
        if implicit_scatter:
            src = self.bname((s.slot, s.level, s.read_version_of_target))
            dst = self.bname((s.slot, s.level, s.write_version))
            L.append(f"  XG_CUDA(cudaMemcpyAsync(p.{dst}, p.{src}, (size_t)(p.e{s.slot}[0] * p.e{s.slot}[1] * "
                     f"p.e{s.slot}[2]) * sizeof(*p.{dst}), cudaMemcpyDeviceToDevice, s));")
        site = gid * 64 + j
        if zbufs:
            # a grid without boundary cells takes the staged z-walk (every tile mask-free)
            L += [f"  if (p.same && xg_zstage_{n}) {{",
                  "    int64_t nz = 0;",
                  f"    XG_TRY(xg_mask_nonzero(G[{s.slot}].mask, &nz));",
                  "    if (nz == 0)"]
            dst = self.bname((s.slot, s.level, s.write_version))
            L += zstage_launch(f"xgk_{n}_{gid}_{tag}_zs", self.elem(zbufs[0][0]), len(zbufs), "    ",
                               [f"p.{self.bname(b)}" for b in zbufs] + [f"p.{dst}"],
                               [f"if (xg_hook_{n}) XG_TRY(xg_hook_{n}(xg_hook_ctx_{n}, {site}, G, "
                                f"{len(self.gen.slots)}, s));", f"xg_prof_launch({site}, s);",
                                f"++xg_zstage_launches_{n};"],
                               [f"xg_prof_end({site}, s);"])
            L += ["  }"]
        L += ["  dim3 block(tl[3], tl[4], tl[5]), grid;",
              "  XG_TRY(xg_tile_grid(p.ntx, p.nty, p.ntz, &grid));",
              f"  if (xg_hook_{n}) XG_TRY(xg_hook_{n}(xg_hook_ctx_{n}, {site}, G, {len(self.gen.slots)}, s));",
              f"  xg_prof_launch({site}, s);",
              f"  if (xg_small_index(p.Z, p.Y, p.X)) xgk_{n}_{gid}_{tag}<int><<<grid, block, 0, s>>>(p);",
              f"  else xgk_{n}_{gid}_{tag}<int64_t><<<grid, block, 0, s>>>(p);",
              "  XG_CUDA(cudaGetLastError());",
              f"  xg_prof_end({site}, s);"]
        if s.implicit:
            L.append(f"  {{ void* t_ = G[{s.slot}].level[{s.level}]; G[{s.slot}].level[{s.level}] = "
                     f"G[{s.slot}].scratch; G[{s.slot}].scratch = t_; }}")
        L += ["  return 0;", "}"]
        self.gen.host_chunks.append("\n".join(L))

    def emit_bnd_single(self, j: int, s) -> None:
        n, gid = self.name, self.gid
        tag = f"s{j}"
        sweeps = [s]
        extra = ["const int64_t* cells", "int64_t ncells"]
        self.gen.device_chunks.append(self.params_struct(tag, sweeps, extra))
        dst = self.bname((s.slot, s.level, s.write_version))
        pre, val = self.value_code(s, False, "    ")
        K = [f"__global__ void __launch_bounds__(256) xgk_{n}_{gid}_{tag}(const __grid_constant__ "
             f"struct xgp_{n}_{gid}_{tag} p) {{"] + self.restrict_locals(sweeps) + [
             "  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < p.ncells; "
             "e += (int64_t)gridDim.x * blockDim.x) {",
             "    const int64_t c = p.cells[e];",
             f"    const int64_t x = c % p.e{s.slot}[2], y = (c / p.e{s.slot}[2]) % p.e{s.slot}[1], "
             f"z = c / (p.e{s.slot}[2] * p.e{s.slot}[1]);",
             "    (void)x; (void)y; (void)z;"]
        K += pre
        if any(s.store_offset):
            oz, oy, ox = s.store_offset
            e = f"p.e{s.slot}"
            K.append(f"    xg_stc({dst}, xg_addr(xg_overstep, z, y, x, {oz}, {oy}, {ox}, {e}[0], {e}[1], {e}[2]), "
                     f"({self.elem(s.slot)})({val}));")
        else:
            K.append(f"    {dst}[c] = {val};")
        K += ["  }", "}"]
        self.gen.device_chunks.append("\n".join(K))
        L = [f"static int xgl_{n}_{gid}_{tag}(xg_grid* G, const struct xgh_{n}_{gid}* h, cudaStream_t s) {{"]
        L += self.check_levels(sweeps, s)
        L += self.fill_params(tag, sweeps, s.slot, s)
        L += [f"  XG_TRY(xg_mask_cells(G[{s.slot}].mask, {s.mask}, &p.cells, &p.ncells));",
              "  if (p.ncells == 0) return 0;",
              f"  if (xg_hook_{n}) XG_TRY(xg_hook_{n}(xg_hook_ctx_{n}, {gid * 64 + j}, G, {len(self.gen.slots)}, s));",
              "  int64_t nb = (p.ncells + 255) / 256; if (nb > 65535) nb = 65535;",
              f"  xg_prof_launch({gid * 64 + j}, s);",
              f"  xgk_{n}_{gid}_{tag}<<<(unsigned)nb, 256, 0, s>>>(p);",
              "  XG_CUDA(cudaGetLastError());",
              f"  xg_prof_end({gid * 64 + j}, s);",
              "  return 0;", "}"]
        self.gen.host_chunks.append("\n".join(L))

    def emit_fused(self, tag: str = "fused", extra_params: list | None = None, extra_args: str = "",
                   extra_fill: list | None = None, final=None, swap: bool = True) -> None:
        """Fused launch of the whole group.  The variant hooks (extra parameters,
        a final per-cell phase, no level exchange) serve the mixed-precision
        residual launch."""
        n, gid = self.name, self.gid
        sweeps = self.g.sweeps
        mains = [j for j, s in enumerate(sweeps) if s.is_main]
        bnds = [j for j, s in enumerate(sweeps) if not s.is_main]
        extra = list(extra_params or [])
        for j in mains:
            extra += [f"const int32_t* m{j}", f"const uint8_t* tzero{j}"]
        for j in bnds:
            extra += [f"const int32_t* bo{j}", f"const int64_t* bc{j}"]
        self.gen.device_chunks.append(self.params_struct(tag, sweeps, extra))
        self.gen.device_chunks.append(self.main_kernel(tag, mains, bnds, final))
        dom = sweeps[mains[0]].slot
        L = [f"static int xgl_{n}_{gid}_{tag}(xg_grid* G, const struct xgh_{n}_{gid}* h, cudaStream_t s"
             f"{extra_args}) {{"]
        L += self.check_levels(sweeps)
        L += self.fill_params(tag, sweeps, dom)
        L += list(extra_fill or [])
        for j in mains + bnds:
            L.append(f"  if (!xg_same_ext(xg_extent(&G[{sweeps[j].slot}]), dom)) return 0;")
        L.append("  int64_t ntiles = 0;")
        for j in mains:
            sj = sweeps[j]
            L += [f"  p.m{j} = xg_mask_device(G[{sj.slot}].mask);",
                  f"  XG_TRY(xg_mask_tiles(G[{sj.slot}].mask, tl, 0, &p.tzero{j}, NULL, NULL, &ntiles));"]
        for j in bnds:
            sj = sweeps[j]
            L.append(f"  XG_TRY(xg_mask_tiles(G[{sj.slot}].mask, tl, {sj.mask}, NULL, &p.bo{j}, &p.bc{j}, &ntiles));")
        for j, offs in self.g.local_checks:
            sj = sweeps[j]
            flat = ", ".join(str(v) for o in offs for v in o)
            L += ["  {", f"    static const int32_t offs[] = {{{flat}}};", "    int ok = 0;",
                  f"    XG_TRY(xg_mask_tile_local(G[{sj.slot}].mask, tl, {sj.mask}, {len(offs)}, offs, "
                  f"xg_overstep, &ok));",
                  "    if (!ok) return 0;", "  }"]
        L += ["  if (ntiles != p.ntz * p.nty * p.ntx) XG_FAIL(\"tile table mismatch\");",
              "  dim3 block(tl[3], tl[4], tl[5]), grid;",
              "  XG_TRY(xg_tile_grid(p.ntx, p.nty, p.ntz, &grid));",
              f"  xg_prof_launch({gid * 64 + 63 if swap else gid * 64 + 62}, s);",
              f"  if (xg_small_index(p.Z, p.Y, p.X)) xgk_{n}_{gid}_{tag}<int><<<grid, block, 0, s>>>(p);",
              f"  else xgk_{n}_{gid}_{tag}<int64_t><<<grid, block, 0, s>>>(p);",
              "  XG_CUDA(cudaGetLastError());",
              f"  xg_prof_end({gid * 64 + 63 if swap else gid * 64 + 62}, s);"]
        for s in sweeps:
            if s.implicit and swap:
                L.append(f"  {{ void* t_ = G[{s.slot}].level[{s.level}]; G[{s.slot}].level[{s.level}] = "
                         f"G[{s.slot}].scratch; G[{s.slot}].scratch = t_; }}")
        L += ["  return 1;", "}"]
        self.gen.host_chunks.append("\n".join(L))


    def emit_loop(self) -> None:
        """Persistent launch of ``K`` iterations of this group (the body of an
        in-place loop): the fused kernel's tile work in a loop over iterations,
        one cooperative launch of at most the resident CTAs, each tile waiting
        for its neighbouring tiles' previous iteration (completion flags, zeroed
        by a memset before the launch).  The launcher returns 1 when it ran, 0
        when the launch does not apply (shapes, tile-local boundary reads, reads
        beyond the neighbouring tiles, more tiles than flags), so the caller falls
        back to one launch per iteration."""
        n, gid = self.name, self.gid
        sweeps = self.g.sweeps
        mains = [j for j, s in enumerate(sweeps) if s.is_main]
        bnds = [j for j, s in enumerate(sweeps) if not s.is_main]
        extra = ["int64_t K", "unsigned* flags", "unsigned* err", "int wrap"]
        for j in mains:
            extra += [f"const int32_t* m{j}", f"const uint8_t* tzero{j}"]
        for j in bnds:
            extra += [f"const int32_t* bo{j}", f"const int64_t* bc{j}"]
        self.gen.device_chunks.append(
            f"#define XG_LOOP_MAX_TILES_{n}_{gid} 65536\n"
            f"__device__ unsigned xg_flags_{n}_{gid}[XG_LOOP_MAX_TILES_{n}_{gid}];\n"
            f"__device__ unsigned xg_sync_{n}_{gid}[2] = {{0u, 0u}};  // [1]: a tile wait gave up")
        self.gen.device_chunks.append(self.params_struct("loop", sweeps, extra))
        self.gen.device_chunks.append(self.main_kernel("loop", mains, bnds, loop=True))
        dom = sweeps[mains[0]].slot
        s0 = sweeps[0]
        offs = sorted({ld.offset for j in mains for _, ld in sweeps[j].loads})
        flat = ", ".join(str(v) for o in offs for v in o)
        L = [f"static int xgl_{n}_{gid}_loop(xg_grid* G, const struct xgh_{n}_{gid}* h, int64_t K, cudaStream_t s) {{"]
        L += self.check_levels(sweeps)
        L += self.fill_params("loop", sweeps, dom)
        for j in mains + bnds:
            L.append(f"  if (!xg_same_ext(xg_extent(&G[{sweeps[j].slot}]), dom)) return 0;")
        L.append("  int64_t ntiles = 0;")
        for j in mains:
            sj = sweeps[j]
            L += [f"  p.m{j} = xg_mask_device(G[{sj.slot}].mask);",
                  f"  XG_TRY(xg_mask_tiles(G[{sj.slot}].mask, tl, 0, &p.tzero{j}, NULL, NULL, &ntiles));"]
        for j in bnds:
            sj = sweeps[j]
            L.append(f"  XG_TRY(xg_mask_tiles(G[{sj.slot}].mask, tl, {sj.mask}, NULL, &p.bo{j}, &p.bc{j}, &ntiles));")
        for j, loffs in self.g.local_checks:
            sj = sweeps[j]
            lflat = ", ".join(str(v) for o in loffs for v in o)
            L += ["  {", f"    static const int32_t offs[] = {{{lflat}}};", "    int ok = 0;",
                  f"    XG_TRY(xg_mask_tile_local(G[{sj.slot}].mask, tl, {sj.mask}, {len(loffs)}, offs, "
                  f"xg_overstep, &ok));",
                  "    if (!ok) return 0;", "  }"]
        L += ["  {  // every main-sweep read of a mask-0 cell lands in its tile or a neighbouring tile",
              f"    static const int32_t offs[] = {{{flat}}};", "    int ok = 0;",
              f"    XG_TRY(xg_mask_tile_reach(G[{sweeps[mains[0]].slot}].mask, tl, {len(offs)}, offs, xg_overstep, "
              f"&ok));",
              "    if (!ok) return 0;", "  }",
              "  if (ntiles != p.ntz * p.nty * p.ntx) XG_FAIL(\"tile table mismatch\");",
              f"  if (K > 0x7fffffffLL || ntiles > XG_LOOP_MAX_TILES_{n}_{gid}) return 0;",
              "  p.K = K;",
              "  p.wrap = xg_overstep == XG_OVERSTEP_WRAP;",
              "  int dev = 0, sms = 0;",
              "  XG_CUDA(cudaGetDevice(&dev));",
              "  static void* flags_addr[64];",
              "  static void* sync_addr[64];",
              "  if (dev < 0 || dev >= 64) return 0;",
              f"  if (!flags_addr[dev]) XG_CUDA(cudaGetSymbolAddress(&flags_addr[dev], xg_flags_{n}_{gid}));",
              f"  if (!sync_addr[dev]) XG_CUDA(cudaGetSymbolAddress(&sync_addr[dev], xg_sync_{n}_{gid}));",
              "  p.flags = (unsigned*)flags_addr[dev];",
              "  p.err = (unsigned*)sync_addr[dev] + 1;",
              "  const dim3 block(tl[3], tl[4], tl[5]);",
              "  const int threads = tl[3] * tl[4] * tl[5];",
              "  if (threads < 27) return 0;  // a tile wait polls its neighbours with threads 0..26",
              "  const bool small = xg_small_index(p.Z, p.Y, p.X);",
              "  int per_sm = 0;",
              f"  if (small) XG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, xgk_{n}_{gid}_loop<int>, "
              "threads, 0));",
              f"  else XG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, xgk_{n}_{gid}_loop<int64_t>, "
              "threads, 0));",
              "  XG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));",
              "  if (per_sm < 1) return 0;",
              "  const int64_t resident = (int64_t)per_sm * sms;",
              "  const int64_t nb = ntiles < resident ? ntiles : resident;",
              "  if (nb < 1) return 0;",
              "  XG_CUDA(cudaMemsetAsync(p.flags, 0, (size_t)ntiles * sizeof(unsigned), s));",
              "  cudaLaunchConfig_t lc;",
              "  memset(&lc, 0, sizeof lc);",
              "  cudaLaunchAttribute at[1];",
              "  at[0].id = cudaLaunchAttributeCooperative;",
              "  at[0].val.cooperative = 1;",
              "  lc.gridDim = dim3((unsigned)nb, 1, 1);",
              "  lc.blockDim = block;",
              "  lc.dynamicSmemBytes = 0;",
              "  lc.stream = s;",
              "  lc.attrs = at;",
              "  lc.numAttrs = 1;",
              f"  xg_prof_launch({gid * 64 + 61}, s);",
              f"  if (small) XG_CUDA(cudaLaunchKernelEx(&lc, xgk_{n}_{gid}_loop<int>, p));",
              f"  else XG_CUDA(cudaLaunchKernelEx(&lc, xgk_{n}_{gid}_loop<int64_t>, p));",
              f"  xg_prof_end({gid * 64 + 61}, s);",
              # K exchanges of level and scratch: the parity of K decides which buffer holds the result
              f"  if (K & 1) {{ void* t_ = G[{s0.slot}].level[{s0.level}]; G[{s0.slot}].level[{s0.level}] = "
              f"G[{s0.slot}].scratch; G[{s0.slot}].scratch = t_; }}",
              "  return 1;", "}"]
        self.gen.host_chunks.append("\n".join(L))


def source_digest(source: str, flags: list) -> str:
    return hashlib.md5(("\n".join(flags) + "\n" + source).encode()).hexdigest()
