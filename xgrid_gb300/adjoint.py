"""Adjoint (reverse-mode) kernels generated from a stencil kernel's DSL body.

For a kernel whose body is one explicit sweep of the target ``u``::

    u'(c) = f( u(c + o_1), ..., u(c + o_m), k(c + q_1), ..., scalars )

(loads of ``u`` from the previous level, coefficient grids ``k`` that the kernel
never writes), one step's vector-Jacobian product in gather form is::

    lam(x)  =      sum_i  lam'(x - o_i) * df/du_i |(x - o_i)
    g_k(x) +=      sum_j  lam'(x - q_j) * df/dk_j |(x - q_j)

where ``df/dL |(c)`` is the symbolic partial derivative of the right-hand side
with respect to load ``L``, evaluated with every load shifted to cell ``c`` —
the forward offsets transposed.  The partials are derived here from the IR
(sum, product and quotient rules, integer powers), the result is emitted as a
CUDA tile kernel in the kernel's arithmetic type, and
``rollout(...)`` wraps forward steps and adjoint steps in a
``torch.autograd.Function`` with checkpoints every ``checkpoint_every`` steps
and recomputation of each segment during the backward pass.

Every cell must be updated each step (all-zero masks), so that the step is a
function of the previous state only.
"""
from __future__ import annotations

import ctypes

from . import analysis, ir
from .log import Logger
from .types import Floating, GridType

B = ir.BinaryOperator
LOG = Logger("xgrid.adjoint")

# z-walk of the adjoint kernel: planes whose loads are issued together, and resident
# 256-thread CTAs per SM asked of ptxas (registers: planes x buffers x loads per plane)
ZWALK_PLANES = 2
ZWALK_BLOCKS = 4
ZWALK_TILE = (64, 4, 64, 64, 4)  # tz, ty, tx, block x, block y


# ------------------------------------------------------------ symbolic algebra
# nodes: ("c", float) | ("p", name) | ("l", (slot, level, offset)) | (op, a, b) | ("neg", a)
ZERO, ONE = ("c", 0.0), ("c", 1.0)


def s_add(a, b):
    if a == ZERO:
        return b
    if b == ZERO:
        return a
    return ("+", a, b)


def s_sub(a, b):
    if b == ZERO:
        return a
    if a == ZERO:
        return s_neg(b)
    return ("-", a, b)


def s_mul(a, b):
    if a == ZERO or b == ZERO:
        return ZERO
    if a == ONE:
        return b
    if b == ONE:
        return a
    return ("*", a, b)


def s_div(a, b):
    if a == ZERO:
        return ZERO
    if b == ONE:
        return a
    return ("/", a, b)


def s_neg(a):
    if a == ZERO:
        return ZERO
    if a[0] == "neg":
        return a[1]
    return ("neg", a)


def diff(node, wrt):
    kind = node[0]
    if kind in ("c", "p"):
        return ZERO
    if kind == "l":
        return ONE if node[1] == wrt else ZERO
    if kind == "neg":
        return s_neg(diff(node[1], wrt))
    a, b = node[1], node[2]
    da, db = diff(a, wrt), diff(b, wrt)
    if kind == "+":
        return s_add(da, db)
    if kind == "-":
        return s_sub(da, db)
    if kind == "*":
        return s_add(s_mul(da, b), s_mul(a, db))
    if kind == "/":
        return s_sub(s_div(da, b), s_div(s_mul(a, db), s_mul(b, b)))
    raise ValueError(kind)


def loads_of(node, out=None):
    out = [] if out is None else out
    if node[0] == "l":
        if node[1] not in out:
            out.append(node[1])
    elif node[0] in ("+", "-", "*", "/"):
        loads_of(node[1], out)
        loads_of(node[2], out)
    elif node[0] == "neg":
        loads_of(node[1], out)
    return out


def shift(node, d):
    """Every load moved by -d (evaluation at cell x - d)."""
    if node[0] == "l":
        slot, level, off = node[1]
        return ("l", (slot, level, tuple(o - s for o, s in zip(off, d))))
    if node[0] in ("+", "-", "*", "/"):
        return (node[0], shift(node[1], d), shift(node[2], d))
    if node[0] == "neg":
        return ("neg", shift(node[1], d))
    return node


class AdjointGenerator:
    """Builds the adjoint CUDA module of one kernel."""

    def __init__(self, gen) -> None:
        from .codegen import SweepGroupEmitter
        self.gen = gen
        d = gen.defn
        body = d.body
        if len(body) != 1 or not isinstance(body[0], ir.Assignment) or not isinstance(body[0].terminal, ir.Stencil):
            LOG.dead(f"kernel '{gen.op.name}': the adjoint needs a body of exactly one grid assignment")
        st = body[0].terminal
        if st.boundary_mask != 0 or any(st.space_offset) or st.time_offset != 0:
            LOG.dead("the adjoint needs a mask-0 assignment to time 0 at offset 0")
        self.stmt = body[0]
        self.target = st.variable.name
        self.slot = gen.slots[self.target]
        ttype = d.scope[self.target].type
        if not isinstance(ttype.element, Floating):
            LOG.dead("the adjoint needs a floating-point grid")
        self.T = "double" if ttype.element.width_bytes == 8 else "float"
        sweep = analysis.collect_sweep(self.stmt, gen.slots, gen.logger)
        if sweep.implicit:
            LOG.dead("the adjoint does not support in-place (time-0) reads of the target")
        groups = analysis.build_groups([sweep], [0], True)
        self.group = groups[0]
        self.em = SweepGroupEmitter(gen, self.group)
        self.em.prepare()
        self.params: dict = {}
        self.expr = self.to_sym(self.stmt.value)
        self.loads = loads_of(self.expr)
        for slot, level, _ in self.loads:
            if slot == self.slot and level == 0:
                LOG.dead("the adjoint needs the target read from the previous level only")

    # IR → algebra (hoisted launch constants become parameters)
    def to_sym(self, e):
        h = self.em.hoist_map.get(id(e))
        if h is not None:
            self.params[h.name] = h
            return ("p", h.name)
        if isinstance(e, ir.Constant):
            return ("c", float(e.value))
        if isinstance(e, ir.Stencil):
            return ("l", (self.gen.slots[e.variable.name], abs(e.time_offset), analysis.pad3(e.space_offset)))
        if isinstance(e, ir.Unary):
            a = self.to_sym(e.right)
            return s_neg(a) if e.operator is ir.UnaryOperator.Neg else a
        if isinstance(e, ir.Cast):
            return self.to_sym(e.value)
        if isinstance(e, ir.Binary):
            div = self.em.div_map.get(id(e))
            if div is not None:  # division by a launch constant: its value is the divisor's d
                return s_div(self.to_sym(e.left), ("p", div.name + ".d"))
            mul = self.em.mul_map.get(id(e))
            if mul is not None:  # product with a launch constant: its value is the scale's m
                h, other = mul
                return s_mul(self.to_sym(other), ("p", h.name + ".m"))
            a, b = self.to_sym(e.left), self.to_sym(e.right)
            if e.operator is B.Add:
                return s_add(a, b)
            if e.operator is B.Sub:
                return s_sub(a, b)
            if e.operator is B.Mul:
                return s_mul(a, b)
            if e.operator is B.Div:
                return s_div(a, b)
            if e.operator is B.Pow and isinstance(e.right, ir.Constant) and float(e.right.value) == 2.0:
                return s_mul(a, a)
        LOG.dead(f"the adjoint cannot differentiate '{type(e).__name__}' expressions")

    def emit_sym(self, node, loadname) -> str:
        T = self.T
        k = node[0]
        if k == "c":
            return f"(({T}){node[1]!r})"
        if k == "p":
            return f"(({T})p.h.{node[1]})"
        if k == "l":
            return loadname(node[1])
        if k == "neg":
            return f"(-{self.emit_sym(node[1], loadname)})"
        return f"({self.emit_sym(node[1], loadname)} {k} {self.emit_sym(node[2], loadname)})"

    def source(self) -> tuple[str, str]:
        """(CUDA source, entry symbol)."""
        from .codegen import c_type
        gen, em = self.gen, self.em
        n = gen.op.name
        T = self.T
        slots_used = sorted({ld[0] for ld in self.loads} | {self.slot})
        # adjoint terms: for every load L of the forward expression, with offset o:
        #   contribution to grad(grid of L)(x) = lam'(x - o) * (df/dL)(x - o)
        terms = {}
        for key in self.loads:
            slot, level, off = key
            d = diff(self.expr, key)
            if d == ZERO:
                continue
            terms.setdefault(slot, []).append((off, shift(d, off)))
        loads_needed = []
        for slot, lst in terms.items():
            for off, d in lst:
                for ld in loads_of(d):
                    if ld not in loads_needed:
                        loads_needed.append(ld)
        lam_offsets = sorted({tuple(-o for o in off) for lst in terms.values() for off, _ in lst})
        names = {}

        def loadname(key):
            return names[key]

        def addr(off):
            oz, oy, ox = off
            return f"xg_addr(xg_overstep, z, y, x, {oz}, {oy}, {ox}, p.Z, p.Y, p.X)"

        lines = [f"struct xgadj_{n} {{", f"  struct xgh_{n}_{self.group.index} h;", "  int64_t Z, Y, X;",
                 "  int32_t tz, ty, tx;", "  int64_t ntz, nty, ntx;",
                 f"  const {T}* lam_in;", f"  {T}* lam_out;"]
        for slot in slots_used:
            lines.append(f"  const {T}* f{slot}[{gen.depth + 1}];")
            lines.append(f"  {T}* g{slot};")
        lines.append("};")
        allofs = [tuple(o for o in off) for off in lam_offsets] + [k[2] for k in loads_needed]
        lo = [min([0] + [o[a_] for o in allofs]) for a_ in range(3)]
        hi = [max([0] + [o[a_] for o in allofs]) for a_ in range(3)]
        from .codegen import CELL_LOOP, TILE_PROLOGUE, zstage_frame, zstage_launch

        from .codegen import SweepGroupEmitter
        axis_name = SweepGroupEmitter.axis_name
        none_mode = gen.cfg.overstep == "none"

        def body(fast):
            out = []
            if not fast and not none_mode:
                used = sorted({(ax, o) for off in allofs for ax, o in zip("zyx", off) if o})
                ext = {"z": "p.Z", "y": "p.Y", "x": "p.X"}
                out += [f"      const int {axis_name(ax, o)} = xg_axis(xg_overstep, {ax} + ({o}), (int){ext[ax]});"
                        for ax, o in used]

            def ld(buf, off):
                oz, oy, ox = off
                if fast:
                    return f"{buf}[c + ({oz}) * sz + ({oy}) * sy + ({ox})]"
                if none_mode:
                    return f"xg_ldc({buf}, {addr(off)})"
                return (f"{buf}[(I){axis_name('z', oz)} * sz + (I){axis_name('y', oy)} * sy + "
                        f"(I){axis_name('x', ox)}]")
            for i, off in enumerate(lam_offsets):
                names[("lam", off)] = f"a{i}"
                out.append(f"      const {T} a{i} = {ld('p.lam_in', off)};")
            for i, key in enumerate(loads_needed):
                slot, level, off = key
                names[key] = f"v{i}"
                out.append(f"      const {T} v{i} = {ld(f'p.f{slot}[{level}]', off)};")
            for slot in slots_used:
                acc = []
                for off, d in terms.get(slot, []):
                    lam = names[("lam", tuple(-o for o in off))]
                    acc.append(f"({lam} * {self.emit_sym(d, loadname)})")
                total = " + ".join(acc) if acc else f"(({T})0)"
                if slot == self.slot:
                    out.append(f"      p.lam_out[c] = {total};")
                else:
                    out.append(f"      if (p.g{slot}) p.g{slot}[c] = p.g{slot}[c] + ({total});")
            return out

        def totals() -> list:
            # (slot, adjoint value of the cell) for lam and every coefficient gradient
            out = []
            for slot in slots_used:
                acc = []
                for off, d in terms.get(slot, []):
                    lam = names[("lam", tuple(-o for o in off))]
                    acc.append(f"({lam} * {self.emit_sym(d, loadname)})")
                out.append((slot, " + ".join(acc) if acc else f"(({T})0)"))
            return out

        def outputs(idx: str, ind: str) -> list:
            out = []
            for slot, total in totals():
                if slot == self.slot:
                    out.append(f"{ind}p.lam_out[{idx}] = {total};")
                else:
                    out.append(f"{ind}if (p.g{slot}) p.g{slot}[{idx}] = p.g{slot}[{idx}] + ({total});")
            return out

        # z-walk (7-point loads, wrapped or clamped edges): every thread walks one (y, x) column
        # through z, z-neighbours from a register window per buffer, four planes per step
        bufs = {}
        for off in lam_offsets:
            bufs.setdefault("lam", ("p.lam_in", set()))[1].add(off)
        for slot, level, off in loads_needed:
            bufs.setdefault((slot, level), (f"p.f{slot}[{level}]", set()))[1].add(off)
        zwalk = not none_mode and all(abs(o[0]) <= 1 and (o[0] == 0 or (o[1] == 0 and o[2] == 0))
                                      for _, offs in bufs.values() for o in offs)

        def zwalk_body() -> list:
            hor = sorted({(o[1], o[2]) for _, offs in bufs.values() for o in offs if o[0] == 0} | {(0, 0)})
            win = {k: offs for k, (_, offs) in bufs.items() if any(o[0] for o in offs)}
            ys = sorted({oy for oy, _ in hor if oy})
            xs = sorted({ox for _, ox in hor if ox})

            def off(oy, ox):
                return f"o_{'m' if oy < 0 else 'p'}{abs(oy)}_{'m' if ox < 0 else 'p'}{abs(ox)}"

            def wv(k):
                return "lam" if k == "lam" else f"f{k[0]}_{k[1]}"
            c0 = off(0, 0)
            L = ["  for (int y = y0 + (int)threadIdx.y; y < y1; y += (int)blockDim.y)",
                 "  for (int x = x0 + (int)threadIdx.x; x < x1; x += (int)blockDim.x) {"]
            L += [f"    const int {axis_name('y', o)} = xg_axis(xg_overstep, y + ({o}), (int)p.Y);" for o in ys]
            L += [f"    const int {axis_name('x', o)} = xg_axis(xg_overstep, x + ({o}), (int)p.X);" for o in xs]
            L += [f"    const I {off(oy, ox)} = (I){axis_name('y', oy)} * sy + (I){axis_name('x', ox)};"
                  for oy, ox in hor]
            L.append("    const int zlo = xg_axis(xg_overstep, z0 - 1, (int)p.Z);")
            for k in win:
                ptr = bufs[k][0]
                L += [f"    {T} w{wv(k)}_m = {ptr}[(I)zlo * sz + {c0}];",
                      f"    {T} w{wv(k)}_c = {ptr}[(I)z0 * sz + {c0}];"]

            def plane(ind, zb, idx_of, tag):
                out = []
                for k, (ptr, offs) in bufs.items():
                    for o in sorted(offs):
                        key = ("lam", o) if k == "lam" else (k[0], k[1], o)
                        if k in win and o[1] == 0 and o[2] == 0:
                            names[key] = idx_of(k, o[0])
                            continue
                        vn = f"h{tag}_{wv(k)}_{off(o[1], o[2])}"
                        out.append(f"{ind}const {T} {vn} = {ptr}[{zb} + {off(o[1], o[2])}];")
                        names[key] = vn
                return out

            U = ZWALK_PLANES
            L += ["    int z = z0;",
                  f"    for (; z + {U} <= z1; z += {U}) {{",
                  "      const I zb0 = (I)z * sz;"]
            L += [f"      const I zb{i} = zb{i - 1} + sz;" for i in range(1, U)]
            L.append(f"      const int zn = xg_axis(xg_overstep, z + {U}, (int)p.Z);")
            for k in win:
                ptr = bufs[k][0]
                L += [f"      const {T} w{wv(k)}_{i + 1} = {ptr}[zb{i + 1} + {c0}];" for i in range(U - 1)]
                L.append(f"      const {T} w{wv(k)}_{U} = {ptr}[(I)zn * sz + {c0}];")
            outs = []
            for i in range(U):
                def idx_of(k, oz, i=i):
                    j = i + oz
                    return f"w{wv(k)}_m" if j == -1 else (f"w{wv(k)}_c" if j == 0 else f"w{wv(k)}_{j}")
                L += plane("      ", f"zb{i}", idx_of, str(i))
                outs += outputs(f"zb{i} + {c0}", "      ")
            L += outs
            for k in win:
                prev = f"w{wv(k)}_c" if U == 1 else f"w{wv(k)}_{U - 1}"
                L += [f"      w{wv(k)}_m = {prev};", f"      w{wv(k)}_c = w{wv(k)}_{U};"]
            L += ["    }",
                  "    for (; z < z1; ++z) {",
                  "      const I zb = (I)z * sz;",
                  "      const int zn = xg_axis(xg_overstep, z + 1, (int)p.Z);"]
            for k in win:
                L.append(f"      const {T} w{wv(k)}_p = {bufs[k][0]}[(I)zn * sz + {c0}];")
            L += plane("      ", "zb", lambda k, oz: f"w{wv(k)}_{'m' if oz < 0 else ('p' if oz > 0 else 'c')}", "r")
            L += outputs(f"zb + {c0}", "      ")
            for k in win:
                L += [f"      w{wv(k)}_m = w{wv(k)}_c;", f"      w{wv(k)}_c = w{wv(k)}_p;"]
            L += ["    }", "  }"]
            return L

        # staged z-walk (planes of lam', u and the coefficients streamed through shared
        # memory): every offset within one cell on every axis
        staged = zwalk and all(max(abs(c) for c in o) <= 1 for _, offs in bufs.values() for o in offs)
        S = []
        if staged:
            keys = list(bufs)
            zl = []
            for i, off in enumerate(lam_offsets):
                names[("lam", off)] = f"a{i}"
                zl.append((f"a{i}", keys.index("lam"), off))
            for i, key in enumerate(loads_needed):
                slot, level, off = key
                names[key] = f"v{i}"
                zl.append((f"v{i}", keys.index((slot, level)), off))
            zo = [("p.lam_out", tot, None, False) if slot == self.slot else (f"p.g{slot}", tot, f"p.g{slot}", True)
                  for slot, tot in totals()]
            S = [zstage_frame(f"xgk_{n}_adjoint_zs", f"struct xgadj_{n}", T, [bufs[k][0] for k in keys], zl, zo)]
        K = S + [f"template <typename I> __global__ void __launch_bounds__(256, {ZWALK_BLOCKS if zwalk else 4}) "
                 f"xgk_{n}_adjoint(const __grid_constant__ struct xgadj_{n} p) {{"] + TILE_PROLOGUE
        if zwalk:
            K += zwalk_body() + ["}"]
        else:
            K += [f"  const bool fast = z0 + ({lo[0]}) >= 0 && z1 - 1 + ({hi[0]}) < p.Z && y0 + ({lo[1]}) >= 0 && "
                  f"y1 - 1 + ({hi[1]}) < p.Y && x0 + ({lo[2]}) >= 0 && x1 - 1 + ({hi[2]}) < p.X;",
                  "  if (fast) {"]
            K += ["  " + l for l in CELL_LOOP] + body(True) + ["    }}", "  } else {"]
            K += ["  " + l for l in CELL_LOOP] + body(False) + ["    }}", "  }", "}"]
        ns = len(gen.slots)
        value_args = [(a, t) for a, t in gen.defn.signature.arguments if not isinstance(t, GridType)]
        H = [f'extern "C" int xg_adjoint_{n}(void* lam_out, const void* lam_in, const void* const* fields, '
             f'void* const* grads, const int64_t* shape, const void* args, size_t nargs, void* stream) {{',
             "  cudaStream_t s = (cudaStream_t)stream;",
             f"  struct xga_{n} xg_a;",
             "  memset(&xg_a, 0, sizeof xg_a);",
             "  if (nargs) memcpy(&xg_a, args, nargs < sizeof xg_a ? nargs : sizeof xg_a);",
             f"  struct xgh_{n}_{self.group.index} xg_h;",
             "  memset(&xg_h, 0, sizeof xg_h);",
             "  {  // the kernel's arguments, by their own names, for the launch constants"]
        for an, at in value_args:
            H.append(f"    {c_type(at)} {an} = xg_a.{an}; (void){an};")
        from .codegen import HostEnv
        H += em.host_hoists(HostEnv(gen), "    ")[2:]
        H += ["  }", f"  struct xgadj_{n} p;", "  memset(&p, 0, sizeof p);", "  p.h = xg_h;",
              "  p.Z = shape[0]; p.Y = shape[1]; p.X = shape[2];",
              f"  p.lam_in = (const {T}*)lam_in; p.lam_out = ({T}*)lam_out;"]
        for slot in slots_used:
            for lv in range(gen.depth + 1):
                H.append(f"  p.f{slot}[{lv}] = (const {T}*)fields[{slot} * {gen.depth + 1} + {lv}];")
            H.append(f"  p.g{slot} = ({T}*)grads[{slot}];")
        if staged:
            H += [f"  if (xg_adjoint_zstage_{n})"]
            H += zstage_launch(f"xgk_{n}_adjoint_zs", T, len(bufs), "  ",
                               [bufs[k][0] for k in bufs] + ["p.lam_out"] + [f"p.g{sl}" for sl in slots_used
                                                                             if sl != self.slot],
                               ["xg_prof_launch(-2, s);"], ["xg_prof_end(-2, s);"])
        tz, ty, tx, bx, by = ZWALK_TILE if zwalk else (2, 16, 32, 32, 8)
        H += [f"  p.tz = {tz}; p.ty = {ty}; p.tx = {tx};",
              "  p.ntz = xg_tiles_along(p.Z, p.tz); p.nty = xg_tiles_along(p.Y, p.ty); p.ntx = xg_tiles_along(p.X, p.tx);",
              f"  dim3 grid, block({bx}, {by}, 1);",
              "  XG_TRY(xg_tile_grid(p.ntx, p.nty, p.ntz, &grid));",
              "  xg_prof_launch(-2, s);",
              f"  if (xg_small_index(p.Z, p.Y, p.X)) xgk_{n}_adjoint<int><<<grid, block, 0, s>>>(p);",
              f"  else xgk_{n}_adjoint<int64_t><<<grid, block, 0, s>>>(p);",
              "  XG_CUDA(cudaGetLastError());",
              "  xg_prof_end(-2, s);",
              "  return 0;", "}"]
        # the module also needs the hoisted-value struct and the argument struct
        hs = [f"struct xgh_{n}_{self.group.index} {{"] + [f"  {h.ctype} {h.name};" for h in em.hoisted]
        if not em.hoisted:
            hs.append("  char xg_empty;")
        hs.append("};")
        ga = [f"struct xga_{n} {{"] + [f"  {c_type(t)} {an};" for an, t in value_args]
        if not value_args:
            ga.append("  char xg_empty;")
        ga.append("};")
        structs = gen.struct_defs()
        sw = [f"static int xg_adjoint_zstage_{n} = 1;  // staged z-walk of the adjoint step (0: register z-walk)",
              f'extern "C" int xg_adjoint_zstage_set_{n}(int on) {{ xg_adjoint_zstage_{n} = on; return 0; }}']
        src = ['#include "xgrid_gen.cuh"', f"static const int xg_overstep = {gen.mode};"] + structs + ga + hs + \
            lines + K + sw + H
        return "\n".join(src) + "\n", f"xg_adjoint_{n}"


def build(op):
    """Compile and load the adjoint module of kernel ``op``; returns (fn, meta)."""
    from .codegen import CudaGenerator
    from .compiler import Compiler, Library
    from .config import get_config
    cfg = get_config()
    gen = CudaGenerator(op, cfg)
    gen.generate()  # typing, depth and struct definitions
    ag = AdjointGenerator(gen)
    src, sym = ag.source()
    # the adjoint has no bit-exactness contract: let nvcc contract multiply-adds
    flags = [f for f in cfg.nvcc_flags if f != "--fmad=false"]
    lib = Library(Compiler(cacheroot=cfg.cacheroot).compile(src, flags))
    fn = lib.entry(sym)
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                   ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_int64), ctypes.c_void_p,
                   ctypes.c_size_t, ctypes.c_void_p]
    meta = {"depth": gen.depth + 1, "target": ag.slot, "nslots": len(gen.slots), "lib": lib, "T": ag.T,
            "source": src}
    return fn, meta


# ------------------------------------------------------------------- autograd
class Rollout:
    """``steps`` forward calls of a one-sweep kernel as a differentiable map.

    ``rollout = Rollout(kernel, steps)`` and then ``u_T = rollout(u0, {"k": kappa},
    (dt,))`` where ``u0`` and the coefficient tensors are CUDA tensors of the grids'
    shape and dtype; gradients flow to ``u0`` and to every coefficient tensor.

    ``checkpoint_every``: ``1`` keeps every state of the forward pass (each step
    writes straight into its slot of a state pool, so keeping them costs no
    copies) and the backward pass runs adjoint steps only; ``k > 1`` keeps a
    copy of the state every ``k`` steps and the backward pass recomputes each
    segment from its checkpoint.  ``None`` (the default) keeps every state when
    ``steps`` states fit in ``state_budget`` bytes (default: a quarter of the
    device memory free at the forward call), else checkpoints every 20 steps.
    """

    def __init__(self, kernel, steps: int, checkpoint_every: int | None = None,
                 state_budget: int | None = None) -> None:
        from .native import NativeKernel
        if kernel.native is None:
            kernel.native = NativeKernel(kernel)
        self.kernel = kernel
        self.native = kernel.native
        self.steps = int(steps)
        if self.steps < 1:
            LOG.dead("a rollout needs at least one step")
        self.every = None if checkpoint_every is None else max(1, int(checkpoint_every))
        self.state_budget = state_budget
        self.fn, self.meta = build(kernel)
        m = self.native.module
        self.target = m.grid_args[self.meta["target"]][0]
        self.grid_names = [n for n, _ in m.grid_args]
        self.value_names = [n for n, _ in m.value_args]
        self.order = m.arg_order
        self.grids = None

    def set_zstage(self, on: bool) -> None:
        """Staged z-walks (planes streamed through shared memory, the default) or
        register z-walks for the forward and the adjoint steps."""
        self.native.set_zstage(on)
        fn = getattr(self.meta["lib"].dylib, f"xg_adjoint_zstage_set_{self.native.module.name}", None)
        if fn is not None:
            fn.restype = ctypes.c_int
            fn(ctypes.c_int(1 if on else 0))

    def checkpoint_interval(self, state_bytes: int) -> int:
        """Steps between kept states for states of ``state_bytes`` (1: every state)."""
        if self.every is not None:
            return self.every
        budget = self.state_budget
        if budget is None:
            import torch
            free, _ = torch.cuda.mem_get_info()
            budget = free // 4
        return 1 if self.steps * state_bytes <= budget else 20

    def _grids(self, shape, dtype_type):
        from .grid import Grid
        if self.grids is None or self.grids[self.target].shape != tuple(shape):
            self.grids = {n: Grid(tuple(shape), dtype_type) for n in self.grid_names}
        return self.grids

    def _call_args(self, grids, values):
        out = []
        for kind, idx in self.order:
            out.append(grids[self.grid_names[idx]] if kind == "grid" else values[idx])
        return out

    def forward_steps(self, grids, values, count: int):
        args = self._call_args(grids, values)
        for _ in range(count):
            self.kernel(*args)

    def forward_pool(self, grids, values, pool, out) -> None:
        """Steps from ``pool[0]``: step i reads state ``pool[i]`` and writes
        ``pool[i + 1]`` (``out`` for the last step), so every state stays without
        copies.  The first step goes through the kernel call (ticks, uploads,
        tables); the others call the module's entry directly with the target's two
        level pointers moved along the pool (the coefficient grids hold the same
        values in every level, so their levels need no rotation)."""
        torch = _torch()
        from . import device, runtime
        ug = grids[self.target]
        ug._extend_time(self.meta["depth"])
        ug._sync_device(False)
        own = [lv.dev for lv in ug._levels]  # the grid's own buffers, put back afterwards
        dst = [pool[i + 1] if i + 1 < self.steps else out for i in range(self.steps)]
        for lv, t in ((0, pool[0]), (1, dst[0])):  # after the call's tick, level 1 is the source, 0 the target
            level = ug._levels[lv]
            level.dev = t.view(-1).view(torch.uint8)
            level.auth = "dev"
        args = self._call_args(grids, values)
        nk = self.native
        graph, nk.use_graph = nk.use_graph, False
        try:
            self.kernel(*args)
        finally:
            nk.use_graph = graph
            for level, buf in zip(ug._levels, own):
                level.dev = buf
                level.auth = "dev"
        if self.steps == 1:
            return
        gl, vals = nk.split(args)
        t = [i for i, g in enumerate(gl) if g is ug][0]
        packed = nk.pack(vals)
        arr = (runtime.XGGrid * len(gl))(*[g.serialize() for g in gl])
        lib = runtime.load()
        pargs = ctypes.cast(ctypes.byref(packed), ctypes.c_void_p) if vals else None
        nargs = ctypes.sizeof(packed) if vals else 0
        stream = device.stream_handle()
        for i in range(1, self.steps):
            arr[t].level[1] = pool[i].data_ptr()
            arr[t].level[0] = dst[i].data_ptr()
            if lib.xg_call(nk.fn_ptr, arr, len(gl), pargs, nargs, None, 0, stream, 0) != 0:
                LOG.dead(f"kernel '{nk.module.name}' failed: {runtime.last_error()}")

    def __call__(self, u0, coefs: dict, values: tuple):
        return _RolloutFn.apply(self, tuple(values), u0, *[coefs[n] for n in self.coef_names(coefs)])

    def coef_names(self, coefs: dict) -> list:
        names = [n for n in self.grid_names if n != self.target]
        missing = [n for n in names if n not in coefs]
        if missing:
            LOG.dead(f"missing coefficient tensors for {missing}")
        return names


def _torch():
    import torch
    return torch


class _RolloutFn:
    """Built lazily so that importing the package does not import torch."""

    _cls = None

    @classmethod
    def apply(cls, *args):
        if cls._cls is None:
            cls._cls = _make_function()
        return cls._cls.apply(*args)


def _make_function():
    torch = _torch()
    from . import device, runtime

    def _hand_back(caller, s, tensors):
        # results made on the backend stream are read on the caller's stream: order the
        # caller after the backend's work, and tell the caching allocator about the use
        caller.wait_stream(s)
        for t in tensors:
            t.record_stream(caller)

    class Fn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, plan, values, u0, *coefs):
            s = device.stream()
            caller = torch.cuda.current_stream()
            s.wait_stream(caller)  # the inputs may still be in production on the caller's stream
            for t in (u0, *coefs):
                t.record_stream(s)
            names = plan.coef_names(dict.fromkeys(plan.grid_names))
            every = plan.checkpoint_interval(u0.numel() * u0.element_size())
            with torch.cuda.stream(s):
                grids = plan._grids(u0.shape, float)
                for n, t in zip(names, coefs):
                    g = grids[n]
                    g._extend_time(plan.meta["depth"])
                    for lv in range(plan.meta["depth"]):
                        g.tensor(lv).copy_(t)
                if every == 1:
                    # state i (before step i) in slot i; the last step writes the output
                    dt = device.torch_dtype(grids[plan.target].numpy_dtype)
                    pool = torch.empty((plan.steps,) + tuple(u0.shape), dtype=dt, device=u0.device)
                    pool[0].copy_(u0)
                    out = torch.empty_like(pool[0])
                    plan.forward_pool(grids, values, pool, out)
                    ctx.states = pool
                else:
                    ug = grids[plan.target]
                    ug.tensor(0).copy_(u0)
                    checkpoints = [u0.detach().clone()]
                    done = 0
                    while done < plan.steps:
                        cnt = min(every, plan.steps - done)
                        plan.forward_steps(grids, values, cnt)
                        done += cnt
                        if done < plan.steps:
                            checkpoints.append(ug.tensor(0).clone())
                    out = ug.tensor(0).clone()
                    ctx.checkpoints = checkpoints
            _hand_back(caller, s, [out])
            ctx.plan, ctx.values, ctx.names, ctx.every = plan, values, names, every
            ctx.save_for_backward(*coefs)
            return out

        @staticmethod
        def backward(ctx, grad_out):
            plan, values, names, every = ctx.plan, ctx.values, ctx.names, ctx.every
            coefs = ctx.saved_tensors
            s = device.stream()
            caller = torch.cuda.current_stream()
            s.wait_stream(caller)
            for t in (grad_out, *coefs):
                t.record_stream(s)
            with torch.cuda.stream(s):
                lam = grad_out.contiguous().clone()
                gcoef = {n: torch.zeros_like(t) for n, t in zip(names, coefs)}
                depth, ns = plan.meta["depth"], plan.meta["nslots"]
                packed = plan.native.pack(list(values))
                shape3 = (ctypes.c_int64 * 3)(*([1] * (3 - lam.dim()) + list(lam.shape)))

                def adjoint_step(state):
                    fields = (ctypes.c_void_p * (ns * depth))()
                    grads = (ctypes.c_void_p * ns)()
                    for slot, n in enumerate(plan.grid_names):
                        if n == plan.target:
                            for lv in range(depth):
                                fields[slot * depth + lv] = state.data_ptr()
                        else:
                            t = coefs[names.index(n)]
                            for lv in range(depth):
                                fields[slot * depth + lv] = t.data_ptr()
                            grads[slot] = gcoef[n].data_ptr()
                    new = torch.empty_like(lam)
                    rc = plan.fn(new.data_ptr(), lam.data_ptr(), fields, grads, shape3,
                                 ctypes.byref(packed) if plan.value_names else None,
                                 ctypes.sizeof(packed) if plan.value_names else 0, device.stream_handle())
                    if rc != 0:
                        LOG.dead(f"adjoint kernel failed: {runtime.last_error()}")
                    return new

                if every == 1:
                    for i in reversed(range(plan.steps)):
                        lam = adjoint_step(ctx.states[i])
                    ctx.states = None
                else:
                    grids = plan._grids(grad_out.shape, float)
                    ug = grids[plan.target]
                    for seg in reversed(range(len(ctx.checkpoints))):
                        start = seg * every
                        cnt = min(every, plan.steps - start)
                        states = [ctx.checkpoints[seg]]
                        ug.tensor(0).copy_(ctx.checkpoints[seg])
                        for _ in range(cnt - 1):
                            plan.forward_steps(grids, values, 1)
                            states.append(ug.tensor(0).clone())
                        for i in reversed(range(cnt)):
                            lam = adjoint_step(states[i])
            _hand_back(caller, s, [lam] + list(gcoef.values()))
            return (None, None, lam) + tuple(gcoef[n] for n in names)

    return Fn
