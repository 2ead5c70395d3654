"""Mixed-precision lowering of affine in-place iteration loops.

A loop of the form (the cavity's pressure iterations, xgrid example
``cavity.py:99-113``)::

    for _ in range(a, b):
        p[0, 0] = f(p[..][0], other fields, scalars)   # mask 0, reads p at time 0
        with xgrid.boundary(k): p[0, 0] = g_k(p[..][0], ...)
        ...

applies the same affine map ``G(p) = L(p) + c`` to ``p`` K times.  With
``xgrid.init(mixed="fp32")`` it runs as defect correction: keep ``p`` (FP64) as
the base and iterate on the defect ``d = p_k - base`` in FP32::

    r      = G(base) - base                 FP64 sweep + boundary phases, rounded once
    d_1    = r
    d_k+1  = L(d_k) + r                     FP32 sweeps: the linear part of the body
    base  += d                              FP64 correction, every ``mixed_every`` iterations

so FP64 arithmetic is only spent on the residual and the correction update.
``L`` is derived symbolically from the DSL body: loads of ``p`` at time 0 become
defect loads, terms that do not depend on ``p`` vanish, coefficients are
evaluated once on the host and rounded to FP32.

The loop qualifies when every sweep of its body writes the same FP64 grid at
time 0 and offset 0, the first sweep is the implicit mask-0 sweep, the others are
boundary sweeps, every right-hand side is affine in that grid's time-0 loads,
and the loop variable is not used in the body.  At run time the lowering also
needs the fused-launch conditions of the group (same extents, boundary reads
inside their tile); otherwise the FP64 loop runs unchanged.
"""
from __future__ import annotations

import dataclasses

from . import analysis, ir
from .types import Floating

B = ir.BinaryOperator

# Work area of a loop in the grid's ``aux`` buffer (xg_mx_layout in xgrid_gen.cuh):
# FP32 residual, two FP32-sized defect buffers, a 16-bit residual copy (rows
# padded to AUX_PITCH elements, each part 256-byte aligned), then AUX_SLOT_BYTES
# of per-launch maxima and an error word.
AUX_PITCH = 32
AUX_SLOT_BYTES = 65536
AUX_BYTES_PER_CELL = 14


def aux_bytes(shape) -> int:
    """Bytes of the work area of a grid of ``shape``."""
    dims = [int(v) for v in shape]
    rest = 1
    for v in dims[:-1]:
        rest *= v
    xp = -(-dims[-1] // AUX_PITCH) * AUX_PITCH
    cells = rest * xp

    def a(v):
        return (v + 255) // 256 * 256
    return 3 * a(cells * 4) + a(cells * 2) + AUX_SLOT_BYTES


def aux_error_offset(shape) -> int:
    """Byte offset of the error word (nonzero after a staging copy timed out)."""
    return aux_bytes(shape) - 4


@dataclasses.dataclass(eq=False)
class MixedPlan:
    loop: ir.For
    target: str
    slot: int
    group: analysis.Group


def _uses_variable(node, name: str) -> bool:
    return any(isinstance(n, ir.Identifier) and n.variable.name == name for n in ir.walk(node))


def degree(e, target: str):
    """Polynomial degree in the target's time-0 loads: 0, 1, or None (not affine)."""
    if isinstance(e, ir.Stencil):
        return 1 if (e.variable.name == target and e.time_offset == 0) else 0
    if isinstance(e, (ir.Constant, ir.Identifier, ir.GridInfo)):
        return 0
    if isinstance(e, ir.Access):
        return 0 if degree(e.value, target) == 0 else None
    if isinstance(e, ir.Unary):
        d = degree(e.right, target)
        if e.operator is ir.UnaryOperator.Not:
            return 0 if d == 0 else None
        return d
    if isinstance(e, ir.Cast):
        d = degree(e.value, target)
        if d == 0:
            return 0
        return d if isinstance(e.type, Floating) else None
    if isinstance(e, ir.Condition):
        ds = [degree(x, target) for x in (e.condition, e.body, e.orelse)]
        return 0 if ds == [0, 0, 0] else None
    if isinstance(e, ir.Call):
        return 0 if all(degree(a, target) == 0 for a in e.arguments) else None
    if isinstance(e, ir.Binary):
        dl, dr = degree(e.left, target), degree(e.right, target)
        if dl is None or dr is None:
            return None
        if e.operator in (B.Add, B.Sub):
            return max(dl, dr)
        if e.operator is B.Mul:
            return dl + dr if dl + dr <= 1 else None
        if e.operator is B.Div:
            return dl if dr == 0 else None
        return 0 if dl == dr == 0 else None
    return None


def match(gen, loop: ir.For):
    """MixedPlan for ``loop`` or None."""
    cfg = gen.cfg
    if cfg.mixed is None or not loop.body:
        return None
    body = loop.body
    if not all(isinstance(s, ir.Assignment) and isinstance(s.terminal, ir.Stencil) for s in body):
        return None
    names = {s.terminal.variable.name for s in body}
    if len(names) != 1:
        return None
    target = names.pop()
    gtype = gen.defn.scope[target].type
    if not (isinstance(gtype.element, Floating) and gtype.element.width_bytes == 8):
        return None
    for i, s in enumerate(body):
        t = s.terminal
        if t.time_offset != 0 or any(t.space_offset):
            return None
        if (i == 0) != (t.boundary_mask == 0):
            return None
        if _uses_variable(s.value, loop.variable.name):
            return None
        if degree(s.value, target) is None:
            return None
    sweeps = [analysis.collect_sweep(s, gen.slots, gen.logger) for s in body]
    if not sweeps[0].implicit:
        return None
    counter = [gen.group_counter[0]]
    groups = analysis.build_groups(sweeps, counter, True)
    if len(groups) != 1 or groups[0].sweeps[0] is not sweeps[0]:
        return None
    return MixedPlan(loop, target, gen.slots[target], groups[0])


class LinearEmitter:
    """FP32 code of the linear part of an affine right-hand side."""

    def __init__(self, mx, target: str, load) -> None:
        self.mx = mx
        self.target = target
        self.load = load  # (ir.Stencil) -> code of the defect load at its offset

    def lin(self, e):
        d = degree(e, self.target)
        if d == 0:
            return None
        if isinstance(e, ir.Stencil):
            return self.load(e)
        if isinstance(e, ir.Unary):
            a = self.lin(e.right)
            return a if e.operator is ir.UnaryOperator.Pos else f"(-{a})"
        if isinstance(e, ir.Cast):
            return self.lin(e.value)
        if isinstance(e, ir.Binary):
            if e.operator in (B.Add, B.Sub):
                a, b = self.lin(e.left), self.lin(e.right)
                if a is None:
                    return b if e.operator is B.Add else f"(-{b})"
                if b is None:
                    return a
                return f"({a} {e.operator.value} {b})"
            if e.operator is B.Mul:
                if degree(e.left, self.target) == 1:
                    return f"({self.lin(e.left)} * {self.mx.coef(e.right)})"
                return f"({self.mx.coef(e.left)} * {self.lin(e.right)})"
            if e.operator is B.Div:
                return f"({self.lin(e.left)} * {self.mx.recip(e.right)})"
        raise AssertionError(f"not affine: {type(e).__name__}")


def coefficients_stencil_free(e, target: str) -> bool:
    """Coefficients of the linear part must be launch constants (no grid loads)."""
    if degree(e, target) == 0:
        return True
    if isinstance(e, ir.Binary) and e.operator in (B.Mul, B.Div):
        parts = [e.left, e.right]
        for x in parts:
            if degree(x, target) == 0 and any(isinstance(n, ir.Stencil) for n in ir.walk(x)):
                return False
        return all(coefficients_stencil_free(x, target) for x in parts)
    if isinstance(e, ir.Binary):
        return all(coefficients_stencil_free(x, target) for x in (e.left, e.right))
    if isinstance(e, ir.Unary):
        return coefficients_stencil_free(e.right, target)
    if isinstance(e, ir.Cast):
        return coefficients_stencil_free(e.value, target)
    return True


class MixedLoopEmitter:
    """Kernels and host driver of one mixed-precision loop."""

    def __init__(self, gen, plan: MixedPlan) -> None:
        from .codegen import DEFAULT_TILING, SweepGroupEmitter
        self.gen = gen
        self.plan = plan
        self.base = SweepGroupEmitter(gen, plan.group)
        self.gid = plan.group.index
        gen.group_counter[0] = self.gid + 1
        dim = gen.defn.scope[plan.target].type.dimension
        gen.group_tiling[self.gid] = DEFAULT_TILING[dim]
        self.coefs: list = []        # (name, host expression, kind)
        self.coef_keys: dict = {}

    # FP32 launch constants of the linear part, evaluated on the host
    def _const(self, e, kind: str) -> str:
        from .codegen import HostEnv
        text = self.gen.expr(e, HostEnv(self.gen))
        key = (kind, text)
        if key not in self.coef_keys:
            name = f"c{len(self.coefs)}"
            self.coef_keys[key] = name
            self.coefs.append((name, text, kind))
        return f"p.k.{self.coef_keys[key]}"

    def coef(self, e) -> str:
        return self._const(e, "mul")

    def recip(self, e) -> str:
        return self._const(e, "recip")

    def emit(self, env, indent: str, out: list) -> None:
        gen, plan = self.gen, self.plan
        n, gid, slot = gen.op.name, self.gid, plan.slot
        b = self.base
        b.prepare()
        b.emit_kernels()
        g = plan.group
        P0 = b.bname((slot, 0, 0))
        S = b.bname((slot, 0, 1))
        # residual launch: r = G(P) - P in FP32 (row pitch X + mx_pad), optionally also as the
        # first defect, and its largest magnitude folded into *mx_max
        b.emit_fused(tag="res", extra_params=["float* mx_r", "float* mx_d", "int64_t mx_pad", "float* mx_max"],
                     extra_args=", float* mx_r, float* mx_d, int64_t mx_pad, float* mx_max",
                     extra_fill=["  p.mx_r = mx_r; p.mx_d = mx_d; p.mx_pad = mx_pad; p.mx_max = mx_max;"],
                     final=(["float xg_amax = 0.f;"],
                            [f"const float rr = (float)({S}[c] - {P0}[c]);",
                             "const I xa = c + ((I)z * (I)p.Y + (I)y) * (I)p.mx_pad;",
                             "p.mx_r[xa] = rr;",
                             "if (p.mx_d) p.mx_d[xa] = rr;",
                             "xg_amax = fmaxf(xg_amax, fabsf(rr));"],
                            ["if (p.mx_max) xg_block_max_atomic(xg_amax, p.mx_max);"]),
                     swap=False)
        from .mixed_tb import TemporalDefect
        self.tb = TemporalDefect(self)
        tb_device = self.tb.device() if self.tb.usable else []
        defect = self.defect_kernel()
        cs = [f"struct xgm_{n}_{gid} {{"] + [f"  float {name};" for name, _, _ in self.coefs]
        if not self.coefs:
            cs.append("  char xg_empty;")
        cs.append("};")
        gen.device_chunks.append("\n".join(cs))
        gen.device_chunks.extend(tb_device)
        gen.device_chunks.extend(defect)
        gen.device_chunks.extend(self.correction_kernel())
        if self.tb.usable:
            gen.host_chunks.append(self.tb.host())
        gen.host_chunks.append(self.host_functions())
        # host block in the kernel body
        v = plan.loop.variable.name
        out.append(f"{indent}{{")
        out.extend(b.host_hoists(env, indent + "  "))
        out.append(f"{indent}  struct xgm_{n}_{gid} xg_hm;")
        out.append(f"{indent}  memset(&xg_hm, 0, sizeof xg_hm);")
        for name, text, kind in self.coefs:
            if kind == "mul":
                out.append(f"{indent}  xg_hm.{name} = (float)({text});")
            else:
                out.append(f"{indent}  xg_hm.{name} = (float)(1.0 / (double)({text}));")
        lp = plan.loop
        out.append(f"{indent}  int64_t xg_K = 0;")
        out.append(f"{indent}  for ({v} = {gen.expr(lp.start, env)}; {v} < {gen.expr(lp.end, env)}; "
                   f"{v} += {gen.expr(lp.step, env)}) ++xg_K;")
        out.append(f"{indent}  if (xg_K > 0) {{")
        out.append(f"{indent}    int xg_mx = xgm_{n}_{gid}_ready(xg_G);")
        out.append(f"{indent}    if (xg_mx < 0) return xg_mx;")
        out.append(f"{indent}    if (xg_mx) XG_TRY(xgm_{n}_{gid}_run(xg_G, &xg_h, &xg_hm, xg_K, xg_s));")
        out.append(f"{indent}    else for (int64_t xg_i = 0; xg_i < xg_K; ++xg_i) XG_TRY(xgl_{n}_{gid}(xg_G, &xg_h, xg_s));")
        out.append(f"{indent}  }}")
        out.append(f"{indent}}}")

    def defect_kernel(self) -> list:
        gen, plan, b = self.gen, self.plan, self.base
        n, gid, target = gen.op.name, self.gid, plan.target
        sweeps = plan.group.sweeps
        main = sweeps[0]
        bnds = list(range(1, len(sweeps)))
        lo, hi = [0, 0, 0], [0, 0, 0]
        for _, ld in main.loads:
            if ld.slot == plan.slot and ld.level == 0:
                for a in range(3):
                    lo[a] = min(lo[a], ld.offset[a])
                    hi[a] = max(hi[a], ld.offset[a])

        def loader(buf: str, fast: bool, idx: str = "c"):
            def load(st):
                oz, oy, ox = analysis.pad3(st.space_offset)
                if fast:
                    off = "".join(f" + ({o}) * {s}" for o, s in ((oz, "sz"), (oy, "sy")) if o) + (f" + ({ox})" if ox else "")
                    return f"{buf}[{idx}{off}]"
                return f"xg_ldc({buf}, xg_addr(xg_overstep, z, y, x, {oz}, {oy}, {ox}, p.Z, p.Y, p.X))"
            return load

        def lin_code(sweep, buf, fast, idx="c"):
            code = LinearEmitter(self, target, loader(buf, fast, idx)).lin(sweep.stmt.value)
            return "0.0f" if code is None else code

        R = 4
        rows = ["    for (int z = z0; z < z1; ++z)",
                f"    for (int yb = y0 + (int)threadIdx.y; yb < y1; yb += {R} * (int)blockDim.y)",
                "    for (int x = x0 + (int)threadIdx.x; x < x1; x += (int)blockDim.x) {"]
        for r in range(R):
            rows += [f"      const int y_{r} = yb + {r} * (int)blockDim.y;",
                     f"      const bool ok_{r} = {'true' if r == 0 else f'y_{r} < y1'};",
                     f"      const I c_{r} = (I)z * sz + (I)y_{r} * sy + (I)x;",
                     f"      const float v_{r} = ok_{r} ? {lin_code(main, 'din', True, f'c_{r}')} + rr[c_{r}] : 0.0f;"]
        for r in range(R):
            rows.append(f"      if (ok_{r}) dout[c_{r}] = v_{r};")
        rows.append("    }")

        params = [f"struct xgp_{n}_{gid}_mxd {{", f"  struct xgm_{n}_{gid} k;", "  int64_t Z, Y, X;",
                  "  int32_t tz, ty, tx;", "  int64_t ntz, nty, ntx;", "  const float* din;", "  float* dout;",
                  "  const float* r;", "  const int32_t* m0;", "  const uint8_t* tzero0;"]
        for j in bnds:
            params += [f"  const int32_t* bo{j};", f"  const int64_t* bc{j};"]
        params.append("};")
        from .codegen import CELL_LOOP, TILE_PROLOGUE
        loop = CELL_LOOP
        K = [f"template <typename I> __global__ void __launch_bounds__(256, 6) xgk_{n}_{gid}_mxd("
             f"const __grid_constant__ struct xgp_{n}_{gid}_mxd p) {{"] + TILE_PROLOGUE + [
             f"  const bool fast = z0 + ({lo[0]}) >= 0 && z1 - 1 + ({hi[0]}) < p.Z && y0 + ({lo[1]}) >= 0 && "
             f"y1 - 1 + ({hi[1]}) < p.Y && x0 + ({lo[2]}) >= 0 && x1 - 1 + ({hi[2]}) < p.X;",
             "  const bool mz = p.tzero0[t] != 0;",
             "  const float* __restrict__ din = p.din;",
             "  float* __restrict__ dout = p.dout;",
             "  const float* __restrict__ rr = p.r;",
             "  if (fast && mz) {  // interior tile without boundary cells: one pass, r added directly"]
        K += rows
        K += ["    return;", "  }",
              "  if (fast) {"]
        K += ["  " + l for l in loop]
        K += [f"      dout[c] = (mz || p.m0[c] == 0) ? {lin_code(main, 'din', True)} : din[c];", "    }}",
              "  } else {"]
        K += ["  " + l for l in loop]
        K += [f"      dout[c] = (mz || p.m0[c] == 0) ? {lin_code(main, 'din', False)} : din[c];", "    }}", "  }"]
        for j in bnds:
            K += ["  __syncthreads();",
                  "  {",
                  "    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);",
                  "    const int nthr = blockDim.x * blockDim.y * blockDim.z;",
                  f"    for (int64_t e = p.bo{j}[t] + tid; e < p.bo{j}[t + 1]; e += nthr) {{",
                  f"      const int64_t c = p.bc{j}[e];",
                  "      const int64_t x = c % p.X, y = (c / p.X) % p.Y, z = c / (p.X * p.Y);",
                  "      (void)x; (void)y; (void)z;",
                  f"      dout[c] = {lin_code(sweeps[j], 'dout', False)};",
                  "    }",
                  "  }"]
        K += ["  __syncthreads();"] + loop + ["    dout[c] = dout[c] + rr[c];", "  }}", "}"]
        return ["\n".join(params), "\n".join(K)]

    def correction_kernel(self) -> list:
        """FP64 correction launch: P += d over each tile, then the loop body's
        boundary phases on P (tile-local, program order), so that boundary cells
        hold exactly what their FP64 rule gives for the corrected interior."""
        from .codegen import CELL_LOOP, TILE_PROLOGUE
        gen, plan, b = self.gen, self.plan, self.base
        n, gid, slot = gen.op.name, self.gid, plan.slot
        sweeps = plan.group.sweeps
        bnds = list(range(1, len(sweeps)))
        bsweeps = [sweeps[j] for j in bnds]
        from .mixed_tb import DSCALE
        P = b.bname((slot, 0, 1))  # boundary phases address the target as version 1
        extra = ["const void* mx_d", "int mx_kind", "const float* mx_slot", "int64_t mx_pad"] + \
            [x for j in bnds for x in (f"const int32_t* bo{j}", f"const int64_t* bc{j}")]
        params = b.params_struct("mxc", bsweeps or [sweeps[0]], extra)
        K = [f"template <typename I> __global__ void __launch_bounds__(256, 6) xgk_{n}_{gid}_mxc("
             f"const __grid_constant__ struct xgp_{n}_{gid}_mxc p) {{"] + TILE_PROLOGUE + b.restrict_locals(bsweeps or [sweeps[0]]) + \
            [f"  const float xg_inv = p.mx_slot ? xg_pow2f(-xg_scale_exp(*p.mx_slot, {DSCALE})) : 1.f;"] + \
            CELL_LOOP + [
             "      const I xa = c + ((I)z * (I)p.Y + (I)y) * (I)p.mx_pad;",
             "      const float dv = p.mx_kind == 0 ? ((const float*)p.mx_d)[xa] : (p.mx_kind == 1 ? "
             "__half2float(((const __half*)p.mx_d)[xa]) : __bfloat162float(((const __nv_bfloat16*)p.mx_d)[xa])) "
             "* xg_inv;",
             f"      {P}[c] = {P}[c] + (double)dv;", "    }}"]
        for j in bnds:
            s = sweeps[j]
            pre, val = b.value_code(s, False, "    ")
            K += ["  __syncthreads();", "  {",
                  "    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);",
                  "    const int nthr = blockDim.x * blockDim.y * blockDim.z;",
                  f"    for (int64_t e = p.bo{j}[t] + tid; e < p.bo{j}[t + 1]; e += nthr) {{",
                  f"    const int64_t c = p.bc{j}[e];",
                  f"    const int64_t x = c % p.X, y = (c / p.X) % p.Y, z = c / (p.X * p.Y);",
                  "    (void)x; (void)y; (void)z;"]
            K += pre
            K += [f"    {P}[c] = {val};", "    }", "  }"]
        K.append("}")
        return [params, "\n".join(K)]

    def host_functions(self) -> str:
        gen, plan, b = self.gen, self.plan, self.base
        n, gid, slot = gen.op.name, self.gid, plan.slot
        sweeps = plan.group.sweeps
        bnds = list(range(1, len(sweeps)))
        L = []
        # run-time applicability (same conditions as the fused launch)
        L += [f"static int xgm_{n}_{gid}_ready(xg_grid* G) {{",
              f"  if (!xg_fuse_{n} || !G[{slot}].scratch || !G[{slot}].aux) return 0;",
              "  xg_mx_aux A;",
              f"  if (xg_mx_layout(&G[{slot}], &A) != 0) return 0;",
              f"  const int32_t* tl = xg_tiling_{n}[{gid}];"]
        for j, offs in plan.group.local_checks:
            flat = ", ".join(str(v) for o in offs for v in o)
            L += ["  {", f"    static const int32_t offs[] = {{{flat}}};", "    int ok = 0;",
                  f"    XG_TRY(xg_mask_tile_local(G[{slot}].mask, tl, {sweeps[j].mask}, {len(offs)}, offs, "
                  f"xg_overstep, &ok));",
                  "    if (!ok) return 0;", "  }"]
        L += ["  return 1;", "}"]
        # FP32 defect launch
        L += [f"static int xgm_{n}_{gid}_defect(xg_grid* G, const struct xgm_{n}_{gid}* hm, const float* din, "
              f"float* dout, const float* r, cudaStream_t s) {{",
              f"  struct xgp_{n}_{gid}_mxd p;",
              "  memset(&p, 0, sizeof p);",
              "  p.k = *hm;",
              f"  const int32_t* tl = xg_tiling_{n}[{gid}];",
              f"  xg_ext e = xg_extent(&G[{slot}]);",
              "  p.Z = e.z; p.Y = e.y; p.X = e.x;",
              "  p.tz = tl[0]; p.ty = tl[1]; p.tx = tl[2];",
              "  p.ntz = xg_tiles_along(p.Z, p.tz); p.nty = xg_tiles_along(p.Y, p.ty); p.ntx = xg_tiles_along(p.X, p.tx);",
              "  p.din = din; p.dout = dout; p.r = r;",
              f"  p.m0 = xg_mask_device(G[{slot}].mask);",
              "  int64_t ntiles = 0;",
              f"  XG_TRY(xg_mask_tiles(G[{slot}].mask, tl, 0, &p.tzero0, NULL, NULL, &ntiles));"]
        for j in bnds:
            L.append(f"  XG_TRY(xg_mask_tiles(G[{slot}].mask, tl, {sweeps[j].mask}, NULL, &p.bo{j}, &p.bc{j}, "
                     f"&ntiles));")
        L += ["  dim3 block(tl[3], tl[4], tl[5]), grid;",
              "  XG_TRY(xg_tile_grid(p.ntx, p.nty, p.ntz, &grid));",
              f"  xg_prof_launch({gid * 64 + 61}, s);",
              f"  if (xg_small_index(p.Z, p.Y, p.X)) xgk_{n}_{gid}_mxd<int><<<grid, block, 0, s>>>(p);",
              f"  else xgk_{n}_{gid}_mxd<int64_t><<<grid, block, 0, s>>>(p);",
              "  XG_CUDA(cudaGetLastError());",
              f"  xg_prof_end({gid * 64 + 61}, s);",
              "  return 0;", "}"]
        # FP64 correction (+ boundary phases)
        bsweeps = [sweeps[j] for j in bnds] or [sweeps[0]]
        P = b.bname((slot, 0, 1))
        L += [f"static int xgm_{n}_{gid}_correct(xg_grid* G, const struct xgh_{n}_{gid}* h, const void* d, "
              f"int kind, const float* slot, int64_t pad, cudaStream_t s) {{"]
        L += b.fill_params("mxc", bsweeps, slot)
        L += [f"  p.{P} = (double*)G[{slot}].level[0];",
              "  p.mx_d = d; p.mx_kind = kind; p.mx_slot = slot; p.mx_pad = pad;",
              "  int64_t ntiles = 0;",
              f"  XG_TRY(xg_mask_tiles(G[{slot}].mask, tl, 0, NULL, NULL, NULL, &ntiles));"]
        for j in bnds:
            L.append(f"  XG_TRY(xg_mask_tiles(G[{slot}].mask, tl, {sweeps[j].mask}, NULL, &p.bo{j}, &p.bc{j}, "
                     f"&ntiles));")
        L += ["  dim3 block(tl[3], tl[4], tl[5]), grid;",
              "  XG_TRY(xg_tile_grid(p.ntx, p.nty, p.ntz, &grid));",
              f"  xg_prof_launch({gid * 64 + 60}, s);",
              f"  if (xg_small_index(p.Z, p.Y, p.X)) xgk_{n}_{gid}_mxc<int><<<grid, block, 0, s>>>(p);",
              f"  else xgk_{n}_{gid}_mxc<int64_t><<<grid, block, 0, s>>>(p);",
              "  XG_CUDA(cudaGetLastError());",
              f"  xg_prof_end({gid * 64 + 60}, s);",
              "  return 0;", "}"]
        # driver
        tb = self.tb.usable
        kind, scaled = self.tb.kind, int(self.tb.scaled)
        L += [f"static int xgm_{n}_{gid}_run(xg_grid* G, const struct xgh_{n}_{gid}* h, "
              f"const struct xgm_{n}_{gid}* hm, int64_t K, cudaStream_t s) {{",
              f"  const xg_ext e = xg_extent(&G[{slot}]);",
              "  xg_mx_aux A;",
              f"  XG_TRY(xg_mx_layout(&G[{slot}], &A));",
              f"  const int64_t m = xg_mixed_every_{n} > 0 ? xg_mixed_every_{n} : K;",
              "  int T = 0, RS = 0;",
              "  int32_t core[3] = {1, 1, 1}, halo[3] = {0, 0, 0};",
              f"  const int tb = {f'xgm_{n}_{gid}_tb_plan(G, &T, &RS, core, halo)' if tb else '0'};",
              "  if (tb < 0) return tb;",
              "  for (int64_t done = 0; done < K;) {",
              "    const int64_t cnt = (K - done) < m ? (K - done) : m;",
              "    const int64_t it = cnt - 1;  // defect iterations after the residual",
              "    const int64_t nl = (tb && it > 0) ? (it + T - 1) / T : 0;"]
        if tb:
            L += ["    if (nl > 0 && nl + 2 <= A.nslots) {",
                  "      // temporally blocked: nl launches of at most T iterations, TMA-staged boxes",
                  f"      if ({scaled}) XG_CUDA(cudaMemsetAsync(A.slots, 0, (size_t)(nl + 1) * sizeof(float), s));",
                  f"      int rc = xgl_{n}_{gid}_res(G, h, s, A.r32, NULL, A.XP - e.x, {scaled} ? A.slots : NULL);",
                  "      if (rc < 0) return rc;",
                  "      if (rc == 0) XG_FAIL(\"mixed-precision residual launch is not applicable\");",
                  "      for (int64_t i = 0; i < nl; ++i) {",
                  "        const int dep = (int)(it / nl + (i < it % nl ? 1 : 0));",
                  "        void* dout = (i & 1) ? A.dB : A.dA;",
                  "        const void* din = (i & 1) ? A.dA : A.dB;",
                  f"        XG_TRY(xgm_{n}_{gid}_tbl(G, hm, &A, dep, RS, core, halo, i == 0, (int)i, din, dout, s));",
                  "      }",
                  f"      XG_TRY(xgm_{n}_{gid}_correct(G, h, ((nl - 1) & 1) ? A.dB : A.dA, {kind}, "
                  f"{scaled} ? A.slots + (nl - 1) : NULL, A.XP - e.x, s));",
                  "    } else {"]
        else:
            L += ["    (void)nl; (void)T; (void)RS; (void)core; (void)halo;", "    {"]
        L += ["      // one FP32 iteration per launch (dense layout)",
              f"      int rc = xgl_{n}_{gid}_res(G, h, s, A.r32, (float*)A.dA, 0, NULL);",
              "      if (rc < 0) return rc;",
              "      if (rc == 0) XG_FAIL(\"mixed-precision residual launch is not applicable\");",
              "      float* din = (float*)A.dA;",
              "      float* dout = (float*)A.dB;",
              "      for (int64_t i = 1; i < cnt; ++i) {",
              f"        XG_TRY(xgm_{n}_{gid}_defect(G, hm, din, dout, A.r32, s));",
              "        float* t_ = din; din = dout; dout = t_;",
              "      }",
              f"      XG_TRY(xgm_{n}_{gid}_correct(G, h, din, 0, NULL, 0, s));",
              "    }",
              "    done += cnt;",
              "  }",
              "  return 0;", "}"]
        return "\n".join(L)
