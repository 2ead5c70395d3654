"""Temporally blocked defect iterations of a mixed-precision loop (2-D grids).

The defect iteration ``d <- L(d) + r`` of ``xgrid_gb300.mixed`` runs ``T``
iterations per launch instead of one.  Each CTA owns a tile of ``TY x TX``
cells and works on a *box*: the tile plus a halo of ``HY = T * sy`` rows and
``HX = roundup(T * sx, 16 bytes / element)`` columns per side (``sy, sx``: reach of the loop
body's main sweep).  Per launch:

1. one thread stages the box of ``d`` and of ``r`` into shared memory with two
   TMA loads (``cp.async.bulk.tensor.2d``, completion on an mbarrier); cells
   outside the grid read as zero;
2. every thread takes a column strip of ``RS`` rows of the box into registers
   (block of 128 x 2 threads, box of 128 x 2*RS cells); vertical neighbours come
   from the thread's own registers, horizontal and strip-edge neighbours from a
   shared copy of the current iterate (two buffers, one barrier per iteration);
3. boxes that contain boundary cells run the loop body's phases in order: the
   main sweep on mask-0 cells, each ``with boundary(k)`` phase on its cells of
   the box (per-tile lists of box-local indices), then ``+ r``;
4. the tile's cells are written back (FP32, or 16-bit with a power-of-two scale
   per field and launch).

Cells at distance ``< k * s`` from an inner box edge are stale after ``k``
iterations; the halo keeps the tile itself exact.  ``xg_mask_box_check`` (run
time, per mask and tiling) proves that the boundary phases never read a stale
cell; when it fails the loop falls back to one iteration per launch.  The FP32
variant performs the same FP32 operations per cell as the one-iteration kernel,
so both give the same bits.
"""
from __future__ import annotations

from . import analysis

BX = 128          # box columns: 32 lanes x 4 columns per lane
NW = 8            # warps per CTA, stacked along y; each owns RS rows of the box
DSCALE = 8        # defect: an input of largest magnitude m is stored as m * 2^s in [2^8, 2^9)
RSCALE = 14       # residual (fixed over the loop): [2^14, 2^15), below the FP16 maximum
STORAGE = {"fp32": ("float", 0, "CU_TENSOR_MAP_DATA_TYPE_FLOAT32"),
           "fp16": ("__half", 1, "CU_TENSOR_MAP_DATA_TYPE_FLOAT16"),
           "bf16": ("__nv_bfloat16", 2, "CU_TENSOR_MAP_DATA_TYPE_BFLOAT16")}


def target_offsets(sweep, slot: int) -> list:
    """Distinct (z, y, x) offsets of the target's time-0 loads in a sweep."""
    out = []
    for _, ld in sweep.loads:
        if ld.slot == slot and ld.level == 0 and ld.version in (0, 1):
            o = tuple(analysis.pad3(ld.offset))
            if o not in out:
                out.append(o)
    return out


class TemporalDefect:
    """Kernel and host launcher of the temporally blocked defect iterations."""

    def __init__(self, mx) -> None:
        from .mixed import LinearEmitter
        self.mx = mx
        self.LinearEmitter = LinearEmitter
        gen, plan = mx.gen, mx.plan
        self.gen = gen
        self.n, self.gid = gen.op.name, mx.gid
        self.slot = plan.slot
        self.target = plan.target
        self.sweeps = plan.group.sweeps
        self.bnds = list(range(1, len(self.sweeps)))
        self.dim = gen.defn.scope[plan.target].type.dimension
        self.dt, self.kind, self.cutype = STORAGE[gen.cfg.mixed]
        self.scaled = self.kind != 0
        # a TMA box must start on a 16-byte boundary: the x halo is a multiple of 4 FP32 or
        # 8 16-bit elements, so that every box's first column (tile origin - halo) is one
        self.xalign = 4 if self.kind == 0 else 8
        self.main_offs = target_offsets(self.sweeps[0], self.slot)
        self.sy = max([abs(o[1]) for o in self.main_offs] + [0])
        self.sx = max([abs(o[2]) for o in self.main_offs] + [0])
        # the register blocks reach one row and one column beyond themselves
        self.usable = (self.dim == 2 and all(o[0] == 0 for o in self.main_offs)
                       and self.sy <= 1 and self.sx <= 1)

    # ----------------------------------------------------------- device code
    def _lin(self, sweep, load) -> str:
        code = self.LinearEmitter(self.mx, self.target, load).lin(sweep.stmt.value)
        return "0.0f" if code is None else code

    def _reg_loader(self, j: int, used: set):
        """Load of the defect at a stencil offset for column ``j`` (0..3) of the
        thread's 4-column block: rows above / at / below come from the register
        rows ``prev`` / ``cur`` / ``nxt``, columns beyond the block from the
        neighbouring lanes (``<row>_w``: lane - 1's last column, ``<row>_e``:
        lane + 1's first column).  ``used`` collects the lane exchanges needed."""
        def load(st):
            oz, oy, ox = analysis.pad3(st.space_offset)
            row = {-1: "prev", 0: "cur", 1: "nxt"}[oy]
            jj = j + ox
            if 0 <= jj <= 3:
                return f"{row}.{'xyzw'[jj]}"
            side = "w" if jj < 0 else "e"
            used.add((row, side))
            return f"{row}_{side}"
        return load

    @staticmethod
    def _box_loader(buf: str):
        def load(st):
            oz, oy, ox = analysis.pad3(st.space_offset)
            return f"{buf}[xg_clampi(c + ({oy}) * BX + ({ox}), 0, BY * BX - 1)]"
        return load

    def device(self) -> list:
        n, gid = self.n, self.gid
        main = self.sweeps[0]
        used: set = set()
        lins = [self._lin(main, self._reg_loader(j, used)) for j in range(4)]
        P = [f"struct xgp_{n}_{gid}_mxt {{",
             "  CUtensorMap md;  // defect in (storage type), box BX x BY",
             "  CUtensorMap mr;  // residual (FP32 on the first launch and in FP32 mode, else storage type)",
             f"  struct xgm_{n}_{gid} k;",
             "  int Y, X, XP, TY, TX, HY, HX, nty, ntx, dep, first, li;",
             "  void* dout;",
             "  void* rout;",
             "  float* sl;",
             "  int* err;",
             "  const int32_t* m0;",
             "  const uint8_t* bzero;"]
        for j in self.bnds:
            P += [f"  const int32_t* bo{j};", f"  const int32_t* bl{j};"]
        P.append("};")
        K = [f"template <typename Dt, int RS>",
             f"__global__ void __launch_bounds__({NW * 32}, 2) xgk_{n}_{gid}_mxt(const __grid_constant__ "
             f"struct xgp_{n}_{gid}_mxt p) {{",
             f"  constexpr int BX = {BX}, NW = {NW}, BY = NW * RS;",
             "  constexpr bool scaled = sizeof(Dt) == 2;",
             "  constexpr unsigned FULL = 0xffffffffu;",
             "  extern __shared__ unsigned char xg_dsm[];",
             "  __shared__ __align__(8) uint64_t xg_bar;",
             "  __shared__ __align__(16) float xg_ex[2][2][NW][BX];  // [parity][first/last row][warp][column]",
             "  float* sA = (float*)(((uintptr_t)xg_dsm + 1023) & ~(uintptr_t)1023);",
             "  float* sB = sA + BY * BX;",
             "  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;",
             "  const int c0 = 4 * lane, r0 = w * RS;  // the thread's block: columns c0..c0+3, rows r0..r0+RS-1",
             "  const int t = blockIdx.x;",
             "  const int ity = t / p.ntx, itx = t - ity * p.ntx;",
             "  const int by = ity * p.TY - p.HY, bx = itx * p.TX - p.HX;",
             "  // stage the boxes of r and (after the first launch) d with TMA",
             "  if (tid == 0) xg_mbar_init(&xg_bar, 1);",
             "  __syncthreads();",
             "  if (tid == 0) {",
             "    const unsigned rb = (p.first || !scaled) ? 4u : (unsigned)sizeof(Dt);",
             "    xg_mbar_expect_tx(&xg_bar, (unsigned)(BY * BX) * (rb + (p.first ? 0u : (unsigned)sizeof(Dt))) + "
             "XG_TMA_TX_EXTRA);",
             "    xg_tma_load_2d(sB, &p.mr, bx, by, &xg_bar);",
             "    if (!p.first) xg_tma_load_2d(sA, &p.md, bx, by, &xg_bar);",
             "  }",
             "  const bool landed = xg_mbar_wait(&xg_bar, 0, XG_GIVEUP_NS);",
             "  if (__syncthreads_or(!landed)) {  // the copy did not complete: report, let it drain, stop",
             "    if (tid == 0) {",
             "      atomicExch(p.err, 1);",
             "      xg_mbar_wait(&xg_bar, 0, XG_WAIT_NS);",
             "    }",
             "    return;",
             "  }",
             "  float4 d[RS], rr[RS];",
             "  {",
             f"    const float ir = (scaled && !p.first) ? xg_pow2f(-xg_scale_exp(p.sl[0], {RSCALE})) : 1.f;",
             f"    const float id = (scaled && !p.first) ? xg_pow2f(-xg_scale_exp(p.sl[p.li - 1], {DSCALE})) : 1.f;",
             "#pragma unroll",
             "    for (int i = 0; i < RS; ++i) {",
             "      const int c = (r0 + i) * BX + c0;",
             "      rr[i] = (p.first || !scaled) ? *(const float4*)(sB + c) : xg_ld4_scaled<Dt>(sB, c, ir);",
             "      d[i] = p.first ? rr[i] : (scaled ? xg_ld4_scaled<Dt>(sA, c, id) : *(const float4*)(sA + c));",
             "    }",
             "  }",
             "  const bool plain = p.bzero[t] != 0;  // no boundary cell in the box",
             "  unsigned mz = 0;  // boxes with boundary cells: bit 4 i + j set when cell (r0 + i, c0 + j) has mask 0",
             "  if (!plain) {",
             "#pragma unroll",
             "    for (int i = 0; i < RS; ++i) {",
             "      const int gy = by + r0 + i;",
             "#pragma unroll",
             "      for (int j = 0; j < 4; ++j) {",
             "        const int gx = bx + c0 + j;",
             "        if (gy >= 0 && gy < p.Y && gx >= 0 && gx < p.X && p.m0[(int64_t)gy * p.X + gx] == 0) "
             "mz |= 1u << (4 * i + j);",
             "      }",
             "    }",
             "  }",
             "  __syncthreads();  // the staged boxes are read: sA and sB become scratch",
             "  for (int k = 0; k < p.dep; ++k) {",
             "    // rows next to the warp's block: last row of the warp above, first row of the warp below",
             "    float (*ex)[NW][BX] = xg_ex[k & 1];",
             "    *(float4*)&ex[0][w][c0] = d[0];",
             "    *(float4*)&ex[1][w][c0] = d[RS - 1];",
             "    __syncthreads();",
             "    const float4 up = w > 0 ? *(const float4*)&ex[1][w - 1][c0] : d[0];",
             "    const float4 dn = w < NW - 1 ? *(const float4*)&ex[0][w + 1][c0] : d[RS - 1];",
             "    float4 prev = up;",
             "#pragma unroll",
             "    for (int i = 0; i < RS; ++i) {",
             "      const float4 cur = d[i];",
             "      const float4 nxt = i + 1 < RS ? d[i + 1 < RS ? i + 1 : i] : dn;"]
        for row, side in sorted(used):
            if side == "w":
                K.append(f"      const float {row}_w = __shfl_up_sync(FULL, {row}.w, 1);")
            else:
                K.append(f"      const float {row}_e = __shfl_down_sync(FULL, {row}.x, 1);")
        K.append("      float4 nv;")
        for j in range(4):
            K.append(f"      nv.{'xyzw'[j]} = {lins[j]};")
        K += ["      if (plain) {",
              "        d[i] = make_float4(nv.x + rr[i].x, nv.y + rr[i].y, nv.z + rr[i].z, nv.w + rr[i].w);",
              "      } else {",
              "        d[i].x = ((mz >> (4 * i)) & 1u) ? nv.x : cur.x;",
              "        d[i].y = ((mz >> (4 * i + 1)) & 1u) ? nv.y : cur.y;",
              "        d[i].z = ((mz >> (4 * i + 2)) & 1u) ? nv.z : cur.z;",
              "        d[i].w = ((mz >> (4 * i + 3)) & 1u) ? nv.w : cur.w;",
              "      }",
              "      prev = cur;",
              "    }",
              "    if (!plain) {  // boundary phases in program order on the box in shared memory, then + r",
              "#pragma unroll",
              "      for (int i = 0; i < RS; ++i) *(float4*)(sB + (r0 + i) * BX + c0) = d[i];",
              "      __syncthreads();"]
        for j in self.bnds:
            K += [f"      for (int e = p.bo{j}[t] + tid; e < p.bo{j}[t + 1]; e += NW * 32) {{",
                  f"        const int c = p.bl{j}[e];",
                  f"        sB[c] = {self._lin(self.sweeps[j], self._box_loader('sB'))};",
                  "      }",
                  "      __syncthreads();"]
        K += ["#pragma unroll",
              "      for (int i = 0; i < RS; ++i) {",
              "        const float4 v = *(const float4*)(sB + (r0 + i) * BX + c0);",
              "        d[i] = make_float4(v.x + rr[i].x, v.y + rr[i].y, v.z + rr[i].z, v.w + rr[i].w);",
              "      }",
              "    }",
              "  }",
              "  // the tile's own cells go back to global memory (the tile's columns are whole 4-column blocks)",
              f"  const float os = scaled ? xg_pow2f(xg_scale_exp(p.sl[p.li], {DSCALE})) : 1.f;",
              f"  const float rs = scaled ? xg_pow2f(xg_scale_exp(p.sl[0], {RSCALE})) : 1.f;",
              "  Dt* __restrict__ dout = (Dt*)p.dout;",
              "  Dt* __restrict__ rout = (Dt*)p.rout;",
              "  const int gx = bx + c0;",
              "  const bool col = c0 >= p.HX && c0 < p.HX + p.TX && gx < p.X;",
              "  float amax = 0.f;",
              "#pragma unroll",
              "  for (int i = 0; i < RS; ++i) {",
              "    const int ly = r0 + i, gy = by + ly;",
              "    if (col && ly >= p.HY && ly < p.HY + p.TY && gy < p.Y) {",
              "      const int64_t a = (int64_t)gy * p.XP + gx;",
              "      const float v[4] = {d[i].x, d[i].y, d[i].z, d[i].w};",
              "      const float q[4] = {rr[i].x, rr[i].y, rr[i].z, rr[i].w};",
              "#pragma unroll",
              "      for (int j = 0; j < 4; ++j) {",
              "        if (gx + j < p.X) {",
              "          dout[a + j] = xg_to_store<Dt>(v[j] * os);",
              "          if (scaled && rout) rout[a + j] = xg_to_store<Dt>(q[j] * rs);",
              "          amax = fmaxf(amax, fabsf(v[j]));",
              "        }",
              "      }",
              "    }",
              "  }",
              "  if (scaled) xg_block_max_atomic(amax, p.sl + p.li + 1);",
              "}"]
        return ["\n".join(P), "\n".join(K)]

    # ------------------------------------------------------------- host code
    def host(self) -> str:
        n, gid, slot, dt = self.n, self.gid, self.slot, self.dt
        cfg = self.gen.cfg
        mo = [v for o in self.main_offs for v in o]
        vals, nof, offs = [], [], []
        for j in self.bnds:
            s = self.sweeps[j]
            os_ = target_offsets(s, self.slot)
            vals.append(s.mask)
            nof.append(len(os_))
            offs += [v for o in os_ for v in o]

        def arr(name, values):
            if not values:
                return [f"  const int32_t* {name} = NULL;"]
            return [f"  static const int32_t {name}[] = {{{', '.join(str(v) for v in values)}}};"]

        L = [f"static int32_t xg_mxt_{n}[2] = {{{int(cfg.mixed_temporal)}, {int(cfg.mixed_rows)}}};",
             f'extern "C" int xg_mixed_tb_{n}(int depth, int rows) {{',
             "  if (depth < 0 || depth > 16) XG_FAIL(\"temporal blocking: depth %d outside 0..16\", depth);",
             "  if (rows >= 0 && rows != 4 && rows != 8) "
             "XG_FAIL(\"temporal blocking: rows per warp must be 4 or 8, not %d\", rows);",
             f"  xg_mxt_{n}[0] = depth;",
             f"  if (rows >= 0) xg_mxt_{n}[1] = rows;",
             "  return 0;",
             "}",
             f"// temporal blocking of the defect iterations: box geometry for this grid, 1 when usable",
             f"static int xgm_{n}_{gid}_tb_plan(xg_grid* G, int* T, int* RS, int32_t* core, int32_t* halo) {{",
             f"  const xg_grid* g = &G[{slot}];",
             f"  if (g->ndim != 2 || xg_mxt_{n}[0] < 1 || !g->mask) return 0;",
             f"  *T = xg_mxt_{n}[0];",
             f"  *RS = xg_mxt_{n}[1];",
             "  if (*RS != 4 && *RS != 8) return 0;",
             f"  halo[0] = 0; halo[1] = *T * {self.sy}; halo[2] = (*T * {self.sx} + {self.xalign - 1}) / "
             f"{self.xalign} * {self.xalign};",
             f"  core[0] = 1; core[1] = {NW} * *RS - 2 * halo[1]; core[2] = {BX} - 2 * halo[2];",
             "  if (core[1] < 1 || core[2] < 8) return 0;",
             f"  const int32_t shrink[3] = {{0, {self.sy}, {self.sx}}};"]
        L += arr("mo", mo) + arr("vals", vals) + arr("nof", nof) + arr("offs", offs)
        L += ["  int ok = 0;",
              f"  XG_TRY(xg_mask_box_check(g->mask, core, halo, shrink, *T, {len(self.main_offs)}, mo, "
              f"{len(vals)}, vals, nof, offs, &ok));",
              "  return ok;",
              "}",
              f"template <int RS>",
              f"static int xgm_{n}_{gid}_go(const struct xgp_{n}_{gid}_mxt& p, int64_t nt, cudaStream_t s) {{",
              "  static int avail = -1;",
              f"  if (avail < 0) XG_TRY(xg_smem_optin(xgk_{n}_{gid}_mxt<{dt}, RS>, &avail));",
              f"  const size_t smem = (size_t)2 * ({NW} * RS) * {BX} * sizeof(float) + 1024;",
              "  if (smem > (size_t)avail) XG_FAIL(\"temporal blocking: %zu bytes of shared memory, %d available\", "
              "smem, avail);",
              f"  xgk_{n}_{gid}_mxt<{dt}, RS><<<(unsigned)nt, {NW * 32}, smem, s>>>(p);",
              "  XG_CUDA(cudaGetLastError());",
              "  return 0;",
              "}",
              f"static int xgm_{n}_{gid}_tbl(xg_grid* G, const struct xgm_{n}_{gid}* hm, const xg_mx_aux* A, "
              f"int dep, int RS, const int32_t* core, const int32_t* halo, int first, int li, const void* din, "
              f"void* dout, cudaStream_t s) {{",
              f"  struct xgp_{n}_{gid}_mxt p;",
              "  memset(&p, 0, sizeof p);",
              "  p.k = *hm;",
              f"  const xg_ext e = xg_extent(&G[{slot}]);",
              "  p.Y = (int)e.y; p.X = (int)e.x; p.XP = (int)A->XP;",
              "  p.TY = core[1]; p.TX = core[2]; p.HY = halo[1]; p.HX = halo[2];",
              "  p.nty = (p.Y + p.TY - 1) / p.TY; p.ntx = (p.X + p.TX - 1) / p.TX;",
              "  p.dep = dep; p.first = first; p.li = li;",
              f"  const int BY = {NW} * RS;",
              f"  const int es = (int)sizeof({dt});",
              f"  if (!first) XG_TRY(xg_tmap_2d(&p.md, din, {self.cutype}, es, e.x, e.y, A->XP * es, {BX}, BY));",
              f"  if (first || !{int(self.scaled)})",
              f"    XG_TRY(xg_tmap_2d(&p.mr, A->r32, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, e.x, e.y, A->XP * 4, {BX}, BY));",
              "  else",
              f"    XG_TRY(xg_tmap_2d(&p.mr, A->r16, {self.cutype}, es, e.x, e.y, A->XP * es, {BX}, BY));",
              "  p.dout = dout;",
              f"  p.rout = (first && {int(self.scaled)}) ? A->r16 : NULL;",
              "  p.sl = A->slots;",
              "  p.err = A->err;",
              f"  p.m0 = xg_mask_device(G[{slot}].mask);",
              "  int64_t nt = 0;",
              f"  XG_TRY(xg_mask_boxes(G[{slot}].mask, core, halo, 0, &p.bzero, NULL, NULL, &nt));"]
        for j in self.bnds:
            L.append(f"  XG_TRY(xg_mask_boxes(G[{slot}].mask, core, halo, {self.sweeps[j].mask}, NULL, &p.bo{j}, "
                     f"&p.bl{j}, &nt));")
        L += ["  if (nt != (int64_t)p.nty * p.ntx) XG_FAIL(\"box table mismatch\");",
              f"  xg_prof_launch({gid * 64 + 59}, s);",
              "  switch (RS) {",
              f"    case 4: XG_TRY(xgm_{n}_{gid}_go<4>(p, nt, s)); break;",
              f"    case 8: XG_TRY(xgm_{n}_{gid}_go<8>(p, nt, s)); break;",
              "    default: XG_FAIL(\"temporal blocking: %d rows per thread is not compiled\", RS);",
              "  }",
              f"  xg_prof_end({gid * 64 + 59}, s);",
              "  return 0;",
              "}"]
        return "\n".join(L)
