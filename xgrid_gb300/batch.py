"""Batched execution of one kernel over many independent problems.

``kernel.batch(problems, steps)`` is equivalent to::

    for _ in range(steps):
        for args in problems:
            kernel(*args)

(problems are independent, so their order does not matter).  Instead of
``steps x len(problems)`` launches it runs one *persistent* launch per step:
``#SM x occupancy`` CTAs pull work items — (problem, tile) pairs, numbered
problem after problem — from an atomic counter, so problems of uneven size
share the GPU without per-problem launches.  Each problem has a device
descriptor holding its time-level pointers, extents, mask tables and the
kernel's launch-invariant scalars (evaluated on the host from that problem's
arguments, as in a regular call).  Time levels rotate through an index: step
``s`` reads level ``k`` from the descriptor's level ``(k - s - 1) mod depth``, the
rotation ``s + 1`` ticks produce.  The ``steps`` launches are captured as one CUDA
graph by the runtime's call cache.

A kernel qualifies when its body is one run of mask-0, explicit grid
assignments (no control flow, no boundary or in-place sweeps) whose grids all
have the same shape within a problem.
"""
from __future__ import annotations

from . import analysis, ir

DEPTH_MAX = 8


def qualifies(gen) -> bool:
    body = gen.defn.body
    if not body or not gen.slots:
        return False
    if not all(isinstance(s, ir.Assignment) and isinstance(s.terminal, ir.Stencil) for s in body):
        return False
    return True


class BatchEmitter:
    """Emits the persistent batched kernel and its two host entry points."""

    def __init__(self, gen, group: analysis.Group, emitter) -> None:
        self.gen = gen
        self.g = group
        self.e = emitter  # the group's SweepGroupEmitter (hoists, buffers, main body)

    @staticmethod
    def usable(group: analysis.Group) -> bool:
        return all(s.is_main and not s.implicit and not any(s.store_offset) for s in group.sweeps)

    def tb_plan(self):
        """(ry, rx) stencil radii when the group can be temporally blocked, else None.

        Temporal blocking advances a tile ``T`` steps per launch inside shared
        memory (halo ``T * r``), which is exact when every step is a pure function
        of the previous one: every grid read is read at t=-1 only, every such grid
        is written at t=0 by exactly one sweep, levels tick with depth 2, edges
        wrap (a wrapped halo cell evolves like the cell it copies), grids have at
        most two dimensions and no cell is masked (checked per call)."""
        gen, g = self.gen, self.g
        if gen.cfg.overstep != "wrap" or not gen.op.tick or gen.depth + 1 != 2:
            return None
        targets = [s.slot for s in g.sweeps]
        if len(set(targets)) != len(targets):
            return None
        ry = rx = 0
        for s in g.sweeps:
            if s.level != 0 or s.implicit or any(s.store_offset):
                return None
            if self.e.elem(s.slot) not in ("float", "double"):
                return None
            for _, ld in s.loads:
                if ld.level != 1 or ld.version != 0 or ld.slot not in targets or ld.offset[0] != 0:
                    return None
                ry, rx = max(ry, abs(ld.offset[1])), max(rx, abs(ld.offset[2]))
        for slot in targets:
            t = gen.defn.signature.arguments[self.e.arg_index(slot)][1]
            if t.dimension > 2:
                return None
        return ry, rx

    def emit_tb(self) -> tuple:
        """Temporally blocked persistent kernel ``xgk_<n>_tb`` and its host entry
        points.  One launch advances every (problem, tile) work item ``T`` steps:
        the tile plus a halo of ``T * r`` cells (wrapped) is loaded into shared
        memory once, steps 1..T-1 update a region that shrinks by ``r`` per step,
        ping-ponging between two shared buffers, and step T writes the tile to
        global memory.  Reads come from one buffer of a ring of three (the two
        levels and the scratch level) and writes go to another, so no launch
        writes a buffer that another CTA still reads; the last launch of a call
        also writes step T-1 so both time levels end where ticking leaves them."""
        from .codegen import SweepEnv
        gen, g, e = self.gen, self.g, self.e
        n, gid = gen.op.name, g.index
        ry, rx = self.tb_plan()
        fields = [s.slot for s in g.sweeps]
        el = {f: e.elem(f) for f in fields}
        K = [f"template <typename I> __global__ void __launch_bounds__(256, 2) xgk_{n}_tb("
             f"const struct xgb_{n}* __restrict__ desc, const int64_t* __restrict__ tile0, int nprob, "
             f"int64_t total, int T, int tby, int tbx, int in_idx, int out_idx, int prev_idx, "
             f"unsigned long long* __restrict__ counter) {{",
             "  extern __shared__ __align__(16) unsigned char xg_smem[];",
             "  __shared__ int64_t item_;",
             "  __shared__ int prob_;",
             "  const int tid = threadIdx.x + blockDim.x * threadIdx.y;",
             f"  const int HY = T * {ry}, HX = T * {rx};",
             "  const int PX = tbx + 2 * HX, PY = tby + 2 * HY;",
             "  unsigned char* sp = xg_smem;"]
        for f in fields:
            for b in "AB":
                K += [f"  {el[f]}* __restrict__ s{b}{f} = ({el[f]}*)sp;",
                      f"  sp += ((size_t)PX * PY * sizeof({el[f]}) + 15) & ~(size_t)15;"]
        K += ["  int64_t next = 0;",
              "  if (tid == 0) next = (int64_t)atomicAdd(counter, 1ull);",
              "  for (;;) {",
              "    if (tid == 0) {",
              "      const int64_t it = next;",
              "      if (it < total) next = (int64_t)atomicAdd(counter, 1ull);",
              "      int lo = 0, hi = nprob - 1;",
              "      if (it < total)",
              "        while (lo < hi) {",
              "          const int mid = (lo + hi + 1) >> 1;",
              "          if (tile0[mid] <= it) lo = mid; else hi = mid - 1;",
              "        }",
              "      item_ = it;",
              "      prob_ = lo;",
              "    }",
              "    __syncthreads();",
              "    const int64_t it = item_;",
              "    const int pr = prob_;",
              "    __syncthreads();",
              "    if (it >= total) break;",
              f"    const struct xgb_{n}& D = desc[pr];",
              f"    const struct xgp_{n}_{gid}_batch& p = D.par;",
              "    const int t = (int)(it - D.tile0tb);",
              "    const int ntx = D.tbn[1];",
              "    const int itx = t % ntx, ity = t / ntx;",
              "    const int X = (int)p.X, Y = (int)p.Y;",
              "    const int x0 = itx * tbx, x1 = min(x0 + tbx, X);",
              "    const int y0 = ity * tby, y1 = min(y0 + tby, Y);",
              "    const int RY = y1 - y0 + 2 * HY, RX = x1 - x0 + 2 * HX;"]
        for f in fields:
            K += [f"    const {el[f]}* __restrict__ in{f} = (const {el[f]}*)D.tb[{f}][in_idx];",
                  f"    {el[f]}* __restrict__ out{f} = ({el[f]}*)D.tb[{f}][out_idx];",
                  f"    {el[f]}* __restrict__ prv{f} = prev_idx >= 0 ? ({el[f]}*)D.tb[{f}][prev_idx] : nullptr;"]
        K += ["    for (int ly = threadIdx.y; ly < RY; ly += blockDim.y) {",
              "      int gy = y0 - HY + ly;",
              "      gy = gy < 0 ? gy + Y : (gy >= Y ? gy - Y : gy);",
              "      const I row = (I)gy * (I)X;",
              "      for (int lx = threadIdx.x; lx < RX; lx += blockDim.x) {",
              "        int gx = x0 - HX + lx;",
              "        gx = gx < 0 ? gx + X : (gx >= X ? gx - X : gx);"]
        K += [f"        xg_cp_async(&sA{f}[ly * PX + lx], &in{f}[row + gx]);" for f in fields]
        K += ["      }", "    }", "    xg_cp_async_wait_all();", "    __syncthreads();"]

        def body(indent, store):
            out = []
            for s in g.sweeps:
                names, local = {}, {}
                for st, ld in s.loads:
                    if ld not in local:
                        vn = f"l{len(local)}_{s.slot}"
                        local[ld] = vn
                        oy, ox = ld.offset[1], ld.offset[2]
                        off = (f" + ({oy}) * PX" if oy else "") + (f" + ({ox})" if ox else "")
                        out.append(f"{indent}const {el[ld.slot]} {vn} = c{ld.slot}[c{off}];")
                    names[id(st)] = local[ld]
                env = SweepEnv(gen, e.hoist_map, names, e.div_map, e.mul_map)
                out.append(f"{indent}{store(s.slot)} = {gen.expr(s.stmt.value, env)};")
            return out

        K += ["    for (int s = 1; s < T; ++s) {"]
        for f in fields:
            K += [f"      const {el[f]}* __restrict__ c{f} = (s & 1) ? sA{f} : sB{f};",
                  f"      {el[f]}* __restrict__ w{f} = (s & 1) ? sB{f} : sA{f};"]
        K += [f"      const int ya = s * {ry}, yb = RY - s * {ry}, xa = s * {rx}, xb = RX - s * {rx};",
              "      for (int ly = ya + (int)threadIdx.y; ly < yb; ly += blockDim.y)",
              "        for (int lx = xa + (int)threadIdx.x; lx < xb; lx += blockDim.x) {",
              "          const int c = ly * PX + lx;"]
        K += body("          ", lambda f: f"w{f}[c]")
        K += ["        }", "      __syncthreads();", "    }", "    {"]
        for f in fields:
            K.append(f"      const {el[f]}* __restrict__ c{f} = (T & 1) ? sA{f} : sB{f};")
        K += ["      for (int ly = HY + (int)threadIdx.y; ly < RY - HY; ly += blockDim.y) {",
              "        const I row = (I)(y0 + ly - HY) * (I)X + (I)(x0 - HX);",
              "        for (int lx = HX + (int)threadIdx.x; lx < RX - HX; lx += blockDim.x) {",
              "          const int c = ly * PX + lx;"]
        K += body("          ", lambda f: f"out{f}[row + lx]")
        K += [f"          if (prev_idx >= 0) prv{f}[row + lx] = c{f}[c];" for f in fields]
        K += ["        }", "      }", "    }", "  }", "}"]

        smem = " + ".join(f"(((size_t)PX * PY * sizeof({el[f]}) + 15) & ~(size_t)15) * 2" for f in fields)
        H = [f"struct xgbt_{n} {{ const void* desc; int64_t total; int64_t steps; unsigned long long* counters; "
             f"int32_t nprob; int32_t small; int32_t blocks; int32_t T; int32_t ty; int32_t tx; int32_t smem; "
             f"int32_t block[3]; }};",
             f"static size_t xg_tb_smem_{n}(int T, int ty, int tx) {{",
             f"  const size_t PX = (size_t)tx + 2 * (size_t)T * {rx}, PY = (size_t)ty + 2 * (size_t)T * {ry};",
             f"  return {smem};",
             "}",
             f'extern "C" int xg_batch_tb_blocks_{n}(int block_threads, int T, int ty, int tx, int* smem, '
             f'int* blocks) {{',
             "  if (T < 1 || ty < 1 || tx < 1) XG_FAIL(\"temporal blocking: T, ty and tx must be positive\");",
             f"  const size_t bytes = xg_tb_smem_{n}(T, ty, tx);",
             "  int dev = 0, sms = 0, per = 0, cap = 0, cap64 = 0;",
             "  XG_CUDA(cudaGetDevice(&dev));",
             "  XG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));",
             f"  XG_TRY(xg_smem_optin(xgk_{n}_tb<int>, &cap));",
             f"  XG_TRY(xg_smem_optin(xgk_{n}_tb<int64_t>, &cap64));",
             "  if (cap64 < cap) cap = cap64;",
             "  if (bytes > (size_t)cap) XG_FAIL(\"temporal blocking: %zu bytes of shared memory per CTA exceed "
             "the %d available\", bytes, cap);",
             f"  XG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, xgk_{n}_tb<int>, block_threads, bytes));",
             "  if (per < 1) XG_FAIL(\"temporal blocking: no CTA of %d threads and %zu bytes fits an SM\", "
             "block_threads, bytes);",
             "  *smem = (int)bytes;",
             "  *blocks = sms * per;",
             "  return 0;",
             "}",
             f'extern "C" int xg_batch_tb_{n}(xg_grid* G, int ngrids, const void* args, size_t nargs, void* ret, '
             f'size_t nret, void* stream) {{',
             "  (void)G; (void)ngrids; (void)ret; (void)nret;",
             "  cudaStream_t s = (cudaStream_t)stream;",
             f"  struct xgbt_{n} b;",
             f"  if (nargs != sizeof b) XG_FAIL(\"{n}: temporal batch argument block has %zu bytes\", nargs);",
             "  memcpy(&b, args, sizeof b);",
             "  if (b.steps < 2) XG_FAIL(\"temporal blocking needs at least two steps\");",
             "  if (b.total <= 0) return 0;",
             "  // launches of at most T steps each, at least two: the first reads level 0, the last",
             "  // reads the scratch level and writes both levels where the ticks leave them",
             "  const int64_t L = (b.steps + b.T - 1) / b.T < 2 ? 2 : (b.steps + b.T - 1) / b.T;",
             "  const int P = (int)(b.steps & 1);  // buffer holding level 0 after the call",
             "  XG_CUDA(cudaMemsetAsync(b.counters, 0, (size_t)L * sizeof(unsigned long long), s));",
             "  dim3 block(b.block[0], b.block[1], b.block[2]);",
             f"  const struct xgb_{n}* d = (const struct xgb_{n}*)b.desc;",
             "  const int64_t* t0 = (const int64_t*)(d + b.nprob) + b.nprob;",
             "  int in = 0;",
             "  for (int64_t i = 0; i < L; ++i) {",
             "    const int dep = (int)(b.steps / L + (i < b.steps % L ? 1 : 0));",
             "    int out, prev = -1;",
             "    if (i == L - 1) { out = P; prev = 1 - P; }",
             "    else if (i == L - 2) out = 2;",
             "    else out = 1 - in;",
             f"    xg_prof_launch({gid * 64 + 58}, s);",
             f"    if (b.small) xgk_{n}_tb<int><<<b.blocks, block, b.smem, s>>>(d, t0, b.nprob, b.total, dep, b.ty, "
             "b.tx, in, out, prev, b.counters + i);",
             f"    else xgk_{n}_tb<int64_t><<<b.blocks, block, b.smem, s>>>(d, t0, b.nprob, b.total, dep, b.ty, "
             "b.tx, in, out, prev, b.counters + i);",
             "    XG_CUDA(cudaGetLastError());",
             f"    xg_prof_end({gid * 64 + 58}, s);",
             "    in = out;",
             "  }",
             "  return 0;",
             "}"]
        return "\n".join(K), H

    def emit(self, value_args) -> list:
        from .codegen import CELL_LOOP, c_type
        gen, g, e = self.gen, self.g, self.e
        n, gid = gen.op.name, g.index
        depth = gen.depth + 1
        mains = list(range(len(g.sweeps)))
        nslots = len(gen.slots)
        extra = []
        for j in mains:
            extra += [f"const int32_t* m{j}", f"const uint8_t* tzero{j}"]
        params = e.params_struct("batch", g.sweeps, extra)
        desc = [f"struct xgb_{n} {{", f"  struct xgp_{n}_{gid}_batch par;",
                f"  void* lv[{nslots}][{depth}];", "  int64_t tile0;",
                f"  void* tb[{nslots}][3];  // temporal blocking: level 0, level 1, scratch",
                "  int64_t tile0tb;", "  int32_t tbn[2];  // tiles along y and x of the temporal tiling", "};"]
        lo, hi = [0, 0, 0], [0, 0, 0]
        for s in g.sweeps:
            for _, ld in s.loads:
                for a in range(3):
                    lo[a] = min(lo[a], ld.offset[a])
                    hi[a] = max(hi[a], ld.offset[a])
        mask_vars = {j: f"mz{j}" for j in mains}
        K = [f"template <typename I> __global__ void __launch_bounds__(256, {e.min_blocks()}) xgk_{n}_batch("
             f"const struct xgb_{n}* __restrict__ desc, const int64_t* __restrict__ tile0, int nprob, "
             f"int64_t total, int rot, unsigned long long* __restrict__ counter) {{",
             "  __shared__ int64_t item_;",
             "  __shared__ int prob_;",
             "  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);",
             "  // work queue: thread 0 takes the next item while the CTA works on the current one",
             "  int64_t next = 0;",
             "  if (tid == 0) next = (int64_t)atomicAdd(counter, 1ull);",
             "  for (;;) {",
             "    if (tid == 0) {",
             "      const int64_t it = next;",
             "      if (it < total) next = (int64_t)atomicAdd(counter, 1ull);",
             "      int lo = 0, hi = nprob - 1;",
             "      if (it < total)",
             "        while (lo < hi) {",
             "          const int mid = (lo + hi + 1) >> 1;",
             "          if (tile0[mid] <= it) lo = mid; else hi = mid - 1;",
             "        }",
             "      item_ = it;",
             "      prob_ = lo;",
             "    }",
             "    __syncthreads();",
             "    const int64_t it = item_;",
             "    const int pr = prob_;",
             "    __syncthreads();",
             "    if (it >= total) break;",
             "    const struct xgb_" + n + "& D = desc[pr];",
             f"    const struct xgp_{n}_{gid}_batch& p = D.par;",
             "    const int t = (int)(it - D.tile0);  // a problem has fewer than 2^31 tiles",
             "    const int ntx = (int)p.ntx, nty = (int)p.nty, ntz = (int)p.ntz;",
             "    const int itx = t % ntx, trow = t / ntx, ity = trow % nty, itz = trow / nty;",
             "    const xg_tile T_ = xg_tile_even(itz, ity, itx, p.Z, p.Y, p.X, p.tx, nty, ntx, ntz);",
             "    const int x0 = T_.x0, x1 = T_.x1, y0 = T_.y0, y1 = T_.y1, z0 = T_.z0, z1 = T_.z1;",
             "    const I sy = (I)p.X, sz = (I)(p.X * p.Y);",
             "    (void)sy; (void)sz;"]
        for b in e.buffers(g.sweeps):
            slot, level, _ = b
            K.append(f"    {e.elem(slot)}* __restrict__ {e.bname(b)} = ({e.elem(slot)}*)D.lv[{slot}]"
                     f"[({level} + rot) % {depth}];")
        K.append(f"    const bool fast = p.same && z0 + ({lo[0]}) >= 0 && z1 - 1 + ({hi[0]}) < p.Z && "
                 f"y0 + ({lo[1]}) >= 0 && y1 - 1 + ({hi[1]}) < p.Y && x0 + ({lo[2]}) >= 0 && "
                 f"x1 - 1 + ({hi[2]}) < p.X;")
        for j in mains:
            K.append(f"    const bool mz{j} = p.tzero{j}[t] != 0;")
        R = e.rows_for(mains)
        K.append("    if (fast) {")
        if R:
            K += e.rows_loop(mains[0], mask_vars[mains[0]], "      ", "fast", R)
            K += ["    } else if (p.same) {"]
            K += e.rows_loop(mains[0], mask_vars[mains[0]], "      ", "edge", R)
            K += ["    } else {"]
        else:
            K += ["  " + l for l in CELL_LOOP]
            K += e.main_body(mains, True, "        ", mask_vars)
            K += ["      }}", "    } else if (p.same) {"]
            K += ["  " + l for l in CELL_LOOP]
            K += e.main_body(mains, "edge", "        ", mask_vars)
            K += ["      }}", "    } else {"]
        K += ["  " + l for l in CELL_LOOP]
        K += e.main_body(mains, False, "        ", mask_vars)
        K += ["      }}", "    }", "  }", "}"]

        # host: descriptors
        H = [f'extern "C" int xg_batch_prepare_{n}(xg_grid* Gall, int nprob, const void* args, size_t stride, '
             f'void* desc_out, size_t desc_bytes, int64_t* total_out, int64_t* max_cells_out, '
             f'const int32_t* tbcfg, int64_t* total_tb_out) {{',
             f"  if (desc_bytes < (size_t)nprob * (sizeof(struct xgb_{n}) + 2 * sizeof(int64_t))) "
             f"XG_FAIL(\"{n}: descriptor buffer of %zu bytes is too small\", desc_bytes);",
             f"  struct xgb_{n}* out = (struct xgb_{n}*)desc_out;",
             "  int64_t* tile0 = (int64_t*)(out + nprob);  // compact copy for the work-queue search",
             "  int64_t* tile0tb = tile0 + nprob;          // the same for the temporal tiling",
             "  int64_t total = 0, max_cells = 0, total_tb = 0;",
             f"  int tb_ok = {1 if self.tb_plan() else 0} && tbcfg != NULL;",
             "  for (int pi = 0; pi < nprob; ++pi) {",
             f"    xg_grid* xg_G = Gall + (size_t)pi * {nslots};",
             "    xg_grid* G = xg_G;",
             f"    struct xga_{n} xg_a;",
             "    memset(&xg_a, 0, sizeof xg_a);",
             f"    if (stride) memcpy(&xg_a, (const char*)args + (size_t)pi * stride, "
             f"stride < sizeof xg_a ? stride : sizeof xg_a);",
             f"    struct xgh_{n}_{gid} xg_h;",
             "    memset(&xg_h, 0, sizeof xg_h);",
             "    {  // the kernel's arguments, by their own names, for the launch constants"]
        for an, at in value_args:
            H.append(f"      {c_type(at)} {an} = xg_a.{an}; (void){an};")
        from .codegen import HostEnv
        H += e.host_hoists(HostEnv(gen), "      ")[2:]
        H += ["    }", "    const struct xgh_" + n + "_" + str(gid) + "* h = &xg_h;"]
        H += ["    " + l.strip() for l in e.fill_params("batch", g.sweeps, g.sweeps[0].slot)]
        H += [f"    if (!p.same) XG_FAIL(\"{n}: every grid of a batched problem needs the same shape\");",
              "    int64_t ntiles = 0;"]
        for j in mains:
            sj = g.sweeps[j]
            H += [f"    p.m{j} = xg_mask_device(G[{sj.slot}].mask);",
                  f"    XG_TRY(xg_mask_tiles(G[{sj.slot}].mask, tl, 0, &p.tzero{j}, NULL, NULL, &ntiles));"]
        H += ["    out[pi].par = p;",
              f"    for (int sl = 0; sl < {nslots}; ++sl)",
              f"      for (int k = 0; k < {depth}; ++k) {{",
              f"        if (G[sl].levels < {depth}) XG_FAIL(\"{n}: grid %d of problem %d has %d levels, {depth} "
              f"needed\", sl, pi, G[sl].levels);",
              "        out[pi].lv[sl][k] = G[sl].level[k];",
              "      }",
              "    out[pi].tile0 = total;",
              "    tile0[pi] = total;",
              "    total += p.ntx * p.nty * p.ntz;",
              "    if (p.X * p.Y * p.Z > max_cells) max_cells = p.X * p.Y * p.Z;",
              "    if (tb_ok) {"]
        ry, rx = self.tb_plan() or (0, 0)
        H += [f"      const int64_t hy = (int64_t)tbcfg[0] * {ry}, hx = (int64_t)tbcfg[0] * {rx};",
              "      int64_t nz = 0;",
              f"      for (int sl = 0; sl < {nslots} && tb_ok; ++sl) {{",
              "        XG_TRY(xg_mask_nonzero(G[sl].mask, &nz));",
              "        if (nz != 0) { tb_ok = 0; xg_set_error(\"temporal blocking needs masks without nonzero "
              "cells\"); }",
              "        else if (!G[sl].scratch) { tb_ok = 0; xg_set_error(\"temporal blocking needs a scratch "
              "level\"); }",
              "        else {",
              "          out[pi].tb[sl][0] = G[sl].level[0];",
              "          out[pi].tb[sl][1] = G[sl].level[1];",
              "          out[pi].tb[sl][2] = G[sl].scratch;",
              "        }",
              "      }",
              "      if (tb_ok && (p.Z != 1 || hy > p.Y || hx > p.X)) {",
              "        tb_ok = 0;",
              "        xg_set_error(\"temporal blocking: the halo exceeds a problem's extent\");",
              "      }",
              "      if (tb_ok) {",
              "        out[pi].tbn[0] = (int32_t)((p.Y + tbcfg[1] - 1) / tbcfg[1]);",
              "        out[pi].tbn[1] = (int32_t)((p.X + tbcfg[2] - 1) / tbcfg[2]);",
              "        out[pi].tile0tb = total_tb;",
              "        tile0tb[pi] = total_tb;",
              "        total_tb += (int64_t)out[pi].tbn[0] * out[pi].tbn[1];",
              "      }",
              "    }",
              "  }",
              "  *total_out = total;",
              "  *max_cells_out = max_cells;",
              "  if (total_tb_out) *total_tb_out = tb_ok ? total_tb : -1;",
              "  return 0;",
              "}"]
        # host: launches (xg_entry_fn signature so the runtime can capture them)
        H += [f"struct xgba_{n} {{ const void* desc; int64_t total; int64_t steps; int64_t step0; "
              f"unsigned long long* counters; int32_t nprob; int32_t tick; int32_t small; int32_t blocks; "
              f"int32_t block[3]; }};",
              f'extern "C" int xg_batch_{n}(xg_grid* G, int ngrids, const void* args, size_t nargs, void* ret, '
              f'size_t nret, void* stream) {{',
              "  (void)G; (void)ngrids; (void)ret; (void)nret;",
              "  cudaStream_t s = (cudaStream_t)stream;",
              f"  struct xgba_{n} b;",
              f"  if (nargs != sizeof b) XG_FAIL(\"{n}: batch argument block has %zu bytes\", nargs);",
              "  memcpy(&b, args, sizeof b);",
              "  if (b.steps <= 0 || b.total <= 0) return 0;",
              "  XG_CUDA(cudaMemsetAsync(b.counters, 0, (size_t)b.steps * sizeof(unsigned long long), s));",
              "  dim3 block(b.block[0], b.block[1], b.block[2]);",
              "  for (int64_t st = 0; st < b.steps; ++st) {",
              f"    const int rot = b.tick ? (int)(({depth} - ((b.step0 + st + 1) % {depth})) % {depth}) : 0;",
              f"    xg_prof_launch({gid * 64 + 59}, s);",
              f"    const struct xgb_{n}* d = (const struct xgb_{n}*)b.desc;",
              "    const int64_t* t0 = (const int64_t*)(d + b.nprob);",
              f"    if (b.small) xgk_{n}_batch<int><<<b.blocks, block, 0, s>>>(d, t0, b.nprob, b.total, rot, "
              "b.counters + st);",
              f"    else xgk_{n}_batch<int64_t><<<b.blocks, block, 0, s>>>(d, t0, b.nprob, b.total, rot, "
              "b.counters + st);",
              "    XG_CUDA(cudaGetLastError());",
              f"    xg_prof_end({gid * 64 + 59}, s);",
              "  }",
              "  return 0;",
              "}",
              f'extern "C" int xg_batch_info_{n}(int32_t* depth, int64_t* desc_size, int32_t* group) {{',
              f"  *depth = {depth}; *desc_size = (int64_t)sizeof(struct xgb_{n}); *group = {gid};",
              "  return 0;",
              "}",
              f'extern "C" int xg_batch_blocks_{n}(int block_threads, int* blocks) {{',
              "  int dev = 0, sms = 0, per = 0;",
              "  XG_CUDA(cudaGetDevice(&dev));",
              "  XG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));",
              f"  XG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, xgk_{n}_batch<int>, block_threads, 0));",
              "  *blocks = sms * (per > 0 ? per : 1);",
              "  return 0;",
              "}"]
        dev = [params, "\n".join(desc), "\n".join(K)]
        if self.tb_plan():
            tk, th = self.emit_tb()
            dev.append(tk)
            H += th
        return dev, "\n".join(H)
