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
from .types import GridType

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
                f"  void* lv[{nslots}][{depth}];", "  int64_t tile0;", "};"]
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
             "    const int x0 = itx * p.tx, x1 = itx == ntx - 1 ? (int)p.X : (itx + 1) * p.tx;",
             "    const int y0 = ity * p.ty, y1 = ity == nty - 1 ? (int)p.Y : (ity + 1) * p.ty;",
             "    const int z0 = itz * p.tz, z1 = itz == ntz - 1 ? (int)p.Z : (itz + 1) * p.tz;",
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
             f'void* desc_out, size_t desc_bytes, int64_t* total_out, int64_t* max_cells_out) {{',
             f"  if (desc_bytes < (size_t)nprob * (sizeof(struct xgb_{n}) + sizeof(int64_t))) "
             f"XG_FAIL(\"{n}: descriptor buffer of %zu bytes is too small\", desc_bytes);",
             f"  struct xgb_{n}* out = (struct xgb_{n}*)desc_out;",
             "  int64_t* tile0 = (int64_t*)(out + nprob);  // compact copy for the work-queue search",
             "  int64_t total = 0, max_cells = 0;",
             "  for (int pi = 0; pi < nprob; ++pi) {",
             f"    xg_grid* G = Gall + (size_t)pi * {nslots};",
             f"    struct xga_{n} a;",
             "    memset(&a, 0, sizeof a);",
             f"    if (stride) memcpy(&a, (const char*)args + (size_t)pi * stride, stride < sizeof a ? stride : sizeof a);"]
        for an, at in value_args:
            H.append(f"    {c_type(at)} {an} = a.{an}; (void){an};")
        from .codegen import HostEnv
        H += e.host_hoists(HostEnv(gen), "    ")
        H += ["    const struct xgh_" + n + "_" + str(gid) + "* h = &h_;"]
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
              "  }",
              "  *total_out = total;",
              "  *max_cells_out = max_cells;",
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
        return [params, "\n".join(desc), "\n".join(K)], "\n".join(H)
