"""Several iterations of an in-place loop per launch, bit-exact (2-D grids).

A loop whose body is one implicit main sweep of a grid ``p``, alone or followed
by boundary phases of ``p`` (the cavity's pressure iterations,
examples/cavity.py:99-113), normally costs one launch per iteration, and at
sizes whose working set sits in L2 the fixed cost of a launch (its ramp and
tail, ~4-5 us on GB300) is a third of an FP64 Jacobi sweep.  Here a launch runs
up to ``TH`` iterations of the group on *boxes*:

* each CTA owns a core of ``cy x cx`` cells (the grid cut into ceil-sized
  cores, ``xg_mask_boxes``) and stages the box (core plus ``TH`` cells of halo
  per side) of ``p`` -- and of the mask when the box holds boundary cells --
  into shared memory; cells outside the grid read 0;
* iteration k computes the cells at distance >= k from the box edge: mask-0
  cells with the main sweep's expression (neighbours from the previous
  iteration's buffer, other grids read from global memory), the others carry
  their value; then every boundary phase on its cells of the box (per-box lists
  of box-local indices), in place, in order;
* the core's cells are written to the scratch level, and the launcher exchanges
  level and scratch once per launch, as after one iteration.

Only grids whose level takes at most a quarter of L2 use it: larger ones stream
from HBM, where the launch ramp is small against a sweep and the halo work is
not repaid (1025^2 FP64 cavity: 0.854 -> 0.761 ms per step with 3 iterations per
launch; 4097^2: 10.08 -> 10.26 ms).

Every cell gets the same operations in the same order as in the one-iteration
kernel, so the results are bit-identical.  The halo of ``TH`` cells keeps the
core exact when main-sweep reads reach one cell; ``xg_mask_box_check`` proves
(per mask and core, cached) that mask-0 cells read inside the grid and that no
boundary phase reads a cell staler than itself, otherwise the loop runs one
launch per iteration.  Overstep mode "none" only (reads beyond the grid are the
zeros of the staged box).
"""
from __future__ import annotations

from . import analysis

THREADS = 256
SITE = 57
MIN_BLOCKS = 2  # resident CTAs per SM asked of ptxas  # profiling site of the launch within its group


def plan(em) -> dict | None:
    """Loads and phases of the group for the temporal kernel, or None when the
    group does not qualify: 2-D grids of the same shape, overstep "none", main
    sweep reach <= 1, boundary phases at the cell itself reading the target at
    offsets <= 1 and other grids at the cell only."""
    gen, g = em.gen, em.g
    if gen.cfg.overstep != "none":
        return None
    sweeps = g.sweeps
    main = sweeps[0]
    slot, level = main.slot, main.level
    if not main.implicit or any(main.store_offset):
        return None
    for s in sweeps:
        t = gen.defn.signature.arguments[em.arg_index(s.slot)][1]
        if t.dimension != 2 or s.slot != slot:
            return None
    main_offs = []
    for _, ld in main.loads:
        o = tuple(analysis.pad3(ld.offset))
        if o[0] != 0 or abs(o[1]) > 1 or abs(o[2]) > 1:
            return None
        if ld.slot != slot and gen.defn.signature.arguments[em.arg_index(ld.slot)][1].dimension != 2:
            return None
        if o not in main_offs:
            main_offs.append(o)
    phases = []
    for j in range(1, len(sweeps)):
        s = sweeps[j]
        if s.is_main or any(s.store_offset) or s.implicit:
            return None
        offs = []
        for _, ld in s.loads:
            o = tuple(analysis.pad3(ld.offset))
            if ld.slot == slot and ld.level == level:
                if o[0] != 0 or abs(o[1]) > 1 or abs(o[2]) > 1:
                    return None
                if o not in offs:
                    offs.append(o)
            elif any(o):
                return None
        phases.append((j, s.mask, offs))
    return {"slot": slot, "level": level, "main_offs": main_offs, "phases": phases}


def emit(em, th: int) -> None:
    """Device kernel and host launcher ``xgl_<name>_<gid>_tloop(G, h, K, s)`` (1:
    ran the K iterations, 0: not applicable, negative: error)."""
    pl = plan(em)
    n, gid = em.name, em.gid
    if pl is None or th < 2:
        em.gen.device_chunks.append(
            f"static int xgl_{n}_{gid}_tloop(xg_grid* G, const struct xgh_{n}_{gid}* h, int64_t K, "
            f"cudaStream_t s) {{ (void)G; (void)h; (void)K; (void)s; return 0; }}")
        return
    g, gen = em.g, em.gen
    sweeps = g.sweeps
    slot, level = pl["slot"], pl["level"]
    T = em.elem(slot)
    src = em.bname((slot, level, sweeps[0].read_version_of_target))
    dst = em.bname((slot, level, sweeps[0].write_version))
    extra = ["int32_t cy, cx, nby, nbx, iters", "const int32_t* m", "const uint8_t* bzero"]
    for j, _, _ in pl["phases"]:
        extra += [f"const int32_t* bo{j}", f"const int32_t* bl{j}"]
    em.gen.device_chunks.append(em.params_struct("tl", sweeps, extra))

    def cell_code(sweep, S: str, indent: str) -> tuple[list, str]:
        """Preload lines and value of ``sweep`` at box cell l / grid cell g: the
        target from shared buffer ``S``, other grids from global memory."""
        from .codegen import SweepEnv
        lines, names, local = [], {}, {}
        for st, ld in sweep.loads:
            if ld not in local:
                vn = f"l{len(local)}"
                local[ld] = vn
                _, oy, ox = analysis.pad3(ld.offset)
                if ld.slot == slot and ld.level == level:
                    lines.append(f"{indent}const {T} {vn} = {S}[l + ({oy}) * BX + ({ox})];")
                else:
                    b = em.bname((ld.slot, ld.level, ld.version))
                    lines.append(f"{indent}const {em.elem(ld.slot)} {vn} = p.{b}[g + ({oy}) * (I)p.X + ({ox})];")
            names[id(st)] = local[ld]
        env = SweepEnv(gen, em.hoist_map, names, em.div_map, em.mul_map)
        return lines, gen.expr(sweep.stmt.value, env)

    K = [f"template <typename I, int BX> __global__ void __launch_bounds__({THREADS}, {MIN_BLOCKS}) "
         f"xgk_{n}_{gid}_tl(const __grid_constant__ struct xgp_{n}_{gid}_tl p) {{",
         f"  constexpr int TH = {th}, NT = {THREADS};",
         "  extern __shared__ __align__(16) unsigned char xg_tl_raw[];",
         "  const int BY = p.cy + 2 * TH, NB = BY * BX;",
         f"  {T}* S0 = ({T}*)xg_tl_raw;",
         f"  {T}* S1 = S0 + NB;",
         "  int32_t* MK = (int32_t*)(S1 + NB);",
         "  const int b = blockIdx.x, iy = b / p.nbx, ix = b % p.nbx;",
         "  const int gy0 = iy * p.cy - TH, gx0 = ix * p.cx - TH;",
         "  const int Y = (int)p.Y, X = (int)p.X;",
         "  const bool zero = p.bzero[b] != 0;",
         "  const int tid = threadIdx.x;",
         f"  const {T}* __restrict__ tin = p.{src};",
         "  // the box of the target (and of the mask when it holds boundary cells); beyond the grid: 0",
         "  for (int l = tid; l < NB; l += NT) {",
         "    const int gy = gy0 + l / BX, gx = gx0 + l % BX;",
         "    const bool in = gy >= 0 && gy < Y && gx >= 0 && gx < X;",
         "    const I g = (I)gy * X + gx;",
         f"    S0[l] = in ? tin[g] : ({T})0;",
         "    if (!zero) MK[l] = in ? p.m[g] : -1;",
         "  }",
         "  __syncthreads();",
         f"  {T}* Sa = S0;",
         f"  {T}* Sb = S1;",
         "  for (int k = 1; k <= p.iters; ++k) {",
         "    // cells at distance >= k from the box edge are exact after iteration k",
         ]
    K += ["    for (int l = tid; l < NB; l += NT) {",
          "      const int ly = l / BX, lx = l % BX;",
          "      const int gy = gy0 + ly, gx = gx0 + lx;",
          "      if (ly < k || ly >= BY - k || lx < k || lx >= BX - k || gy < 0 || gy >= Y || gx < 0 || gx >= X) "
          "continue;",
          "      const I g = (I)gy * X + gx;",
          "      (void)g;",
          "      if (zero || MK[l] == 0) {"]
    pre, val = cell_code(sweeps[0], "Sa", "        ")
    K += pre + [f"        Sb[l] = {val};",
                "      } else {",
                "        Sb[l] = Sa[l];",
                "      }",
                "    }",
                "    __syncthreads();"]
    for j, _, _ in pl["phases"]:
        pre, val = cell_code(sweeps[j], "Sb", "        ")
        K += ["    if (!zero) {",
              f"      for (int e = p.bo{j}[b] + tid; e < p.bo{j}[b + 1]; e += NT) {{",
              f"        const int l = p.bl{j}[e];",
              "        const int ly = l / BX, lx = l % BX;",
              "        if (ly < k || ly >= BY - k || lx < k || lx >= BX - k) continue;",
              "        const I g = (I)(gy0 + ly) * X + (gx0 + lx);",
              "        (void)g;"]
        K += pre + [f"        Sb[l] = {val};", "      }", "    }", "    __syncthreads();"]
    K += [f"    {T}* t_ = Sa; Sa = Sb; Sb = t_;",
          "  }",
          f"  {T}* __restrict__ out = p.{dst};",
          "  for (int l = tid; l < NB; l += NT) {",
          "    const int ly = l / BX, lx = l % BX;",
          "    const int gy = gy0 + ly, gx = gx0 + lx;",
          "    if (ly < TH || ly >= TH + p.cy || lx < TH || lx >= TH + p.cx || gy >= Y || gx >= X) continue;",
          "    out[(I)gy * X + gx] = Sa[l];",
          "  }",
          "}"]
    em.gen.device_chunks.append("\n".join(K))

    # host launcher
    mo = pl["main_offs"]
    vals = [v for _, v, _ in pl["phases"]]
    nof = [len(o) for _, _, o in pl["phases"]]
    offs = [v for _, _, o in pl["phases"] for t in o for v in t]

    def arr(name, typ, xs):
        return [f"  static const {typ} {name}[] = {{{', '.join(str(v) for v in xs) if xs else '0'}}};"]
    site = gid * 64 + SITE
    bxs = (64, 96, 128)
    L = [f"static int xgl_{n}_{gid}_tloop(xg_grid* G, const struct xgh_{n}_{gid}* h, int64_t K, cudaStream_t s) {{",
         f"  constexpr int TH = {th};",
         f"  if (!xg_tloop_{n} || G[{slot}].ndim != 2) return 0;"]
    L += em.check_levels(sweeps)
    L += em.fill_params("tl", sweeps, slot)
    L += [f"  if (!p.same || p.Y > 0x3fffffffLL || p.X > 0x3fffffffLL) return 0;",
          "  {  // grids whose level is more than a quarter of L2 stream from HBM: launches are not their",
          "     // bottleneck, and the boxes' halo work is not repaid (measured at 4097^2 FP64)",
          "    static int l2 = -1;",
          "    if (l2 < 0) {",
          "      int dev = 0;",
          "      XG_CUDA(cudaGetDevice(&dev));",
          "      XG_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));",
          "    }",
          f"    if ((double)p.Y * (double)p.X * sizeof({T}) > 0.25 * l2) return 0;",
          "  }"]
    L += arr("mo", "int32_t", [v for t in mo for v in t]) + arr("vals", "int32_t", vals)
    L += arr("nof", "int32_t", nof) + arr("offs", "int32_t", offs)
    L += ["  // core of a box: the (rows, box width) pair whose busiest SM has the fewest box cells",
          "  static int64_t key_y = -1, key_x = -1;",
          "  static int cy = 0, bx = 0;",
          "  if (key_y != p.Y || key_x != p.X) {",
          "    int dev = 0, sms = 0;",
          "    XG_CUDA(cudaGetDevice(&dev));",
          "    XG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));",
          "    int64_t best = -1;",
          f"    for (int w : {{{', '.join(str(v) for v in bxs)}}}) {{",
          "      const int cx = w - 2 * TH;",
          "      for (int r = 4; r <= 40; ++r) {",
          f"        const size_t smem = (size_t)(r + 2 * TH) * w * (2 * sizeof({T}) + sizeof(int32_t));",
          "        const int per_sm = (int)((228 * 1024) / (smem + 1024)) < 4 ? (int)((228 * 1024) / (smem + 1024)) : 4;",
          "        if (per_sm < 1) continue;",
          "        const int64_t nb = ((p.Y + r - 1) / r) * ((p.X + cx - 1) / cx);",
          "        const int64_t slots = (int64_t)sms * per_sm;",
          "        const int64_t cost = ((nb + slots - 1) / slots) * (int64_t)(r + 2 * TH) * w;",
          "        if (best < 0 || cost < best) { best = cost; cy = r; bx = w; }",
          "      }",
          "    }",
          "    key_y = p.Y; key_x = p.X;",
          "  }",
          "  const int32_t core[3] = {1, cy, bx - 2 * TH}, halo[3] = {0, TH, TH}, shrink[3] = {0, 1, 1};",
          "  int ok = 0;",
          f"  XG_TRY(xg_mask_box_check(G[{slot}].mask, core, halo, shrink, TH, {len(mo)}, mo, {len(vals)}, vals, nof, "
          "offs, &ok));",
          "  if (!ok) return 0;",
          "  int64_t nb = 0;",
          f"  XG_TRY(xg_mask_boxes(G[{slot}].mask, core, halo, 0, &p.bzero, NULL, NULL, &nb));"]
    for j, v, _ in pl["phases"]:
        L.append(f"  XG_TRY(xg_mask_boxes(G[{slot}].mask, core, halo, {v}, NULL, &p.bo{j}, &p.bl{j}, &nb));")
    L += ["  // (the tables above exist from here on, also for calls of one iteration: a later call of",
          "  //  several may come from an entry that may not build them)",
          "  if (K < 2 || nb > 0x7fffffffLL) return 0;",
          f"  p.m = xg_mask_device(G[{slot}].mask);",
          "  p.cy = cy; p.cx = bx - 2 * TH;",
          "  p.nby = (int32_t)((p.Y + p.cy - 1) / p.cy); p.nbx = (int32_t)((p.X + p.cx - 1) / p.cx);",
          f"  const size_t smem = (size_t)(cy + 2 * TH) * bx * (2 * sizeof({T}) + sizeof(int32_t));",
          "  const bool small = xg_small_index(p.Z, p.Y, p.X);"]
    for w in bxs:
        for it, tag in (("int", "32"), ("int64_t", "64")):
            L += [f"  static int avail_{w}_{tag} = -1;",
                  f"  if (avail_{w}_{tag} < 0) XG_TRY(xg_smem_optin(xgk_{n}_{gid}_tl<{it}, {w}>, &avail_{w}_{tag}));",
                  f"  if (bx == {w} && smem > (size_t)avail_{w}_{tag}) return 0;"]
    L += ["  for (int64_t done = 0; done < K;) {",
          "    p.iters = (int32_t)(K - done < TH ? K - done : TH);",
          f"    p.{src} = ({T}*)G[{slot}].level[{level}];",
          f"    p.{dst} = ({T}*)G[{slot}].scratch;",
          f"    xg_prof_launch({site}, s);"]
    first = True
    for w in bxs:
        cond = "if" if first else "else if"
        first = False
        L += [f"    {cond} (bx == {w}) {{",
              f"      if (small) xgk_{n}_{gid}_tl<int, {w}><<<(unsigned)nb, {THREADS}, smem, s>>>(p);",
              f"      else xgk_{n}_{gid}_tl<int64_t, {w}><<<(unsigned)nb, {THREADS}, smem, s>>>(p);",
              "    }"]
    L += ["    XG_CUDA(cudaGetLastError());",
          f"    xg_prof_end({site}, s);",
          f"    {{ void* t_ = G[{slot}].level[{level}]; G[{slot}].level[{level}] = G[{slot}].scratch; "
          f"G[{slot}].scratch = t_; }}",
          "    done += p.iters;",
          "  }",
          "  return 1;",
          "}"]
    em.gen.device_chunks.append("\n".join(L))
