// Helpers shared by every generated kernel module (the .cu files that
// xgrid_gb300.codegen writes into the cache root).  Device code here is the
// addressing of the stencil templates; host code is the launch plumbing.
#pragma once
#include <cuda.h>  // CUtensorMap and its enums only; the encoder is reached through the runtime
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdbool.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "xgrid_gb300.h"
#include "xgrid_internal.h"

#define XG_HD static __host__ __device__ __forceinline__

// Report a CUDA error through the runtime's error channel and return -1.
#define XG_CUDA(call)                                                                       \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      char m_[512];                                                                         \
      snprintf(m_, sizeof m_, "%s: %s (%s)", #call, cudaGetErrorName(e_), cudaGetErrorString(e_)); \
      xg_set_error(m_);                                                                     \
      return -1;                                                                            \
    }                                                                                       \
  } while (0)

#define XG_TRY(call)            \
  do {                          \
    int r_ = (call);            \
    if (r_ < 0) return r_;      \
  } while (0)

#define XG_FAIL(...)                            \
  do {                                          \
    char m_[512];                               \
    snprintf(m_, sizeof m_, __VA_ARGS__);       \
    xg_set_error(m_);                           \
    return -1;                                  \
  } while (0)

// x*x with the conversions of pow(x, 2.0) / powf(x, 2.0): gcc folds those calls
// to one multiplication, so this keeps the generated C's results.
XG_HD double xg_sq_d(double a) { return a * a; }
XG_HD float xg_sq_f(float a) { return a * a; }

// ---------------------------------------------------------------------------
// Division by a divisor known before the launch (a loop-invariant subtree).
//
// Method: Brisebarre, Muller & Raina, "Accelerating correctly rounded
// floating-point division when the divisor is known in advance", IEEE Trans.
// Computers 53(8), 2004, followed by one Markstein correction step.  With
// zh = RN(1/d) and zl = RN(1/d - zh) precomputed on the host,
//     q  = RN(x*zh + RN(x*zl))        within 1 ulp of x/d (a faithful quotient)
//     r  = x - q*d                    exact (one fma) for a faithful q
//     q' = RN(q + r*zh)               = RN(x/d) by Markstein's theorem
// as long as nothing underflows or overflows.  The host derives from d the
// window of x exponents where that holds; outside it (and for d not normal,
// x = 0, inf, NaN, tiny or huge) the IEEE division runs instead, so the result
// is RN(x/d) for every x.
// Multiplication by a launch-invariant factor m.  When m = +-2^s the product is
// exact unless it leaves the normal range, so for a normal x with a normal
// result it is x with s added to its exponent (and the sign flipped for m < 0):
// integer instructions only, which matters where the FP64 pipe bounds a sweep.
// Zeros keep their magnitude; subnormal or out-of-range products, inf and NaN
// take the FP64 multiply.  Either way the result is RN(x*m).
struct xg_scale {
  double m;
  int s;             // exponent of |m| when p2
  unsigned hs;       // s << 20: added to the high word of x
  unsigned sg;       // sign bit of m, in the high word
  int p2;            // |m| is a power of two
};

static inline xg_scale xg_make_scale(double m) {
  xg_scale k;
  memset(&k, 0, sizeof k);
  k.m = m;
  if (!isfinite(m) || m == 0.0 || fpclassify(m) != FP_NORMAL) return k;
  int ex = 0;
  const double fr = frexp(m, &ex);  // |fr| in [0.5, 1)
  if (fabs(fr) != 0.5) return k;
  k.s = ex - 1;
  k.hs = (unsigned)k.s << 20;
  k.sg = m < 0 ? 0x80000000u : 0u;
  k.p2 = 1;
  return k;
}

__device__ __forceinline__ double xg_mulk(double x, const xg_scale& k) {
  if (k.p2) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned e = (hi >> 20) & 0x7ffu;
    if (e - 1u <= 2045u && (unsigned)((int)e + k.s - 1) <= 2045u)
      return __hiloint2double((int)((hi + k.hs) ^ k.sg), (int)lo);
    if (((hi << 1) | lo) == 0u) return __hiloint2double((int)(hi ^ k.sg), (int)lo);
  }
  return __dmul_rn(x, k.m);
}

struct xg_divisor {
  double d, zh, zl;
  unsigned lo, span;  // fast path when (biased exponent of x) - lo <= span (unsigned)
  int ok;
  xg_scale rz;        // d = +-2^s: x/d = x * 2^-s exactly (rz.p2 set)
};

static inline xg_divisor xg_make_divisor(double d) {
  xg_divisor k;
  memset(&k, 0, sizeof k);
  k.d = d;
  if (!isfinite(d) || d == 0.0 || fpclassify(d) != FP_NORMAL) return k;
  const double zh = 1.0 / d;
  if (!isfinite(zh) || fpclassify(zh) != FP_NORMAL) return k;
  if (fma(-zh, d, 1.0) == 0.0) k.rz = xg_make_scale(zh);  // 1/d exact: a power of two
  const double e = fma(-zh, d, 1.0);  // 1 - zh*d, exact for zh = RN(1/d)
  k.zh = zh;
  k.zl = e / d;
  const int ed = ilogb(d);
  // |x| >= 2^-900 * max(1, |d|) keeps x*zl, the residual and r*zh normal;
  // |x/d| <= 2^1000 keeps every intermediate finite.
  int lo = -900 + (ed > 0 ? ed : 0);
  int hi = 1000 + ed;
  if (hi > 1023) hi = 1023;
  if (hi < lo) return k;
  k.lo = (unsigned)(lo + 1023);
  k.span = (unsigned)(hi - lo);
  k.ok = 1;
  return k;
}

__device__ __forceinline__ double xg_divk(double x, const xg_divisor& k) {
  if (k.rz.p2) return xg_mulk(x, k.rz);  // x/d and x*(1/d) are the same real number
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  if (k.ok && e - k.lo <= k.span) {
    const double u = __dmul_rn(x, k.zl);
    const double q = __fma_rn(x, k.zh, u);
    const double r = __fma_rn(-q, k.d, x);
    return __fma_rn(r, k.zh, q);
  }
  if ((b << 1) == 0ull && k.ok) return __dmul_rn(x, k.zh);  // +-0 / d: zero with the quotient's sign
  return x / k.d;
}

// Collapsed (z, y, x) view of a C-order shape of 1..3 dimensions.
struct xg_ext {
  int64_t z, y, x;
};

static inline xg_ext xg_extent(const xg_grid* g) {
  xg_ext e{1, 1, 1};
  if (g->ndim == 1) {
    e.x = g->shape[0];
  } else if (g->ndim == 2) {
    e.y = g->shape[0];
    e.x = g->shape[1];
  } else {
    e.z = g->shape[0];
    e.y = g->shape[1];
    e.x = g->shape[2];
  }
  return e;
}

static inline bool xg_same_ext(xg_ext a, xg_ext b) { return a.z == b.z && a.y == b.y && a.x == b.x; }

// Linear index of (z+oz, y+oy, x+ox) in a grid of extent (Z, Y, X) under an
// overstep mode; -1 when mode "none" leaves the allocation.
//   wrap : periodic per axis            (xgrid/lang/generator.py:172-173)
//   limit: clamped per axis              (xgrid/lang/generator.py:174-175)
//   none : row-major flattened offset    (xgrid/lang/generator.py:176-179)
// Periodic index: one compare-and-add for offsets up to one period (the
// stencil case), a remainder only beyond that.
__device__ __forceinline__ int64_t xg_wrap(int64_t c, int64_t n) {
  if (c < 0) {
    c += n;
    if (c < 0) c = ((c % n) + n) % n;
  } else if (c >= n) {
    c -= n;
    if (c >= n) c %= n;
  }
  return c;
}

__device__ __forceinline__ int64_t xg_addr(int mode, int64_t z, int64_t y, int64_t x, int oz, int oy, int ox,
                                           int64_t Z, int64_t Y, int64_t X) {
  if (mode == XG_OVERSTEP_NONE) {
    int64_t t = ((z + oz) * Y + (y + oy)) * X + (x + ox);
    return (t < 0 || t >= Z * Y * X) ? -1 : t;
  }
  int64_t cz = z + oz, cy = y + oy, cx = x + ox;
  if (mode == XG_OVERSTEP_WRAP) {
    cz = xg_wrap(cz, Z);
    cy = xg_wrap(cy, Y);
    cx = xg_wrap(cx, X);
  } else {
    cz = cz < 0 ? 0 : (cz >= Z ? Z - 1 : cz);
    cy = cy < 0 ? 0 : (cy >= Y ? Y - 1 : cy);
    cx = cx < 0 ? 0 : (cx >= X ? X - 1 : cx);
  }
  return (cz * Y + cy) * X + cx;
}

// One coordinate of an edge tile under wrap or limit (the same rules as
// xg_addr, computed once per cell and axis offset instead of once per load).
__device__ __forceinline__ int xg_axis(int mode, int c, int n) {
  if (mode == XG_OVERSTEP_WRAP) {
    if (c < 0) {
      c += n;
      if (c < 0) c = ((c % n) + n) % n;
    } else if (c >= n) {
      c -= n;
      if (c >= n) c %= n;
    }
    return c;
  }
  return c < 0 ? 0 : (c >= n ? n - 1 : c);
}

// Flattened neighbour under "none": -1 outside the allocation.
__device__ __forceinline__ int64_t xg_flat(int64_t t, int64_t total) { return (t < 0 || t >= total) ? -1 : t; }

template <typename T>
__device__ __forceinline__ T xg_ldc(const T* p, int64_t i) {
  if (i < 0) {
    T zero;
    memset(&zero, 0, sizeof(T));
    return zero;
  }
  return p[i];
}

template <typename T>
__device__ __forceinline__ void xg_stc(T* p, int64_t i, T v) {
  if (i >= 0) p[i] = v;
}

// Tile bounds: axis of extent n cut into max(1, n / t) tiles of t cells, the last
// one absorbing the remainder (so that it is never narrower than t).
__device__ __forceinline__ void xg_tile_range(int64_t n, int32_t t, int64_t nt, int64_t i, int64_t* lo, int64_t* hi) {
  *lo = i * t;
  *hi = (i == nt - 1) ? n : (i + 1) * t;
}

// Tiles along an axis of n cells for tiles of at least t cells, or -t tiles when t is
// negative (z and y only; xg_tile_of has the rule).
static inline int64_t xg_tiles_along(int64_t n, int32_t t) {
  return t < 0 ? (n < -(int64_t)t ? n : -(int64_t)t) : (n / t > 0 ? n / t : 1);
}

// The tile of the calling CTA: the launch grid is (ntx, nty, ntz) tiles, so the
// tile coordinates are the block indices (no division); t is the linear tile id
// used by the mask tables.
struct xg_tile {
  int z0, z1, y0, y1, x0, x1;
  int64_t t;
};

// Tile (iz, iy, ix): along z and y, tile i of nt covers [i * n / nt, (i + 1) * n / nt)
// (even split, tiles differ by at most one cell); along x, tiles of tx cells with the
// last one absorbing the remainder (columns stay aligned to the warps).
__device__ __forceinline__ xg_tile xg_tile_even(int64_t iz, int64_t iy, int64_t ix, int64_t Z, int64_t Y, int64_t X,
                                                int tx, int64_t nty, int64_t ntx, int64_t ntz) {
  xg_tile T;
  T.t = (iz * nty + iy) * ntx + ix;
  T.x0 = (int)(ix * tx);
  T.x1 = (ix == ntx - 1) ? (int)X : (int)((ix + 1) * tx);
  T.y0 = (int)(iy * Y / nty);
  T.y1 = (int)((iy + 1) * Y / nty);
  T.z0 = (int)(iz * Z / ntz);
  T.z1 = (int)((iz + 1) * Z / ntz);
  return T;
}

__device__ __forceinline__ xg_tile xg_tile_of(int64_t Z, int64_t Y, int64_t X, int tz, int ty, int tx,
                                              int64_t nty, int64_t ntx, int64_t ntz) {
  (void)tz; (void)ty;
  return xg_tile_even(blockIdx.z, blockIdx.y, blockIdx.x, Z, Y, X, tx, nty, ntx, ntz);
}

// Tile kernels are instantiated for int and int64_t linear indices; the 32-bit
// one (fewer integer instructions per load) runs when every index fits and the
// runtime's test switch (xg_force_wide_index) is off.
static inline bool xg_small_index(int64_t Z, int64_t Y, int64_t X) {
  return Z * Y * X < (1LL << 31) - 1 && !xg_wide_index_forced();
}

// Launch grid of a tiling; fails when an axis exceeds what CUDA allows.
static inline int xg_tile_grid(int64_t ntx, int64_t nty, int64_t ntz, dim3* grid) {
  if (ntx > 2147483647LL || nty > 65535 || ntz > 65535) {
    xg_set_error("tiling needs more than 65535 tiles along y or z; use larger tiles");
    return -1;
  }
  *grid = dim3((unsigned)ntx, (unsigned)nty, (unsigned)ntz);
  return 0;
}

// ---------------------------------------------------------------------------
// Tensor-memory-accelerator (TMA) staging of 2-D boxes into shared memory.
//
// A box of bx x by elements at (x, y) of a row-pitched 2-D array lands in
// shared memory as by rows of bx elements; elements outside the array read as
// zero.  Rules the callers keep: the array base is 16-byte aligned, the pitch
// and bx * element size are multiples of 16 bytes, and every x coordinate times
// the element size is a multiple of 16 bytes (negative x included).
typedef CUresult (*xg_tmap_encode_fn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                      const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                      CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static inline int xg_tmap_2d(CUtensorMap* map, const void* base, CUtensorMapDataType type, int elem, int64_t X,
                             int64_t Y, int64_t pitch_bytes, int bx, int by) {
  static xg_tmap_encode_fn enc = NULL;
  if (!enc) {
    void* fn = NULL;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    XG_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !fn) XG_FAIL("cuTensorMapEncodeTiled is not available from the driver");
    enc = (xg_tmap_encode_fn)fn;
  }
  if (((uintptr_t)base & 15) || (pitch_bytes & 15) || ((bx * elem) & 15) || bx > 256 || by > 256 || X < 1 || Y < 1)
    XG_FAIL("TMA box: base %p, pitch %lld B, box %d x %d of %d-byte elements breaks the alignment rules", base,
            (long long)pitch_bytes, bx, by, elem);
  const cuuint64_t dims[2] = {(cuuint64_t)X, (cuuint64_t)Y};
  const cuuint64_t strides[1] = {(cuuint64_t)pitch_bytes};
  const cuuint32_t box[2] = {(cuuint32_t)bx, (cuuint32_t)by};
  const cuuint32_t step[2] = {1, 1};
  const CUresult r = enc(map, type, 2, (void*)base, dims, strides, box, step, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) XG_FAIL("cuTensorMapEncodeTiled failed with status %d", (int)r);
  return 0;
}

__device__ __forceinline__ unsigned xg_smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void xg_mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(xg_smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void xg_mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(xg_smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void xg_tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          xg_smem_addr(dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(xg_smem_addr(bar))
      : "memory");
}

// Bounded waits.  Every device-side wait gives up after XG_WAIT_NS nanoseconds of
// the global timer (about a second; the copies and barriers it waits for take
// microseconds).  The waits whose give-up path reports an error and leaves (the
// first wait for a TMA staging copy, the neighbour-tile wait of a persistent loop)
// use XG_GIVEUP_NS, the same by default.  A module compiled with XG_FAIL_WAITS
// makes those waits unable to succeed, to test the give-up paths: the tile wait
// polls once, and a TMA staging barrier expects 16 bytes more than its copies
// deliver (the copies themselves still land, and the CTA drains them before it
// leaves; XG_DRAIN_NS bounds that wait).
#ifndef XG_WAIT_NS
#define XG_WAIT_NS 1000000000ull
#endif
#ifdef XG_FAIL_WAITS
#define XG_GIVEUP_NS 0ull
#define XG_TMA_TX_EXTRA 16u
#define XG_DRAIN_NS 20000000ull  // the copies land in microseconds; their barrier never completes here
#else
#define XG_GIVEUP_NS XG_WAIT_NS
#define XG_TMA_TX_EXTRA 0u
#define XG_DRAIN_NS XG_WAIT_NS
#endif
#define XG_WAIT_POLLS_MAX (1u << 30)  // a second bound that does not depend on the timer

__device__ __forceinline__ uint64_t xg_now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait for phase `parity` of an mbarrier for at most `limit_ns`; false when it did not complete.
__device__ __forceinline__ bool xg_mbar_wait(uint64_t* bar, unsigned parity, uint64_t limit_ns) {
  const uint64_t t0 = xg_now_ns();
  for (unsigned i = 0; i < XG_WAIT_POLLS_MAX; ++i) {
    unsigned done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(xg_smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
    if (xg_now_ns() - t0 >= limit_ns) return false;
  }
  return false;
}

// ---------------------------------------------------------------------------
// Persistent loop kernels: one cooperative launch runs K iterations of a launch
// group, each CTA walking the tiles blockIdx.x, blockIdx.x + gridDim.x, ... of
// every iteration in turn, each tile waiting only for its neighbouring tiles.

// Tile number t of a (ntz, nty, ntx) tiling, numbered like xg_tile_of.
__device__ __forceinline__ xg_tile xg_tile_at(int64_t t, int64_t Z, int64_t Y, int64_t X, int tz, int ty, int tx,
                                              int64_t nty, int64_t ntx, int64_t ntz) {
  (void)tz; (void)ty;
  return xg_tile_even(t / (ntx * nty), (t / ntx) % nty, t % ntx, Z, Y, X, tx, nty, ntx, ntz);
}

// Completion flags of a persistent loop launch: flags[t] counts the iterations
// tile t has completed (zero at launch).  Iteration k of a tile reads the cells
// its neighbouring tiles wrote in iteration k - 1 and overwrites the buffer
// they read in iteration k - 1, so it may start once every tile of its 3 x 3 x 3
// neighbourhood (tile coordinates, wrapped across the grid when the grid's edges
// wrap) has completed k iterations -- no grid-wide barrier.  Threads 0..26 each
// poll one neighbour's flag with acquire loads; the wait gives up after
// XG_GIVEUP_NS, sets the error word and returns false.  The launch is
// cooperative, so every CTA whose tiles are waited for is resident.
__device__ __forceinline__ bool xg_tile_wait(const unsigned* flags, int64_t t, int64_t ntz, int64_t nty,
                                             int64_t ntx, int wrap, unsigned need, unsigned* err) {
  __shared__ int ok_;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  if (tid == 0) ok_ = 1;
  __syncthreads();
  if (tid < 27 && tid != 13) {
    const int64_t n[3] = {ntz, nty, ntx};
    int64_t c[3] = {t / (ntx * nty), (t / ntx) % nty, t % ntx};
    const int d[3] = {tid / 9 - 1, (tid / 3) % 3 - 1, tid % 3 - 1};
    bool skip = false;
    for (int a = 0; a < 3; ++a) {
      if (d[a] == 0) continue;
      if (n[a] == 1) { skip = true; break; }
      int64_t v = c[a] + d[a];
      if (v < 0 || v >= n[a]) {
        if (!wrap) { skip = true; break; }
        v = (v + n[a]) % n[a];
      }
      c[a] = v;
    }
    if (!skip) {
      const unsigned* f = flags + (c[0] * nty + c[1]) * ntx + c[2];
      const uint64_t t0 = xg_now_ns();
      int ok = 0;
      for (unsigned i = 0; i < XG_WAIT_POLLS_MAX; ++i) {
        unsigned v;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(f) : "memory");
        if ((int)(v - need) >= 0) {
          ok = 1;
          break;
        }
        if (xg_now_ns() - t0 >= XG_GIVEUP_NS) break;
      }
      if (!ok) atomicExch(&ok_, 0);
    }
  }
  __syncthreads();
  if (ok_) return true;
  if (tid == 0) atomicExch((int*)err, 1);
  return false;
}

// Tile t has completed `done` iterations: every thread's writes, then the flag (release).
__device__ __forceinline__ void xg_tile_done(unsigned* flags, int64_t t, unsigned done) {
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
    __threadfence();
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(flags + t), "r"(done) : "memory");
  }
}

// ---------------------------------------------------------------------------
// Power-of-two storage scales of 16-bit fields.  For a field whose largest
// magnitude is m, xg_scale_exp(m, A) = A - floor(log2 m) (clamped to the normal
// exponent range), so m * 2^s lies in [2^A, 2^(A+1)); multiplying by 2^s and by
// 2^-s is exact in FP32.  Zero, inf and NaN give s = 0.
__device__ __forceinline__ int xg_scale_exp(float m, int A) {
  const int b = __float_as_int(m);
  if (!(m > 0.f) || b >= 0x7f800000) return 0;
  const int s = A - (((b >> 23) & 0xff) - 127);
  return s < -126 ? -126 : (s > 126 ? 126 : s);
}

__device__ __forceinline__ float xg_pow2f(int s) { return __int_as_float((s + 127) << 23); }

template <typename T>
__device__ __forceinline__ T xg_to_store(float v);
template <>
__device__ __forceinline__ float xg_to_store<float>(float v) {
  return v;
}
template <>
__device__ __forceinline__ __half xg_to_store<__half>(float v) {
  return __float2half_rn(v);
}
template <>
__device__ __forceinline__ __nv_bfloat16 xg_to_store<__nv_bfloat16>(float v) {
  return __float2bfloat16_rn(v);
}
__device__ __forceinline__ float xg_from_store(float v) { return v; }
__device__ __forceinline__ float xg_from_store(__half v) { return __half2float(v); }
__device__ __forceinline__ float xg_from_store(__nv_bfloat16 v) { return __bfloat162float(v); }

// Four consecutive stored values at element `idx` of a shared-memory array of T,
// converted to FP32 and multiplied by `scale` (a power of two: exact).
template <typename T>
__device__ __forceinline__ float4 xg_ld4_scaled(const void* base, int idx, float scale) {
  const T* h = (const T*)base + idx;
  return make_float4(xg_from_store(h[0]) * scale, xg_from_store(h[1]) * scale, xg_from_store(h[2]) * scale,
                     xg_from_store(h[3]) * scale);
}

// Largest value over the block (every thread calls it; v >= 0 or NaN) folded
// into *dst with an integer atomicMax (non-negative floats order like their bits).
__device__ __forceinline__ void xg_block_max_atomic(float v, float* dst) {
  __shared__ float red[32];
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthr = blockDim.x * blockDim.y * blockDim.z;
  for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((tid & 31) == 0) red[tid >> 5] = v;
  __syncthreads();
  if (tid == 0) {
    float m = 0.f;
    for (int w = 0; w < (nthr + 31) / 32; ++w) m = fmaxf(m, red[w]);
    atomicMax((int*)dst, __float_as_int(m));
  }
}

// Work area of a mixed-precision loop in xg_grid.aux: the FP32 residual, two
// defect buffers of FP32 size, a 16-bit copy of the residual, then a block of
// per-launch maxima with an error word at its end.  Rows are padded to a
// multiple of 32 elements so that TMA boxes can address them.
#define XG_MX_PITCH 32
#define XG_MX_SLOT_BYTES 65536
struct xg_mx_aux {
  float* r32;
  void* dA;
  void* dB;
  void* r16;
  float* slots;
  int* err;
  int64_t XP, nslots;
};

static inline size_t xg_align256(size_t v) { return (v + 255) & ~(size_t)255; }

static inline int xg_mx_layout(const xg_grid* g, xg_mx_aux* a) {
  const xg_ext e = xg_extent(g);
  a->XP = (e.x + XG_MX_PITCH - 1) / XG_MX_PITCH * XG_MX_PITCH;
  const size_t np = (size_t)(e.z * e.y) * (size_t)a->XP;
  const size_t o_dA = xg_align256(np * 4), o_dB = o_dA + xg_align256(np * 4), o_r16 = o_dB + xg_align256(np * 4);
  const size_t o_sl = o_r16 + xg_align256(np * 2), total = o_sl + XG_MX_SLOT_BYTES;
  if (!g->aux || (size_t)g->aux_bytes < total)
    XG_FAIL("mixed-precision work area has %lld bytes, %zu needed", (long long)g->aux_bytes, total);
  unsigned char* b = (unsigned char*)g->aux;
  a->r32 = (float*)b;
  a->dA = b + o_dA;
  a->dB = b + o_dB;
  a->r16 = b + o_r16;
  a->slots = (float*)(b + o_sl);
  a->nslots = XG_MX_SLOT_BYTES / 4 - 1;
  a->err = (int*)(b + o_sl + XG_MX_SLOT_BYTES - 4);
  return 0;
}

__device__ __forceinline__ int xg_clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Raise a kernel's dynamic shared-memory limit to the most the device allows
// next to the kernel's static shared memory; *avail receives that limit.  The
// limit is a property of the function, shared by every later launch and graph
// replay, so it is set to the maximum once rather than to one launch's size.
template <typename K>
static inline int xg_smem_optin(K* kernel, int* avail) {
  int dev = 0, cap = 0;
  XG_CUDA(cudaGetDevice(&dev));
  XG_CUDA(cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  XG_CUDA(cudaFuncGetAttributes(&fa, kernel));
  const int dyn = cap - (int)fa.sharedSizeBytes;
  XG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
  if (avail) *avail = dyn;
  return 0;
}

// Chunk length along z of a staged z-walk launch over a Z x Y x X grid cut into
// (ty, tx) column blocks, one CTA per (block, chunk): the chunk count per column
// minimises ceil(CTAs / SMs) * (planes per chunk + 1), the planes that the
// busiest SM streams when every CTA costs its own planes plus its two halo
// planes at half weight (neighbouring chunks read them too, often from L2).
// Chunks hold at least 8 planes.  *nt receives the CTA count.
static inline int xg_zstage_chunks(int64_t Z, int64_t Y, int64_t X, int ty, int tx, int* zlen, int64_t* nt) {
  static int nsm = 0;
  if (nsm == 0) {
    int dev = 0;
    XG_CUDA(cudaGetDevice(&dev));
    XG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    if (nsm < 1) nsm = 1;
  }
  const int64_t ncb = ((X + tx - 1) / tx) * ((Y + ty - 1) / ty);
  int64_t cmax = Z / 8 > 1 ? Z / 8 : 1;
  if (cmax > 4096) cmax = 4096;
  int64_t best_len = Z, best_cost = -1;
  for (int64_t c = 1; c <= cmax; ++c) {
    const int64_t len = (Z + c - 1) / c, chunks = (Z + len - 1) / len;
    const int64_t cost = ((ncb * chunks + nsm - 1) / nsm) * (len + 1);
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      best_len = len;
    }
  }
  if (best_len > 0x7fffffffLL) XG_FAIL("staged z-walk: chunk of %lld planes", (long long)best_len);
  *zlen = (int)best_len;
  *nt = ncb * ((Z + best_len - 1) / best_len);
  return 0;
}

// ---------------------------------------------------------------------------
// Binary64 addition on the integer pipe.
//
// GB300 issues FP64 arithmetic at a small fraction of its integer rate, so FP64
// sweeps are bound by the FP64 pipe.  xg_dadd_i(a, b) returns RN(a + b) (IEEE
// 754 round to nearest, ties to even) with integer instructions: the larger
// operand's significand sits at bits 62..10 of a 64-bit word, the smaller one
// is shifted right by the exponent difference with every bit shifted out
// OR-ed into bit 0 (sticky), the two are added or subtracted, the sum is
// normalised back to bits 62..10 and rounded at bit 10.  Ten bits below the
// last significand bit make the sticky bit irrelevant except to break exact
// ties, so the rounding is the IEEE one.  Zeros, subnormals, infinities, NaN
// and sums that leave the normal range take the hardware operation, so the
// result is RN(a + b) for every input.  Generated sweeps send part of their
// FP64 additions here so that the FP64 and the integer pipes both work.
template <bool SUB>
__device__ __forceinline__ double xg_dadd_core(double a, double b) {
  const unsigned long long M = 0x7fffffffffffffffull;
  const unsigned long long A = (unsigned long long)__double_as_longlong(a);
  const unsigned long long B = (unsigned long long)__double_as_longlong(b) ^ (SUB ? ~M : 0ull);
  const unsigned long long MA = A & M, MB = B & M;
  if ((unsigned)(MA >> 52) - 1u > 2045u || (unsigned)(MB >> 52) - 1u > 2045u) {
    if (MB == 0ull && MA != 0ull) return a;                           // x +- 0 = x
    if (MA == 0ull && MB != 0ull) return __longlong_as_double((long long)B);  // 0 + y, 0 - y
    return SUB ? __dsub_rn(a, b) : __dadd_rn(a, b);
  }
  const bool sw = MA < MB;
  const unsigned long long X = sw ? B : A, Y = sw ? A : B;  // X: larger magnitude, its sign is the result's
  const unsigned long long MX = sw ? MB : MA, MY = sw ? MA : MB;
  const int ex = (int)(MX >> 52);
  const int d = ex - (int)(MY >> 52);
  const unsigned long long F = 0x000fffffffffffffull, H = 0x0010000000000000ull;
  const unsigned long long mx = ((MX & F) | H) << 10;
  const unsigned long long my = ((MY & F) | H) << 10;
  const int k = d < 63 ? d : 63;
  unsigned long long sy = my >> k;
  sy |= (unsigned long long)((sy << k) != my);
  unsigned long long s;
  int e = ex;
  if (((X ^ Y) >> 63) == 0ull) {
    s = mx + sy;  // < 2^64
    const unsigned long long c = s >> 63;
    s = (s >> c) | (s & c);
    e += (int)c;
  } else {
    s = mx - sy;
    if (s == 0ull) return 0.0;  // exact cancellation is +0 under round to nearest
    const int z = __clzll((long long)s) - 1;
    s <<= z;
    e -= z;
  }
  if (e < 1 || e > 2046) return SUB ? __dsub_rn(a, b) : __dadd_rn(a, b);
  s += 0x1ffull + ((s >> 10) & 1ull);
  const unsigned long long r = ((unsigned long long)(e - 1) << 52) + (s >> 10);  // a carry bumps the exponent
  return __longlong_as_double((long long)(r | (X & ~M)));
}

__device__ __forceinline__ double xg_dadd_i(double a, double b) { return xg_dadd_core<false>(a, b); }
__device__ __forceinline__ double xg_dsub_i(double a, double b) { return xg_dadd_core<true>(a, b); }

// Asynchronous copy of one element from global to shared memory (cp.async): a
// thread issues all of its tile's copies back to back without a register round
// trip, then waits once (xg_cp_async_wait_all) before the block barrier.
template <typename T>
__device__ __forceinline__ void xg_cp_async(T* dst, const T* src) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8 || sizeof(T) == 16, "cp.async copies 4, 8 or 16 bytes");
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(xg_smem_addr(dst)), "l"(src), "n"(sizeof(T))
               : "memory");
}

// 16 bytes from global to shared memory, both 16-byte aligned, through L2 only
// (cp.async.cg): staged planes are read once per CTA.
template <typename T>
__device__ __forceinline__ void xg_cp_async16(T* dst, const T* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(xg_smem_addr(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void xg_cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// Close the group of this thread's cp.async copies issued since the last commit (an empty
// group is legal), and wait until at most N of its groups are still in flight.
__device__ __forceinline__ void xg_cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void xg_cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
