// Helpers shared by every generated kernel module (the .cu files that
// xgrid_gb300.codegen writes into the cache root).  Device code here is the
// addressing of the stencil templates; host code is the launch plumbing.
#pragma once
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
__device__ __forceinline__ int64_t xg_addr(int mode, int64_t z, int64_t y, int64_t x, int oz, int oy, int ox,
                                           int64_t Z, int64_t Y, int64_t X) {
  if (mode == XG_OVERSTEP_NONE) {
    int64_t t = ((z + oz) * Y + (y + oy)) * X + (x + ox);
    return (t < 0 || t >= Z * Y * X) ? -1 : t;
  }
  int64_t cz = z + oz, cy = y + oy, cx = x + ox;
  if (mode == XG_OVERSTEP_WRAP) {
    cz = ((cz % Z) + Z) % Z;
    cy = ((cy % Y) + Y) % Y;
    cx = ((cx % X) + X) % X;
  } else {
    cz = cz < 0 ? 0 : (cz >= Z ? Z - 1 : cz);
    cy = cy < 0 ? 0 : (cy >= Y ? Y - 1 : cy);
    cx = cx < 0 ? 0 : (cx >= X ? X - 1 : cx);
  }
  return (cz * Y + cy) * X + cx;
}

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

static inline int64_t xg_tiles_along(int64_t n, int32_t t) { return n / t > 0 ? n / t : 1; }
