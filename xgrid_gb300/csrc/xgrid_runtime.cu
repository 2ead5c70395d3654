// Runtime of the GB300 stencil backend: error channel, boundary-mask index
// tables and the CUDA-graph call cache.  C ABI declared in include/xgrid_gb300.h.
//
// The reference filters every sweep cell by `boundary_mask[id] == k`
// (xgrid/lang/generator.py:295-298), so a boundary sweep scans the whole grid to
// update O(N) cells.  Here the mask is precompiled once per upload into
//   * per-value cell lists (a boundary sweep launches over its list only), and
//   * per-tiling tables: a "tile has only mask-0 cells" flag (the interior
//     sweep skips the mask read there) and the cells of each nonzero value
//     grouped by tile (a fused launch processes its own tile's boundary cells).
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <list>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "xgrid_gb300.h"
#include "xgrid_internal.h"

namespace {

thread_local std::string g_error;
// Mask versions are unique in the process: a new mask (whose handle and level
// buffers may reuse freed addresses) can never match a cached graph of an old one.
std::atomic<uint64_t> g_mask_versions{0};
// set while a no-alloc entry point runs: building a missing table is an error
thread_local int g_noalloc_scope = 0;

int fail(const std::string& msg) {
  g_error = msg;
  return -1;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

#define XG_CUDA(call)                                   \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

template <typename T>
int upload(const std::vector<T>& host, T** dev) {
  *dev = nullptr;
  if (g_noalloc_scope)
    return fail("xgrid: a boundary-mask table needed by this call is not built yet, and an entry point that "
                "may not allocate is running; make one regular call with the same grids first");
  size_t bytes = std::max<size_t>(host.size(), 1) * sizeof(T);
  XG_CUDA(cudaMalloc(reinterpret_cast<void**>(dev), bytes));
  if (!host.empty()) XG_CUDA(cudaMemcpy(*dev, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}

struct TileKey {
  int32_t tz, ty, tx;
  bool operator<(const TileKey& o) const {
    return std::tie(tz, ty, tx) < std::tie(o.tz, o.ty, o.tx);
  }
};

struct Csr {
  int32_t* off = nullptr;
  int64_t* cells = nullptr;
};

struct Tiles {
  int64_t ntiles = 0;
  int32_t nt[3] = {1, 1, 1};
  uint8_t* zero = nullptr;
  std::map<int32_t, Csr> csr;
};

// Tiling of exactly `core` cells per tile (ceil division: the last tile of an
// axis may reach past the grid), each tile read with `halo` extra cells per side.
struct BoxKey {
  int32_t core[3], halo[3];
  bool operator<(const BoxKey& o) const {
    return std::lexicographical_compare(core, core + 3, o.core, o.core + 3) ||
           (std::equal(core, core + 3, o.core) && std::lexicographical_compare(halo, halo + 3, o.halo, o.halo + 3));
  }
};

struct BoxCsr {
  int32_t* off = nullptr;
  int32_t* local = nullptr;
};

struct Boxes {
  int64_t ntiles = 0;
  int64_t nt[3] = {1, 1, 1};
  uint8_t* zero = nullptr;
  std::map<int32_t, BoxCsr> csr;
};

}  // namespace

struct xg_mask {
  int ndim = 0;
  int64_t ext[3] = {1, 1, 1};  // collapsed z, y, x extents
  int64_t total = 0;
  uint64_t version = 0;
  std::vector<int32_t> host;
  int32_t* dev = nullptr;
  std::map<int32_t, std::vector<int64_t>> cells;      // nonzero value -> sorted cells
  std::map<int32_t, int64_t*> cells_dev;
  std::map<TileKey, Tiles> tiles;
  std::map<BoxKey, Boxes> boxes;
  std::map<std::string, int> local_cache;

  void release_tables() {
    for (auto& kv : cells_dev) cudaFree(kv.second);
    cells_dev.clear();
    for (auto& kv : tiles) {
      cudaFree(kv.second.zero);
      for (auto& c : kv.second.csr) {
        cudaFree(c.second.off);
        cudaFree(c.second.cells);
      }
    }
    tiles.clear();
    for (auto& kv : boxes) {
      cudaFree(kv.second.zero);
      for (auto& c : kv.second.csr) {
        cudaFree(c.second.off);
        cudaFree(c.second.local);
      }
    }
    boxes.clear();
    local_cache.clear();
  }
};

namespace {

// Tilings (tz, ty, tx), the rule xg_tile_of in the generated code follows: the z and y
// axes are split evenly into nt = max(1, n / t) tiles -- or into -t tiles when t is
// negative -- tile i covering [i * n / nt, (i + 1) * n / nt), so their tiles differ by
// at most one cell; the x axis has tiles of tx cells, the last one absorbing the
// remainder, so that tile columns stay aligned to the warps that sweep them.
inline int64_t tile_count(int64_t n, int32_t t) {
  return t < 0 ? std::min<int64_t>(n, -(int64_t)t) : std::max<int64_t>(1, n / t);
}
inline int64_t tile_of_even(int64_t c, int64_t n, int64_t nt) { return ((c + 1) * nt - 1) / n; }
inline int64_t tile_of_last(int64_t c, int32_t t, int64_t nt) { return std::min<int64_t>(c / t, nt - 1); }
// shortest tile along an axis
inline int64_t tile_min(int axis, int64_t n, int32_t t, int64_t nt) { return axis == 2 ? (nt > 1 ? t : n) : n / nt; }
inline bool tiling_valid(const int32_t* t) { return t[0] != 0 && t[1] != 0 && t[2] >= 1; }

int64_t tile_id(const xg_mask* m, const Tiles& T, const TileKey& k, int64_t lin) {
  int64_t x = lin % m->ext[2];
  int64_t y = (lin / m->ext[2]) % m->ext[1];
  int64_t z = lin / (m->ext[2] * m->ext[1]);
  int64_t iz = tile_of_even(z, m->ext[0], T.nt[0]), iy = tile_of_even(y, m->ext[1], T.nt[1]),
          ix = tile_of_last(x, k.tx, T.nt[2]);
  return (iz * T.nt[1] + iy) * T.nt[2] + ix;
}

// Linear index addressed from (z,y,x)+(oz,oy,ox) under an overstep mode, or -1
// when the access falls outside the allocation in mode "none".
int64_t address(const xg_mask* m, int64_t lin, const int32_t* o, int overstep) {
  int64_t X = m->ext[2], Y = m->ext[1], Z = m->ext[0];
  int64_t x = lin % X, y = (lin / X) % Y, z = lin / (X * Y);
  if (overstep == XG_OVERSTEP_NONE) {
    int64_t t = lin + (int64_t)o[0] * X * Y + (int64_t)o[1] * X + o[2];
    return (t < 0 || t >= m->total) ? -1 : t;
  }
  int64_t c[3] = {z + o[0], y + o[1], x + o[2]}, n[3] = {Z, Y, X};
  for (int d = 0; d < 3; ++d) {
    if (overstep == XG_OVERSTEP_WRAP) {
      c[d] = ((c[d] % n[d]) + n[d]) % n[d];
    } else {
      c[d] = std::min<int64_t>(std::max<int64_t>(c[d], 0), n[d] - 1);
    }
  }
  return (c[0] * Y + c[1]) * X + c[2];
}

// Range of tile indices along one axis whose box [i*c - h, i*c + c + h) holds coordinate x.
inline void box_range(int64_t x, int32_t c, int32_t h, int64_t nt, int64_t* lo, int64_t* hi) {
  // i*c - h <= x          ->  i <= floor((x + h) / c)
  // x < i*c + c + h       ->  i*c > x - c - h  ->  i >= floor((x - c - h) / c) + 1
  const int64_t a = x - c - h;
  const int64_t fl = a >= 0 ? a / c : -((-a + c - 1) / c);
  *lo = std::max<int64_t>(fl + 1, 0);
  *hi = std::min<int64_t>((x + h) / c, nt - 1);
}

// Distance of coordinate x to the nearest box edge that lies inside the grid
// (cells beyond it are not in the box but exist in the grid), or a large value.
inline int64_t inner_distance(int64_t x, int64_t i, int32_t c, int32_t h, int64_t n) {
  const int64_t lo = i * c - h, hi = i * c + c + h;
  int64_t d = INT64_MAX / 4;
  if (lo > 0) d = std::min<int64_t>(d, x - lo);
  if (hi < n) d = std::min<int64_t>(d, hi - 1 - x);
  return d;
}

// ---------------------------------------------------------------- graph cache
struct GraphEntry {
  std::vector<uint8_t> key;
  bool captured = false;
  cudaGraphExec_t exec = nullptr;
  std::vector<std::array<void*, XG_MAX_LEVELS + 1>> post;  // level[] + scratch per grid
  std::vector<uint8_t> ret;
};

std::mutex g_graph_mu;
std::list<GraphEntry> g_graphs;  // most recently used first
constexpr size_t kMaxGraphs = 32;

std::vector<uint8_t> make_key(xg_entry_fn fn, const xg_grid* g, int n, const void* args, size_t nargs) {
  std::vector<uint8_t> k;
  auto put = [&k](const void* p, size_t b) {
    const uint8_t* c = static_cast<const uint8_t*>(p);
    k.insert(k.end(), c, c + b);
  };
  put(&fn, sizeof(fn));
  put(&n, sizeof(n));
  put(&nargs, sizeof(nargs));
  if (nargs) put(args, nargs);
  for (int i = 0; i < n; ++i) {
    put(&g[i].ndim, sizeof(int32_t));
    put(&g[i].levels, sizeof(int32_t));
    put(g[i].shape, sizeof(g[i].shape));
    put(g[i].level, sizeof(g[i].level));
    put(&g[i].scratch, sizeof(void*));
    put(&g[i].mask, sizeof(void*));
    put(&g[i].aux, sizeof(void*));
    uint64_t v = g[i].mask ? g[i].mask->version : 0;
    put(&v, sizeof(v));
  }
  return k;
}

}  // namespace

extern "C" {

int xg_graph_clear(xg_entry_fn fn);

const char* xg_last_error(void) { return g_error.c_str(); }

void xg_internal_noalloc_scope(int on) { g_noalloc_scope = on; }

void xg_set_error(const char* message) { g_error = message ? message : ""; }

int xg_runtime_version(void) { return 1; }

int xg_mask_create(int ndim, const int64_t* shape, xg_mask** out) {
  if (!out) return fail("xg_mask_create: null output");
  if (ndim < 1 || ndim > XG_MAX_DIM) return fail("xg_mask_create: grids must have 1 to 3 dimensions");
  xg_mask* m = new xg_mask();
  m->ndim = ndim;
  int64_t e[3] = {1, 1, 1};
  for (int d = 0; d < ndim; ++d) {
    if (shape[d] <= 0) {
      delete m;
      return fail("xg_mask_create: every extent must be positive");
    }
    e[3 - ndim + d] = shape[d];
  }
  std::memcpy(m->ext, e, sizeof(e));
  m->total = e[0] * e[1] * e[2];
  *out = m;
  return 0;
}

int xg_mask_destroy(xg_mask* m) {
  if (!m) return 0;
  // cached graphs may reference this mask's tables: drop them, and let work in
  // flight finish, before freeing
  xg_graph_clear(nullptr);
  cudaDeviceSynchronize();
  m->release_tables();
  cudaFree(m->dev);
  delete m;
  return 0;
}

int xg_mask_upload(xg_mask* m, const int32_t* host) {
  if (!m || !host) return fail("xg_mask_upload: null argument");
  m->release_tables();
  m->host.assign(host, host + m->total);
  m->cells.clear();
  for (int64_t i = 0; i < m->total; ++i)
    if (m->host[i] != 0) m->cells[m->host[i]].push_back(i);
  if (!m->dev) XG_CUDA(cudaMalloc(reinterpret_cast<void**>(&m->dev), m->total * sizeof(int32_t)));
  XG_CUDA(cudaMemcpy(m->dev, m->host.data(), m->total * sizeof(int32_t), cudaMemcpyHostToDevice));
  m->version = ++g_mask_versions;
  return 0;
}

uint64_t xg_mask_version(const xg_mask* m) { return m ? m->version : 0; }

const int32_t* xg_mask_device(const xg_mask* m) { return m ? m->dev : nullptr; }

int xg_mask_cells(xg_mask* m, int32_t value, const int64_t** cells, int64_t* count) {
  if (!m || !cells || !count) return fail("xg_mask_cells: null argument");
  if (value == 0) return fail("xg_mask_cells: mask value 0 has no cell list");
  auto it = m->cells.find(value);
  if (it == m->cells.end()) {
    *cells = nullptr;
    *count = 0;
    return 0;
  }
  auto d = m->cells_dev.find(value);
  if (d == m->cells_dev.end()) {
    int64_t* p = nullptr;
    if (upload(it->second, &p)) return -1;
    d = m->cells_dev.emplace(value, p).first;
  }
  *cells = d->second;
  *count = static_cast<int64_t>(it->second.size());
  return 0;
}

int xg_mask_nonzero(const xg_mask* m, int64_t* count) {
  if (!m || !count) return fail("xg_mask_nonzero: null argument");
  int64_t n = 0;
  for (const auto& kv : m->cells) n += static_cast<int64_t>(kv.second.size());
  *count = n;
  return 0;
}

int xg_mask_tiles(xg_mask* m, const int32_t* tile, int32_t value, const uint8_t** tile_zero,
                  const int32_t** csr_off, const int64_t** csr_cells, int64_t* ntiles) {
  if (!m || !tile) return fail("xg_mask_tiles: null argument");
  if (!tiling_valid(tile)) return fail("xg_mask_tiles: tile extents must be nonzero (x positive)");
  TileKey key{tile[0], tile[1], tile[2]};
  auto it = m->tiles.find(key);
  if (it == m->tiles.end()) {
    Tiles T;
    T.nt[0] = (int32_t)tile_count(m->ext[0], key.tz);
    T.nt[1] = (int32_t)tile_count(m->ext[1], key.ty);
    T.nt[2] = (int32_t)tile_count(m->ext[2], key.tx);
    T.ntiles = (int64_t)T.nt[0] * T.nt[1] * T.nt[2];
    if (T.ntiles > INT32_MAX) return fail("xg_mask_tiles: too many tiles");
    std::vector<uint8_t> zero(T.ntiles, 1);
    for (auto& kv : m->cells)
      for (int64_t c : kv.second) zero[tile_id(m, T, key, c)] = 0;
    if (upload(zero, &T.zero)) return -1;
    it = m->tiles.emplace(key, T).first;
  }
  Tiles& T = it->second;
  if (tile_zero) *tile_zero = T.zero;
  if (ntiles) *ntiles = T.ntiles;
  if (value != 0 && (csr_off || csr_cells)) {
    auto c = T.csr.find(value);
    if (c == T.csr.end()) {
      std::vector<int32_t> off(T.ntiles + 1, 0);
      std::vector<int64_t> sorted;
      auto cv = m->cells.find(value);
      if (cv != m->cells.end()) {
        std::vector<std::pair<int64_t, int64_t>> tagged;
        tagged.reserve(cv->second.size());
        for (int64_t cell : cv->second) tagged.emplace_back(tile_id(m, T, key, cell), cell);
        std::sort(tagged.begin(), tagged.end());
        for (auto& p : tagged) {
          off[p.first + 1] += 1;
          sorted.push_back(p.second);
        }
        for (int64_t t = 0; t < T.ntiles; ++t) off[t + 1] += off[t];
      }
      Csr csr;
      if (upload(off, &csr.off) || upload(sorted, &csr.cells)) return -1;
      c = T.csr.emplace(value, csr).first;
    }
    if (csr_off) *csr_off = c->second.off;
    if (csr_cells) *csr_cells = c->second.cells;
  }
  return 0;
}

int xg_mask_tile_local(xg_mask* m, const int32_t* tile, int32_t value, int noff, const int32_t* offsets,
                       int overstep, int* ok) {
  if (!m || !tile || !ok || (noff > 0 && !offsets)) return fail("xg_mask_tile_local: null argument");
  std::string ck(reinterpret_cast<const char*>(tile), 3 * sizeof(int32_t));
  ck.append(reinterpret_cast<const char*>(&value), sizeof(value));
  ck.append(reinterpret_cast<const char*>(&overstep), sizeof(overstep));
  ck.append(reinterpret_cast<const char*>(offsets), (size_t)noff * 3 * sizeof(int32_t));
  auto hit = m->local_cache.find(ck);
  if (hit != m->local_cache.end()) {
    *ok = hit->second;
    return 0;
  }
  if (xg_mask_tiles(m, tile, 0, nullptr, nullptr, nullptr, nullptr)) return -1;
  TileKey key{tile[0], tile[1], tile[2]};
  const Tiles& T = m->tiles.at(key);
  int result = 1;
  auto cv = m->cells.find(value);
  if (cv != m->cells.end()) {
    for (int64_t c : cv->second) {
      int64_t own = tile_id(m, T, key, c);
      for (int k = 0; k < noff && result; ++k) {
        int64_t t = address(m, c, offsets + 3 * k, overstep);
        if (t >= 0 && tile_id(m, T, key, t) != own) result = 0;
      }
      if (!result) break;
    }
  }
  m->local_cache.emplace(ck, result);
  *ok = result;
  return 0;
}

int xg_mask_tile_reach(xg_mask* m, const int32_t* tile, int noff, const int32_t* offsets, int overstep, int* ok) {
  if (!m || !tile || !ok || (noff > 0 && !offsets)) return fail("xg_mask_tile_reach: null argument");
  const int32_t ext[3] = {tile[0], tile[1], tile[2]};
  int64_t nt[3], reach[3] = {0, 0, 0};
  for (int a = 0; a < 3; ++a) {
    if (!tiling_valid(ext)) return fail("xg_mask_tile_reach: tile extents must be nonzero (x positive)");
    nt[a] = tile_count(m->ext[a], ext[a]);
    for (int k = 0; k < noff; ++k) reach[a] = std::max<int64_t>(reach[a], std::abs(offsets[3 * k + a]));
  }
  // a read may reach the next tile along an axis, never the one after it: the reach
  // must not exceed the shortest tile
  for (int a = 0; a < 3; ++a)
    if (nt[a] > 1 && reach[a] > tile_min(a, m->ext[a], ext[a], nt[a])) {
      *ok = 0;
      return 0;
    }
  if (overstep != XG_OVERSTEP_NONE) {  // clamped reads stay put, wrapped reads reach the wrapped neighbour
    *ok = 1;
    return 0;
  }
  std::string ck("reach");
  ck.append(reinterpret_cast<const char*>(tile), 3 * sizeof(int32_t));
  ck.append(reinterpret_cast<const char*>(offsets), (size_t)noff * 3 * sizeof(int32_t));
  auto hit = m->local_cache.find(ck);
  if (hit != m->local_cache.end()) {
    *ok = hit->second;
    return 0;
  }
  // overstep "none" addresses the flattened index: a read past a row or plane end of
  // the grid lands at the other end of the next row or plane.  Only mask-0 cells
  // within the reach of the grid's outer faces can do that; check those.
  int result = 1;
  const int64_t X = m->ext[2], Y = m->ext[1], Z = m->ext[0];
  auto tile_of3 = [&](int64_t lin, int64_t* c) {
    const int64_t x = lin % X, y = (lin / X) % Y, z = lin / (X * Y);
    c[0] = tile_of_even(z, Z, nt[0]);
    c[1] = tile_of_even(y, Y, nt[1]);
    c[2] = tile_of_last(x, ext[2], nt[2]);
  };
  for (int64_t z = 0; z < Z && result; ++z)
    for (int64_t y = 0; y < Y && result; ++y) {
      const bool face_zy = z < reach[0] || z >= Z - reach[0] || y < reach[1] || y >= Y - reach[1];
      for (int64_t x = 0; x < X && result; ++x) {
        if (!face_zy && x >= reach[2] && x < X - reach[2]) {
          x = X - reach[2] - 1;  // skip the interior of the row
          continue;
        }
        const int64_t lin = (z * Y + y) * X + x;
        if (m->host[lin] != 0) continue;
        int64_t own[3];
        tile_of3(lin, own);
        for (int k = 0; k < noff && result; ++k) {
          const int64_t t = address(m, lin, offsets + 3 * k, overstep);
          if (t < 0) continue;  // outside the allocation: the kernel reads zero there
          int64_t c[3];
          tile_of3(t, c);
          for (int a = 0; a < 3; ++a)
            if (std::abs(c[a] - own[a]) > 1) result = 0;
        }
      }
    }
  m->local_cache.emplace(ck, result);
  *ok = result;
  return 0;
}

int xg_mask_boxes(xg_mask* m, const int32_t* core, const int32_t* halo, int32_t value, const uint8_t** box_zero,
                  const int32_t** off, const int32_t** local, int64_t* ntiles) {
  if (!m || !core || !halo) return fail("xg_mask_boxes: null argument");
  for (int a = 0; a < 3; ++a)
    if (core[a] < 1 || halo[a] < 0) return fail("xg_mask_boxes: core extents must be positive, halos non-negative");
  const int64_t box[3] = {core[0] + 2LL * halo[0], core[1] + 2LL * halo[1], core[2] + 2LL * halo[2]};
  if (box[0] * box[1] * box[2] > INT32_MAX) return fail("xg_mask_boxes: box too large");
  BoxKey key;
  std::copy(core, core + 3, key.core);
  std::copy(halo, halo + 3, key.halo);
  auto it = m->boxes.find(key);
  if (it == m->boxes.end()) {
    Boxes B;
    for (int a = 0; a < 3; ++a) B.nt[a] = (m->ext[a] + core[a] - 1) / core[a];
    B.ntiles = B.nt[0] * B.nt[1] * B.nt[2];
    if (B.ntiles > INT32_MAX) return fail("xg_mask_boxes: too many tiles");
    std::vector<uint8_t> zero(B.ntiles, 1);
    for (auto& kv : m->cells)
      for (int64_t c : kv.second) {
        const int64_t co[3] = {c / (m->ext[1] * m->ext[2]), (c / m->ext[2]) % m->ext[1], c % m->ext[2]};
        int64_t lo[3], hi[3];
        for (int a = 0; a < 3; ++a) box_range(co[a], core[a], halo[a], B.nt[a], &lo[a], &hi[a]);
        for (int64_t iz = lo[0]; iz <= hi[0]; ++iz)
          for (int64_t iy = lo[1]; iy <= hi[1]; ++iy)
            for (int64_t ix = lo[2]; ix <= hi[2]; ++ix) zero[(iz * B.nt[1] + iy) * B.nt[2] + ix] = 0;
      }
    if (upload(zero, &B.zero)) return -1;
    it = m->boxes.emplace(key, B).first;
  }
  Boxes& B = it->second;
  if (box_zero) *box_zero = B.zero;
  if (ntiles) *ntiles = B.ntiles;
  if (value != 0 && (off || local)) {
    auto c = B.csr.find(value);
    if (c == B.csr.end()) {
      std::vector<std::pair<int64_t, int32_t>> tagged;
      auto cv = m->cells.find(value);
      if (cv != m->cells.end())
        for (int64_t cell : cv->second) {
          const int64_t co[3] = {cell / (m->ext[1] * m->ext[2]), (cell / m->ext[2]) % m->ext[1], cell % m->ext[2]};
          int64_t lo[3], hi[3];
          for (int a = 0; a < 3; ++a) box_range(co[a], core[a], halo[a], B.nt[a], &lo[a], &hi[a]);
          for (int64_t iz = lo[0]; iz <= hi[0]; ++iz)
            for (int64_t iy = lo[1]; iy <= hi[1]; ++iy)
              for (int64_t ix = lo[2]; ix <= hi[2]; ++ix) {
                const int64_t lz = co[0] - (iz * core[0] - halo[0]), ly = co[1] - (iy * core[1] - halo[1]),
                              lx = co[2] - (ix * core[2] - halo[2]);
                tagged.emplace_back((iz * B.nt[1] + iy) * B.nt[2] + ix, (int32_t)((lz * box[1] + ly) * box[2] + lx));
              }
        }
      std::sort(tagged.begin(), tagged.end());
      std::vector<int32_t> offs(B.ntiles + 1, 0), locs;
      locs.reserve(tagged.size());
      for (auto& p : tagged) {
        offs[p.first + 1] += 1;
        locs.push_back(p.second);
      }
      for (int64_t t = 0; t < B.ntiles; ++t) offs[t + 1] += offs[t];
      if (offs[B.ntiles] < 0 || tagged.size() > (size_t)INT32_MAX) return fail("xg_mask_boxes: too many cells");
      BoxCsr csr;
      if (upload(offs, &csr.off) || upload(locs, &csr.local)) return -1;
      c = B.csr.emplace(value, csr).first;
    }
    if (off) *off = c->second.off;
    if (local) *local = c->second.local;
  }
  return 0;
}

int xg_mask_box_check(xg_mask* m, const int32_t* core, const int32_t* halo, const int32_t* shrink, int32_t depth,
                      int nmain, const int32_t* main_offsets, int nphase, const int32_t* values, const int32_t* noffs,
                      const int32_t* offsets, int* ok) {
  if (!m || !core || !halo || !shrink || !ok || (nmain > 0 && !main_offsets) ||
      (nphase > 0 && (!values || !noffs)))
    return fail("xg_mask_box_check: null argument");
  std::string ck("box");
  auto put = [&ck](const void* p, size_t b) { ck.append(static_cast<const char*>(p), b); };
  put(core, 12);
  put(halo, 12);
  put(shrink, 12);
  put(&depth, 4);
  put(&nmain, 4);
  put(main_offsets, (size_t)nmain * 12);
  put(&nphase, 4);
  int total = 0;
  for (int p = 0; p < nphase; ++p) total += noffs[p];
  put(values, (size_t)nphase * 4);
  put(noffs, (size_t)nphase * 4);
  if (total) put(offsets, (size_t)total * 12);
  auto hit = m->local_cache.find(ck);
  if (hit != m->local_cache.end()) {
    *ok = hit->second;
    return 0;
  }
  const int64_t* n = m->ext;
  auto inside = [n](const int64_t* c) { return c[0] >= 0 && c[0] < n[0] && c[1] >= 0 && c[1] < n[1] && c[2] >= 0 && c[2] < n[2]; };
  int result = 1;
  // (1) mask-0 cells read inside the grid; only cells within the reach of an edge can fail
  int32_t reach[3] = {0, 0, 0};
  for (int k = 0; k < nmain; ++k)
    for (int a = 0; a < 3; ++a) reach[a] = std::max(reach[a], std::abs(main_offsets[3 * k + a]));
  for (int64_t z = 0; z < n[0] && result; ++z)
    for (int64_t y = 0; y < n[1] && result; ++y) {
      const bool band = z < reach[0] || z >= n[0] - reach[0] || y < reach[1] || y >= n[1] - reach[1];
      for (int64_t x = 0; x < n[2] && result; x = (band || x >= n[2] - reach[2] || x + 1 < reach[2]) ? x + 1
                                                                                                 : n[2] - reach[2]) {
        if (m->host[(z * n[1] + y) * n[2] + x] != 0) continue;
        for (int k = 0; k < nmain; ++k) {
          const int64_t c[3] = {z + main_offsets[3 * k], y + main_offsets[3 * k + 1], x + main_offsets[3 * k + 2]};
          if (!inside(c)) {
            result = 0;
            break;
          }
        }
      }
    }
  // (2) boundary phases: reads inside the grid, never of their own mask value, and never
  //     closer to an inner box edge than the cell itself (up to the depth's halo)
  int base = 0;
  for (int p = 0; p < nphase && result; base += noffs[p], ++p) {
    auto cv = m->cells.find(values[p]);
    if (cv == m->cells.end()) continue;
    int64_t nt[3];
    for (int a = 0; a < 3; ++a) nt[a] = (n[a] + core[a] - 1) / core[a];
    for (int64_t cell : cv->second) {
      const int64_t co[3] = {cell / (n[1] * n[2]), (cell / n[2]) % n[1], cell % n[2]};
      int64_t lo[3], hi[3];
      for (int a = 0; a < 3; ++a) box_range(co[a], core[a], halo[a], nt[a], &lo[a], &hi[a]);
      for (int k = 0; k < noffs[p] && result; ++k) {
        const int32_t* o = offsets + 3 * (base + k);
        const int64_t src[3] = {co[0] + o[0], co[1] + o[1], co[2] + o[2]};
        if (!inside(src) || m->host[(src[0] * n[1] + src[1]) * n[2] + src[2]] == values[p]) {
          result = 0;
          break;
        }
        for (int a = 0; a < 3 && result; ++a) {
          if (o[a] == 0) continue;
          const int64_t need = (int64_t)depth * shrink[a];
          const int64_t i0 = a == 0 ? lo[0] : (a == 1 ? lo[1] : lo[2]), i1 = a == 0 ? hi[0] : (a == 1 ? hi[1] : hi[2]);
          for (int64_t i = i0; i <= i1; ++i) {
            const int64_t dc = inner_distance(co[a], i, core[a], halo[a], n[a]);
            const int64_t ds = inner_distance(src[a], i, core[a], halo[a], n[a]);
            if (ds < std::min(dc, need)) {
              result = 0;
              break;
            }
          }
        }
      }
      if (!result) break;
    }
  }
  m->local_cache.emplace(ck, result);
  *ok = result;
  return 0;
}

int xg_call(xg_entry_fn fn, xg_grid* grids, int ngrids, const void* args, size_t nargs, void* ret, size_t nret,
            void* stream, int use_graph) {
  if (!fn) return fail("xg_call: null entry point");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!use_graph || s == nullptr) return fn(grids, ngrids, args, nargs, ret, nret, stream);

  std::vector<uint8_t> key = make_key(fn, grids, ngrids, args, nargs);
  std::unique_lock<std::mutex> lock(g_graph_mu);
  auto it = std::find_if(g_graphs.begin(), g_graphs.end(), [&](const GraphEntry& e) { return e.key == key; });
  if (it == g_graphs.end()) {
    // first sighting: run eagerly (this builds any mask tables the body needs)
    GraphEntry e;
    e.key = key;
    g_graphs.push_front(std::move(e));
    while (g_graphs.size() > kMaxGraphs) {
      if (g_graphs.back().exec) cudaGraphExecDestroy(g_graphs.back().exec);
      g_graphs.pop_back();
    }
    lock.unlock();
    return fn(grids, ngrids, args, nargs, ret, nret, stream);
  }
  g_graphs.splice(g_graphs.begin(), g_graphs, it);
  GraphEntry& e = g_graphs.front();
  if (!e.captured) {
    XG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int rc = fn(grids, ngrids, args, nargs, ret, nret, stream);
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (rc != 0) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
    cudaError_t ie = cudaGraphInstantiate(&e.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) return cuda_fail(ie, "cudaGraphInstantiate");
    e.captured = true;
    e.post.resize(ngrids);
    for (int i = 0; i < ngrids; ++i) {
      std::copy(grids[i].level, grids[i].level + XG_MAX_LEVELS, e.post[i].begin());
      e.post[i][XG_MAX_LEVELS] = grids[i].scratch;
    }
    e.ret.assign(static_cast<uint8_t*>(ret), static_cast<uint8_t*>(ret) + (ret ? nret : 0));
  } else {
    for (int i = 0; i < ngrids; ++i) {
      std::copy(e.post[i].begin(), e.post[i].begin() + XG_MAX_LEVELS, grids[i].level);
      grids[i].scratch = e.post[i][XG_MAX_LEVELS];
    }
    if (ret && nret) std::memcpy(ret, e.ret.data(), std::min(nret, e.ret.size()));
  }
  XG_CUDA(cudaGraphLaunch(e.exec, s));
  return 0;
}

int xg_graph_clear(xg_entry_fn fn) {
  std::lock_guard<std::mutex> lock(g_graph_mu);
  for (auto it = g_graphs.begin(); it != g_graphs.end();) {
    xg_entry_fn owner;
    std::memcpy(&owner, it->key.data(), sizeof(owner));
    if (fn == nullptr || owner == fn) {
      if (it->exec) cudaGraphExecDestroy(it->exec);
      it = g_graphs.erase(it);
    } else {
      ++it;
    }
  }
  return 0;
}

// ------------------------------------------------------------ launch accounting
namespace {
struct ProfRec {
  int32_t group;
  cudaEvent_t start, stop;
};
std::mutex g_prof_mu;
int g_prof_on = 0;
int64_t g_launches = 0;
std::vector<ProfRec> g_prof;
std::vector<cudaEvent_t> g_event_pool;
cudaEvent_t pooled_event() {
  if (!g_event_pool.empty()) {
    cudaEvent_t e = g_event_pool.back();
    g_event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}
}  // namespace

namespace {
std::atomic<int> g_wide_index{0};
}

void xg_force_wide_index(int on) { g_wide_index.store(on ? 1 : 0); }

int xg_wide_index_forced(void) { return g_wide_index.load(std::memory_order_relaxed); }

int xg_memcpy(void* dst, const void* src, size_t bytes, void* stream) {
  if (bytes == 0) return 0;
  if (!dst || !src) return fail("xg_memcpy: null pointer");
  XG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, static_cast<cudaStream_t>(stream)));
  return 0;
}

void xg_prof_enable(int on) {
  std::lock_guard<std::mutex> lock(g_prof_mu);
  g_prof_on = on;
}

int xg_prof_enabled(void) { return g_prof_on; }

// While `stream` is being captured into a CUDA graph the events become event-record
// nodes of the graph (cudaEventRecordExternal): every replay of the graph records
// them again, so xg_prof_read then gives the launch durations of the latest replay.
static bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(s, &st) == cudaSuccess && st == cudaStreamCaptureStatusActive;
}

static void prof_record(cudaEvent_t e, cudaStream_t s) {
  if (capturing(s))
    cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
  else
    cudaEventRecord(e, s);
}

void xg_prof_launch(int group, void* stream) {
  std::lock_guard<std::mutex> lock(g_prof_mu);
  g_launches += 1;
  if (!g_prof_on) return;
  if (g_prof_on == 2 && !capturing(static_cast<cudaStream_t>(stream))) return;
  ProfRec r{group, pooled_event(), pooled_event()};
  prof_record(r.start, static_cast<cudaStream_t>(stream));
  g_prof.push_back(r);
}

void xg_prof_end(int group, void* stream) {
  std::lock_guard<std::mutex> lock(g_prof_mu);
  if (!g_prof_on || g_prof.empty() || g_prof.back().group != group) return;
  prof_record(g_prof.back().stop, static_cast<cudaStream_t>(stream));
}

int64_t xg_prof_launches(void) {
  std::lock_guard<std::mutex> lock(g_prof_mu);
  return g_launches;
}

int xg_prof_read(int64_t max, int32_t* groups, float* ms, int64_t* count) {
  std::lock_guard<std::mutex> lock(g_prof_mu);
  int64_t n = std::min<int64_t>(max, (int64_t)g_prof.size());
  for (int64_t i = 0; i < n; ++i) {
    XG_CUDA(cudaEventSynchronize(g_prof[i].stop));
    float t = 0.f;
    XG_CUDA(cudaEventElapsedTime(&t, g_prof[i].start, g_prof[i].stop));
    if (groups) groups[i] = g_prof[i].group;
    if (ms) ms[i] = t;
  }
  if (count) *count = (int64_t)g_prof.size();
  return 0;
}

void xg_prof_reset(void) {
  std::lock_guard<std::mutex> lock(g_prof_mu);
  for (auto& r : g_prof) {
    g_event_pool.push_back(r.start);
    g_event_pool.push_back(r.stop);
  }
  g_prof.clear();
  g_launches = 0;
}

int64_t xg_graph_count(void) {
  std::lock_guard<std::mutex> lock(g_graph_mu);
  int64_t n = 0;
  for (auto& e : g_graphs) n += e.captured ? 1 : 0;
  return n;
}

}  // extern "C"
