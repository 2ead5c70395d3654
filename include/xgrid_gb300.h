/*
 * xgrid_gb300.h — C ABI of the GB300 stencil backend.
 *
 * Two kinds of shared objects export this ABI:
 *
 *  1. libxgrid_gb300.so, the runtime (xgrid_gb300/csrc/xgrid_runtime.cu): error
 *     channel, device-resident boundary masks and their index tables, and the
 *     CUDA-graph call cache.
 *  2. One generated module per @xgrid.kernel (cacheroot/<md5>.cu.so), which
 *     exports one entry point  xg_kernel_<name>  of type xg_entry_fn.
 *
 * Every function returns 0 on success and a negative status on failure; the
 * message is then available from xg_last_error() (thread-local).  Python raises
 * it as an Exception, which keeps the reference convention that every failure
 * surfaces as a Python Exception (xgrid/util/logging.py:58-60).
 *
 * No torch or CUDA C++ types appear in the signatures: device memory is passed
 * as plain pointers, CUDA streams as void*.
 */
#ifndef XGRID_GB300_H
#define XGRID_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XG_MAX_DIM 3
#define XG_MAX_LEVELS 8

/* Overstep modes (xgrid/util/init.py:48, xgrid/lang/generator.py:172-177). */
#define XG_OVERSTEP_NONE 0
#define XG_OVERSTEP_LIMIT 1
#define XG_OVERSTEP_WRAP 2

typedef struct xg_mask xg_mask;

/*
 * One grid argument.  Replaces the by-value C struct
 *   struct __Grid<N>d_<T> { int32_t time; int32_t shape[N]; T** data; int32_t* boundary_mask; }
 * that the reference passes to its generated C function
 * (xgrid/lang/generator.py:144-165, xgrid/util/typing/reference.py:34-65,
 *  serialised by xgrid/xgrid/__init__.py:60-68).
 * Differences: level pointers and the scratch buffer are DEVICE pointers, the
 * mask is a runtime handle with derived index tables, and the struct is passed
 * by pointer so that the callee can report the level/scratch exchange of an
 * in-place (Jacobi) sweep back to the caller.
 */
typedef struct xg_grid {
    int32_t ndim;                  /* 1..XG_MAX_DIM                                  */
    int32_t levels;                /* number of valid entries of level[] (the "time") */
    int64_t shape[XG_MAX_DIM];     /* C-order extents, shape[ndim-1] is contiguous    */
    void* level[XG_MAX_LEVELS];    /* level[0] = now, level[k] = k calls ago          */
    void* scratch;                 /* device buffer of one level, exchanged with
                                      level[0] by two-phase sweeps (may be NULL)      */
    xg_mask* mask;                 /* boundary mask handle                            */
    void* aux;                     /* device work area of mixed-precision loops
                                      (residual, defect and scale fields; may be
                                      NULL); zero it when allocating: its last 4
                                      bytes are an error word that a kernel sets to
                                      1 when a TMA staging copy does not complete    */
    int64_t aux_bytes;             /* size of aux                                     */
} xg_grid;

/*
 * Entry point of a generated kernel module: runs the body of one
 * @xgrid.kernel on `stream`.  Replaces the generated C function
 *   <ret> <name>(struct __Grid.. g0, ..., scalars..., structs...)
 * (xgrid/lang/generator.py:184-226) that Operator.__call__ invokes through
 * Library.function (xgrid/lang/operator.py:29-41, xgrid/util/ffi.py:13-35).
 * `grids` holds the grid arguments in declaration order, `args` the remaining
 * arguments packed as a C struct in declaration order (natural alignment),
 * `ret` receives the return value (nret bytes).  The call is asynchronous on
 * `stream` except for kernels that return a value.
 */
typedef int (*xg_entry_fn)(xg_grid* grids, int ngrids, const void* args, size_t nargs,
                           void* ret, size_t nret, void* stream);

/*
 * Launch hook of a generated module (no counterpart in the reference, which
 * runs one grid in one process).  A module exports
 *     int xg_set_hook_<name>(xg_launch_hook_fn fn, void* ctx);
 * With a hook set, every single-sweep launch first calls fn(ctx, site, grids,
 * ngrids, stream), site = launch group * 64 + sweep index within the group:
 * the slab decomposition refreshes the halo rows of the buffers that sweep
 * reads across slabs there (xgrid_gb300.slab).  A nonzero return fails the
 * call.  Fused launches, persistent loops and mixed-precision loops call no
 * hook: callers that set one run the module with fusion off and without them.
 */
typedef int (*xg_launch_hook_fn)(void* ctx, int site, xg_grid* grids, int ngrids, void* stream);

/*
 * No-alloc variant of an entry point (no counterpart in the reference).
 * A kernel declared with @xgrid.kernel(noalloc=True) also exports
 *     xg_kernel_<name>_noalloc
 * with the signature of xg_entry_fn and the same results as xg_kernel_<name>.
 * It is meant for callers that cannot call cudaMalloc: code running under a
 * fixed device-memory budget, inside another framework's allocator, or in a
 * real-time loop where an allocation may block.  The scratch level that an
 * in-place (two-phase) sweep needs comes from a static __device__ array of
 * 64 MiB in the module (held by every GPU that loads the module until the
 * process exits) instead of grids[i].scratch, which is ignored; calls that
 * need more than 64 MiB of scratch fail with an error.  The call allocates
 * nothing: it fails instead if a boundary-mask table it needs has not been
 * built by an earlier regular call with the same grids.  Its first call on a
 * device looks up the array's device address (do it before any stream
 * capture).  All calls share the array, so calls that overlap on the GPU
 * race; the caller's level pointers are never replaced.
 */
typedef xg_entry_fn xg_noalloc_entry_fn;
#define XG_DECLARE_NOALLOC_ENTRY(name)                                                   \
    int xg_kernel_##name##_noalloc(xg_grid* grids, int ngrids, const void* args, size_t nargs, \
                                   void* ret, size_t nret, void* stream)

/* ---- errors -------------------------------------------------------------- */
const char* xg_last_error(void);
void xg_set_error(const char* message);
int xg_runtime_version(void);

/* ---- boundary masks ------------------------------------------------------ */
/* Replaces Grid.boundary (xgrid/xgrid/__init__.py:40-41): an int32 array of the
 * grid's shape whose value k selects the `with xgrid.boundary(k)` sweeps that
 * update a cell (xgrid/lang/generator.py:295-298). */
int xg_mask_create(int ndim, const int64_t* shape, xg_mask** out);
/* Frees the mask and its tables; drops every cached graph first. */
int xg_mask_destroy(xg_mask* mask);
/* Copy a host mask in, rebuild the per-value cell lists, upload (synchronous).
 * Every upload gets a version number that is unique in the process. */
int xg_mask_upload(xg_mask* mask, const int32_t* host);
uint64_t xg_mask_version(const xg_mask* mask);
const int32_t* xg_mask_device(const xg_mask* mask);
/* Device list of the cells (row-major linear indices, ascending) whose mask
 * equals `value` (value != 0). */
int xg_mask_cells(xg_mask* mask, int32_t value, const int64_t** cells, int64_t* count);
/* Number of cells whose mask is nonzero (host-side count, no device work).
 * Runtime helper with no counterpart in the reference. */
int xg_mask_nonzero(const xg_mask* mask, int64_t* count);
/* Tile tables for a tiling of `tile` = {tz, ty, tx} cells (the last tile of
 * each axis absorbs the remainder):  *tile_zero[t] = 1 when every cell of tile
 * t has mask 0;  *csr_off/*csr_cells list the cells of mask `value` grouped by
 * tile (csr_off has ntiles+1 entries).  Device pointers, owned by the mask. */
int xg_mask_tiles(xg_mask* mask, const int32_t* tile, int32_t value,
                  const uint8_t** tile_zero, const int32_t** csr_off,
                  const int64_t** csr_cells, int64_t* ntiles);
/* 1 in *ok when, for every cell c of mask `value` and each of the `noff`
 * offsets (noff x 3, order z,y,x), the cell addressed from c under `overstep`
 * lies in the same tile as c (reads outside the grid count as local). */
int xg_mask_tile_local(xg_mask* mask, const int32_t* tile, int32_t value, int noff,
                       const int32_t* offsets, int overstep, int* ok);
/* 1 in *ok when every read of a mask-0 cell at one of the `noff` offsets (noff x 3,
 * order z,y,x) under `overstep` lands in the cell's tile or in a tile next to it
 * (along each axis at most one tile away, wrapped across the grid under "wrap"):
 * the condition under which a persistent loop launch lets each tile wait only for
 * its neighbouring tiles.  Reads outside the allocation count as local. */
int xg_mask_tile_reach(xg_mask* mask, const int32_t* tile, int noff, const int32_t* offsets, int overstep,
                       int* ok);
/* Box tables of temporally blocked launches (runtime helpers with no
 * counterpart in the reference, which sweeps once per statement).  Tiles have
 * exactly core = {tz, ty, tx} cells (the last tile of an axis may reach past
 * the grid) and are read with halo = {hz, hy, hx} cells per side (the "box").
 * *box_zero[t] = 1 when every grid cell in tile t's box has mask 0; for
 * value != 0, *off (ntiles+1 entries) and *local list per tile the cells of
 * mask `value` inside its box as box-local indices ((z*BY + y)*BX + x). */
int xg_mask_boxes(xg_mask* mask, const int32_t* core, const int32_t* halo, int32_t value,
                  const uint8_t** box_zero, const int32_t** off, const int32_t** local,
                  int64_t* ntiles);
/* 1 in *ok when `depth` iterations of an in-place sweep group can run inside
 * each box without reading stale cells: every mask-0 cell's `nmain` offsets
 * (nmain x 3, z,y,x) stay in the grid; and for each of the `nphase` boundary
 * phases (mask values[p], noffs[p] offsets, consecutive in `offsets`), every
 * read of a cell of that value stays in the grid, reads no cell of the same
 * value, and lies no closer to an inner box edge than the cell itself (up to
 * depth * shrink[a] along axis a, shrink being the main sweep's reach). */
int xg_mask_box_check(xg_mask* mask, const int32_t* core, const int32_t* halo, const int32_t* shrink,
                      int32_t depth, int nmain, const int32_t* main_offsets, int nphase,
                      const int32_t* values, const int32_t* noffs, const int32_t* offsets, int* ok);

/* ---- graph-cached calls -------------------------------------------------- */
/* Call `fn` and cache the launches it makes as a CUDA graph keyed by the
 * argument bytes and the grid pointers; later calls with the same key replay
 * the graph and restore the level/scratch exchange and the return value.  The
 * first call with a key runs eagerly (it may build mask tables).  use_graph = 0
 * always calls eagerly. */
int xg_call(xg_entry_fn fn, xg_grid* grids, int ngrids, const void* args, size_t nargs,
            void* ret, size_t nret, void* stream, int use_graph);
/* Drop every cached graph of `fn` (all when fn is NULL). */
int xg_graph_clear(xg_entry_fn fn);
int64_t xg_graph_count(void);

/* ---- host mirror copies --------------------------------------------------- */
/* Asynchronous copy of `bytes` on `stream` between a grid level and its
 * page-locked host mirror (either direction; cudaMemcpyAsync with the direction
 * inferred from the pointers).  Carries the numpy <-> device transfers behind
 * Grid.now / Grid._data and the upload before a call (the reference hands its
 * numpy levels to the C code directly, xgrid/xgrid/__init__.py:60-68). */
int xg_memcpy(void* dst, const void* src, size_t bytes, void* stream);

/* ---- index width ----------------------------------------------------------- */
/* Every tile kernel exists for 32-bit and 64-bit linear indices; the 64-bit one
 * runs for grids of 2^31 cells or more.  xg_force_wide_index(1) makes every
 * later launch take the 64-bit kernels (a test switch: the two must give the
 * same bits; cached CUDA graphs keep the kernels they captured). */
void xg_force_wide_index(int on);
int xg_wide_index_forced(void);

/* ---- launch accounting (used by generated modules and the benchmark) ----- */
/* Generated modules call xg_prof_launch() before every kernel launch and
 * xg_prof_end() after it.  Both only count unless profiling is on; with
 * profiling on, CUDA events are recorded around each launch on its stream and
 * xg_prof_read() returns (group id, milliseconds) per launch.  A call captured
 * into a CUDA graph while profiling is on gets its events as event-record nodes
 * of the graph: each replay records them again, and xg_prof_read() then returns
 * the durations of the launches of the latest replay.  xg_prof_enable(2) records
 * only launches that are being captured (graph nodes), xg_prof_enable(1) all. */
void xg_prof_enable(int on);
int xg_prof_enabled(void);
void xg_prof_launch(int group, void* stream);
void xg_prof_end(int group, void* stream);
int64_t xg_prof_launches(void);
int xg_prof_read(int64_t max, int32_t* groups, float* ms, int64_t* count);
void xg_prof_reset(void);

#ifdef __cplusplus
}
#endif
#endif /* XGRID_GB300_H */
