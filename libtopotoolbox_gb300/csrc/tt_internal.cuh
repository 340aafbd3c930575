// Internal declarations shared by the CUDA translation units of libtt_cuda.
//
// Layout conventions (include/topotoolbox.h:284-290): a grid has m = dims[0]
// rows along the fastest (contiguous) axis i and n = dims[1] columns along j;
// pixel (i, j) lives at p = j * m + i.  Tiles are 32 x 32 pixels, numbered
// column-major: tile (ti, tj) has id tj * tiles_m + ti.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <cstdio>

#include "../../include/tt_cuda.h"

namespace tt {

constexpr int kTile = 32;          // tile side (pixels)
constexpr int kHalo = kTile + 2;   // tile plus one-pixel halo ring
constexpr int kPitch = kHalo + 1;  // padded row pitch in shared memory (35):
                                   // (3c + r) mod 32 is conflict-free both
                                   // along r and along c.

struct GridDims {
  int64_t m;  // dims[0], fastest
  int64_t n;  // dims[1]
  int tm;     // tiles along i
  int tn;     // tiles along j
  __host__ __device__ int64_t cells() const { return m * n; }
  __host__ __device__ int tiles() const { return tm * tn; }
};

inline GridDims make_dims(const ptrdiff_t dims[2]) {
  GridDims g;
  g.m = dims[0];
  g.n = dims[1];
  g.tm = (int)((g.m + kTile - 1) / kTile);
  g.tn = (int)((g.n + kTile - 1) / kTile);
  return g;
}

// D8 neighbour offsets in the bit order of include/topotoolbox.h:807-816,
// for column-major (order 0) arrays: bit k points to (i + di[k], j + dj[k]).
// Row-major (order 1) swaps the two tables (src/flow_routing.c:39-49).
// The two offset tables {0,1,1,1,0,-1,-1,-1} and {1,1,0,-1,-1,-1,0,1}, stored
// as 2-bit fields (offset + 1) so a data-dependent k needs no memory lookup.
constexpr unsigned kD8A = 0x1A9u;   // {0,1,1,1,0,-1,-1,-1} + 1
constexpr unsigned kD8B = 0x901Au;  // {1,1,0,-1,-1,-1,0,1} + 1
__host__ __device__ __forceinline__ int d8_di(int k, unsigned order) {
  return (int)((((order & 1) ? kD8B : kD8A) >> (2 * k)) & 3u) - 1;
}
__host__ __device__ __forceinline__ int d8_dj(int k, unsigned order) {
  return (int)((((order & 1) ? kD8A : kD8B) >> (2 * k)) & 3u) - 1;
}

// Index of the highest set bit, as the reference decodes a direction byte
// (src/flow_accumulation.c:63-67).
__device__ __forceinline__ int d8_bit(unsigned d) { return 31 - __clz(d); }

// Slot in a list appended to by many threads: the threads that call it
// together take consecutive slots with one atomic on the shared counter
// (one per group of converged threads, not one per element, so a counter
// that millions of elements append to does not serialise at one address).
__device__ __forceinline__ int append_slot(int *counter) {
  namespace cg = cooperative_groups;
  cg::coalesced_group g = cg::coalesced_threads();
  int base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(counter, (int)g.size());
  return g.shfl(base, 0) + (int)g.thread_rank();
}

// ------------------------------------------------------------------
// Status, launch accounting, workspace
// ------------------------------------------------------------------

void set_status(tt_cuda_status s);
tt_cuda_status get_status();
void note_launch(int count = 1);
bool cuda_ok(cudaError_t e, const char *what);

#define TT_LAUNCH(kernel, grid, block, smem, stream, ...)                   \
  do {                                                                      \
    kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);             \
    ::tt::note_launch();                                                    \
  } while (0)

#define TT_CHECK(expr)                                                      \
  do {                                                                      \
    if (!::tt::cuda_ok((expr), #expr)) return TT_CUDA_ERR_CUDA;            \
  } while (0)

// Returns any status other than success to the caller.
#define TT_TRY_STATUS(expr)                 \
  do {                                      \
    tt_cuda_status _s = (expr);             \
    if (_s != TT_CUDA_SUCCESS) return _s;   \
  } while (0)

// A grow-only bump allocator over one device allocation per device.  Every
// public call resets it on entry and carves its scratch from it; calls are
// serialised per device (see DeviceLock).
class Workspace {
 public:
  // Returns nullptr when the device allocation fails.
  void *take(size_t bytes);
  void reset() { used_ = 0; }
  // Ensure `bytes` total capacity, reallocating if needed.  Must be called
  // before take() in a call; invalidates earlier pointers.
  bool reserve(size_t bytes);
  void release();
  size_t capacity() const { return cap_; }

 private:
  char *base_ = nullptr;
  size_t cap_ = 0;
  size_t used_ = 0;
};

// Deferred status (a batch captured into a CUDA graph, and device-pointer
// calls between tt_cuda_defer_begin and tt_cuda_defer_end): when a sink is
// set, stages record their status words into it with device copies instead
// of reading them back and synchronising the stream.  Each record is
// kRecordInts ints: {kind, a, b, c}.
constexpr int kRecordInts = 4;
enum : int { REC_RELAX = 1, REC_FOREST = 2 };
struct StatusSink {
  int *dev;      // device array of records
  int capacity;  // records
  int next;      // next free record
};
StatusSink *status_sink();               // nullptr unless deferring
// Reserves a record and returns its device address, or nullptr when full
// (the stage then reads its status back itself).
int *sink_record(int kind, cudaStream_t st);
// The first failure among `count` records read back to the host.
tt_cuda_status sink_status(const int *records, int count);

// For the life of the scope, this thread's stages record into `sink` and
// take their scratch from `ws` (and the pipeline's staging from `io`, when
// given) instead of the device's shared workspaces; the previous settings
// come back at its end.  Work left in flight on a private workspace keeps
// it busy, which the device's shared one must never be.
class SinkScope {
 public:
  SinkScope(StatusSink *sink, Workspace *ws, Workspace *io = nullptr);
  ~SinkScope();
  SinkScope(const SinkScope &) = delete;
  SinkScope &operator=(const SinkScope &) = delete;

 private:
  StatusSink *sink_;
  Workspace *ws_, *io_;
};

Workspace &workspace();          // of the current device (or the override)
void *pinned_scratch();          // 4 KiB of pinned host memory per device
int64_t max_rounds();
// Sweep schedule of the relaxations (0..5) for this thread's calls.
int relax_schedule();
void set_last_rounds(int64_t r);

// RAII lock of the current device's call mutex.
class DeviceLock {
 public:
  DeviceLock();
  ~DeviceLock();

 private:
  int dev_;
};

inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// Launch geometry: a persistent grid sized to the SM count.
int sm_count();

// ------------------------------------------------------------------
// Stage entry points (device pointers, enqueued on `st`).  Each returns a
// status; iterative stages synchronise `st`.
// ------------------------------------------------------------------

// `bounded`: on large grids, start from the fill of a max-pooled DEM (the
// same result, fewer tile visits); off for canvases of many DEMs, whose NaN
// gutters make that bound useless.
tt_cuda_status fill_dev(float *f, const float *dem, const uint8_t *bc,
                        const GridDims &g, cudaStream_t st, bool bounded = true);
// Grayscale reconstruction by dilation: marker := R(marker, mask).
tt_cuda_status reconstruct_dev(float *marker, const float *mask,
                               const GridDims &g, cudaStream_t st);
tt_cuda_status identifyflats_dev(int32_t *flags, const float *dem,
                                 const GridDims &g,
                                 unsigned long long *count_dev,
                                 cudaStream_t st);
// Tile flags of the relaxations: a tile waits with its edge ring or its
// whole interior to be evaluated.
enum : int { DIRTY_EDGE = 1, DIRTY_FULL = 2 };
// Marks dirty (whole interior) the tiles whose pixels or halo hold pixel
// (i, j) of an m x n grid with tm tiles along i.
__device__ __forceinline__ void mark_tiles_near(int *dirty, int tm, int64_t i, int64_t j,
                                                int64_t m, int64_t n) {
  const int ti0 = (int)((i > 0 ? i - 1 : 0) / kTile), ti1 = (int)((i + 1 < m ? i + 1 : i) / kTile);
  const int tj0 = (int)((j > 0 ? j - 1 : 0) / kTile), tj1 = (int)((j + 1 < n ? j + 1 : j) / kTile);
  for (int tj = tj0; tj <= tj1; tj++)
    for (int ti = ti0; ti <= ti1; ti++) dirty[tj * tm + ti] = DIRTY_FULL;
}

// The gwdt start written by the costs pass (pipeline entry points, which do
// not return the costs): the costs array becomes the relaxation's cost
// array (halved, NaN at non-flat pixels), `dist` gets 1 at presills, +INF at
// other flats and 0 elsewhere, and the tiles around presills are marked in
// `dirty` (zeroed
// by the caller, one int per tile).
struct GwdtSeed {
  float *dist;
  int *dirty;
};
tt_cuda_status costs_dev(float *costs, ptrdiff_t *conncomps,
                         const int32_t *flats, const float *orig,
                         const float *filled, const GridDims &g,
                         cudaStream_t st, const GwdtSeed *seed = nullptr);
tt_cuda_status gwdt_dev(float *dist, ptrdiff_t *prev, const float *costs,
                        const int32_t *flats, const GridDims &g,
                        cudaStream_t st);
// gwdt from the start a costs pass with a GwdtSeed wrote (`costs` in the
// relaxation's form, `dirty` its tile flags).
tt_cuda_status gwdt_seeded_dev(float *dist, const float *costs, const int32_t *flats,
                               int *dirty, const GridDims &g, cudaStream_t st);
tt_cuda_status directions_dev(uint8_t *dir, const float *dem,
                              const float *dist, const int32_t *flats,
                              const GridDims &g, unsigned order,
                              cudaStream_t st);
// Topological node order (every donor before its receiver) from directions.
tt_cuda_status node_order_dev(ptrdiff_t *node, const uint8_t *dir,
                              const GridDims &g, unsigned order,
                              cudaStream_t st);
tt_cuda_status accumulate_dev(float *acc, const uint8_t *dir,
                              const float *weights, const GridDims &g,
                              cudaStream_t st);
// Exact subtree pixel counts (int) of the forest of `dir`.
// Node order and accumulation from one forest contraction; `acc_done(ctx)`
// (may be null) runs once the accumulation is enqueued, before the node
// order's sort.
tt_cuda_status node_order_acc_dev(ptrdiff_t *node, float *acc, const uint8_t *dir,
                                  const float *weights, const GridDims &g,
                                  cudaStream_t st,
                                  tt_cuda_status (*acc_done)(void *) = nullptr,
                                  void *ctx = nullptr);
tt_cuda_status count_dev(int *count, const uint8_t *dir, const GridDims &g, cudaStream_t st);
tt_cuda_status accumulate_backward_dev(float *grad_w, const uint8_t *dir,
                                       const float *grad_acc,
                                       const GridDims &g, cudaStream_t st);
tt_cuda_status gradient2_dev(float *p0, float *p1, const float *dem,
                             float cellsize, const GridDims &g,
                             cudaStream_t st);
// Hillshade of tile columns [jt0, jt1) only (DEM columns 32 * jt0 - 2 to
// 32 * jt1 + 1 must be in place).
tt_cuda_status hillshade_cols_dev(float *out, const float *dem, float azimuth,
                                  float altitude, float cellsize, const GridDims &g,
                                  int jt0, int jt1, cudaStream_t st);
tt_cuda_status hillshade_dev(float *out, const float *dem, float azimuth,
                             float altitude, float cellsize, const GridDims &g,
                             cudaStream_t st);
tt_cuda_status hillshade_backward_dev(float *grad_dem, const float *dem,
                                      const float *grad_out, float azimuth,
                                      float altitude, float cellsize,
                                      const GridDims &g, cudaStream_t st);

// Edge-list forms.
tt_cuda_status edgelist_dev(ptrdiff_t *source, ptrdiff_t *target, int64_t *count,
                            const ptrdiff_t *node, const uint8_t *dir, const GridDims &g,
                            unsigned order, cudaStream_t st);
tt_cuda_status accumulate_edgelist_dev(float *acc, const ptrdiff_t *source,
                                       const ptrdiff_t *target, const float *fraction,
                                       const float *weights, int64_t E, const GridDims &g,
                                       cudaStream_t st);
// The list-order sweep out[tgt] += frac[e] * out[src] over any edge list
// of nodes [0, N): out = w (or 1) first, then every edge in list order
// (FP64 sums, deterministic).  `out` may equal `w`.
tt_cuda_status edge_sweep_dev(float *out, const float *w, const ptrdiff_t *source,
                              const ptrdiff_t *target, const float *frac, int64_t E, int64_t N,
                              cudaStream_t st);
// The same list-order sweep in the (|, &) semiring, exact:
// out[tgt] |= out[src] & in[e] in list order, or with `up`
// out[src] |= out[tgt] & in[e] in reverse list order.  out = w first; `out`
// may equal `w`.
tt_cuda_status edge_sweep_u32_dev(uint32_t *out, const uint32_t *w, const ptrdiff_t *source,
                                  const ptrdiff_t *target, const uint32_t *in, int64_t E,
                                  int64_t N, bool up, cudaStream_t st);
// 1 + the largest node index named by the edge list (INT64_MAX for a
// negative index), read back to the host.
tt_cuda_status edge_node_count_dev(const ptrdiff_t *source, const ptrdiff_t *target, int64_t E,
                                   int64_t *count, cudaStream_t st);
tt_cuda_status drainagebasins_dev(ptrdiff_t *basins, const ptrdiff_t *source,
                                  const ptrdiff_t *target, int64_t E, const GridDims &g,
                                  cudaStream_t st);
tt_cuda_status degree_dev(uint8_t *indegree, uint8_t *outdegree, const ptrdiff_t *source,
                          const ptrdiff_t *target, int64_t N, int64_t E, cudaStream_t st);

// Exclusive scan of n ints: out[k] = sum of in[0..k); the total lands in
// off[scan_blocks_for(n)].  cnt and off hold scan_blocks_for(n) + 1 ints.
int scan_blocks_for(int64_t n);
tt_cuda_status scan_exclusive_dev(const int *in, int64_t n, int *out, int *cnt, int *off,
                                  cudaStream_t st);

// Graphflood single-flow graph (row-major dim = {rows, cols}).
tt_cuda_status sfgraph_dev(const double *topo, size_t *rcv, double *dist, size_t *donors,
                           uint8_t *ndonors, size_t *stack, const uint8_t *bcs, int64_t rows,
                           int64_t cols, double dx, bool d8, cudaStream_t st);
tt_cuda_status sf_drainage_area_dev(double *area, const size_t *rcv, int64_t rows,
                                    int64_t cols, double dx, cudaStream_t st);

// Sun vector of src/hillshade.c:104-106, evaluated in double and rounded.
void sun_vector(float azimuth, float altitude, float *sx, float *sy, float *sz);

}  // namespace tt
