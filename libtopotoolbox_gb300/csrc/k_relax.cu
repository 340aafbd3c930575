// Tile relaxation engine for the two monotone fixpoint problems of the
// pipeline:
//
//  * sink filling (src/fillsinks.c:23-77, src/reconstruct.c:68-312), stated
//    in the un-negated elevation space:  f(p) = max(dem(p), min of f over the
//    3x3 neighbourhood), iterated downwards from f = dem on bc == 1 and +INF
//    elsewhere.  The reference computes the same fixpoint as
//    -reconstruct(-dem) by raster scans plus a FIFO queue.
//  * the gray-weighted distance transform (src/gwdt.c:290-351):
//    d(v) = min(d(v), d(u) + chamfer(u,v) * (c(u) + c(v)) / 2) over flat
//    neighbours u, from d = 1 at presills and +INF at other flats.  The
//    reference runs Dijkstra; label correcting reaches the same minimum over
//    float-evaluated paths because fl(d + w) is monotone in d and never below
//    d, so every distance is bit-identical.
//
// Both updates only ever lower a value, and any order of updates converges
// to the same fixpoint, so tiles can be relaxed concurrently and races
// between neighbouring tiles are benign.
//
// Work decomposition: one warp owns one 32 x 32 tile.  It stages the tile and
// a one-pixel halo in shared memory and runs directional Gauss-Seidel sweeps
// (down, up, right, left along the two axes, each lane carrying one line)
// until four consecutive sweeps change nothing.  Changed cells are written
// back with a float atomic minimum; a changed edge or corner pushes the
// neighbouring tile onto a global work queue.
//
// Scheduling: one persistent launch.  Warp w of W owns the tiles
// w, w + W, w + 2W, ... and keeps scanning their "dirty" flags (32 at a time
// with a ballot); a warp that relaxes a tile and changes an edge marks the
// neighbouring tile dirty, so information crosses tile borders as soon as a
// tile finishes, with no host round trips and no shared queue to contend on.
// A tile has a single owner, so no two warps relax it at once.  A pending
// counter (dirty + running tiles) detects termination: it is raised before a
// flag is set and lowered only after the owner has finished the tile, so it
// cannot reach zero while work remains.  Every wait is bounded: a warp that
// idles too long, or a run that exceeds its visit budget, raises an abort
// flag and all warps return with an error status.
#include <algorithm>
#include <cmath>
#include <mutex>

#include "tt_internal.cuh"

namespace tt {
namespace {

constexpr int kWarps = 4;        // tiles per block
constexpr int kMaxSweeps = 256;  // per tile visit; a capped tile re-enqueues
constexpr float kSqrt2 = 1.41421356237309504880f;

enum Kind { FILL = 0, GWDT = 1 };

struct WarpTile {
  float s[kHalo][kPitch];  // state: f (fill) or dist (gwdt); [c][r]
  float a[kHalo][kPitch];  // aux: dem (fill) or costs (gwdt)
  uint64_t flat[kHalo];    // gwdt: flat bit per row of column c (rows 0..33)
  uint32_t dirty[kHalo];   // changed interior rows (bit r-1) of column c
  uint32_t need[kHalo];    // interior rows of column c to re-evaluate
};

// Control block (device memory, zero-initialised).
struct QueueCtl {
  unsigned long long visits;  // tiles relaxed so far
  int pending;                // dirty + running tiles
  int abort;                  // ABORT_* bits
};

enum : int { ABORT_SPIN = 1, ABORT_VISITS = 2 };

constexpr long long kSpinLimit = 1LL << 22;  // idle scans before giving up

struct RelaxArgs {
  float *state;
  const float *aux;
  const int32_t *flats;
  int64_t m, n;
  int tm, tn;
  QueueCtl *ctl;
  int *dirty;  // per tile: 1 while waiting to be relaxed
  unsigned long long max_visits;
};

// Dirty flag values: 1 = a halo pixel changed (re-evaluate the edge ring),
// 2 = evaluate every pixel (first visit, or a visit that hit its sweep cap).
enum : int { DIRTY_EDGE = 1, DIRTY_FULL = 2 };

__device__ __forceinline__ void mark_dirty(const RelaxArgs &a, int t, int v) {
  atomicAdd(&a.ctl->pending, 1);
  if (atomicMax(&a.dirty[t], v) != 0) atomicSub(&a.ctl->pending, 1);
}

__device__ __forceinline__ void push_tile(const RelaxArgs &a, int ti, int tj,
                                          int v = DIRTY_EDGE) {
  if (ti < 0 || tj < 0 || ti >= a.tm || tj >= a.tn) return;
  mark_dirty(a, tj * a.tm + ti, v);
}

// The update at pixel (c, r) from all eight neighbours.  Neighbour values may
// be old or new: every value is an upper bound of the fixpoint, so any mix
// gives a valid (and never higher) result.
template <int KIND>
__device__ __forceinline__ float relax8(const WarpTile &t, int c, int r, float cur) {
  if (KIND == FILL) {
    float lo = cur;
#pragma unroll
    for (int dc = -1; dc <= 1; dc++)
#pragma unroll
      for (int dr = -1; dr <= 1; dr++)
        if (dc || dr) lo = fminf(lo, t.s[c + dc][r + dr]);
    const float z = t.a[c][r];
    return (lo > z) ? lo : z;
  } else {
    if (!((t.flat[c] >> r) & 1)) return cur;
    const float cs = t.a[c][r];
    float best = cur;
#pragma unroll
    for (int dc = -1; dc <= 1; dc++) {
      const uint64_t fc = t.flat[c + dc];
#pragma unroll
      for (int dr = -1; dr <= 1; dr++) {
        if (!(dc || dr)) continue;
        if (!((fc >> (r + dr)) & 1)) continue;
        const float ch = (dc && dr) ? kSqrt2 : 1.0f;
        const float w = __fmul_rn(__fmul_rn(ch, __fadd_rn(cs, t.a[c + dc][r + dr])), 0.5f);
        const float prop = __fadd_rn(t.s[c + dc][r + dr], w);
        if (prop < best) best = prop;
      }
    }
    return best;
  }
}

// Work-proportional Gauss-Seidel sweeps.  need[c] marks the interior pixels
// of column c whose neighbourhood changed since they were last evaluated
// against all eight neighbours; only those are evaluated, a step with no
// marked pixel is skipped by the whole warp, and a pixel that changes marks
// its eight neighbours.  An unmarked pixel therefore cannot be lowered by any
// neighbour, and the tile is at its local fixpoint exactly when no pixel is
// marked.

// Sweep along r (lane = column c).  dir = +1 down, -1 up.
template <int KIND>
__device__ void sweep_rows(WarpTile &t, int lane, int dir) {
  const int c = lane + 1;
  uint32_t nd = t.need[c];
  uint32_t dmask = 0;
  for (int s = 0; s < kTile; s++) {
    const int r = dir > 0 ? 1 + s : kTile - s;
    const uint32_t bit = 1u << (r - 1);
    const bool act = (nd & bit) != 0;
    if (!__any_sync(0xffffffffu, act)) continue;
    uint32_t mark = 0;
    if (act) {
      nd &= ~bit;
      const float cur = t.s[c][r];
      const float nv = relax8<KIND>(t, c, r, cur);
      if (nv < cur) {
        t.s[c][r] = nv;
        dmask |= bit;
        mark = bit | (bit << 1) | (bit >> 1);
      }
    }
    // neighbours in this column and in the two adjacent columns
    const uint32_t from_left = __shfl_up_sync(0xffffffffu, mark, 1);
    const uint32_t from_right = __shfl_down_sync(0xffffffffu, mark, 1);
    nd |= (mark & ~bit) | (lane > 0 ? from_left : 0u) | (lane < 31 ? from_right : 0u);
    __syncwarp();
  }
  t.need[c] = nd;
  t.dirty[c] |= dmask;
  __syncwarp();
}

// Sweep along c (lane = row r).  dir = +1 right, -1 left.
template <int KIND>
__device__ void sweep_cols(WarpTile &t, int lane, int dir) {
  const int r = lane + 1;
  for (int s = 0; s < kTile; s++) {
    const int c = dir > 0 ? 1 + s : kTile - s;
    const uint32_t w = t.need[c];
    if (w == 0) continue;  // warp-uniform (shared word)
    const bool act = (w >> lane) & 1u;
    bool ch = false;
    if (act) {
      const float cur = t.s[c][r];
      const float nv = relax8<KIND>(t, c, r, cur);
      ch = nv < cur;
      if (ch) t.s[c][r] = nv;
    }
    const unsigned b = __ballot_sync(0xffffffffu, ch);
    __syncwarp();
    if (lane == 0) {
      // every marked pixel of column c was evaluated in this step; pixels next
      // to one that changed (in this column and the two adjacent ones) must
      // be evaluated again
      const uint32_t d3 = b | (b << 1) | (b >> 1);
      t.need[c] = (b << 1) | (b >> 1);
      if (c > 1) t.need[c - 1] |= d3;
      if (c < kTile) t.need[c + 1] |= d3;
      t.dirty[c] |= b;
    }
    __syncwarp();
  }
}

template <int KIND>
__device__ void relax_tile(const RelaxArgs &a, WarpTile &t, int lane, int tile, int mode);

template <int KIND>
__global__ void __launch_bounds__(kWarps * 32)
relax_persistent_kernel(RelaxArgs a) {
  __shared__ WarpTile tiles[kWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpTile &t = tiles[warp];
  const int W = gridDim.x * kWarps;
  const int wid = blockIdx.x * kWarps + warp;
  const int T = a.tm * a.tn;
  long long idle = 0;
  for (;;) {
    if (*(volatile int *)&a.ctl->abort) break;
    if (lane == 0 && *(volatile unsigned long long *)&a.ctl->visits >= a.max_visits)
      atomicOr(&a.ctl->abort, ABORT_VISITS);
    bool did = false;
    for (int base = wid; base < T; base += W * 32) {
      const int mine = base + lane * W;
      int f = (mine < T) ? *(volatile int *)&a.dirty[mine] : 0;
      unsigned mask = __ballot_sync(0xffffffffu, f != 0);
      while (mask) {
        const int l = __ffs(mask) - 1;
        mask &= mask - 1;
        const int tile = base + l * W;
        int got = 0;
        if (lane == 0) {
          got = atomicExch(&a.dirty[tile], 0);
          if (got) {
            atomicAdd(&a.ctl->visits, 1ULL);  // no return: no round trip
            __threadfence();
          }
        }
        got = __shfl_sync(0xffffffffu, got, 0);
        if (!got) continue;
        did = true;
        relax_tile<KIND>(a, t, lane, tile, got);
        if (lane == 0) {
          __threadfence();
          atomicSub(&a.ctl->pending, 1);
        }
        __syncwarp();
      }
    }
    if (did) {
      idle = 0;
      continue;
    }
    int stop = 0;
    if (lane == 0) {
      if (*(volatile int *)&a.ctl->pending <= 0) {
        stop = 1;
      } else if (++idle > kSpinLimit) {
        atomicOr(&a.ctl->abort, ABORT_SPIN);
        stop = 1;
      } else {
        __nanosleep(idle < 64 ? 64 : 512);
      }
    }
    if (__shfl_sync(0xffffffffu, stop, 0)) break;
  }
}

// Relaxes one tile to its local fixpoint and marks changed neighbours dirty.
template <int KIND>
__device__ void relax_tile(const RelaxArgs &a, WarpTile &t, int lane, int tile, int mode) {
  {
    const int ti = tile % a.tm, tj = tile / a.tm;
    const int64_t i0 = (int64_t)ti * kTile, j0 = (int64_t)tj * kTile;

    // Stage tile + halo.  Lane r loads row r (and lanes 0, 1 rows 32, 33).
    // Loads are issued a chunk of columns at a time into registers before
    // any of them is consumed, so one visit waits for a few memory latencies
    // instead of one per column.
    constexpr int kChunk = 9;  // 34 columns = 9 + 9 + 9 + 7
    const int r_lo = lane, r_hi = lane + 32;
    const int64_t i_lo = i0 - 1 + r_lo, i_hi = i0 - 1 + r_hi;
    const bool ilo_ok = i_lo >= 0 && i_lo < a.m;
    const bool ihi_ok = r_hi < kHalo && i_hi < a.m;
    for (int c0 = 0; c0 < kHalo; c0 += kChunk) {
      float s_lo[kChunk], a_lo[kChunk], s_hi[kChunk], a_hi[kChunk];
      int f_lo[kChunk], f_hi[kChunk];
#pragma unroll
      for (int u = 0; u < kChunk; u++) {
        const int c = c0 + u;
        const int64_t j = j0 - 1 + c;
        const bool jok = c < kHalo && j >= 0 && j < a.n;
        s_lo[u] = INFINITY;
        a_lo[u] = (KIND == FILL) ? INFINITY : 0.0f;
        s_hi[u] = INFINITY;
        a_hi[u] = (KIND == FILL) ? INFINITY : 0.0f;
        f_lo[u] = 0;
        f_hi[u] = 0;
        if (jok && ilo_ok) {
          const int64_t p = j * a.m + i_lo;
          s_lo[u] = __ldcg(&a.state[p]);  // L2: other SMs update it concurrently
          a_lo[u] = a.aux[p];
          if (KIND == GWDT) f_lo[u] = a.flats[p];
        }
        if (jok && ihi_ok) {
          const int64_t p = j * a.m + i_hi;
          s_hi[u] = __ldcg(&a.state[p]);
          a_hi[u] = a.aux[p];
          if (KIND == GWDT) f_hi[u] = a.flats[p];
        }
      }
#pragma unroll
      for (int u = 0; u < kChunk; u++) {
        const int c = c0 + u;
        if (c >= kHalo) break;
        t.s[c][r_lo] = s_lo[u];
        t.a[c][r_lo] = a_lo[u];
        if (r_hi < kHalo) {
          t.s[c][r_hi] = s_hi[u];
          t.a[c][r_hi] = a_hi[u];
        }
        uint32_t flo = 0, fhi = 0;
        if (KIND == GWDT) {
          flo = __ballot_sync(0xffffffffu, f_lo[u] & 1);
          fhi = __ballot_sync(0xffffffffu, f_hi[u] & 1);
        }
        if (lane == 0) {
          t.dirty[c] = 0;
          t.need[c] = (mode == DIRTY_FULL || c == 1 || c == kTile) ? 0xffffffffu
                                                                    : 0x80000001u;
          if (KIND == GWDT) t.flat[c] = (uint64_t)flo | ((uint64_t)(fhi & 3u) << 32);
        }
      }
    }
    __syncwarp();

    // Sweep until no pixel is marked for re-evaluation: the local fixpoint.
    bool done = false;
    int sweeps = 0, k = 0;
    while (sweeps < kMaxSweeps) {
      if (!__any_sync(0xffffffffu, t.need[lane + 1] != 0)) {
        done = true;
        break;
      }
      switch (k) {
        case 0: sweep_rows<KIND>(t, lane, +1); break;
        case 1: sweep_rows<KIND>(t, lane, -1); break;
        case 2: sweep_cols<KIND>(t, lane, +1); break;
        default: sweep_cols<KIND>(t, lane, -1); break;
      }
      k = (k + 1) & 3;
      sweeps++;
    }
    __syncwarp();

    // Write back changed cells (coalesced per column) and collect edge flags.
    uint32_t top = 0, bottom = 0;
    for (int c = 1; c <= kTile; c++) {
      uint32_t dm = t.dirty[c];
      if (!dm) continue;
      int64_t j = j0 + c - 1;
      int64_t i = i0 + lane;
      if ((dm >> lane) & 1u) {
        if (j < a.n && i < a.m) a.state[j * a.m + i] = t.s[c][lane + 1];
      }
      top |= dm & 1u;
      bottom |= (dm >> 31) & 1u;
    }
    __threadfence();  // publish this lane's writes before any push below
    __syncwarp();
    {  // lanes 0..8 mark one neighbour each, concurrently
      const uint32_t left = t.dirty[1], right = t.dirty[kTile];
      switch (lane) {
        case 0: if (top) push_tile(a, ti - 1, tj); break;
        case 1: if (bottom) push_tile(a, ti + 1, tj); break;
        case 2: if (left) push_tile(a, ti, tj - 1); break;
        case 3: if (right) push_tile(a, ti, tj + 1); break;
        case 4: if (left & 1u) push_tile(a, ti - 1, tj - 1); break;
        case 5: if ((left >> 31) & 1u) push_tile(a, ti + 1, tj - 1); break;
        case 6: if (right & 1u) push_tile(a, ti - 1, tj + 1); break;
        case 7: if ((right >> 31) & 1u) push_tile(a, ti + 1, tj + 1); break;
        case 8: if (!done) push_tile(a, ti, tj, DIRTY_FULL); break;  // capped
        default: break;
      }
      __threadfence();  // the pending increments land before the owner's decrement
    }
    __syncwarp();
  }
}

// f = dem where bc == 1 (and where dem is NaN), +INF elsewhere
// (src/fillsinks.c:24-37 in the un-negated space).
__global__ void fill_init_kernel(float *__restrict__ f, const float *__restrict__ dem,
                                 const uint8_t *__restrict__ bc, int64_t N) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    float z = dem[p];
    f[p] = (bc[p] == 1 || isnan(z)) ? z : INFINITY;
  }
}

// Reconstruction by dilation in the un-negated space: f = -min(marker, mask),
// z = -mask.
__global__ void negate_pair_kernel(float *__restrict__ f, float *__restrict__ z,
                                   const float *__restrict__ marker,
                                   const float *__restrict__ mask, int64_t N) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    float mk = mask[p], mr = marker[p];
    z[p] = -mk;
    f[p] = isnan(mk) ? -mk : -(mr < mk ? mr : mk);
  }
}

__global__ void negate_kernel(float *__restrict__ out, const float *__restrict__ in,
                              int64_t N) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x)
    out[p] = -in[p];
}

// Mark every tile dirty (fill starts everywhere).
__global__ void dirty_all_kernel(int *dirty, QueueCtl *ctl, int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    dirty[t] = DIRTY_FULL;
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->pending = n;
}

// dist = 1 at presills, +INF at other flats, 0 elsewhere; flag every tile
// whose pixels or halo contain a presill (plain stores: idempotent).
__global__ void gwdt_init_kernel(float *__restrict__ dist,
                                 const int32_t *__restrict__ flats, int64_t m,
                                 int64_t n, RelaxArgs qa) {
  const int64_t N = m * n;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    int32_t f = flats[p];
    float d = 0.0f;
    if (f & 1) d = (f & 4) ? 1.0f : INFINITY;
    dist[p] = d;
    if ((f & 5) == 5) {
      int64_t i = p % m, j = p / m;
      int ti0 = (int)((i > 0 ? i - 1 : 0) / kTile), ti1 = (int)((i + 1 < m ? i + 1 : i) / kTile);
      int tj0 = (int)((j > 0 ? j - 1 : 0) / kTile), tj1 = (int)((j + 1 < n ? j + 1 : j) / kTile);
      for (int tj = tj0; tj <= tj1; tj++)
        for (int ti = ti0; ti <= ti1; ti++) {
          int *fl = &qa.dirty[tj * qa.tm + ti];
          if (*fl == 0) *fl = DIRTY_FULL;
        }
    }
  }
}

// pending = number of flagged tiles (the persistent launch starts after).
__global__ void count_dirty_kernel(const int *__restrict__ dirty, int n, QueueCtl *ctl) {
  int c = 0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    c += dirty[t] != 0;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(&ctl->pending, c);
}

// A valid back-link for every reached flat: the first flat neighbour u (in
// the neighbour order of src/gwdt.c:318-320) with d(v) == d(u) + w(u, v).
__global__ void gwdt_prev_kernel(ptrdiff_t *__restrict__ prev,
                                 const float *__restrict__ dist,
                                 const float *__restrict__ costs,
                                 const int32_t *__restrict__ flats, int64_t m,
                                 int64_t n) {
  const int64_t N = m * n;
  const int di[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
  const int dj[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    ptrdiff_t pr = p;
    int32_t f = flats[p];
    float d = dist[p];
    if ((f & 1) && !(f & 4) && d < INFINITY) {
      int64_t i = p % m, j = p / m;
      float cp = costs[p];
      for (int k = 0; k < 8; k++) {
        int64_t ni = i + di[k], nj = j + dj[k];
        if (ni < 0 || ni >= m || nj < 0 || nj >= n) continue;
        int64_t q = nj * m + ni;
        if (!(flats[q] & 1)) continue;
        float ch = (di[k] != 0 && dj[k] != 0) ? kSqrt2 : 1.0f;
        float w = __fmul_rn(__fmul_rn(ch, __fadd_rn(cp, costs[q])), 0.5f);
        if (__fadd_rn(dist[q], w) == d) {
          pr = q;
          break;
        }
      }
    }
    prev[p] = pr;
  }
}

int elementwise_grid(int64_t N) {
  int64_t b = (N + 255) / 256;
  int64_t cap = (int64_t)sm_count() * 16;
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}

// Host driver: mark the starting tiles, run one persistent launch, read the
// status.
template <int KIND>
tt_cuda_status run_queue(float *state, const float *aux, const int32_t *flats,
                         const GridDims &g, cudaStream_t st) {
  const int T = g.tiles();
  Workspace &ws = workspace();
  size_t need = align_up(sizeof(QueueCtl)) + align_up((size_t)T * 4);
  if (!ws.reserve(need)) return TT_CUDA_ERR_ALLOC;
  QueueCtl *ctl = (QueueCtl *)ws.take(sizeof(QueueCtl));
  int *dirty = (int *)ws.take((size_t)T * 4);
  QueueCtl *hctl = (QueueCtl *)pinned_scratch();
  if (!hctl) return TT_CUDA_ERR_ALLOC;

  RelaxArgs ra{state, aux, flats, g.m, g.n, g.tm, g.tn, ctl, dirty, 0};
  const int64_t cap_rounds = max_rounds();
  ra.max_visits = (unsigned long long)T * (unsigned long long)std::min<int64_t>(cap_rounds, 1LL << 20);
  TT_CHECK(cudaMemsetAsync(ctl, 0, sizeof(QueueCtl), st));
  const int tgrid = (T + 255) / 256;
  if (KIND == FILL) {
    TT_LAUNCH(dirty_all_kernel, tgrid, 256, 0, st, dirty, ctl, T);
  } else {
    TT_CHECK(cudaMemsetAsync(dirty, 0, (size_t)T * 4, st));
    TT_LAUNCH(gwdt_init_kernel, elementwise_grid(g.cells()), 256, 0, st, state, flats,
              g.m, g.n, ra);
    TT_LAUNCH(count_dirty_kernel, std::min(tgrid, sm_count() * 4), 256, 0, st, dirty, T, ctl);
  }
  TT_CHECK(cudaGetLastError());
  static int blocks_per_sm[2] = {0, 0};
  if (!blocks_per_sm[KIND]) {
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, relax_persistent_kernel<KIND>,
                                                  kWarps * 32, 0);
    blocks_per_sm[KIND] = b > 0 ? b : 1;
  }
  // No more warps than tiles (each warp owns at least one tile).
  int grid = sm_count() * blocks_per_sm[KIND];
  grid = std::max(1, std::min(grid, (T + kWarps - 1) / kWarps));
  TT_LAUNCH(relax_persistent_kernel<KIND>, grid, kWarps * 32, 0, st, ra);
  TT_CHECK(cudaGetLastError());
  if (status_sink()) {  // deferred: record the abort word, no round trip
    int *rec = sink_record(REC_RELAX, st);
    if (rec) TT_CHECK(cudaMemcpyAsync(rec + 1, &ctl->abort, sizeof(int),
                                      cudaMemcpyDeviceToDevice, st));
    return TT_CUDA_SUCCESS;
  }
  TT_CHECK(cudaMemcpyAsync(hctl, ctl, sizeof(QueueCtl), cudaMemcpyDeviceToHost, st));
  TT_CHECK(cudaStreamSynchronize(st));
  // Tile visits per tile, reported as "rounds".
  set_last_rounds((int64_t)(hctl->visits / (unsigned long long)(T > 0 ? T : 1)));
  if (hctl->abort) return TT_CUDA_ERR_NOT_CONVERGED;
  return TT_CUDA_SUCCESS;
}

}  // namespace

tt_cuda_status fill_dev(float *f, const float *dem, const uint8_t *bc,
                        const GridDims &g, cudaStream_t st) {
  TT_LAUNCH(fill_init_kernel, elementwise_grid(g.cells()), 256, 0, st, f, dem,
            bc, g.cells());
  TT_CHECK(cudaGetLastError());
  return run_queue<FILL>(f, dem, nullptr, g, st);
}

tt_cuda_status reconstruct_dev(float *marker, const float *mask,
                               const GridDims &g, cudaStream_t st) {
  // The negated copies live in the io-independent scratch of this call.
  const int64_t N = g.cells();
  float *buf = nullptr;
  TT_CHECK(cudaMallocAsync((void **)&buf, (size_t)N * 8, st));
  float *f = buf, *z = buf + N;
  TT_LAUNCH(negate_pair_kernel, elementwise_grid(N), 256, 0, st, f, z, marker, mask, N);
  tt_cuda_status s = run_queue<FILL>(f, z, nullptr, g, st);
  if (s == TT_CUDA_SUCCESS || s == TT_CUDA_ERR_NOT_CONVERGED)
    TT_LAUNCH(negate_kernel, elementwise_grid(N), 256, 0, st, marker, f, N);
  cudaFreeAsync(buf, st);
  return s;
}

tt_cuda_status gwdt_dev(float *dist, ptrdiff_t *prev, const float *costs,
                        const int32_t *flats, const GridDims &g,
                        cudaStream_t st) {
  tt_cuda_status s = run_queue<GWDT>(dist, costs, flats, g, st);
  if ((s == TT_CUDA_SUCCESS || s == TT_CUDA_ERR_NOT_CONVERGED) && prev) {
    TT_LAUNCH(gwdt_prev_kernel, elementwise_grid(g.cells()), 256, 0, st, prev,
              dist, costs, flats, g.m, g.n);
    TT_CHECK(cudaGetLastError());
  }
  return s;
}

// ------------------------------------------------------------------
// Sink filling that allocates nothing (tt_cuda_fillsinks_noalloc_dev).
//
// For callers that cannot allocate device memory once they are running: a
// framework whose own pool already holds the device's memory, or a loop
// that must not pay for cudaMalloc/cudaFree (both can synchronise the whole
// device).  The only scratch of the fill -- the control block and one flag
// per 32 x 32 tile -- lives in the file-scope array below, sized for
// kNoAllocMaxTiles tiles; every device that loads this library holds it
// until the process exits.  All calls share it: each call clears what must
// start at zero, and calls that overlap on the GPU race on it.
// ------------------------------------------------------------------
constexpr int kNoAllocMaxTiles = 65536;  // e.g. 8192 x 8192 pixels
constexpr int kNoAllocHeaderWords = 64;  // control block, padded to 256 bytes
static __device__ __align__(256) int g_fill_scratch[kNoAllocHeaderWords + kNoAllocMaxTiles];

namespace {
void *g_fill_scratch_addr[64];  // device address of g_fill_scratch, per device
std::mutex g_fill_scratch_mu;

// Set-up, once per device, with that device current.
tt_cuda_status fill_scratch_address(void **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return TT_CUDA_ERR_CUDA;
  }
  if (dev < 0 || dev >= 64) return TT_CUDA_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(g_fill_scratch_mu);
  if (!g_fill_scratch_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_fill_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return TT_CUDA_ERR_CUDA;
    }
    g_fill_scratch_addr[dev] = p;
  }
  *out = g_fill_scratch_addr[dev];
  return TT_CUDA_SUCCESS;
}

tt_cuda_status fill_noalloc(float *f, const float *dem, const uint8_t *bc,
                            const GridDims &g, cudaStream_t st) {
  void *base = nullptr;
  tt_cuda_status s = fill_scratch_address(&base);
  if (s != TT_CUDA_SUCCESS) return s;
  QueueCtl *ctl = (QueueCtl *)base;
  int *dirty = (int *)base + kNoAllocHeaderWords;
  const int T = g.tiles();
  TT_LAUNCH(fill_init_kernel, elementwise_grid(g.cells()), 256, 0, st, f, dem, bc,
            g.cells());
  TT_CHECK(cudaMemsetAsync(ctl, 0, sizeof(QueueCtl), st));
  TT_LAUNCH(dirty_all_kernel, (T + 255) / 256, 256, 0, st, dirty, ctl, T);
  TT_CHECK(cudaGetLastError());
  RelaxArgs ra{f, dem, nullptr, g.m, g.n, g.tm, g.tn, ctl, dirty, 0};
  ra.max_visits = (unsigned long long)T *
                  (unsigned long long)std::min<int64_t>(max_rounds(), 1LL << 20);
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, relax_persistent_kernel<FILL>,
                                                kWarps * 32, 0);
  int grid = sm_count() * (b > 0 ? b : 1);
  grid = std::max(1, std::min(grid, (T + kWarps - 1) / kWarps));
  TT_LAUNCH(relax_persistent_kernel<FILL>, grid, kWarps * 32, 0, st, ra);
  TT_CHECK(cudaGetLastError());
  QueueCtl h;  // read back into host stack memory: no pinned allocation
  TT_CHECK(cudaMemcpyAsync(&h, ctl, sizeof(QueueCtl), cudaMemcpyDeviceToHost, st));
  TT_CHECK(cudaStreamSynchronize(st));
  set_last_rounds((int64_t)(h.visits / (unsigned long long)(T > 0 ? T : 1)));
  return h.abort ? TT_CUDA_ERR_NOT_CONVERGED : TT_CUDA_SUCCESS;
}
}  // namespace

}  // namespace tt

extern "C" tt_cuda_status tt_cuda_fillsinks_noalloc_dev(float *output,
                                                        const float *dem,
                                                        const uint8_t *bc,
                                                        const ptrdiff_t dims[2],
                                                        void *stream) {
  using namespace tt;
  tt_cuda_status s = TT_CUDA_SUCCESS;
  if (!output || !dem || !bc || !dims || dims[0] <= 0 || dims[1] <= 0 ||
      dims[0] >= (1LL << 31) || dims[1] >= (1LL << 31) ||
      dims[0] * dims[1] >= (1LL << 31)) {
    s = TT_CUDA_ERR_INVALID_ARGUMENT;
  } else {
    GridDims g = make_dims(dims);
    int ndev = 0;
    if (g.tiles() > kNoAllocMaxTiles) {
      s = TT_CUDA_ERR_INVALID_ARGUMENT;  // beyond the static scratch
    } else if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      s = TT_CUDA_ERR_NO_DEVICE;
    } else {
      DeviceLock lock;
      s = fill_noalloc(output, dem, bc, g, (cudaStream_t)stream);
      if (s == TT_CUDA_ERR_CUDA) cudaGetLastError();
    }
  }
  set_status(s);
  return s;
}
