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
// Scheduling: one persistent launch.  Every warp pops a tile from the queue
// (a ring buffer with monotone head/tail counters), relaxes it and pushes the
// neighbours it changed, so information crosses tile borders as soon as a
// tile finishes, with no host round trips.  A per-tile "queued" flag keeps a
// tile in the queue at most once; it is cleared when the tile is popped,
// before its halo is read, so later changes re-queue it.  A tile may then be
// relaxed by two warps at once: both results are valid upper bounds, and
// because the pointwise minimum of two fixpoints of either update is again a
// fixpoint, the atomic-minimum write keeps the result exact.  A pending
// counter (queued + running tiles) detects termination.  Every wait is
// bounded: a warp that spins too long, or a run that exceeds its visit
// budget, raises an abort flag and all warps return with an error status.
#include <algorithm>
#include <cmath>

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
};

// Queue control block (device memory, zero-initialised except `cap`).
struct QueueCtl {
  unsigned long long head;    // next slot to pop
  unsigned long long tail;    // next slot to push
  unsigned long long visits;  // tiles relaxed so far
  int pending;                // queued + running tiles
  int abort;                  // ABORT_* bits
};

enum : int { ABORT_SPIN = 1, ABORT_VISITS = 2 };

constexpr long long kSpinLimit = 1LL << 22;  // idle polls before giving up

struct RelaxArgs {
  float *state;
  const float *aux;
  const int32_t *flats;
  int64_t m, n;
  int tm, tn;
  QueueCtl *ctl;
  int *q;       // ring of tile ids, -1 = empty slot
  int *inq;     // per tile: 1 while queued
  unsigned long long cap;  // ring capacity (> number of tiles)
  unsigned long long max_visits;
};

__device__ __forceinline__ void q_push(const RelaxArgs &a, int t) {
  if (atomicExch(&a.inq[t], 1) != 0) return;  // already queued
  atomicAdd(&a.ctl->pending, 1);
  unsigned long long pos = atomicAdd(&a.ctl->tail, 1ULL);
  int *slot = &a.q[pos % a.cap];
  // The slot's previous entry has been claimed by a popper (at most `tiles`
  // entries are ever queued and cap exceeds that); wait until it took it.
  for (long long k = 0; atomicCAS(slot, -1, t) != -1; k++) {
    if (k > kSpinLimit) {
      atomicOr(&a.ctl->abort, ABORT_SPIN);
      return;
    }
    __nanosleep(64);
  }
}

__device__ __forceinline__ void push_tile(const RelaxArgs &a, int ti, int tj) {
  if (ti < 0 || tj < 0 || ti >= a.tm || tj >= a.tn) return;
  q_push(a, tj * a.tm + ti);
}

// Claims the next queued tile, or returns -1 when the queue is empty.
__device__ __forceinline__ int q_pop(const RelaxArgs &a) {
  volatile unsigned long long *vh = &a.ctl->head;
  volatile unsigned long long *vt = &a.ctl->tail;
  unsigned long long h = *vh;
  for (;;) {
    if (h >= *vt) return -1;
    unsigned long long old = atomicCAS(&a.ctl->head, h, h + 1);
    if (old == h) break;
    h = old;
  }
  int *slot = &a.q[h % a.cap];
  int v;
  for (long long k = 0; (v = atomicExch(slot, -1)) < 0; k++) {
    if (k > kSpinLimit) {
      atomicOr(&a.ctl->abort, ABORT_SPIN);
      return -1;
    }
    __nanosleep(32);
  }
  return v;
}

// Float minimum through integer atomics (values are never NaN here).
__device__ __forceinline__ void atomic_min_float(float *addr, float v) {
  if (!signbit(v))
    atomicMin((int *)addr, __float_as_int(v));
  else
    atomicMax((unsigned int *)addr, __float_as_uint(v));
}

template <int KIND>
__device__ __forceinline__ float relax_one(const WarpTile &t, int c, int r,
                                           int c0, int r0, int c1, int r1,
                                           int c2, int r2, float cur) {
  if (KIND == FILL) {
    float lo = fminf(fminf(fminf(cur, t.s[c0][r0]), t.s[c1][r1]), t.s[c2][r2]);
    float z = t.a[c][r];
    return (lo > z) ? lo : z;
  } else {
    if (!((t.flat[c] >> r) & 1)) return cur;
    float cs = t.a[c][r];
    float best = cur;
    const int cc[3] = {c0, c1, c2}, rr[3] = {r0, r1, r2};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      if (!((t.flat[cc[k]] >> rr[k]) & 1)) continue;
      float ch = (cc[k] != c && rr[k] != r) ? kSqrt2 : 1.0f;
      float w = __fmul_rn(__fmul_rn(ch, __fadd_rn(cs, t.a[cc[k]][rr[k]])), 0.5f);
      float prop = __fadd_rn(t.s[cc[k]][rr[k]], w);
      if (prop < best) best = prop;
    }
    return best;
  }
}

// Sweep along r (lane = column).  dir = +1 down, -1 up.
template <int KIND>
__device__ bool sweep_rows(WarpTile &t, int lane, int dir) {
  const int c = lane + 1;
  bool changed = false;
  uint32_t dmask = 0;
  for (int s = 0; s < kTile; s++) {
    int r = dir > 0 ? 1 + s : kTile - s;
    int rp = r - dir;
    float cur = t.s[c][r];
    float nv = relax_one<KIND>(t, c, r, c - 1, rp, c, rp, c + 1, rp, cur);
    if (nv < cur) {
      t.s[c][r] = nv;
      dmask |= 1u << (r - 1);
      changed = true;
    }
    __syncwarp();
  }
  t.dirty[c] |= dmask;
  __syncwarp();
  return __any_sync(0xffffffffu, changed);
}

// Sweep along c (lane = row).  dir = +1 right, -1 left.
template <int KIND>
__device__ bool sweep_cols(WarpTile &t, int lane, int dir) {
  const int r = lane + 1;
  bool any = false;
  for (int s = 0; s < kTile; s++) {
    int c = dir > 0 ? 1 + s : kTile - s;
    int cp = c - dir;
    float cur = t.s[c][r];
    float nv = relax_one<KIND>(t, c, r, cp, r - 1, cp, r, cp, r + 1, cur);
    bool ch = nv < cur;
    if (ch) t.s[c][r] = nv;
    unsigned b = __ballot_sync(0xffffffffu, ch);
    if (b) {
      any = true;
      if (lane == 0) t.dirty[c] |= b;
    }
    __syncwarp();
  }
  return any;
}

template <int KIND>
__global__ void __launch_bounds__(kWarps * 32)
relax_persistent_kernel(RelaxArgs a) {
  __shared__ WarpTile tiles[kWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpTile &t = tiles[warp];
  long long idle = 0;
  for (;;) {
    int tile = -1, stop = 0;
    if (lane == 0) {
      if (*(volatile int *)&a.ctl->abort) {
        stop = 1;
      } else {
        tile = q_pop(a);
        if (tile < 0) {
          if (*(volatile int *)&a.ctl->pending == 0) {
            stop = 1;
          } else if (++idle > kSpinLimit) {
            atomicOr(&a.ctl->abort, ABORT_SPIN);
            stop = 1;
          } else {
            __nanosleep(idle < 64 ? 100 : 1000);
          }
        } else {
          idle = 0;
          atomicExch(&a.inq[tile], 0);  // later changes re-queue this tile
          if (atomicAdd(&a.ctl->visits, 1ULL) >= a.max_visits)
            atomicOr(&a.ctl->abort, ABORT_VISITS);
          __threadfence();
        }
      }
    }
    stop = __shfl_sync(0xffffffffu, stop, 0);
    if (stop) break;
    tile = __shfl_sync(0xffffffffu, tile, 0);
    if (tile < 0) continue;
    const int ti = tile % a.tm, tj = tile / a.tm;
    const int64_t i0 = (int64_t)ti * kTile, j0 = (int64_t)tj * kTile;

    // Stage tile + halo.  Lane r loads row r (and lanes 0,1 rows 32,33).
    for (int c = 0; c < kHalo; c++) {
      int64_t j = j0 - 1 + c;
      bool jok = j >= 0 && j < a.n;
      uint32_t flo = 0, fhi = 0;
      for (int half = 0; half < 2; half++) {
        int r = lane + half * 32;
        bool act = r < kHalo;
        int64_t i = i0 - 1 + r;
        bool ok = act && jok && i >= 0 && i < a.m;
        float sv = INFINITY, av = (KIND == FILL) ? INFINITY : 0.0f;
        bool fl = false;
        if (ok) {
          int64_t p = j * a.m + i;
          sv = __ldcg(&a.state[p]);  // L2: other SMs update it concurrently
          av = a.aux[p];
          if (KIND == GWDT) fl = (a.flats[p] & 1) != 0;
        }
        if (act) {
          t.s[c][r] = sv;
          t.a[c][r] = av;
        }
        if (KIND == GWDT) {
          unsigned b = __ballot_sync(0xffffffffu, fl);
          if (half == 0) flo = b; else fhi = b;
        }
      }
      if (lane == 0) {
        t.dirty[c] = 0;
        if (KIND == GWDT) t.flat[c] = (uint64_t)flo | ((uint64_t)(fhi & 3u) << 32);
      }
    }
    __syncwarp();

    int quiet = 0, sweeps = 0, k = 0;
    while (quiet < 4 && sweeps < kMaxSweeps) {
      bool ch;
      switch (k) {
        case 0: ch = sweep_rows<KIND>(t, lane, +1); break;
        case 1: ch = sweep_rows<KIND>(t, lane, -1); break;
        case 2: ch = sweep_cols<KIND>(t, lane, +1); break;
        default: ch = sweep_cols<KIND>(t, lane, -1); break;
      }
      quiet = ch ? 0 : quiet + 1;
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
        if (j < a.n && i < a.m) atomic_min_float(&a.state[j * a.m + i], t.s[c][lane + 1]);
      }
      top |= dm & 1u;
      bottom |= (dm >> 31) & 1u;
    }
    __threadfence();  // publish this lane's writes before any push below
    __syncwarp();
    if (lane == 0) {
      uint32_t left = t.dirty[1], right = t.dirty[kTile];
      if (top) push_tile(a, ti - 1, tj);
      if (bottom) push_tile(a, ti + 1, tj);
      if (left) push_tile(a, ti, tj - 1);
      if (right) push_tile(a, ti, tj + 1);
      if (left & 1u) push_tile(a, ti - 1, tj - 1);
      if ((left >> 31) & 1u) push_tile(a, ti + 1, tj - 1);
      if (right & 1u) push_tile(a, ti - 1, tj + 1);
      if ((right >> 31) & 1u) push_tile(a, ti + 1, tj + 1);
      if (quiet < 4) push_tile(a, ti, tj);  // capped: come back later
      __threadfence();
      atomicSub(&a.ctl->pending, 1);
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

// Queue every tile (fill starts everywhere).
__global__ void queue_all_kernel(int *q, int *inq, QueueCtl *ctl, int n,
                                 unsigned long long cap) {
  for (unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
       t < cap; t += (unsigned long long)gridDim.x * blockDim.x) {
    q[t] = t < (unsigned long long)n ? (int)t : -1;
    if (t < (unsigned long long)n) inq[t] = 1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->tail = n;
    ctl->pending = n;
  }
}

__global__ void queue_clear_kernel(int *q, int *inq, int n, unsigned long long cap) {
  for (unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
       t < cap; t += (unsigned long long)gridDim.x * blockDim.x) {
    q[t] = -1;
    if (t < (unsigned long long)n) inq[t] = 0;
  }
}

// dist = 1 at presills, +INF at other flats, 0 elsewhere; enqueue every tile
// whose pixels or halo contain a presill.
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
        for (int ti = ti0; ti <= ti1; ti++) q_push(qa, tj * qa.tm + ti);
    }
  }
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

// Host driver: set up the queue, run one persistent launch, read the status.
template <int KIND>
tt_cuda_status run_queue(float *state, const float *aux, const int32_t *flats,
                         const GridDims &g, cudaStream_t st) {
  const int T = g.tiles();
  const unsigned long long cap = 2ULL * (unsigned long long)T + 64;
  Workspace &ws = workspace();
  size_t need = align_up(sizeof(QueueCtl)) + align_up(cap * 4) + align_up((size_t)T * 4);
  if (!ws.reserve(need)) return TT_CUDA_ERR_ALLOC;
  QueueCtl *ctl = (QueueCtl *)ws.take(sizeof(QueueCtl));
  int *q = (int *)ws.take(cap * 4);
  int *inq = (int *)ws.take((size_t)T * 4);
  QueueCtl *hctl = (QueueCtl *)pinned_scratch();
  if (!hctl) return TT_CUDA_ERR_ALLOC;

  RelaxArgs ra{state, aux, flats, g.m, g.n, g.tm, g.tn, ctl, q, inq, cap, 0};
  const int64_t cap_rounds = max_rounds();
  ra.max_visits = (unsigned long long)T * (unsigned long long)std::min<int64_t>(cap_rounds, 1LL << 20);
  TT_CHECK(cudaMemsetAsync(ctl, 0, sizeof(QueueCtl), st));
  const int qgrid = (int)std::min<unsigned long long>((cap + 255) / 256, (unsigned long long)sm_count() * 16);
  if (KIND == FILL) {
    TT_LAUNCH(queue_all_kernel, qgrid, 256, 0, st, q, inq, ctl, T, cap);
  } else {
    TT_LAUNCH(queue_clear_kernel, qgrid, 256, 0, st, q, inq, T, cap);
    TT_LAUNCH(gwdt_init_kernel, elementwise_grid(g.cells()), 256, 0, st, state, flats,
              g.m, g.n, ra);
  }
  TT_CHECK(cudaGetLastError());
  static int blocks_per_sm[2] = {0, 0};
  if (!blocks_per_sm[KIND]) {
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, relax_persistent_kernel<KIND>,
                                                  kWarps * 32, 0);
    blocks_per_sm[KIND] = b > 0 ? b : 1;
  }
  const int grid = sm_count() * blocks_per_sm[KIND];
  TT_LAUNCH(relax_persistent_kernel<KIND>, grid, kWarps * 32, 0, st, ra);
  TT_CHECK(cudaGetLastError());
  TT_CHECK(cudaMemcpyAsync(hctl, ctl, sizeof(QueueCtl), cudaMemcpyDeviceToHost, st));
  TT_CHECK(cudaStreamSynchronize(st));
  // Report tile visits per tile as "rounds" (comparable to a sweep count).
  set_last_rounds((int64_t)(hctl->visits / (unsigned long long)(T > 0 ? T : 1)));
  if (hctl->abort & ABORT_VISITS) return TT_CUDA_ERR_NOT_CONVERGED;
  if (hctl->abort & ABORT_SPIN) return TT_CUDA_ERR_NOT_CONVERGED;
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

}  // namespace tt
