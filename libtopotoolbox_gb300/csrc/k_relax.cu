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
// back; a changed edge or corner enqueues the neighbouring tile for the next
// round.  The host launches rounds until the queue is empty.
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

struct RelaxArgs {
  float *state;
  const float *aux;
  const int32_t *flats;
  int64_t m, n;
  int tm, tn;
  const int *list_in;
  const int *count_in;
  int *list_out;
  int *count_out;
  int *mark;
  int round;
};

__device__ __forceinline__ void push_tile(const RelaxArgs &a, int ti, int tj) {
  if (ti < 0 || tj < 0 || ti >= a.tm || tj >= a.tn) return;
  int t = tj * a.tm + ti;
  int next = a.round + 1;
  if (atomicMax(&a.mark[t], next) < next) {
    int slot = atomicAdd(a.count_out, 1);
    a.list_out[slot] = t;
  }
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
relax_round_kernel(RelaxArgs a) {
  __shared__ WarpTile tiles[kWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpTile &t = tiles[warp];
  const int count = *(volatile const int *)a.count_in;
  for (int w = blockIdx.x * kWarps + warp; w < count; w += gridDim.x * kWarps) {
    const int tile = a.list_in[w];
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
          sv = a.state[p];
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
        if (j < a.n && i < a.m) a.state[j * a.m + i] = t.s[c][lane + 1];
      }
      top |= dm & 1u;
      bottom |= (dm >> 31) & 1u;
    }
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
      if (quiet < 4) push_tile(a, ti, tj);  // capped: come back next round
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

__global__ void iota_kernel(int *list, int *mark, int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    list[t] = t;
    mark[t] = 1;
  }
}

// dist = 1 at presills, +INF at other flats, 0 elsewhere; enqueue every tile
// whose pixels or halo contain a presill.
__global__ void gwdt_init_kernel(float *__restrict__ dist,
                                 const int32_t *__restrict__ flats, int64_t m,
                                 int64_t n, int tm, int tn, int *list, int *count,
                                 int *mark) {
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
          int t = tj * tm + ti;
          if (atomicMax(&mark[t], 1) < 1) list[atomicAdd(count, 1)] = t;
        }
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

// Host driver of the round loop.  `init` fills the initial list.
template <int KIND>
tt_cuda_status run_rounds(float *state, const float *aux, const int32_t *flats,
                          const GridDims &g, cudaStream_t st) {
  const int T = g.tiles();
  Workspace &ws = workspace();
  size_t need = 3 * align_up((size_t)T * 4) + 256 * 2;
  if (!ws.reserve(need)) return TT_CUDA_ERR_ALLOC;
  int *lists[2] = {(int *)ws.take((size_t)T * 4), (int *)ws.take((size_t)T * 4)};
  int *mark = (int *)ws.take((size_t)T * 4);
  int *counts = (int *)ws.take(256);
  int *hcount = (int *)pinned_scratch();
  if (!hcount) return TT_CUDA_ERR_ALLOC;

  TT_CHECK(cudaMemsetAsync(mark, 0, (size_t)T * 4, st));
  TT_CHECK(cudaMemsetAsync(counts, 0, 2 * sizeof(int) * 2, st));
  if (KIND == FILL) {
    TT_LAUNCH(iota_kernel, (T + 255) / 256, 256, 0, st, lists[1], mark, T);
    TT_CHECK(cudaMemcpyAsync(counts + 1, &T, sizeof(int), cudaMemcpyHostToDevice, st));
    TT_CHECK(cudaStreamSynchronize(st));  // T lives on the host stack
  } else {
    TT_LAUNCH(gwdt_init_kernel, elementwise_grid(g.cells()), 256, 0, st, state,
              flats, g.m, g.n, g.tm, g.tn, lists[1], counts + 1, mark);
  }
  TT_CHECK(cudaGetLastError());

  const int grid = sm_count() * 8;
  const int64_t cap = max_rounds();
  int64_t round = 1;  // the initial list is round 1, stored in slot 1
  const int batch = 8;
  for (;;) {
    const int nb = (int)std::min<int64_t>(batch, cap - round + 1);
    if (nb <= 0) {
      set_last_rounds(round - 1);
      return TT_CUDA_ERR_NOT_CONVERGED;
    }
    for (int b = 0; b < nb; b++) {
      int in = (int)(round & 1), out = (int)((round + 1) & 1);
      TT_CHECK(cudaMemsetAsync(counts + out, 0, sizeof(int), st));
      RelaxArgs ra{state, aux, flats, g.m, g.n, g.tm, g.tn, lists[in],
                   counts + in, lists[out], counts + out, mark, (int)round};
      TT_LAUNCH(relax_round_kernel<KIND>, grid, kWarps * 32, 0, st, ra);
      round++;
    }
    TT_CHECK(cudaGetLastError());
    TT_CHECK(cudaMemcpyAsync(hcount, counts + (round & 1), sizeof(int),
                             cudaMemcpyDeviceToHost, st));
    TT_CHECK(cudaStreamSynchronize(st));
    if (*hcount == 0) break;
  }
  set_last_rounds(round - 1);
  return TT_CUDA_SUCCESS;
}

}  // namespace

tt_cuda_status fill_dev(float *f, const float *dem, const uint8_t *bc,
                        const GridDims &g, cudaStream_t st) {
  TT_LAUNCH(fill_init_kernel, elementwise_grid(g.cells()), 256, 0, st, f, dem,
            bc, g.cells());
  TT_CHECK(cudaGetLastError());
  return run_rounds<FILL>(f, dem, nullptr, g, st);
}

tt_cuda_status reconstruct_dev(float *marker, const float *mask,
                               const GridDims &g, cudaStream_t st) {
  // The negated copies live in the io-independent scratch of this call.
  const int64_t N = g.cells();
  float *buf = nullptr;
  TT_CHECK(cudaMallocAsync((void **)&buf, (size_t)N * 8, st));
  float *f = buf, *z = buf + N;
  TT_LAUNCH(negate_pair_kernel, elementwise_grid(N), 256, 0, st, f, z, marker, mask, N);
  tt_cuda_status s = run_rounds<FILL>(f, z, nullptr, g, st);
  if (s == TT_CUDA_SUCCESS || s == TT_CUDA_ERR_NOT_CONVERGED)
    TT_LAUNCH(negate_kernel, elementwise_grid(N), 256, 0, st, marker, f, N);
  cudaFreeAsync(buf, st);
  return s;
}

tt_cuda_status gwdt_dev(float *dist, ptrdiff_t *prev, const float *costs,
                        const int32_t *flats, const GridDims &g,
                        cudaStream_t st) {
  tt_cuda_status s = run_rounds<GWDT>(dist, costs, flats, g, st);
  if ((s == TT_CUDA_SUCCESS || s == TT_CUDA_ERR_NOT_CONVERGED) && prev) {
    TT_LAUNCH(gwdt_prev_kernel, elementwise_grid(g.cells()), 256, 0, st, prev,
              dist, costs, flats, g.m, g.n);
    TT_CHECK(cudaGetLastError());
  }
  return s;
}

}  // namespace tt
