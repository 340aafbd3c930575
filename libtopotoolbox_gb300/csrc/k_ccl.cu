// gwdt_computecosts (src/gwdt.c:167-278) on the GPU.
//
// Flat pixels are labelled into 8-connected components with a lock-free
// union-find: every label points at a smaller or equal linear index, and a
// union links the larger root under the smaller one with atomicMin, retrying
// when another thread relinked it first.  The maximum depth
// (filled - original) of each component is an order-independent maximum,
// taken with atomicMax on an order-preserving integer image of the float, so
// the costs
//
//     cost = (float)((double)(float)(maxdepth - depth) + 0.1)
//
// are bit-identical to the reference (the difference is taken in float and
// the 0.1 offset added in double, src/gwdt.c:247-277).  The label stored in
// `conncomps` is the smallest linear index among the component's pixels of
// maximal depth; the reference picks one of those pixels by its scan-order
// union-find (src/gwdt.c:141-153), which can differ when depths tie.
#include <algorithm>
#include <climits>

#include "tt_internal.cuh"

namespace tt {
namespace {

__device__ __forceinline__ int ordered_key(float x) {
  int b = __float_as_int(x);
  return b >= 0 ? b : b ^ 0x7fffffff;
}
__device__ __forceinline__ float key_to_float(int k) {
  return __int_as_float(k >= 0 ? k : k ^ 0x7fffffff);
}

__device__ __forceinline__ int uf_find(const int *L, int x) {
  int y = ((volatile const int *)L)[x];
  while (y != x) {
    x = y;
    y = ((volatile const int *)L)[x];
  }
  return x;
}

__device__ void uf_union(int *L, int a, int b) {
  for (int it = 0; it < (1 << 30); it++) {
    a = uf_find(L, a);
    b = uf_find(L, b);
    if (a == b) return;
    if (a < b) {
      int old = atomicMin(&L[b], a);
      if (old == b) return;
      b = old;
    } else {
      int old = atomicMin(&L[a], b);
      if (old == a) return;
      a = old;
    }
  }
}

// Tile-local labelling: one warp per 32 x 32 tile runs the union-find in
// shared memory over the tile's internal edges, then writes for every flat
// pixel the global index of its tile-local root (the smallest index of its
// tile-local component).  Roots get their max-depth and argmax slots reset.
constexpr int kCclWarps = 4;

__device__ __forceinline__ int sfind(const int *lab, int x) {
  int y = ((volatile const int *)lab)[x];
  while (y != x) {
    x = y;
    y = ((volatile const int *)lab)[x];
  }
  return x;
}

__device__ void sunion(int *lab, int a, int b) {
  for (int it = 0; it < 4096; it++) {
    a = sfind(lab, a);
    b = sfind(lab, b);
    if (a == b) return;
    if (a < b) {
      int old = atomicMin(&lab[b], a);
      if (old == b) return;
      b = old;
    } else {
      int old = atomicMin(&lab[a], b);
      if (old == a) return;
      a = old;
    }
  }
}

__global__ void __launch_bounds__(kCclWarps * 32)
ccl_tile_kernel(int *__restrict__ L, int *__restrict__ maxkey,
                int *__restrict__ argmax, const int32_t *__restrict__ flats,
                int64_t m, int64_t n, int tm, int tn) {
  __shared__ int lab[kCclWarps][kTile * kTile];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int *lb = lab[warp];
  const int T = tm * tn;
  for (int tile = blockIdx.x * kCclWarps + warp; tile < T; tile += gridDim.x * kCclWarps) {
    const int ti = tile % tm, tj = tile / tm;
    const int64_t i0 = (int64_t)ti * kTile, j0 = (int64_t)tj * kTile;
    const int ii = lane;
    const int64_t i = i0 + ii;
    for (int jj = 0; jj < kTile; jj++) {
      const int64_t j = j0 + jj;
      bool f = i < m && j < n && (flats[j * m + i] & 1);
      lb[jj * kTile + ii] = f ? jj * kTile + ii : -1;
    }
    __syncwarp();
    // internal edges to the earlier neighbours (i-1,j), (i-1,j-1), (i,j-1), (i+1,j-1)
    for (int jj = 0; jj < kTile; jj++) {
      const int loc = jj * kTile + ii;
      if (lb[loc] < 0) continue;
      const int di[4] = {-1, -1, 0, 1};
      const int dj[4] = {0, -1, -1, -1};
#pragma unroll
      for (int k = 0; k < 4; k++) {
        int qi = ii + di[k], qj = jj + dj[k];
        if (qi < 0 || qi >= kTile || qj < 0) continue;
        int q = qj * kTile + qi;
        if (((volatile int *)lb)[q] >= 0) sunion(lb, loc, q);
      }
    }
    __syncwarp();
    for (int jj = 0; jj < kTile; jj++) {
      const int64_t j = j0 + jj;
      if (i >= m || j >= n) continue;
      const int loc = jj * kTile + ii;
      int v = -1;
      if (lb[loc] >= 0) {
        int r = sfind(lb, loc);
        v = (int)((j0 + r / kTile) * m + (i0 + r % kTile));
        if (r == loc) {
          maxkey[j * m + i] = INT_MIN;
          argmax[j * m + i] = INT_MAX;
        }
      }
      L[j * m + i] = v;
    }
    __syncwarp();
  }
}

// Edges that cross tile borders: from the last row, the last column and the
// first column of every tile to the neighbours (i+1,j), (i,j+1), (i+1,j+1),
// (i+1,j-1) lying in another tile.
__global__ void ccl_border_kernel(int *__restrict__ L,
                                  const int32_t *__restrict__ flats, int64_t m,
                                  int64_t n, int tm, int tn) {
  const int T = tm * tn;
  // 32 last-row + 32 last-column + 32 first-column candidates per tile
  const int64_t total = (int64_t)T * 96;
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < total;
       w += (int64_t)gridDim.x * blockDim.x) {
    const int tile = (int)(w / 96), k = (int)(w % 96);
    const int ti = tile % tm, tj = tile / tm;
    int ii, jj;
    if (k < 32) { ii = kTile - 1; jj = k; }
    else if (k < 64) { ii = k - 32; jj = kTile - 1; }
    else { ii = k - 64; jj = 0; }
    const int64_t i = (int64_t)ti * kTile + ii, j = (int64_t)tj * kTile + jj;
    if (i >= m || j >= n) continue;
    const int64_t p = j * m + i;
    if (!(flats[p] & 1)) continue;
    const int di[4] = {1, 0, 1, 1};
    const int dj[4] = {0, 1, 1, -1};
#pragma unroll
    for (int e = 0; e < 4; e++) {
      int64_t qi = i + di[e], qj = j + dj[e];
      if (qi >= m || qj < 0 || qj >= n) continue;
      if (qi / kTile == ti && qj / kTile == tj) continue;  // internal edge
      int64_t q = qj * m + qi;
      if (flats[q] & 1) uf_union(L, (int)p, (int)q);
    }
  }
}

__global__ void ccl_max_kernel(int *__restrict__ L, int *__restrict__ maxkey,
                               const int32_t *__restrict__ flats,
                               const float *__restrict__ orig,
                               const float *__restrict__ filled, int64_t N) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    if (!(flats[p] & 1)) continue;
    int r = uf_find(L, (int)p);
    L[p] = r;
    float depth = __fsub_rn(filled[p], orig[p]);
    if (!isnan(depth)) atomicMax(&maxkey[r], ordered_key(depth));
  }
}

__global__ void ccl_argmax_kernel(const int *__restrict__ L,
                                  const int *__restrict__ maxkey,
                                  int *__restrict__ argmax,
                                  const int32_t *__restrict__ flats,
                                  const float *__restrict__ orig,
                                  const float *__restrict__ filled, int64_t N) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    if (!(flats[p] & 1)) continue;
    int r = L[p];
    float depth = __fsub_rn(filled[p], orig[p]);
    if (!isnan(depth) && ordered_key(depth) == maxkey[r]) atomicMin(&argmax[r], (int)p);
  }
}

__global__ void costs_kernel(float *__restrict__ costs,
                             ptrdiff_t *__restrict__ conncomps,
                             const int *__restrict__ L,
                             const int *__restrict__ maxkey,
                             const int *__restrict__ argmax,
                             const int32_t *__restrict__ flats,
                             const float *__restrict__ orig,
                             const float *__restrict__ filled, int64_t N) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    float c = 0.0f;
    ptrdiff_t lab = 0;
    if (flats[p] & 1) {
      int r = L[p];
      float maxd = key_to_float(maxkey[r]);
      float depth = __fsub_rn(filled[p], orig[p]);
      float diff = __fsub_rn(maxd, depth);
      c = __double2float_rn(__dadd_rn((double)diff, 0.1));
      int a = argmax[r];
      lab = (a == INT_MAX) ? r : a;
    }
    costs[p] = c;
    conncomps[p] = lab;
  }
}

int ew_grid(int64_t N) {
  int64_t b = (N + 255) / 256;
  int64_t cap = (int64_t)sm_count() * 16;
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}

}  // namespace

tt_cuda_status costs_dev(float *costs, ptrdiff_t *conncomps,
                         const int32_t *flats, const float *orig,
                         const float *filled, const GridDims &g,
                         cudaStream_t st) {
  const int64_t N = g.cells();
  Workspace &ws = workspace();
  if (!ws.reserve(3 * align_up((size_t)N * 4))) return TT_CUDA_ERR_ALLOC;
  int *L = (int *)ws.take((size_t)N * 4);
  int *maxkey = (int *)ws.take((size_t)N * 4);
  int *argmax = (int *)ws.take((size_t)N * 4);
  const int grid = ew_grid(N);
  const int T = g.tiles();
  const int tgrid = (int)std::min<int64_t>((T + kCclWarps - 1) / kCclWarps,
                                           (int64_t)sm_count() * 16);
  TT_LAUNCH(ccl_tile_kernel, tgrid, kCclWarps * 32, 0, st, L, maxkey, argmax, flats,
            g.m, g.n, g.tm, g.tn);
  TT_LAUNCH(ccl_border_kernel, ew_grid((int64_t)T * 96), 256, 0, st, L, flats, g.m,
            g.n, g.tm, g.tn);
  TT_LAUNCH(ccl_max_kernel, grid, 256, 0, st, L, maxkey, flats, orig, filled, N);
  TT_LAUNCH(ccl_argmax_kernel, grid, 256, 0, st, L, maxkey, argmax, flats, orig, filled, N);
  TT_LAUNCH(costs_kernel, grid, 256, 0, st, costs, conncomps, L, maxkey, argmax,
            flats, orig, filled, N);
  TT_CHECK(cudaGetLastError());
  return TT_CUDA_SUCCESS;
}

}  // namespace tt
