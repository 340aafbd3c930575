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

__global__ void ccl_init_kernel(int *__restrict__ L, int *__restrict__ maxkey,
                                int *__restrict__ argmax,
                                const int32_t *__restrict__ flats, int64_t N) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    bool f = flats[p] & 1;
    L[p] = f ? (int)p : -1;
    if (f) {
      maxkey[p] = INT_MIN;
      argmax[p] = INT_MAX;
    }
  }
}

__global__ void ccl_merge_kernel(int *__restrict__ L,
                                 const int32_t *__restrict__ flats, int64_t m,
                                 int64_t n) {
  const int64_t N = m * n;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    if (!(flats[p] & 1)) continue;
    int64_t i = p % m, j = p / m;
    // Every 8-connected edge once: the four neighbours earlier in scan order.
    const int di[4] = {-1, -1, 0, 1};
    const int dj[4] = {0, -1, -1, -1};
#pragma unroll
    for (int k = 0; k < 4; k++) {
      int64_t ni = i + di[k], nj = j + dj[k];
      if (ni < 0 || ni >= m || nj < 0) continue;
      int64_t q = nj * m + ni;
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
  TT_LAUNCH(ccl_init_kernel, grid, 256, 0, st, L, maxkey, argmax, flats, N);
  TT_LAUNCH(ccl_merge_kernel, grid, 256, 0, st, L, flats, g.m, g.n);
  TT_LAUNCH(ccl_max_kernel, grid, 256, 0, st, L, maxkey, flats, orig, filled, N);
  TT_LAUNCH(ccl_argmax_kernel, grid, 256, 0, st, L, maxkey, argmax, flats, orig, filled, N);
  TT_LAUNCH(costs_kernel, grid, 256, 0, st, costs, conncomps, L, maxkey, argmax,
            flats, orig, filled, N);
  TT_CHECK(cudaGetLastError());
  return TT_CUDA_SUCCESS;
}

}  // namespace tt
