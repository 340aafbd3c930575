// Edge-list forms of the D8 forest, the callers of the path's outputs:
//
//  * flow_routing_d8_edgelist (src/flow_routing.c:258-312): one edge
//    (u, receiver(u)) per pixel u with a direction, listed in `node` order.
//    An order-preserving compaction: per-block counts, one scan, scatter.
//  * flow_accumulation_edgelist (src/flow_accumulation.c:10-30) on an edge
//    list of a D8 forest with unit fractions, listed in topological order:
//    the edges are turned back into a direction grid and summed by the exact
//    forest contraction.  Every other list (fractions, several edges out of a
//    pixel, non-neighbours, any order) takes the general sweep of
//    k_edgeflow.cu.
//  * drainagebasins (src/drainagebasins.c:6-27): the reference labels basins
//    in a reverse sweep over a topologically ordered edge list (every edge
//    out of a pixel is listed after every edge into it).  Running backwards,
//    the sweep therefore meets each basin first at the basin's last-listed
//    edge, whose target is the basin's root, and numbers basins in
//    decreasing order of that edge's index.  Here: each pixel's parent is the
//    target of its first-listed out-edge (the one the backward sweep applies
//    last), roots come from pointer jumping, a basin's key is its largest
//    edge index (distinct per basin), and its label is 1 + the number of
//    basins with a larger key (a scan over marked edge indices, no sort).
//    The labels equal the reference's on the same list.
//  * edgelist_degree (src/streamquad.c:209-224): atomic in/out-degree
//    counters wrapped to uint8 as the reference's counters wrap.
#include <algorithm>
#include <climits>

#include "tt_internal.cuh"

namespace tt {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanPer = 8;                         // elements per thread
constexpr int kScanBlock = kScanThreads * kScanPer;  // 2048 per block

// Exclusive scan of one int per thread over the block; returns the block
// total through *total.
__device__ int block_exclusive_scan(int v, int *total) {
  __shared__ int warp_sums[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < kScanThreads / 32) warp_sums[lane] = wi - w;  // exclusive
    if (lane == kScanThreads / 32 - 1) *total = wi;
  }
  __syncthreads();
  const int r = warp_sums[warp] + incl - v;
  __syncthreads();
  return r;
}

// Exclusive scan of the per-block counts by one block; off[nb] = total.
__global__ void scan_blocks_kernel(const int *__restrict__ cnt, int *__restrict__ off, int nb) {
  __shared__ int total;
  int carry = 0;
  for (int base = 0; base < nb; base += kScanThreads) {
    const int k = base + threadIdx.x;
    const int v = k < nb ? cnt[k] : 0;
    const int ex = block_exclusive_scan(v, &total);
    if (k < nb) off[k] = carry + ex;
    __syncthreads();
    carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) off[nb] = carry;
}

// ---- flow_routing_d8_edgelist -------------------------------------------

struct EdgeArgs {
  const ptrdiff_t *node;
  const uint8_t *dir;
  int64_t N;
  ptrdiff_t off[8];  // linear offset of direction bit r (memory order)
};

__device__ __forceinline__ int edge_flags(const EdgeArgs &a, int64_t k0, ptrdiff_t *u) {
  int f = 0;
#pragma unroll
  for (int s = 0; s < kScanPer; s++) {
    const int64_t k = k0 + s;
    u[s] = k < a.N ? a.node[k] : 0;
  }
#pragma unroll
  for (int s = 0; s < kScanPer; s++)
    if (k0 + s < a.N && a.dir[u[s]] != 0) f |= 1 << s;
  return f;
}

__global__ void edge_count_kernel(EdgeArgs a, int *__restrict__ cnt) {
  __shared__ int total;
  const int64_t k0 = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanPer;
  ptrdiff_t u[kScanPer];
  const int f = edge_flags(a, k0, u);
  block_exclusive_scan(__popc(f), &total);
  if (threadIdx.x == 0) cnt[blockIdx.x] = total;
}

__global__ void edge_scatter_kernel(EdgeArgs a, const int *__restrict__ off,
                                    ptrdiff_t *__restrict__ source,
                                    ptrdiff_t *__restrict__ target) {
  __shared__ int total;
  const int64_t k0 = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanPer;
  ptrdiff_t u[kScanPer];
  const int f = edge_flags(a, k0, u);
  int pos = off[blockIdx.x] + block_exclusive_scan(__popc(f), &total);
#pragma unroll
  for (int s = 0; s < kScanPer; s++) {
    if (!((f >> s) & 1)) continue;
    const unsigned d = a.dir[u[s]];
    source[pos] = u[s];
    target[pos] = u[s] + a.off[31 - __clz(d)];
    pos++;
  }
}

// ---- flow_accumulation_edgelist -------------------------------------------

enum : int {
  EL_BAD_INDEX = 1,
  EL_NOT_NEIGHBOUR = 2,
  EL_DUPLICATE = 4,
  EL_FRACTION = 8,
  EL_CYCLE = 16,  // a pointer-jumping fixpoint that still has an out-edge
  EL_ORDER = 32   // an edge into a pixel listed after the pixel's out-edge
};

// Direction bit of each source from its edge (bit k of the column-major
// convention of flow_accumulation: (i + di[k], j + dj[k])).
__global__ void edges_to_dir_kernel(const ptrdiff_t *__restrict__ source,
                                    const ptrdiff_t *__restrict__ target,
                                    const float *__restrict__ fraction, int64_t E,
                                    int64_t m, int64_t n, uint8_t *__restrict__ dir,
                                    int *__restrict__ seen, int *__restrict__ maxin,
                                    int *__restrict__ err) {
  const int64_t N = m * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = source[e], v = target[e];
    if (u < 0 || u >= N || v < 0 || v >= N) {
      atomicOr(err, EL_BAD_INDEX);
      continue;
    }
    atomicMax(&maxin[v], (int)e);
    if (fraction[e] != 1.0f) atomicOr(err, EL_FRACTION);
    const int64_t i = u % m, j = u / m, vi = v % m, vj = v / m;
    const int64_t di = vi - i, dj = vj - j;
    int k = -1;
#pragma unroll
    for (int b = 0; b < 8; b++)
      if (d8_di(b, 0) == di && d8_dj(b, 0) == dj) k = b;
    if (k < 0) {
      atomicOr(err, EL_NOT_NEIGHBOUR);
      continue;
    }
    if (atomicAdd(&seen[u], 1) != 0) {
      atomicOr(err, EL_DUPLICATE);
      continue;
    }
    dir[u] = (uint8_t)(1u << k);
  }
}

// The forest sum equals the list-order sweep only when every edge into a
// pixel is listed before the pixel's own out-edge.
__global__ void edges_order_kernel(const ptrdiff_t *__restrict__ source, int64_t E, int64_t N,
                                   const int *__restrict__ maxin, int *__restrict__ err) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = source[e];
    if (u >= 0 && u < N && maxin[u] > (int)e) atomicOr(err, EL_ORDER);
  }
}

// ---- drainagebasins ---------------------------------------------------------

__global__ void basins_init_kernel(int *__restrict__ first, int *__restrict__ parent,
                                   int64_t N) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    first[p] = INT_MAX;
    parent[p] = (int)p;
  }
}

// first[u] = index of u's first-listed out-edge.
__global__ void basins_first_kernel(const ptrdiff_t *__restrict__ source, int64_t E,
                                    int64_t N, int *__restrict__ first, int *__restrict__ err) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = source[e];
    if (u < 0 || u >= N) {
      atomicOr(err, EL_BAD_INDEX);
      continue;
    }
    atomicMin(&first[u], (int)e);
  }
}

__global__ void basins_parent_kernel(const ptrdiff_t *__restrict__ source,
                                     const ptrdiff_t *__restrict__ target, int64_t E,
                                     int64_t N, const int *__restrict__ first,
                                     int *__restrict__ parent, int *__restrict__ err) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = source[e], v = target[e];
    if (u < 0 || u >= N || v < 0 || v >= N) {
      atomicOr(err, EL_BAD_INDEX);
      continue;
    }
    if (first[u] == (int)e) parent[u] = (int)v;
  }
}

// One block per 32 x 32 tile: every pixel's in-tile terminal (a root, or an
// exit: a pixel whose parent lies in another tile) by pointer jumping in
// shared memory; exits are appended to a list.  J[p] = p for roots and
// parent(p) for exits (the coarse pointer the next kernel jumps on).
__global__ void __launch_bounds__(256)
basins_tile_kernel(const int *__restrict__ parent, int64_t m, int64_t n, int tm, int tn,
                   int *__restrict__ term, int *__restrict__ J, int *__restrict__ exits,
                   int *__restrict__ nexits, int *__restrict__ err) {
  __shared__ int ptr[kTile * kTile];
  const int T = tm * tn;
  for (int tile = blockIdx.x; tile < T; tile += gridDim.x) {
    const int ti = tile % tm, tj = tile / tm;
    const int64_t i0 = (int64_t)ti * kTile, j0 = (int64_t)tj * kTile;
    for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
      const int64_t i = i0 + (e & 31), j = j0 + (e >> 5);
      int v = e;
      if (i < m && j < n) {
        const int64_t p = j * m + i, q = parent[p];
        const int64_t qi = q % m, qj = q / m;
        if (q != p && qi >= i0 && qi < i0 + kTile && qj >= j0 && qj < j0 + kTile)
          v = (int)((qj - j0) * kTile + (qi - i0));
      }
      ptr[e] = v;
    }
    __syncthreads();
    for (int round = 0; round < 12; round++) {
      int moved = 0;
      for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
        const int a = ptr[e], b = ptr[a];
        if (a != b) {
          ptr[e] = b;
          moved = 1;
        }
      }
      if (!__syncthreads_or(moved)) break;
    }
    for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
      const int64_t i = i0 + (e & 31), j = j0 + (e >> 5);
      if (i >= m || j >= n) continue;
      const int64_t p = j * m + i;
      const int t = ptr[e];
      if (ptr[t] != t) atomicOr(err, EL_CYCLE);  // chain never ended in-tile
      term[p] = (int)((j0 + (t >> 5)) * m + (i0 + (t & 31)));
      if (t == e) {  // a terminal: root, or exit with its parent outside
        const int q = parent[p];
        J[p] = q;
        if (q != (int)p) exits[append_slot(nexits)] = (int)p;
      }
    }
    __syncthreads();
  }
}

// Coarse pointers: an exit's pointer starts at its parent's in-tile
// terminal; one round of jumping over the exit list.
__global__ void exits_init_kernel(const int *__restrict__ exits, const int *__restrict__ nexits,
                                  const int *__restrict__ term, int *__restrict__ J) {
  const int E = *nexits;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < E; k += gridDim.x * blockDim.x) {
    const int x = exits[k];
    J[x] = term[J[x]];
  }
}

__global__ void exits_jump_kernel(const int *__restrict__ exits, const int *__restrict__ nexits,
                                  int *__restrict__ J, int *__restrict__ changed) {
  const int E = *nexits;
  int c = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < E; k += gridDim.x * blockDim.x) {
    const int x = exits[k];
    const int a = J[x], b = J[a];
    if (a != b) {
      J[x] = b;
      c = 1;
    }
  }
  if (__any_sync(0xffffffffu, c) && (threadIdx.x & 31) == 0) atomicOr(changed, 1);
}

__global__ void basins_root_kernel(const int *__restrict__ term, const int *__restrict__ J,
                                   int64_t N, int *__restrict__ root) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x)
    root[p] = J[term[p]];
}

// key[root] = largest edge index among the pixels of the basin.  A root
// must have no out-edge; one that has lies on a cycle of the edge list.
// Large basins put millions of pixels on one key: lanes with the same root
// are reduced first and one atomic per root and warp is issued.
__global__ void basins_key_kernel(const int *__restrict__ root, const int *__restrict__ first,
                                  int64_t N, int *__restrict__ key, int *__restrict__ err) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < N;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = base + threadIdx.x;  // whole warps iterate together
    const bool in = p < N;
    const int f = in ? first[p] : INT_MAX;
    const int r = in ? root[p] : -1;
    if (in && r == (int)p && f != INT_MAX) atomicOr(err, EL_CYCLE);
    const unsigned grp = __match_any_sync(0xffffffffu, r);
    const int mx = __reduce_max_sync(grp, f == INT_MAX ? -1 : f);
    if (in && lane == __ffs(grp) - 1 && mx >= 0) atomicMax(&key[r], mx);
  }
}

__global__ void basins_mark_kernel(const int *__restrict__ key, int64_t N,
                                   int *__restrict__ mark) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int k = key[p];
    if (k >= 0) mark[k] = 1;
  }
}

// Exclusive scan of `mark` (block counts come from scan_blocks_kernel).
__global__ void mark_count_kernel(const int *__restrict__ mark, int64_t E, int *__restrict__ cnt) {
  __shared__ int total;
  const int64_t k0 = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanPer;
  int c = 0;
#pragma unroll
  for (int s = 0; s < kScanPer; s++) c += (k0 + s < E) ? mark[k0 + s] : 0;
  block_exclusive_scan(c, &total);
  if (threadIdx.x == 0) cnt[blockIdx.x] = total;
}

__global__ void mark_scan_kernel(const int *__restrict__ mark, int64_t E,
                                 const int *__restrict__ off, int *__restrict__ ex) {
  __shared__ int total;
  const int64_t k0 = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanPer;
  int v[kScanPer], c = 0;
#pragma unroll
  for (int s = 0; s < kScanPer; s++) {
    v[s] = (k0 + s < E) ? mark[k0 + s] : 0;
    c += v[s];
  }
  int run = off[blockIdx.x] + block_exclusive_scan(c, &total);
#pragma unroll
  for (int s = 0; s < kScanPer; s++) {
    if (k0 + s < E) ex[k0 + s] = run;
    run += v[s];
  }
}

// label = K - (marks before the basin's key); pixels on no edge keep 0.
__global__ void basins_label_kernel(const int *__restrict__ root, const int *__restrict__ key,
                                    const int *__restrict__ ex, const int *__restrict__ total,
                                    int64_t N, ptrdiff_t *__restrict__ basins) {
  const int K = *total;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int k = key[root[p]];
    basins[p] = k >= 0 ? (ptrdiff_t)(K - ex[k]) : 0;
  }
}

// ---- edgelist_degree ---------------------------------------------------------

__global__ void degree_count_kernel(const ptrdiff_t *__restrict__ source,
                                    const ptrdiff_t *__restrict__ target, int64_t E,
                                    int64_t N, int *__restrict__ indeg,
                                    int *__restrict__ outdeg, int *__restrict__ err) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = source[e], v = target[e];
    if (u < 0 || u >= N || v < 0 || v >= N) {
      atomicOr(err, EL_BAD_INDEX);
      continue;
    }
    atomicAdd(&indeg[v], 1);
    atomicAdd(&outdeg[u], 1);
  }
}

__global__ void degree_narrow_kernel(const int *__restrict__ indeg, const int *__restrict__ outdeg,
                                     int64_t N, uint8_t *__restrict__ in8,
                                     uint8_t *__restrict__ out8) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    in8[p] = (uint8_t)indeg[p];  // wraps modulo 256 like a uint8 counter
    out8[p] = (uint8_t)outdeg[p];
  }
}

int grid_for(int64_t n) {
  const int64_t b = (n + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * 32;
  return (int)std::max<int64_t>(1, std::min(b, cap));
}

tt_cuda_status read_err(const int *err_dev, cudaStream_t st, int *out) {
  int *h = (int *)pinned_scratch();
  if (!h) return TT_CUDA_ERR_ALLOC;
  TT_CHECK(cudaMemcpyAsync(h, err_dev, sizeof(int), cudaMemcpyDeviceToHost, st));
  TT_CHECK(cudaStreamSynchronize(st));
  *out = *h;
  return TT_CUDA_SUCCESS;
}

}  // namespace

tt_cuda_status edgelist_dev(ptrdiff_t *source, ptrdiff_t *target, int64_t *count,
                            const ptrdiff_t *node, const uint8_t *dir, const GridDims &g,
                            unsigned order, cudaStream_t st) {
  const int64_t N = g.cells();
  const int nb = (int)((N + kScanBlock - 1) / kScanBlock);
  Workspace &ws = workspace();
  if (!ws.reserve(2 * align_up((size_t)(nb + 1) * 4))) return TT_CUDA_ERR_ALLOC;
  int *cnt = (int *)ws.take((size_t)(nb + 1) * 4);
  int *off = (int *)ws.take((size_t)(nb + 1) * 4);
  EdgeArgs a;
  a.node = node;
  a.dir = dir;
  a.N = N;
  const ptrdiff_t s0 = (order & 1) ? g.m : 1, s1 = (order & 1) ? 1 : g.m;
  const ptrdiff_t offs[8] = {s1, s0 + s1, s0, s0 - s1, -s1, -s0 - s1, -s0, -s0 + s1};
  for (int r = 0; r < 8; r++) a.off[r] = offs[r];
  TT_LAUNCH(edge_count_kernel, nb, kScanThreads, 0, st, a, cnt);
  TT_LAUNCH(scan_blocks_kernel, 1, kScanThreads, 0, st, cnt, off, nb);
  TT_LAUNCH(edge_scatter_kernel, nb, kScanThreads, 0, st, a, off, source, target);
  TT_CHECK(cudaGetLastError());
  int *h = (int *)pinned_scratch();
  if (!h) return TT_CUDA_ERR_ALLOC;
  TT_CHECK(cudaMemcpyAsync(h, off + nb, sizeof(int), cudaMemcpyDeviceToHost, st));
  TT_CHECK(cudaStreamSynchronize(st));
  *count = *h;
  return TT_CUDA_SUCCESS;
}

tt_cuda_status accumulate_edgelist_dev(float *acc, const ptrdiff_t *source,
                                       const ptrdiff_t *target, const float *fraction,
                                       const float *weights, int64_t E, const GridDims &g,
                                       cudaStream_t st) {
  const int64_t N = g.cells();
  // The direction grid and the duplicate counters must outlive the
  // accumulation, which may grow (and so move) the shared workspace: they
  // get a stream-ordered allocation of their own.
  uint8_t *dir = nullptr;
  int *seen = nullptr, *maxin = nullptr, *err = nullptr;
  TT_CHECK(cudaMallocAsync((void **)&dir, (size_t)N + 256, st));
  TT_CHECK(cudaMallocAsync((void **)&seen, (size_t)N * 8 + 256, st));
  maxin = seen + N;
  err = seen + 2 * N;
  TT_CHECK(cudaMemsetAsync(dir, 0, (size_t)N, st));
  TT_CHECK(cudaMemsetAsync(seen, 0, (size_t)N * 4, st));
  TT_CHECK(cudaMemsetAsync(maxin, 0xff, (size_t)N * 4, st));  // -1: no edge in
  TT_CHECK(cudaMemsetAsync(err, 0, 4, st));
  if (E > 0) {
    TT_LAUNCH(edges_to_dir_kernel, grid_for(E), 256, 0, st, source, target, fraction, E, g.m,
              g.n, dir, seen, maxin, err);
    TT_LAUNCH(edges_order_kernel, grid_for(E), 256, 0, st, source, E, N, maxin, err);
  }
  TT_CHECK(cudaGetLastError());
  int e = 0;
  tt_cuda_status s = read_err(err, st, &e);
  if (s == TT_CUDA_SUCCESS && (e & EL_BAD_INDEX)) s = TT_CUDA_ERR_INVALID_ARGUMENT;
  if (s == TT_CUDA_SUCCESS && e)  // not a D8 forest in topological order
    s = edge_sweep_dev(acc, weights, source, target, fraction, E, N, st);
  else if (s == TT_CUDA_SUCCESS)
    s = accumulate_dev(acc, dir, weights, g, st);
  cudaFreeAsync(dir, st);
  cudaFreeAsync(seen, st);
  return s;
}

tt_cuda_status drainagebasins_dev(ptrdiff_t *basins, const ptrdiff_t *source,
                                  const ptrdiff_t *target, int64_t E, const GridDims &g,
                                  cudaStream_t st) {
  const int64_t N = g.cells();
  const int64_t Em = std::max<int64_t>(E, 1);
  const int nb = (int)((Em + kScanBlock - 1) / kScanBlock);
  Workspace &ws = workspace();
  const size_t need = 6 * align_up((size_t)N * 4) + 2 * align_up((size_t)Em * 4) +
                      2 * align_up((size_t)(nb + 1) * 4) + 256;
  if (!ws.reserve(need)) return TT_CUDA_ERR_ALLOC;
  int *ctl = (int *)ws.take(256);  // [0] error bits, [1] changed, [2] exit count
  int *first = (int *)ws.take((size_t)N * 4);
  int *pa = (int *)ws.take((size_t)N * 4);
  int *pb = (int *)ws.take((size_t)N * 4);
  int *key = (int *)ws.take((size_t)N * 4);
  int *rootp = (int *)ws.take((size_t)N * 4);
  int *ex_list = (int *)ws.take((size_t)N * 4);
  int *mark = (int *)ws.take((size_t)Em * 4);
  int *ex = (int *)ws.take((size_t)Em * 4);
  int *cnt = (int *)ws.take((size_t)(nb + 1) * 4);
  int *off = (int *)ws.take((size_t)(nb + 1) * 4);
  const int gN = grid_for(N), gE = grid_for(E);
  TT_CHECK(cudaMemsetAsync(ctl, 0, 256, st));
  TT_LAUNCH(basins_init_kernel, gN, 256, 0, st, first, pa, N);
  TT_LAUNCH(basins_first_kernel, gE, 256, 0, st, source, E, N, first, ctl);
  TT_LAUNCH(basins_parent_kernel, gE, 256, 0, st, source, target, E, N, first, pa, ctl);
  TT_CHECK(cudaGetLastError());
  // Roots: in-tile terminals by pointer jumping in shared memory, then
  // jumping over the exits only, then every pixel through its terminal.
  int *term = pb, *J = key, *root = rootp;  // key is free until the keys are taken
  int *exits = ex_list, *nexits = ctl + 2;
  TT_LAUNCH(basins_tile_kernel, (int)std::min<int64_t>(g.tiles(), INT_MAX), 256,
            0, st, pa, g.m, g.n, g.tm, g.tn, term, J, exits, nexits, ctl);
  TT_LAUNCH(exits_init_kernel, gN, 256, 0, st, exits, nexits, term, J);
  int *h = (int *)pinned_scratch();
  if (!h) return TT_CUDA_ERR_ALLOC;
  bool converged = false;
  for (int round = 0; round < 40; round += 4) {
    TT_CHECK(cudaMemsetAsync(ctl + 1, 0, 4, st));
    for (int k = 0; k < 4; k++)
      TT_LAUNCH(exits_jump_kernel, gN, 256, 0, st, exits, nexits, J, ctl + 1);
    TT_CHECK(cudaGetLastError());
    TT_CHECK(cudaMemcpyAsync(h, ctl, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    TT_CHECK(cudaStreamSynchronize(st));
    if (h[0] & EL_BAD_INDEX) return TT_CUDA_ERR_INVALID_ARGUMENT;
    if (h[0] & EL_CYCLE) return TT_CUDA_ERR_CYCLE;
    if (!h[1]) {
      converged = true;
      break;
    }
  }
  if (!converged) return TT_CUDA_ERR_CYCLE;
  TT_LAUNCH(basins_root_kernel, gN, 256, 0, st, term, J, N, root);
  int *cur = root;
  TT_CHECK(cudaMemsetAsync(key, 0xff, (size_t)N * 4, st));  // -1: no edge in basin
  TT_CHECK(cudaMemsetAsync(mark, 0, (size_t)Em * 4, st));
  TT_LAUNCH(basins_key_kernel, gN, 256, 0, st, cur, first, N, key, ctl);
  TT_LAUNCH(basins_mark_kernel, gN, 256, 0, st, key, N, mark);
  TT_LAUNCH(mark_count_kernel, nb, kScanThreads, 0, st, mark, Em, cnt);
  TT_LAUNCH(scan_blocks_kernel, 1, kScanThreads, 0, st, cnt, off, nb);
  TT_LAUNCH(mark_scan_kernel, nb, kScanThreads, 0, st, mark, Em, off, ex);
  TT_LAUNCH(basins_label_kernel, gN, 256, 0, st, cur, key, ex, off + nb, N, basins);
  TT_CHECK(cudaGetLastError());
  int e = 0;
  TT_TRY_STATUS(read_err(ctl, st, &e));
  if (e & EL_CYCLE) return TT_CUDA_ERR_CYCLE;
  if (e) return TT_CUDA_ERR_INVALID_ARGUMENT;
  return TT_CUDA_SUCCESS;
}

int scan_blocks_for(int64_t n) {
  return (int)((std::max<int64_t>(n, 1) + kScanBlock - 1) / kScanBlock);
}

tt_cuda_status scan_exclusive_dev(const int *in, int64_t n, int *out, int *cnt, int *off,
                                  cudaStream_t st) {
  const int nb = scan_blocks_for(n);
  TT_LAUNCH(mark_count_kernel, nb, kScanThreads, 0, st, in, n, cnt);
  TT_LAUNCH(scan_blocks_kernel, 1, kScanThreads, 0, st, cnt, off, nb);
  TT_LAUNCH(mark_scan_kernel, nb, kScanThreads, 0, st, in, n, off, out);
  TT_CHECK(cudaGetLastError());
  return TT_CUDA_SUCCESS;
}

tt_cuda_status degree_dev(uint8_t *indegree, uint8_t *outdegree, const ptrdiff_t *source,
                          const ptrdiff_t *target, int64_t N, int64_t E, cudaStream_t st) {
  Workspace &ws = workspace();
  if (!ws.reserve(2 * align_up((size_t)N * 4) + 256)) return TT_CUDA_ERR_ALLOC;
  int *err = (int *)ws.take(256);
  int *in = (int *)ws.take((size_t)N * 4);
  int *out = (int *)ws.take((size_t)N * 4);
  TT_CHECK(cudaMemsetAsync(err, 0, 4, st));
  TT_CHECK(cudaMemsetAsync(in, 0, (size_t)N * 4, st));
  TT_CHECK(cudaMemsetAsync(out, 0, (size_t)N * 4, st));
  TT_LAUNCH(degree_count_kernel, grid_for(E), 256, 0, st, source, target, E, N, in, out, err);
  TT_LAUNCH(degree_narrow_kernel, grid_for(N), 256, 0, st, in, out, N, indegree, outdegree);
  TT_CHECK(cudaGetLastError());
  int e = 0;
  tt_cuda_status s = read_err(err, st, &e);
  if (s == TT_CUDA_SUCCESS && e) return TT_CUDA_ERR_INVALID_ARGUMENT;
  return s;
}

}  // namespace tt
