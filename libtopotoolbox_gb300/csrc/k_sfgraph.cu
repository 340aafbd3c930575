// Graphflood's single-flow graph (src/graphflood/sfgraph.c:27-113) and its
// drainage area (src/graphflood/gf_flowacc.c:19-35) on the GPU.
//
// Layout: row-major `dim` = {rows, cols}, node = row * cols + col, FP64
// elevations and graphflood's own boundary codes (src/graphflood/gf_utils.c:
// a node can give with BC 1, 3, 6, 7, 8, 9 and receive with BC 1, 3, 4, 5,
// 6, 7, 9; neighbours never wrap across the first/last row or column).  In
// the tile convention of the other kernels the grid is m = cols pixels along
// the fast axis i and n = rows along j.
//
//  * receivers: a stencil per node, the first strict maximum of
//    (z - z_n) / distance in double over the neighbours in graphflood's
//    order — bit-identical to the reference;
//  * donors: every node lists the neighbours that drain into it in
//    increasing node index, as the reference's inversion loop does;
//  * the Braun-Willett stack: a depth-first preorder from every root in node
//    order, donors in listed order.  In that preorder a node follows its
//    receiver after the whole subtrees of the donors listed before it, so
//        pos(v) = pos(receiver) + 1 + sum of sizes of earlier donors
//    and a root's position is the total size of the roots before it.  Sizes
//    are exact subtree pixel counts from the forest contraction; positions
//    are root-ward path sums of those offsets (pointer jumping inside each
//    tile in shared memory, then over the tile exits only).  The stack is
//    therefore the reference's, bit for bit;
//  * drainage area: cell_area * (subtree size), minus the node itself at
//    roots, which the reference leaves out.  The reference adds multiples of
//    cell_area in stack order, so the two agree exactly whenever those sums
//    are exact (cell_area a multiple of a power of two, as for integer cell
//    sizes) and to a few ulps otherwise.
#include <algorithm>
#include <climits>
#include <cmath>

#include "tt_internal.cuh"

namespace tt {
namespace {

__device__ __forceinline__ bool gf_can_give(uint8_t b) {
  return b == 1 || b == 3 || b == 6 || b == 7 || b == 8 || b == 9;
}
__device__ __forceinline__ bool gf_can_receive(uint8_t b) {
  return b == 1 || b == 3 || b == 4 || b == 5 || b == 6 || b == 7 || b == 9;
}

struct SfArgs {
  const double *topo;
  const uint8_t *bcs;
  int64_t rows, cols;
  bool d8;
  double dist[8];  // neighbour distances in graphflood's order
};

// Graphflood's neighbour n as (row, col) offsets: D8 order
// (-1,-1) (-1,0) (-1,1) (0,-1) (0,1) (1,-1) (1,0) (1,1); D4 order
// (-1,0) (0,-1) (0,1) (1,0).
__device__ __forceinline__ void gf_offset(int n, bool d8, int *dr, int *dc) {
  if (d8) {
    *dr = n < 3 ? -1 : (n < 5 ? 0 : 1);
    *dc = (n == 0 || n == 3 || n == 5) ? -1 : ((n == 1 || n == 6) ? 0 : 1);
  } else {
    *dr = n == 0 ? -1 : (n == 3 ? 1 : 0);
    *dc = n == 1 ? -1 : (n == 2 ? 1 : 0);
  }
}

// Receivers, distances and the direction byte of the tile convention (bit k:
// (i + d8_di(k), j + d8_dj(k)) with i = col, j = row); 0 at roots.
__global__ void sf_receivers_kernel(SfArgs a, size_t *__restrict__ rcv,
                                    double *__restrict__ dist, uint8_t *__restrict__ dir,
                                    int *__restrict__ parent) {
  const int64_t N = a.rows * a.cols;
  const int K = a.d8 ? 8 : 4;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N;
       v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = v / a.cols, c = v % a.cols;
    int64_t best = v;
    double bestd = 0.0, slope = 0.0;
    int bdr = 0, bdc = 0;
    if (gf_can_give(a.bcs[v])) {
      const double z = a.topo[v];
      for (int n = 0; n < K; n++) {
        int dr, dc;
        gf_offset(n, a.d8, &dr, &dc);
        const int64_t rr = r + dr, cc = c + dc;
        if (rr < 0 || rr >= a.rows || cc < 0 || cc >= a.cols) continue;
        const int64_t q = rr * a.cols + cc;
        if (!gf_can_receive(a.bcs[q])) continue;
        const double d = a.dist[n];
        const double s = __ddiv_rn(__dsub_rn(z, a.topo[q]), d);
        if (s > slope) {
          best = q;
          bestd = d;
          slope = s;
          bdr = dr;
          bdc = dc;
        }
      }
    }
    rcv[v] = (size_t)best;
    dist[v] = bestd;
    parent[v] = (int)best;
    uint8_t bits = 0;
    if (best != v)
      for (int k = 0; k < 8; k++)
        if (d8_di(k, 0) == bdc && d8_dj(k, 0) == bdr) bits = (uint8_t)(1u << k);
    dir[v] = bits;
  }
}

// Donors of every node in increasing node index (the D8 offsets of
// graphflood's order are already increasing), K slots per node.
__global__ void sf_donors_kernel(const size_t *__restrict__ rcv, int64_t rows, int64_t cols,
                                 int K, size_t *__restrict__ donors,
                                 uint8_t *__restrict__ ndonors) {
  const int64_t N = rows * cols;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N;
       v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = v / cols, c = v % cols;
    int cnt = 0;
    for (int n = 0; n < 8; n++) {
      int dr, dc;
      gf_offset(n, true, &dr, &dc);
      const int64_t rr = r + dr, cc = c + dc;
      if (rr < 0 || rr >= rows || cc < 0 || cc >= cols) continue;
      const int64_t q = rr * cols + cc;
      if (rcv[q] == (size_t)v && cnt < K) donors[v * K + cnt++] = (size_t)q;
    }
    ndonors[v] = (uint8_t)cnt;
  }
}

// ---- Root-ward path sums --------------------------------------------------
// out(p) = sum of val over the path from p to its root, both ends included.
// One block per 32 x 32 tile jumps (pointer, partial sum) pairs in shared
// memory until every pixel points at its in-tile terminal (a root, or an
// exit: a pixel whose parent lies in another tile); psum(p) then holds the
// sum up to the terminal, terminal excluded.  Terminals are finished by
// double-buffered jumping over the exits alone.

__global__ void __launch_bounds__(256)
rw_tile_kernel(const int *__restrict__ parent, const int *__restrict__ val, int64_t m,
               int64_t n, int tm, int tn, int *__restrict__ term, int *__restrict__ psum,
               int *__restrict__ accA, int *__restrict__ xA, int *__restrict__ accB,
               int *__restrict__ xB, int *__restrict__ exits, int *__restrict__ nexits,
               int *__restrict__ err) {
  __shared__ int ptr[kTile * kTile];
  __shared__ int sum[kTile * kTile];
  constexpr int kPer = kTile * kTile / 256;
  const int T = tm * tn;
  for (int tile = blockIdx.x; tile < T; tile += gridDim.x) {
    const int ti = tile % tm, tj = tile / tm;
    const int64_t i0 = (int64_t)ti * kTile, j0 = (int64_t)tj * kTile;
    for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
      const int64_t i = i0 + (e & 31), j = j0 + (e >> 5);
      int v = e, s = 0;
      if (i < m && j < n) {
        const int64_t p = j * m + i, q = parent[p];
        const int64_t qi = q % m, qj = q / m;
        if (q != p && qi >= i0 && qi < i0 + kTile && qj >= j0 && qj < j0 + kTile) {
          v = (int)((qj - j0) * kTile + (qi - i0));
          s = val[p];
        }
      }
      ptr[e] = v;
      sum[e] = s;
    }
    __syncthreads();
    for (int round = 0; round < 12; round++) {
      int np[kPer], ns[kPer], moved = 0;
#pragma unroll
      for (int u = 0; u < kPer; u++) {
        const int e = threadIdx.x + u * 256;
        const int a = ptr[e];
        np[u] = ptr[a];
        ns[u] = sum[e] + (a != e ? sum[a] : 0);
        moved |= np[u] != a;
      }
      __syncthreads();
#pragma unroll
      for (int u = 0; u < kPer; u++) {
        const int e = threadIdx.x + u * 256;
        ptr[e] = np[u];
        sum[e] = ns[u];
      }
      if (!__syncthreads_or(moved)) break;
    }
    for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
      const int64_t i = i0 + (e & 31), j = j0 + (e >> 5);
      if (i >= m || j >= n) continue;
      const int64_t p = j * m + i;
      const int t = ptr[e];
      if (ptr[t] != t) atomicOr(err, 1);  // a chain that never ended in-tile
      term[p] = (int)((j0 + (t >> 5)) * m + (i0 + (t & 31)));
      psum[p] = sum[e];
      if (t == e) {
        const int q = parent[p];
        if (q == (int)p) {  // root: finished
          accA[p] = accB[p] = val[p];
          xA[p] = xB[p] = -1;
        } else {
          const int64_t qi = q % m, qj = q / m;
          if (qi >= i0 && qi < i0 + kTile && qj >= j0 && qj < j0 + kTile)
            atomicOr(err, 1);  // a terminal whose parent is in-tile: a cycle
          exits[append_slot(nexits)] = (int)p;
        }
      }
    }
    __syncthreads();
  }
}

__global__ void rw_exits_init_kernel(const int *__restrict__ exits, const int *__restrict__ nexits,
                                     const int *__restrict__ parent, const int *__restrict__ val,
                                     const int *__restrict__ term, const int *__restrict__ psum,
                                     int *__restrict__ acc, int *__restrict__ x) {
  const int E = *nexits;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < E; k += gridDim.x * blockDim.x) {
    const int p = exits[k], q = parent[p];
    acc[p] = val[p] + psum[q];
    x[p] = term[q];
  }
}

__global__ void rw_exits_jump_kernel(const int *__restrict__ exits, const int *__restrict__ nexits,
                                     const int *__restrict__ accI, const int *__restrict__ xI,
                                     int *__restrict__ accO, int *__restrict__ xO,
                                     int *__restrict__ changed) {
  const int E = *nexits;
  int c = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < E; k += gridDim.x * blockDim.x) {
    const int p = exits[k], y = xI[p];
    if (y >= 0) {
      accO[p] = accI[p] + accI[y];
      xO[p] = xI[y];
      c = 1;
    } else {
      accO[p] = accI[p];
      xO[p] = -1;
    }
  }
  if (__any_sync(0xffffffffu, c) && (threadIdx.x & 31) == 0) atomicOr(changed, 1);
}

__global__ void rw_final_kernel(const int *__restrict__ term, const int *__restrict__ psum,
                                const int *__restrict__ acc, int64_t N, int *__restrict__ out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x)
    out[p] = psum[p] + acc[term[p]];
}

// ---- Stack positions ---------------------------------------------------------

// val(v) = 1 + sizes of the donors listed before v at v's receiver; a root's
// val is its base (set after the scan of root sizes).
__global__ void sf_offsets_kernel(const int *__restrict__ parent, const int *__restrict__ size,
                                  const size_t *__restrict__ donors,
                                  const uint8_t *__restrict__ ndonors, int K, int64_t N,
                                  int *__restrict__ val, int *__restrict__ rootsz) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N;
       v += (int64_t)gridDim.x * blockDim.x) {
    const int p = parent[v];
    if (p == (int)v) {
      rootsz[v] = size[v];
      val[v] = 0;
      continue;
    }
    rootsz[v] = 0;
    int off = 1;
    const int nd = ndonors[p];
    for (int k = 0; k < nd; k++) {
      const size_t s = donors[(size_t)p * K + k];
      if (s < (size_t)v) off += size[s];
    }
    val[v] = off;
  }
}

__global__ void sf_root_base_kernel(const int *__restrict__ parent, const int *__restrict__ base,
                                    int64_t N, int *__restrict__ val) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N;
       v += (int64_t)gridDim.x * blockDim.x)
    if (parent[v] == (int)v) val[v] = base[v];
}

__global__ void sf_stack_kernel(const int *__restrict__ pos, int64_t N, size_t *__restrict__ stack) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N;
       v += (int64_t)gridDim.x * blockDim.x)
    stack[pos[v]] = (size_t)v;
}

// ---- Drainage area from receivers ---------------------------------------------

// Receiver indices back to direction bytes and parents; anything but the
// node itself or one of its eight neighbours is refused.
__global__ void sf_rcv_to_dir_kernel(const size_t *__restrict__ rcv, int64_t rows, int64_t cols,
                                     uint8_t *__restrict__ dir, int *__restrict__ parent,
                                     int *__restrict__ err) {
  const int64_t N = rows * cols;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N;
       v += (int64_t)gridDim.x * blockDim.x) {
    const size_t q = rcv[v];
    uint8_t bits = 0;
    int par = (int)v;
    if (q >= (size_t)N) {
      atomicOr(err, 2);
    } else if (q != (size_t)v) {
      const int64_t dr = (int64_t)(q / cols) - v / cols, dc = (int64_t)(q % cols) - v % cols;
      for (int k = 0; k < 8; k++)
        if (d8_di(k, 0) == dc && d8_dj(k, 0) == dr) bits = (uint8_t)(1u << k);
      if (!bits) atomicOr(err, 2);
      par = (int)q;
    }
    dir[v] = bits;
    parent[v] = par;
  }
}

__global__ void sf_area_kernel(const int *__restrict__ size, const int *__restrict__ parent,
                               int64_t N, double cell_area, double *__restrict__ area) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N;
       v += (int64_t)gridDim.x * blockDim.x) {
    const int s = size[v] - (parent[v] == (int)v ? 1 : 0);
    area[v] = __dmul_rn(cell_area, (double)s);
  }
}

int sf_grid(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)sm_count() * 32));
}

}  // namespace

namespace {

// Scratch of one call, in one stream-ordered allocation (the forest
// contraction inside grows the shared workspace, which would move anything
// taken from it before).
struct SfScratch {
  char *base = nullptr;
  size_t used = 0;
  void *take(size_t bytes) {
    void *p = base + used;
    used += align_up(bytes);
    return p;
  }
};

// out = root-ward inclusive path sums of val over the forest `parent`.
tt_cuda_status rootward_sum(int *out, const int *parent, const int *val, const GridDims &g,
                            SfScratch &s, cudaStream_t st) {
  const int64_t N = g.cells();
  int *ctl = (int *)s.take(256);  // [0] error, [1] changed, [2] exit count
  int *term = (int *)s.take(N * 4), *psum = (int *)s.take(N * 4);
  int *acc[2] = {(int *)s.take(N * 4), (int *)s.take(N * 4)};
  int *x[2] = {(int *)s.take(N * 4), (int *)s.take(N * 4)};
  int *exits = (int *)s.take(N * 4);
  TT_CHECK(cudaMemsetAsync(ctl, 0, 256, st));
  const int gN = sf_grid(N);
  TT_LAUNCH(rw_tile_kernel, (int)std::min<int64_t>(g.tiles(), INT_MAX), 256, 0,
            st, parent, val, g.m, g.n, g.tm, g.tn, term, psum, acc[0], x[0], acc[1], x[1],
            exits, ctl + 2, ctl);
  TT_LAUNCH(rw_exits_init_kernel, gN, 256, 0, st, exits, ctl + 2, parent, val, term, psum,
            acc[0], x[0]);
  int *h = (int *)pinned_scratch();
  if (!h) return TT_CUDA_ERR_ALLOC;
  int cur = 0;
  bool converged = false;
  for (int round = 0; round < 40; round += 4) {
    TT_CHECK(cudaMemsetAsync(ctl + 1, 0, 4, st));
    for (int k = 0; k < 4; k++) {
      TT_LAUNCH(rw_exits_jump_kernel, gN, 256, 0, st, exits, ctl + 2, acc[cur], x[cur],
                acc[cur ^ 1], x[cur ^ 1], ctl + 1);
      cur ^= 1;
    }
    TT_CHECK(cudaGetLastError());
    TT_CHECK(cudaMemcpyAsync(h, ctl, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    TT_CHECK(cudaStreamSynchronize(st));
    if (h[0]) return TT_CUDA_ERR_CYCLE;
    if (!h[1]) {
      converged = true;
      break;
    }
  }
  if (!converged) return TT_CUDA_ERR_CYCLE;
  TT_LAUNCH(rw_final_kernel, gN, 256, 0, st, term, psum, acc[cur], N, out);
  TT_CHECK(cudaGetLastError());
  return TT_CUDA_SUCCESS;
}

size_t rootward_bytes(int64_t N) { return 256 + 7 * align_up((size_t)N * 4); }

SfArgs sf_args(const double *topo, const uint8_t *bcs, int64_t rows, int64_t cols, double dx,
               bool d8) {
  SfArgs a;
  a.topo = topo;
  a.bcs = bcs;
  a.rows = rows;
  a.cols = cols;
  a.d8 = d8;
  // src/graphflood/gf_utils.c generate_offsetdx_D8 / _D4
  const double diag = (double)std::sqrt(2.0) * dx;
  const double d8v[8] = {diag, dx, diag, dx, dx, diag, dx, diag};
  for (int k = 0; k < 8; k++) a.dist[k] = d8 ? d8v[k] : dx;
  return a;
}

}  // namespace

tt_cuda_status sfgraph_dev(const double *topo, size_t *rcv, double *dist, size_t *donors,
                           uint8_t *ndonors, size_t *stack, const uint8_t *bcs, int64_t rows,
                           int64_t cols, double dx, bool d8, cudaStream_t st) {
  const int64_t N = rows * cols;
  const int K = d8 ? 8 : 4;
  const ptrdiff_t dims[2] = {cols, rows};  // tile convention: m = cols, n = rows
  const GridDims g = make_dims(dims);
  const int nb = scan_blocks_for(N);
  SfScratch s;
  const size_t bytes = align_up((size_t)N) + 5 * align_up((size_t)N * 4) +
                       2 * align_up((size_t)(nb + 1) * 4) + rootward_bytes(N);
  TT_CHECK(cudaMallocAsync((void **)&s.base, bytes, st));
  uint8_t *dir = (uint8_t *)s.take(N);
  int *parent = (int *)s.take(N * 4), *size = (int *)s.take(N * 4);
  int *val = (int *)s.take(N * 4), *rootsz = (int *)s.take(N * 4);
  int *pos = (int *)s.take(N * 4);
  int *cnt = (int *)s.take((nb + 1) * 4), *off = (int *)s.take((nb + 1) * 4);
  const int gN = sf_grid(N);
  tt_cuda_status r = TT_CUDA_SUCCESS;
  do {
    TT_LAUNCH(sf_receivers_kernel, gN, 256, 0, st, sf_args(topo, bcs, rows, cols, dx, d8), rcv,
              dist, dir, parent);
    TT_LAUNCH(sf_donors_kernel, gN, 256, 0, st, rcv, rows, cols, K, donors, ndonors);
    if (!cuda_ok(cudaGetLastError(), "sf receivers")) {
      r = TT_CUDA_ERR_CUDA;
      break;
    }
    r = count_dev(size, dir, g, st);
    if (r != TT_CUDA_SUCCESS) break;
    TT_LAUNCH(sf_offsets_kernel, gN, 256, 0, st, parent, size, donors, ndonors, K, N, val,
              rootsz);
    // root bases: exclusive scan of root sizes in node order (into pos)
    r = scan_exclusive_dev(rootsz, N, pos, cnt, off, st);
    if (r != TT_CUDA_SUCCESS) break;
    TT_LAUNCH(sf_root_base_kernel, gN, 256, 0, st, parent, pos, N, val);
    r = rootward_sum(pos, parent, val, g, s, st);
    if (r != TT_CUDA_SUCCESS) break;
    TT_LAUNCH(sf_stack_kernel, gN, 256, 0, st, pos, N, stack);
    if (!cuda_ok(cudaGetLastError(), "sf stack")) r = TT_CUDA_ERR_CUDA;
  } while (0);
  cudaFreeAsync(s.base, st);
  return r;
}

tt_cuda_status sf_drainage_area_dev(double *area, const size_t *rcv, int64_t rows,
                                    int64_t cols, double dx, cudaStream_t st) {
  const int64_t N = rows * cols;
  const ptrdiff_t dims[2] = {cols, rows};
  const GridDims g = make_dims(dims);
  SfScratch s;
  TT_CHECK(cudaMallocAsync((void **)&s.base, 256 + align_up((size_t)N) +
                                                 2 * align_up((size_t)N * 4), st));
  int *err = (int *)s.take(256);
  uint8_t *dir = (uint8_t *)s.take(N);
  int *parent = (int *)s.take(N * 4), *size = (int *)s.take(N * 4);
  tt_cuda_status r = TT_CUDA_SUCCESS;
  do {
    if (!cuda_ok(cudaMemsetAsync(err, 0, 4, st), "memset")) {
      r = TT_CUDA_ERR_CUDA;
      break;
    }
    TT_LAUNCH(sf_rcv_to_dir_kernel, sf_grid(N), 256, 0, st, rcv, rows, cols, dir, parent, err);
    int *h = (int *)pinned_scratch();
    if (!h) {
      r = TT_CUDA_ERR_ALLOC;
      break;
    }
    if (!cuda_ok(cudaMemcpyAsync(h, err, 4, cudaMemcpyDeviceToHost, st), "copy") ||
        !cuda_ok(cudaStreamSynchronize(st), "sync")) {
      r = TT_CUDA_ERR_CUDA;
      break;
    }
    if (*h) {
      r = TT_CUDA_ERR_INVALID_ARGUMENT;
      break;
    }
    r = count_dev(size, dir, g, st);
    if (r != TT_CUDA_SUCCESS) break;
    TT_LAUNCH(sf_area_kernel, sf_grid(N), 256, 0, st, size, parent, N, dx * dx, area);
    if (!cuda_ok(cudaGetLastError(), "sf area")) r = TT_CUDA_ERR_CUDA;
  } while (0);
  cudaFreeAsync(s.base, st);
  return r;
}

}  // namespace tt
