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
//
// Work decomposition: one warp per 32 x 32 tile labels the tile's internal
// edges in shared memory (with path halving) and reduces each tile-local
// component to its maximum depth and the smallest pixel attaining it; only
// edges that cross tile borders touch the global union-find, and the global
// maximum / argmax take one atomic per (tile, component), not per pixel.
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

// Root of x; labels always point at smaller or equal indices.  Path halving
// only ever lowers a label (atomicMin), so it is safe under concurrent unions.
__device__ __forceinline__ int uf_find(int *L, int x) {
  volatile int *vL = L;
  int p = vL[x];
  while (p != x) {
    int gp = vL[p];
    if (gp < p) atomicMin(&L[x], gp);
    x = p;
    p = gp;
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

constexpr int kCclWarps = 4;

// Shared-memory union-find over run ids (see ccl_tile_kernel).
__device__ __forceinline__ int sfind(int *lab, int x) {
  volatile int *v = lab;
  int p = v[x];
  while (p != x) {
    const int gp = v[p];
    if (gp < p) atomicMin(&lab[x], gp);
    x = p;
    p = gp;
  }
  return x;
}

__device__ void sunion(int *lab, int a, int b) {
  for (int it = 0; it < 4096; it++) {
    a = sfind(lab, a);
    b = sfind(lab, b);
    if (a == b) return;
    if (a < b) {
      const int old = atomicMin(&lab[b], a);
      if (old == b) return;
      b = old;
    } else {
      const int old = atomicMin(&lab[a], b);
      if (old == a) return;
      a = old;
    }
  }
}

// Bits s.. of the run of set bits that starts at bit s of m.
__device__ __forceinline__ uint32_t run_mask(uint32_t m, int s) {
  const uint32_t tail = ~(m >> s);
  const int len = tail ? __ffs(tail) - 1 : 32 - s;
  return len >= 32 ? 0xffffffffu : (((1u << len) - 1u) << s);
}

// Start bit of the run containing bit b (b set in m, starts = run starts).
__device__ __forceinline__ int run_start(uint32_t starts, int b) {
  const uint32_t below = starts & (b == 31 ? 0xffffffffu : ((2u << b) - 1u));
  return 31 - __clz(below);
}

// A component's maximum depth key and the smallest tile index attaining it,
// packed so that one 64-bit maximum reduces both: the key (sign flipped to
// order as unsigned) above, 1023 - index below.  0 means no key.
__device__ __forceinline__ unsigned long long pack_best(int key, int loc) {
  return ((unsigned long long)((unsigned)key ^ 0x80000000u) << 32) | (unsigned)(1023 - loc);
}

struct CclTile {
  // Union-find over run ids (column * 32 + first row).  Two run starts of
  // one column are at least two rows apart, so start >> 1 gives every run
  // its own 64-bit slot: once every run knows its root, lab64 holds the
  // per-root reduction (pack_best), and each run parks its own best in
  // key64 at its start (its pixels' keys are read by then).
  union {
    int lab[kTile * kTile];
    unsigned long long lab64[kTile * kTile / 2];
  };
  union {
    int key[kTile * kTile];  // per pixel: depth key (INT_MIN: none)
    unsigned long long key64[kTile * kTile / 2];
  };
  int16_t root[kTile * kTile];  // per pixel: local root, -1 for non-flats
  uint32_t starts[kTile];       // run starts of each column
};

// One warp per tile.  Each lane owns one column's flat mask (32 bits): a
// vertical run of flats is connected by construction, so the union-find only
// runs over runs, uniting each run with the runs of the next column that
// touch it (8-connectivity = its extent grown by one row).  Every pixel then
// takes the root of its run; each tile-local component is reduced to its
// maximum depth and the smallest pixel attaining it.
__global__ void __launch_bounds__(kCclWarps * 32)
ccl_tile_kernel(int *__restrict__ L, int *__restrict__ lmax, int *__restrict__ larg,
                unsigned long long *__restrict__ best,
                int *__restrict__ roots, int *__restrict__ nroots,
                uint4 *__restrict__ edges,
                const int32_t *__restrict__ flats, const float *__restrict__ orig,
                const float *__restrict__ filled, int64_t m, int64_t n, int tm, int tn) {
  __shared__ CclTile tiles[kCclWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  CclTile &t = tiles[warp];
  const int T = tm * tn;
  for (int tile = blockIdx.x * kCclWarps + warp; tile < T; tile += gridDim.x * kCclWarps) {
    const int ti = tile % tm, tj = tile / tm;
    const int64_t i0 = (int64_t)ti * kTile, j0 = (int64_t)tj * kTile;
    const int64_t i = i0 + lane;  // lane = row for the per-pixel phases
    uint32_t my_mask = 0;
    // Eight columns at a time: every load of the batch is issued (from a
    // clamped, always valid address) before any result is used.
    const int64_t icl = i < m ? i : m - 1;
    for (int j8 = 0; j8 < kTile; j8 += 8) {
      int fv[8];
      float fl[8], og[8];
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const int64_t j = j0 + j8 + u;
        const int64_t p = (j < n ? j : n - 1) * m + icl;
        fv[u] = flats[p];
        fl[u] = filled[p];
        og[u] = orig[p];
      }
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const int jj = j8 + u;
        const bool f = i < m && j0 + jj < n && (fv[u] & 1);
        int k = INT_MIN;
        if (f) {
          const float d = __fsub_rn(fl[u], og[u]);
          if (!isnan(d)) k = ordered_key(d);
        }
        t.key[jj * kTile + lane] = k;
        t.root[jj * kTile + lane] = -1;
        const uint32_t b = __ballot_sync(0xffffffffu, f);
        if (lane == jj) my_mask = b;
      }
    }
    {  // the tile's edge flat masks for the border pass: top and bottom row
       // (bit = column), left and right column (bit = row)
      const uint32_t top = __ballot_sync(0xffffffffu, my_mask & 1u);
      const uint32_t bottom = __ballot_sync(0xffffffffu, (my_mask >> 31) & 1u);
      const uint32_t left = __shfl_sync(0xffffffffu, my_mask, 0);
      const uint32_t right = __shfl_sync(0xffffffffu, my_mask, kTile - 1);
      if (lane == 0) edges[tile] = make_uint4(top, bottom, left, right);
    }
    // Tiles without flats (most of them) and tiles that are flat throughout
    // (inside large flats) take short paths with the same results as the
    // general one below.
    const bool full = i0 + kTile <= m && j0 + kTile <= n;
    if (!__any_sync(0xffffffffu, my_mask != 0)) {
      __syncwarp();  // no labels: L is only ever read at flat pixels
      continue;
    }
    if (full && __all_sync(0xffffffffu, my_mask == 0xffffffffu)) {
      // one component; its root is run 0 (column 0, row 0) at pixel (i0, j0)
      int kmax = INT_MIN;
      for (int jj = 0; jj < kTile; jj++) kmax = max(kmax, t.key[jj * kTile + lane]);
      kmax = __reduce_max_sync(0xffffffffu, kmax);
      int first = INT_MAX;  // smallest tile index attaining the maximum
      if (kmax != INT_MIN)
        for (int jj = 0; jj < kTile; jj++)
          if (t.key[jj * kTile + lane] == kmax) {
            first = jj * kTile + lane;
            break;
          }
      first = __reduce_min_sync(0xffffffffu, first);
      const int64_t rootp = j0 * m + i0;
      for (int jj = 0; jj < kTile; jj++) {
        const int64_t gp = (j0 + jj) * m + i;
        L[gp] = (int)rootp;
        if (jj || lane) larg[gp] = -1;
      }
      if (lane == 0) {
        lmax[rootp] = kmax;
        larg[rootp] = first == INT_MAX
                          ? INT_MAX
                          : (int)((j0 + first / kTile) * m + (i0 + first % kTile));
        best[rootp] = 0ULL;
        roots[atomicAdd(nroots, 1)] = (int)rootp;
      }
      __syncwarp();
      continue;
    }
    // lane = column c from here to the unions
    const uint32_t M = my_mask, S = M & ~(M << 1);
    t.starts[lane] = S;
    for (uint32_t s = S; s; s &= s - 1) {
      const int r = __ffs(s) - 1;
      t.lab[lane * kTile + r] = lane * kTile + r;
    }
    __syncwarp();
    const uint32_t M1 = __shfl_down_sync(0xffffffffu, M, 1);
    const uint32_t S1 = __shfl_down_sync(0xffffffffu, S, 1);
    if (lane < kTile - 1) {
      for (uint32_t rs = S1; rs; rs &= rs - 1) {
        const int s1 = __ffs(rs) - 1;
        const uint32_t rm = run_mask(M1, s1);
        uint32_t ov = M & (rm | (rm << 1) | (rm >> 1));
        while (ov) {
          const int s0 = run_start(S, __ffs(ov) - 1);
          sunion(t.lab, lane * kTile + s0, (lane + 1) * kTile + s1);
          ov &= ~run_mask(M, s0);
        }
      }
    }
    __syncwarp();
    // lane = column: every pixel of a run takes the run's root, and the run
    // parks its best (largest key, first pixel attaining it) at its start
    for (uint32_t s = S; s; s &= s - 1) {
      const int s0 = __ffs(s) - 1;
      const int r = sfind(t.lab, lane * kTile + s0);
      int km = INT_MIN, kl = 0;
      for (uint32_t b = run_mask(M, s0); b; b &= b - 1) {
        const int loc = lane * kTile + __ffs(b) - 1;
        t.root[loc] = (int16_t)r;
        const int k = t.key[loc];
        if (k > km) {  // strictly: the first (smallest) pixel keeps a tie
          km = k;
          kl = loc;
        }
      }
      t.key64[(lane * kTile + s0) >> 1] = km == INT_MIN ? 0ULL : pack_best(km, kl);
    }
    __syncwarp();
    {  // local roots: clear their reduction slot and list them (one
       // reservation per tile, lane = column)
      uint32_t rs = 0;
      for (uint32_t s = S; s; s &= s - 1) {
        const int loc = lane * kTile + __ffs(s) - 1;
        if (t.root[loc] == loc) {
          t.lab64[loc >> 1] = 0ULL;
          rs |= s & (~s + 1u);
        }
      }
      const int mine = __popc(rs);
      int incl = mine;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      int base = 0;
      if (lane == 0 && total) base = atomicAdd(nroots, total);
      base = __shfl_sync(0xffffffffu, base, 0) + incl - mine;
      for (uint32_t b = rs; b; b &= b - 1)
        roots[base++] = (int)((j0 + lane) * m + (i0 + __ffs(b) - 1));
    }
    __syncwarp();
    // one 64-bit maximum per run folds its best into its root
    for (uint32_t s = S; s; s &= s - 1) {
      const int loc = lane * kTile + __ffs(s) - 1;
      const unsigned long long v = t.key64[loc >> 1];
      if (v) atomicMax(&t.lab64[t.root[loc] >> 1], v);
    }
    __syncwarp();
    // lane = row: labels and the roots' maximum / argmax, coalesced per column
    for (int jj = 0; jj < kTile; jj++) {
      const int64_t j = j0 + jj;
      const bool in = i < m && j < n;
      const int64_t gp = j * m + i;
      const int loc = jj * kTile + lane;
      const int r = t.root[loc];
      if (!in || r < 0) continue;  // L is only ever read at flat pixels
      if (r == loc) {
        const unsigned long long v = t.lab64[loc >> 1];
        const int a = 1023 - (int)(v & 1023u);
        lmax[gp] = v ? (int)((unsigned)(v >> 32) ^ 0x80000000u) : INT_MIN;
        larg[gp] = v ? (int)((j0 + a / kTile) * m + (i0 + a % kTile)) : INT_MAX;
        best[gp] = 0ULL;
      } else {
        larg[gp] = -1;  // not a local root
      }
      L[gp] = (int)((j0 + r / kTile) * m + (i0 + r % kTile));
    }
    __syncwarp();
  }
}

// Edges that cross tile borders, from the tiles' edge masks (one thread per
// tile; bit k of a row mask is column k, of a column mask row k).  Flat
// pixels next to each other along one tile edge are already connected
// inside the tile, so a border needs one union per pair of touching runs
// (8-connectivity: a run on one side touches the other side's pixels from
// one position before its start to one after its end), not one per pixel.
// Per tile: the border with the tile below (its bottom row against their
// top row), the border with the tile to the right (right column against
// their left column), and the two corners: (31, 31) against (0, 0) of the
// tile below-right, (31, 0) against (0, 31) of the tile below-left.
__device__ void unite_runs(int *L, uint32_t a, uint32_t b, int64_t pa0, int64_t pa_step,
                           int64_t pb0, int64_t pb_step) {
  const uint32_t sb = b & ~(b << 1);  // run starts of b
  for (uint32_t ra = a & ~(a << 1); ra; ra &= ra - 1) {
    const int s0 = __ffs(ra) - 1;
    const uint32_t rm = run_mask(a, s0);
    uint32_t ov = b & (rm | (rm << 1) | (rm >> 1));
    while (ov) {
      const int t0 = run_start(sb, __ffs(ov) - 1);
      uf_union(L, (int)(pa0 + s0 * pa_step), (int)(pb0 + t0 * pb_step));
      ov &= ~run_mask(b, t0);
    }
  }
}

__global__ void ccl_border_kernel(int *__restrict__ L, const uint4 *__restrict__ edges,
                                  int64_t m, int tm, int tn) {
  const int T = tm * tn;
  for (int tile = blockIdx.x * blockDim.x + threadIdx.x; tile < T;
       tile += gridDim.x * blockDim.x) {
    const int ti = tile % tm, tj = tile / tm;
    const int64_t i0 = (int64_t)ti * kTile, j0 = (int64_t)tj * kTile;
    const uint4 e = edges[tile];  // top, bottom, left, right
    if (ti + 1 < tm) {
      const uint4 d = edges[tile + 1];  // the tile below
      if (e.y && d.x)  // bottom row (i0 + 31, j0 + k) against row i0 + 32
        unite_runs(L, e.y, d.x, j0 * m + i0 + kTile - 1, m, j0 * m + i0 + kTile, m);
      if (tj + 1 < tn && (e.y >> 31) && (edges[tile + 1 + tm].x & 1u))
        uf_union(L, (int)((j0 + kTile - 1) * m + i0 + kTile - 1),
                 (int)((j0 + kTile) * m + i0 + kTile));
      if (tj > 0 && (e.y & 1u) && (edges[tile + 1 - tm].x >> 31))
        uf_union(L, (int)(j0 * m + i0 + kTile - 1), (int)((j0 - 1) * m + i0 + kTile));
    }
    if (tj + 1 < tn) {
      const uint4 r = edges[tile + tm];  // the tile to the right
      if (e.w && r.z)  // right column (i0 + k, j0 + 31) against column j0 + 32
        unite_runs(L, e.w, r.z, (j0 + kTile - 1) * m + i0, 1, (j0 + kTile) * m + i0, 1);
    }
  }
}

// A component's maximum depth key and the smallest pixel attaining it,
// packed so that one 64-bit maximum over its local roots reduces both: the
// key (sign flipped to order as unsigned) above, 2^31 - 1 - pixel below.
// 0 means no key.
__device__ __forceinline__ unsigned long long pack_root(int key, int pixel) {
  return ((unsigned long long)((unsigned)key ^ 0x80000000u) << 32) |
         (unsigned)(0x7fffffff - pixel);
}
__device__ __forceinline__ int root_key(unsigned long long v) {
  return v ? (int)((unsigned)(v >> 32) ^ 0x80000000u) : INT_MIN;
}
__device__ __forceinline__ int root_arg(unsigned long long v) {
  return v ? 0x7fffffff - (int)(unsigned)(v & 0xffffffffu) : INT_MAX;
}

// Local roots (a compact list) fold their maximum and its first pixel into
// their global root with one 64-bit maximum, and then point straight at it,
// so any flat pixel p reaches its root in two steps: L[L[p]] (every label
// above a pixel is a local root).  The roots are final here (every union
// is done), and a label only ever moves down to the root, so pointing a
// local root at it while other threads still walk through it is safe.
__global__ void ccl_root_kernel(int *__restrict__ L, const int *__restrict__ lmax,
                                const int *__restrict__ larg, const int *__restrict__ roots,
                                const int *__restrict__ nroots,
                                unsigned long long *__restrict__ best) {
  const int K = *nroots;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x) {
    const int p = roots[k];
    const int R = uf_find(L, p);
    const int key = lmax[p];
    if (key != INT_MIN) atomicMax(&best[R], pack_root(key, larg[p]));
    atomicMin(&L[p], R);
  }
}

// Four pixels per thread: each level of the dependent gather (a pixel's
// local root, its global root, the root's maximum and argmax) is issued for
// all four before any result is used.  Labels are read at flat pixels only
// (the labelling writes none elsewhere); `conncomps` may be null (the
// pipeline needs the costs alone).
constexpr int kCostPer = 4;

template <bool SEED>
__global__ void costs_kernel(float *__restrict__ costs,
                             ptrdiff_t *__restrict__ conncomps, int *__restrict__ L,
                             const unsigned long long *__restrict__ best,
                             const int32_t *__restrict__ flats,
                             const float *__restrict__ orig,
                             const float *__restrict__ filled, int64_t N,
                             GwdtSeed seed, int64_t m, int64_t n, int tm) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p0 < N;
       p0 += kCostPer * stride) {
    int fv[kCostPer], l1[kCostPer], R[kCostPer], mk[kCostPer], am[kCostPer];
    float fl[kCostPer], og[kCostPer];
#pragma unroll
    for (int u = 0; u < kCostPer; u++) {
      const int64_t p = p0 + u * stride;
      fv[u] = p < N ? flats[p] : 0;
    }
    // the depths are read with the labels, at flat pixels only: the same
    // dependent level, two thirds fewer bytes where flats are a third
#pragma unroll
    for (int u = 0; u < kCostPer; u++) {
      const int64_t p = p0 + u * stride;
      const bool f = fv[u] & 1;
      l1[u] = f ? L[p] : -1;
      fl[u] = f ? filled[p] : 0.f;
      og[u] = f ? orig[p] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < kCostPer; u++) R[u] = l1[u] >= 0 ? L[l1[u]] : -1;
#pragma unroll
    for (int u = 0; u < kCostPer; u++) {
      const unsigned long long v = R[u] >= 0 ? best[R[u]] : 0ULL;
      mk[u] = root_key(v);
      am[u] = root_arg(v);
    }
#pragma unroll
    for (int u = 0; u < kCostPer; u++) {
      const int64_t p = p0 + u * stride;
      if (p >= N) continue;
      float c = 0.0f;
      ptrdiff_t lab = 0;
      if (R[u] >= 0) {
        const float maxd = key_to_float(mk[u]);
        const float depth = __fsub_rn(fl[u], og[u]);
        const float diff = __fsub_rn(maxd, depth);
        c = __double2float_rn(__dadd_rn((double)diff, 0.1));
        lab = (am[u] == INT_MAX) ? R[u] : am[u];
      }
      if (SEED) {  // the gwdt start (src/gwdt.c:296-308) instead of plain costs
        const int32_t f = fv[u];
        costs[p] = (f & 1) ? c * 0.5f : NAN;  // halved: c >= 0.1, exact
        seed.dist[p] = (f & 5) == 5 ? 1.0f : (f & 1) ? INFINITY : 0.0f;
        if ((f & 5) == 5) mark_tiles_near(seed.dirty, tm, p % m, p / m, m, n);
      } else {
        costs[p] = c;
      }
      if (conncomps) conncomps[p] = lab;
    }
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
                         cudaStream_t st, const GwdtSeed *seed) {
  const int64_t N = g.cells();
  Workspace &ws = workspace();
  const int T = g.tiles();
  if (!ws.reserve(4 * align_up((size_t)N * 4) + align_up((size_t)N * 8) +
                  align_up((size_t)T * 16) + 256))
    return TT_CUDA_ERR_ALLOC;
  int *nroots = (int *)ws.take(256);
  uint4 *edges = (uint4 *)ws.take((size_t)T * 16);
  int *roots = (int *)ws.take((size_t)N * 4);
  int *L = (int *)ws.take((size_t)N * 4);
  int *lmax = (int *)ws.take((size_t)N * 4);
  int *larg = (int *)ws.take((size_t)N * 4);
  unsigned long long *best = (unsigned long long *)ws.take((size_t)N * 8);
  const int grid = ew_grid(N);
  // one tile per warp: the block scheduler evens out tiles whose labelling
  // takes longer (many runs, many unions)
  const int tgrid = (int)std::min<int64_t>((T + kCclWarps - 1) / kCclWarps, INT_MAX);
  TT_CHECK(cudaMemsetAsync(nroots, 0, sizeof(int), st));
  TT_LAUNCH(ccl_tile_kernel, tgrid, kCclWarps * 32, 0, st, L, lmax, larg, best, roots,
            nroots, edges, flats, orig, filled, g.m, g.n, g.tm, g.tn);
  TT_LAUNCH(ccl_border_kernel, ew_grid(T), 256, 0, st, L, edges, g.m, g.tm, g.tn);
  TT_LAUNCH(ccl_root_kernel, grid, 256, 0, st, L, lmax, larg, roots, nroots, best);
  const int cgrid = (int)std::min<int64_t>((N + 1023) / 1024, (int64_t)sm_count() * 32);
  if (seed)
    TT_LAUNCH(costs_kernel<true>, cgrid, 256, 0, st, costs, conncomps, L, best,
              flats, orig, filled, N, *seed, g.m, g.n, g.tm);
  else
    TT_LAUNCH(costs_kernel<false>, cgrid, 256, 0, st, costs, conncomps, L, best,
              flats, orig, filled, N, GwdtSeed{nullptr, nullptr}, g.m, g.n, g.tm);
  TT_CHECK(cudaGetLastError());
  return TT_CUDA_SUCCESS;
}

}  // namespace tt
