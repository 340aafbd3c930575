// Receiver-forest kernels: flow accumulation (src/flow_accumulation.c:32-80),
// a topological node order for flow_routing_d8_carve
// (src/flow_routing.c:135-256), and the adjoint of weighted accumulation.
//
// The D8 directions define a forest (every pixel has at most one receiver).
// The reference walks it sequentially (a DFS for the order, then one pass in
// that order for the sums).  Here the forest is contracted in two levels:
//
//  1. Tile level (one 128-thread block per 32 x 32 tile, shared memory).
//     Pixels whose receiver lies outside their tile are the tile's exits E.
//     Inside a tile sums are taken with a "last arriver continues" walk:
//     every in-tile leaf starts a thread that adds its value into its
//     receiver and decrements the receiver's count of pending in-tile
//     donors; the thread that brings the count to zero owns the now-complete
//     receiver and continues downstream.
//     For each entry pixel (one with a donor in another tile) the walk also
//     records the exit its in-tile path reaches and the number of steps.
//  2. Coarse level (global memory).  The exits form a smaller forest
//     e -> exit reached from receiver(e); the same last-arriver walk runs on
//     it with global atomics.  A final tile pass injects each entry pixel's
//     inflow and repeats the in-tile walk to produce every pixel's total.
//
// Sums are exact: weights are converted to 64-bit fixed point with a
// power-of-two scale 2^k1 chosen from max|w| * N so no partial sum can
// overflow, and integer addition is associative, so the result is
// independent of the order of the walk and identical from run to run (no
// float atomics).  Unit weights use scale 1 (exact pixel counts).  Each
// total is rounded once to float32.
//
// One scale bounds the rounding of every weight by 2^-(k1+1) in absolute
// terms, which is too coarse for weights far below max|w| (a 1e-6 headwater
// weight beside unit weights on 2.7e8 pixels).  When the smallest nonzero
// |w| asks for a finer scale, the same contraction runs again at scales
// k1 + d, k1 + 2d, ... with sums taken modulo 2^64 (wrapping integer adds are
// still exact and associative).  Pass i's total X_i differs from
// 2^d * X_(i-1) by less than N * 2^d <= 2^61 units, so the 64-bit residue of
// X_i and that of X_(i-1) determine X_i exactly; the finest total, rebuilt
// from the exact first total and the per-pass corrections in double-double,
// is rounded once to float32.
//
// The node order sorts pixels by the length of their longest upstream path
// h (0 at sources): a receiver's h exceeds each donor's, so ascending h is a
// topological order.  h is computed by the same two-level walk with max
// instead of sum, then a counting sort places pixels by h.  Pixels with equal
// h have no mutual constraint; their relative order follows atomic slot
// reservation and may vary between runs.
//
// The adjoint grad_w(u) = sum of grad_acc over the path from u to its outlet
// is a root-ward path sum: pointer jumping inside each tile (10 synchronous
// rounds in shared memory) and over the exits, in float-float (two-float)
// arithmetic.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <type_traits>

#include <cuda/atomic>

#include "tt_internal.cuh"

namespace tt {
namespace {

constexpr int kTileCells = kTile * kTile;

enum : int {
  RL_NONE = -4,    // outside the grid (partial tile)
  RL_BADDIR = -3,  // direction points off the grid: treated as an outlet
  RL_EXIT = -2,    // receiver lies in another tile
  RL_ROOT = -1     // outlet or sink (direction 0)
};

enum : int { ERR_CYCLE = 1, ERR_BADDIR = 2, ERR_WEIGHT = 4 };

// One exit of the coarse forest, updated as a unit by a 128-bit
// compare-and-swap: a donor adds its total, raises the longest path and
// counts itself off in one atomic step, so the donor that takes `pend` to
// zero reads the complete totals from the swap itself.
struct __align__(16) CoarseCell {
  long long sum;  // fixed-point total (local, then with all coarse donors)
  int h;          // longest upstream path
  int pend;       // coarse donors not yet arrived
};

struct UpArgs {
  const uint8_t *dir;
  int64_t m, n;
  int tm, tn;
  unsigned order;
  const float *w;  // nullptr: unit weights
  int wshift;      // fixed-point scale 2^wshift
  int phase;       // 1: local pass (forest_up_kernel), 3: final pass (forest_fin_kernel)
  bool want_acc;
  bool want_h;
  CoarseCell *ccell;  // per exit id: sums, longest path, pending coarse donors
  CoarseCell *cell;   // per exit pixel: final totals, read by the final pass
  void *lacc;        // per pixel: in-tile (local) total, long long (int for unit counts)
  int16_t *lrl;      // per pixel: local receiver or RL_* code
  uint8_t *emask;    // per tile and ring pixel: directions of donors in other tiles
  int *xmap;        // per entry pixel: id of the exit reached in-tile, or -1
  int *xsteps;      // per entry pixel: steps to that exit
  int *elist;       // per exit id: the exit's pixel
  int *ecount;
  float *acc_out;
  long long *raw_out;  // when set: the fixed-point totals instead of acc_out
  int *count_out;  // unit weights: the exact count as int (or nullptr)
  int *h_out;
  int *hmax;
  int *err;
  // Deferred weighted sums: {passes, k1, d} computed on the device.  When
  // set, this launch is pass `pass` (scale k1 + pass * d); a pass at or past
  // `passes` does nothing, and a single-pass plan writes acc_out directly.
  const int *plan;
  int pass;
};

__device__ __forceinline__ bool pass_unused(const UpArgs &a) {
  return a.plan && a.pass >= a.plan[0];
}
__device__ __forceinline__ int pass_shift(const UpArgs &a) {
  return a.plan ? a.plan[1] + a.pass * a.plan[2] : a.wshift;
}

__device__ __forceinline__ long long to_fixed(float w, int k, int *err) {
  unsigned bits = __float_as_uint(w);
  int e = (bits >> 23) & 0xff;
  unsigned mant = bits & 0x7fffffu;
  if (e == 255) {
    atomicOr(err, ERR_WEIGHT);
    return 0;
  }
  if (e == 0)
    e = 1;
  else
    mant |= 0x800000u;
  int sh = e - 150 + k;  // value = mant * 2^(e-150)
  long long v;
  if (sh >= 0)  // modulo 2^64 (a multiple of 2^64 is 0) at the finer scales
    v = sh < 64 ? (long long)((unsigned long long)mant << sh) : 0;
  else if (sh > -40)
    v = ((long long)mant + (1LL << (-sh - 1))) >> (-sh);
  else
    v = 0;
  return (bits >> 31) ? (long long)(0ULL - (unsigned long long)v) : v;
}

// Receiver code of tile pixel (ii, jj).
__device__ __forceinline__ int local_receiver(const uint8_t (*dir)[36], int ii,
                                              int jj, int64_t i, int64_t j,
                                              int64_t m, int64_t n,
                                              unsigned order) {
  if (i >= m || j >= n) return RL_NONE;
  unsigned d = dir[jj + 1][ii + 1];
  if (d == 0) return RL_ROOT;
  int k = d8_bit(d);
  int di = d8_di(k, order), dj = d8_dj(k, order);
  int64_t gi = i + di, gj = j + dj;
  if (gi < 0 || gi >= m || gj < 0 || gj >= n) return RL_BADDIR;
  int ti = ii + di, tj = jj + dj;
  if (ti >= 0 && ti < kTile && tj >= 0 && tj < kTile) return tj * kTile + ti;
  return RL_EXIT;
}

// One 128-thread block per tile.
//  1. receivers (local index or RL_* code), the count of in-tile donors of
//     every pixel, initial values (weight); the 124 ring pixels, one per
//     thread, look for donors in other tiles and, in the final pass, add
//     their inflow;
//  2. "last arriver continues": every in-tile leaf starts a walk that adds
//     its value into its receiver and decrements the receiver's count of
//     pending donors; the walker that brings the count to zero owns the now
//     complete receiver and continues downstream.  No barriers, and every
//     pixel is owned exactly once unless it lies on or below a cycle;
//  3. every entry pixel (ring pixel with a donor in another tile) follows
//     its receivers to the in-tile terminal and records it with the number
//     of steps (first pass only).
constexpr int kUpThreads = 128;
// Resident blocks per SM for the two tile passes (up to 56 and 40
// registers a thread, no spills; shared memory allows 10 and 15): walks
// wait at block barriers for the block's longest chain, so more resident
// blocks keep the SM busy meanwhile.
constexpr int kUpBlocks = 9;
constexpr int kFinBlocks = 11;
constexpr int kRing = 4 * kTile - 4;  // 124 ring pixels

// Tile sums: 64-bit fixed point for weights, 32-bit pixel counts for unit
// weights (a count never exceeds the 2^31 - 1 pixels a grid may hold), which
// halves the local totals' traffic and the shared-memory atomics' width.
template <bool U32>
using AccT = typename std::conditional<U32, int, long long>::type;
__device__ __forceinline__ void acc_add(int *p, int v) { atomicAdd(p, v); }
__device__ __forceinline__ void acc_add(long long *p, long long v) {
  atomicAdd((unsigned long long *)p, (unsigned long long)v);
}

template <typename AT>
struct UpTile {
  uint8_t dir[kHalo][36];   // [c][r], one-pixel halo
  int16_t rl[kTileCells];   // local receiver or an RL_* code
  int16_t leaf[kTileCells];  // in-tile leaves, in the order the walks take them
  int pend[kTileCells];     // in-tile donors not yet arrived
  AT acc[kTileCells];
  int h[kTileCells];
  int nvalid;
  int owned;
  int bad;
  int nleaf;
  int next;  // next entry of `leaf` to walk
};

// Pixel index (jj * 32 + ii) of ring pixel k, 0 <= k < 124.
__device__ __forceinline__ int ring_pixel(int k) {
  if (k < kTile) return k * kTile;                      // ii = 0
  if (k < 2 * kTile) return (k - kTile) * kTile + kTile - 1;  // ii = 31
  if (k < 3 * kTile - 2) return k - 2 * kTile + 1;       // jj = 0, ii = 1..30
  return (kTile - 1) * kTile + (k - 3 * kTile + 3);     // jj = 31, ii = 1..30
}

// Receiver code of the pixel at tile position (ii, jj) with direction byte
// d, neighbour order ORDER.  `inner`: the tile and its one-pixel halo lie in
// the grid, so every receiver is on the grid.
template <unsigned ORDER>
__device__ __forceinline__ int tile_receiver(unsigned d, int ii, int jj, bool inner,
                                             int64_t i0, int64_t j0, int64_t m, int64_t n) {
  if (d == 0) return RL_ROOT;
  constexpr unsigned A = ORDER ? kD8B : kD8A, B = ORDER ? kD8A : kD8B;
  const int k = d8_bit(d);
  const int di = (int)((A >> (2 * k)) & 3u) - 1, dj = (int)((B >> (2 * k)) & 3u) - 1;
  const int ni = ii + di, nj = jj + dj;
  if (!inner) {
    const int64_t gi = i0 + ni, gj = j0 + nj;
    if (gi < 0 || gi >= m || gj < 0 || gj >= n) return RL_BADDIR;
  }
  if ((unsigned)ni < (unsigned)kTile && (unsigned)nj < (unsigned)kTile) return nj * kTile + ni;
  return RL_EXIT;
}

// Stages the tile's directions with a one-pixel halo (0 off the grid).
__device__ __forceinline__ void stage_dirs(uint8_t (*dir)[36], const uint8_t *__restrict__ g,
                                           int64_t i0, int64_t j0, int64_t m, int64_t n,
                                           bool inner, int tid) {
  constexpr int kL = (kHalo * kHalo + kUpThreads - 1) / kUpThreads;
  uint8_t v[kL];
  const uint8_t *base = g + (j0 - 1) * m + (i0 - 1);  // only dereferenced in the grid
#pragma unroll
  for (int u = 0; u < kL; u++) {
    const int e = tid + u * kUpThreads;
    const int c = e / kHalo, r = e % kHalo;
    if (inner) {
      v[u] = e < kHalo * kHalo ? base[(int64_t)c * m + r] : 0;
    } else {
      const int64_t i = i0 - 1 + r, j = j0 - 1 + c;
      v[u] = (e < kHalo * kHalo && i >= 0 && i < m && j >= 0 && j < n) ? g[j * m + i] : 0;
    }
  }
#pragma unroll
  for (int u = 0; u < kL; u++) {
    const int e = tid + u * kUpThreads;
    if (e < kHalo * kHalo) dir[e / kHalo][e % kHalo] = v[u];
  }
}

// Thread tid owns tile pixels e = tid + 128 u (u = 0..7): row ii = tid % 32,
// columns jj = tid / 32 + 4 u, so its global indices advance by 4 m.
constexpr int kPerThread = kTileCells / kUpThreads;  // 8

template <bool ACC, bool H, unsigned ORDER, bool U32>
__global__ void __launch_bounds__(kUpThreads, kUpBlocks) forest_up_kernel(UpArgs a) {
  using AT = AccT<U32>;
  __shared__ UpTile<AT> t;
  const int tid = threadIdx.x;
  const int ii = tid & (kTile - 1), jb = tid >> 5;
  const int T = a.tm * a.tn;
  if (pass_unused(a)) return;
  const int wshift = pass_shift(a);
  for (int tile = blockIdx.x; tile < T; tile += gridDim.x) {
    const int ti = tile % a.tm, tj = tile / a.tm;
    const int64_t i0 = (int64_t)ti * kTile, j0 = (int64_t)tj * kTile;
    const bool inner = i0 >= 1 && j0 >= 1 && i0 + kTile + 1 <= a.m && j0 + kTile + 1 <= a.n;
    stage_dirs(t.dir, a.dir, i0, j0, a.m, a.n, inner, tid);
#pragma unroll
    for (int u = 0; u < kPerThread; u++) t.pend[tid + u * kUpThreads] = 0;
    if (tid == 0) {
      t.nvalid = 0;
      t.owned = 0;
      t.bad = 0;
      t.nleaf = 0;
      t.next = 0;
    }
    __syncthreads();

    const int64_t g0 = (j0 + jb) * a.m + i0 + ii;  // global index of u = 0
    const int64_t gstep = 4 * a.m;
    const bool row_in = i0 + ii < a.m;
    int nvalid = 0, bad = 0;
#pragma unroll
    for (int u = 0; u < kPerThread; u++) {
      const int jj = jb + 4 * u, e = tid + u * kUpThreads;
      const bool in = inner || (row_in && j0 + jj < a.n);
      const int rl = in ? tile_receiver<ORDER>(t.dir[jj + 1][ii + 1], ii, jj, inner, i0, j0,
                                               a.m, a.n)
                        : RL_NONE;
      t.rl[e] = (int16_t)rl;
      bad |= rl == RL_BADDIR;
      if (rl >= 0) atomicAdd(&t.pend[rl], 1);
      if (ACC)
        t.acc[e] = !in ? AT(0)
                   : (U32 || !a.w) ? AT(1)
                                   : AT(to_fixed(a.w[g0 + u * gstep], wshift, a.err));
      if (H) t.h[e] = 0;
      nvalid += in;
    }
    if (nvalid) atomicAdd(&t.nvalid, nvalid);
    if (bad) t.bad = 1;
    __syncthreads();

    // Ring pixels with donors in other tiles (entry pixels).
    bool entry = false;
    int re = 0;
    if (tid < kRing) {
      re = ring_pixel(tid);
      const int ri = re % kTile, rj = re / kTile;
      unsigned ne = 0;
      if (t.rl[re] != RL_NONE) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
          constexpr unsigned A = ORDER ? kD8B : kD8A, B = ORDER ? kD8A : kD8B;
          const int di = (int)((A >> (2 * k)) & 3u) - 1, dj = (int)((B >> (2 * k)) & 3u) - 1;
          const int qr = ri + 1 - di, qc = rj + 1 - dj;  // halo coordinates of q
          if (qr >= 1 && qr <= kTile && qc >= 1 && qc <= kTile) continue;
          const unsigned dq = t.dir[qc][qr];
          if (dq != 0 && d8_bit(dq) == k) ne |= 1u << k;
        }
        entry = ne != 0;
      }
      a.emask[(size_t)tile * kRing + tid] = (uint8_t)ne;
    }
    // Leaves, listed before any walk starts (a walk empties counts).
#pragma unroll
    for (int u = 0; u < kPerThread; u++) {
      const int e = tid + u * kUpThreads;
      if (t.rl[e] != RL_NONE && t.pend[e] == 0) t.leaf[atomicAdd(&t.nleaf, 1)] = (int16_t)e;
    }
    __syncthreads();

    // Last arriver continues.  A thread whose walk ends takes the next leaf
    // from the list, so the threads of a warp stay busy until the list is
    // empty instead of each stepping through its own leaves' walks.
    int owned = 0;
    {
      const int nleaf = t.nleaf;
      int cur = -1;
      AT v = 0;
      int hv = 0;
      for (int guard = 0; guard < 2 * kTileCells + 2; guard++) {
        if (cur < 0) {
          const int k = atomicAdd(&t.next, 1);
          if (k >= nleaf) break;
          cur = t.leaf[k];
          if (ACC) v = t.acc[cur];
          if (H) hv = t.h[cur];
          owned++;
        }
        const int q = t.rl[cur];
        if (q < 0) {  // exit, outlet or grid edge: nothing further in-tile
          cur = -1;
          continue;
        }
        if (ACC) acc_add(&t.acc[q], v);
        if (H) atomicMax(&t.h[q], hv + 1);
        cuda::atomic_ref<int, cuda::thread_scope_block> pend(t.pend[q]);
        if (pend.fetch_sub(1, cuda::std::memory_order_acq_rel) != 1) {
          cur = -1;
          continue;
        }
        cur = q;  // every donor of q has arrived: q is complete
        owned++;
        if (ACC) v = t.acc[cur];
        if (H) hv = t.h[cur];
      }
    }
    if (owned) atomicAdd(&t.owned, owned);
    __syncthreads();
    if (tid == 0 && t.owned != t.nvalid) atomicOr(a.err, ERR_CYCLE);

#pragma unroll
    for (int u = 0; u < kPerThread; u++) {
      const int jj = jb + 4 * u, e = tid + u * kUpThreads;
      if (!(inner || (row_in && j0 + jj < a.n))) continue;
      const int64_t gp = g0 + u * gstep;
      if (ACC) static_cast<AT *>(a.lacc)[gp] = t.acc[e];  // local totals for the final pass
      if (H) a.h_out[gp] = t.h[e];
      const int rl = t.rl[e];
      a.lrl[gp] = (int16_t)rl;
      if (rl != RL_EXIT) continue;
      const int id = append_slot(a.ecount);  // dense exit ids
      a.ccell[id] = CoarseCell{ACC ? (long long)t.acc[e] : 0LL, H ? t.h[e] : 0, 0};
      a.elist[id] = (int)gp;
      t.pend[e] = id;  // the counts are spent: keep the exit's id there
    }
    __syncthreads();
    if (entry) {  // the in-tile terminal of an entry pixel and its distance
      int cur = re, steps = 0;
      for (; steps < kTileCells && t.rl[cur] >= 0; steps++) cur = t.rl[cur];
      const int x = t.rl[cur] == RL_EXIT ? t.pend[cur] : -1;
      const int64_t gp = (j0 + re / kTile) * a.m + (i0 + re % kTile);
      a.xmap[gp] = x;
      a.xsteps[gp] = steps;
    }
    if (tid == 0 && t.bad) atomicOr(a.err, ERR_BADDIR);
    __syncthreads();
  }
}

// Final pass: a pixel's total is its local total plus the inflow of every
// entry pixel whose in-tile path passes through it.  The first pass left the
// local totals, every pixel's receiver code and, per ring pixel, the
// directions of its donors in other tiles.  Each entry pixel (one thread per
// ring pixel) gathers its inflow from the coarse cells of those donors and
// walks its path to the terminal, adding the inflow and raising h to
// (longest path into the entry) + (steps walked).
template <typename AT>
struct FinTile {
  AT acc[kTileCells];
  int h[kTileCells];
  int16_t rl[kTileCells];
};

template <bool ACC, bool H, unsigned ORDER, bool U32>
__global__ void __launch_bounds__(kUpThreads, kFinBlocks) forest_fin_kernel(UpArgs a) {
  using AT = AccT<U32>;
  __shared__ FinTile<AT> t;
  const int tid = threadIdx.x;
  const int ii = tid & (kTile - 1), jb = tid >> 5;
  const int T = a.tm * a.tn;
  if (pass_unused(a)) return;
  const int wshift = pass_shift(a);
  // a deferred single-pass plan needs no combination: write floats
  long long *const raw_out = (a.plan && a.plan[0] == 1) ? nullptr : a.raw_out;
  int hm = 0;  // largest height this thread wrote, over all its tiles
  for (int tile = blockIdx.x; tile < T; tile += gridDim.x) {
    const int ti = tile % a.tm, tj = tile / a.tm;
    const int64_t i0 = (int64_t)ti * kTile, j0 = (int64_t)tj * kTile;
    const bool full = i0 + kTile <= a.m && j0 + kTile <= a.n;
    const bool row_in = i0 + ii < a.m;
    const int64_t g0 = (j0 + jb) * a.m + i0 + ii;
    const int64_t gstep = 4 * a.m;
#pragma unroll
    for (int u = 0; u < kPerThread; u++) {  // local totals and receivers
      const int e = tid + u * kUpThreads;
      const bool in = full || (row_in && j0 + jb + 4 * u < a.n);
      const int64_t gp = g0 + u * gstep;
      if (ACC) t.acc[e] = in ? static_cast<const AT *>(a.lacc)[gp] : AT(0);
      if (H) t.h[e] = in ? a.h_out[gp] : 0;
      t.rl[e] = in ? a.lrl[gp] : (int16_t)RL_NONE;
    }
    unsigned mask = 0;
    if (tid < kRing) mask = a.emask[(size_t)tile * kRing + tid];
    __syncthreads();

    if (mask) {  // an entry pixel: carry its inflow down its path
      const int re = ring_pixel(tid);
      const int64_t p = (j0 + re / kTile) * a.m + (i0 + re % kTile);
      long long inflow = 0;
      int hin = 0;
      for (unsigned mk = mask; mk; mk &= mk - 1) {
        const int k = __ffs(mk) - 1;
        constexpr unsigned A = ORDER ? kD8B : kD8A, B = ORDER ? kD8A : kD8B;
        const int di = (int)((A >> (2 * k)) & 3u) - 1, dj = (int)((B >> (2 * k)) & 3u) - 1;
        const CoarseCell cq = a.cell[p - dj * a.m - di];
        if (ACC) inflow += cq.sum;
        if (H) hin = max(hin, cq.h + 1);
      }
      int cur = re;
      for (int d = 0; d < kTileCells; d++) {
        if (ACC && inflow) acc_add(&t.acc[cur], (AT)inflow);
        if (H) atomicMax(&t.h[cur], hin + d);
        const int q = t.rl[cur];
        if (q < 0) break;
        cur = q;
      }
    }
    __syncthreads();

#pragma unroll
    for (int u = 0; u < kPerThread; u++) {
      const int e = tid + u * kUpThreads;
      if (!(full || (row_in && j0 + jb + 4 * u < a.n))) continue;
      const int64_t gp = g0 + u * gstep;
      if (ACC) {
        if (a.count_out) {
          a.count_out[gp] = (int)t.acc[e];
        } else if (raw_out) {
          raw_out[gp] = t.acc[e];
        } else {
          const float v = U32 ? __int2float_rn((int)t.acc[e]) : __ll2float_rn(t.acc[e]);
          a.acc_out[gp] = wshift ? ldexpf(v, -wshift) : v;
        }
      }
      if (H) {
        a.h_out[gp] = t.h[e];
        hm = max(hm, t.h[e]);
      }
    }
    __syncthreads();
  }
  // One atomic per warp on the shared maximum, not one per thread and tile.
  if (H) {
    hm = __reduce_max_sync(0xffffffffu, hm);
    if ((tid & 31) == 0 && hm) atomicMax(a.hmax, hm);
  }
}

__device__ __forceinline__ int64_t receiver_of(const uint8_t *dir, int64_t p,
                                               int64_t m, unsigned order) {
  unsigned d = dir[p];
  int k = d8_bit(d);
  int64_t i = p % m, j = p / m;
  return (j + d8_dj(k, order)) * m + (i + d8_di(k, order));
}

// Coarse links, over exit ids: link(e) = {next exit, hops}, the exit
// reached in-tile from receiver(e) and 1 + the steps to it.
__global__ void coarse_link_kernel(const int *__restrict__ elist,
                                   const int *__restrict__ ecount,
                                   const uint8_t *__restrict__ dir, int64_t m,
                                   unsigned order, const int *__restrict__ xmap,
                                   const int *__restrict__ xsteps,
                                   int2 *__restrict__ link,
                                   CoarseCell *__restrict__ ccell) {
  const int E = *ecount;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < E; a += gridDim.x * blockDim.x) {
    const int64_t r = receiver_of(dir, elist[a], m, order);
    const int nx = xmap[r];
    link[a] = make_int2(nx, 1 + xsteps[r]);
    if (nx >= 0) atomicAdd(&ccell[nx].pend, 1);
  }
}

// Lists the exits without coarse donors and packs every exit's coarse
// in-degree into the high half of its link's hop count (hops <= 1025).
__global__ void coarse_leaves_kernel(const int *__restrict__ ecount,
                                     const CoarseCell *__restrict__ ccell,
                                     int2 *__restrict__ link, int *__restrict__ leaves,
                                     int *__restrict__ lcount) {
  const int E = *ecount;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < E; a += gridDim.x * blockDim.x) {
    const int pend = ccell[a].pend;
    link[a].y |= pend << 16;
    if (pend == 0) leaves[append_slot(lcount)] = a;
  }
}

// Relaxed 128-bit compare-and-swap: (lo, hi) holds the expected value on
// entry and the value found on return.
__device__ __forceinline__ void cas128(CoarseCell *p, unsigned long long &lo,
                                       unsigned long long &hi, unsigned long long nlo,
                                       unsigned long long nhi) {
  asm volatile(
      "{\n\t.reg .b128 c, v, d;\n\tmov.b128 c, {%0, %1};\n\tmov.b128 v, {%2, %3};\n\t"
      "atom.global.cas.b128 d, [%4], c, v;\n\tmov.b128 {%0, %1}, d;\n\t}"
      : "+l"(lo), "+l"(hi)
      : "l"(nlo), "l"(nhi), "l"(p)
      : "memory");
}

// Last-arriver walk over the exits: a walker owns a complete exit, folds its
// totals into the next exit downstream with one compare-and-swap, and
// continues only if it was the last donor to arrive.  The next exit's link
// is loaded together with its cell, so a hop costs two dependent accesses;
// into an exit with a single coarse donor (most hops along a river) the
// walker is the only arrival, so it combines and stores without the swap:
// one dependent access per hop.
__global__ void coarse_walk_kernel(const int *__restrict__ leaves,
                                   const int *__restrict__ lcount,
                                   const int2 *__restrict__ link,
                                   CoarseCell *ccell, int *processed, int limit) {
  const int L = *lcount;
  int n_done = 0;  // exits this thread completed, over all its leaves
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < L; a += gridDim.x * blockDim.x) {
    const int e0 = leaves[a];
    // A leaf has no coarse donors: its cell was completed by earlier kernels.
    const longlong2 c0 = __ldcg(reinterpret_cast<const longlong2 *>(&ccell[e0]));
    long long v = c0.x;
    int hv = (int)(unsigned)(unsigned long long)c0.y;
    int2 l = link[e0];
    for (int guard = 0; guard < limit; guard++) {
      n_done++;
      const int nx = l.x;
      if (nx < 0) break;
      const longlong2 g = __ldcg(reinterpret_cast<const longlong2 *>(&ccell[nx]));
      const int2 ln = link[nx];
      const int hops = l.y & 0xffff;
      if ((ln.y >> 16) == 1) {  // the only coarse donor of nx: no other writer
        const long long sum = g.x + v;
        const int h = max((int)(unsigned)(unsigned long long)g.y, hv + hops);
        __stcg(reinterpret_cast<longlong2 *>(&ccell[nx]),
               make_longlong2(sum, (long long)(unsigned long long)(unsigned)h));
        v = sum;
        hv = h;
        l = ln;
        continue;
      }
      unsigned long long lo = (unsigned long long)g.x, hi = (unsigned long long)g.y;
      unsigned long long nlo, nhi;
      for (;;) {
        const int oh = (int)(unsigned)hi, op = (int)(unsigned)(hi >> 32);
        nlo = lo + (unsigned long long)v;
        nhi = (unsigned long long)(unsigned)max(oh, hv + hops) |
              ((unsigned long long)(unsigned)(op - 1) << 32);
        const unsigned long long elo = lo, ehi = hi;
        cas128(&ccell[nx], lo, hi, nlo, nhi);
        if (lo == elo && hi == ehi) break;  // swapped
      }
      if ((int)(unsigned)(hi >> 32) != 1) break;  // other donors still to come
      v = (long long)nlo;  // every donor of nx has arrived: its totals are final
      hv = (int)(unsigned)nhi;
      l = ln;
    }
  }
  // One atomic per warp on the shared count, not one per leaf.
  n_done = __reduce_add_sync(0xffffffffu, n_done);
  if ((threadIdx.x & 31) == 0 && n_done) atomicAdd(processed, n_done);
}

// Final exit totals back to pixel-indexed cells for the final tile pass.
__global__ void coarse_scatter_kernel(const int *__restrict__ ecount,
                                      const int *__restrict__ elist,
                                      const CoarseCell *__restrict__ ccell,
                                      CoarseCell *__restrict__ cell) {
  const int E = *ecount;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < E; a += gridDim.x * blockDim.x)
    cell[elist[a]] = ccell[a];
}

// ------------------------------------------------------------------
// Node order: histogram of h, exclusive scan, scatter.
// ------------------------------------------------------------------
constexpr int kSmallBins = 256;

// Bins of the height histogram, read on the device from the maximum height
// of the contraction: heights 0 .. hmax, never more than N.  Heights outside
// the bins (only possible when the contraction reported a cycle) are skipped.
__device__ __forceinline__ int height_bins(const int *hmax, int64_t N) {
  const int64_t H = (int64_t)*hmax + 1;
  return (int)(H < N ? (H > 0 ? H : 0) : N);
}

__global__ void clear_bins_kernel(int *__restrict__ hist, int *__restrict__ cursor,
                                  const int *__restrict__ hmax, int64_t N) {
  const int H = height_bins(hmax, N);
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < H; b += gridDim.x * blockDim.x) {
    hist[b] = 0;
    cursor[b] = 0;
  }
}

__global__ void h_hist_kernel(const int *__restrict__ h, int64_t N,
                              int *__restrict__ hist, const int *__restrict__ hmax) {
  __shared__ int sb[kSmallBins];
  const int H = height_bins(hmax, N);
  for (int b = threadIdx.x; b < kSmallBins; b += blockDim.x) sb[b] = 0;
  __syncthreads();
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    int v = h[p];
    if ((unsigned)v >= (unsigned)H) continue;
    if (v < kSmallBins) {
      atomicAdd(&sb[v], 1);
    } else {
      unsigned grp = __match_any_sync(__activemask(), v);
      int leader = __ffs(grp) - 1;
      if ((int)(threadIdx.x & 31) == leader) atomicAdd(&hist[v], __popc(grp));
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kSmallBins; b += blockDim.x)
    if (sb[b]) atomicAdd(&hist[b], sb[b]);
}

// Exclusive scan of the height bins by one block of 1024 threads.
__global__ void __launch_bounds__(1024) scan_kernel(const int *__restrict__ in,
                                                    int *__restrict__ out,
                                                    const int *__restrict__ hmax, int64_t N) {
  __shared__ int part[1024];
  const int tid = threadIdx.x;
  const int n = height_bins(hmax, N);
  const int chunk = (n + 1023) / 1024;
  const int b0 = tid * chunk, b1 = min(n, b0 + chunk);
  int s = 0;
  for (int k = b0; k < b1; k++) s += in[k];
  part[tid] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    int v = tid >= off ? part[tid - off] : 0;
    __syncthreads();
    part[tid] += v;
    __syncthreads();
  }
  int run = tid > 0 ? part[tid - 1] : 0;
  for (int k = b0; k < b1; k++) {
    int v = in[k];
    out[k] = run;
    run += v;
  }
}

constexpr int kScatterPer = 8;  // elements per thread per chunk

__global__ void node_scatter_kernel(const int *__restrict__ h, int64_t N,
                                    const int *__restrict__ off,
                                    int *__restrict__ cursor,
                                    ptrdiff_t *__restrict__ node,
                                    const int *__restrict__ hmax) {
  __shared__ int cnt[kSmallBins];
  __shared__ int base[kSmallBins];
  const int H = height_bins(hmax, N);
  // Chunks of blockDim * kScatterPer pixels: count small bins in shared
  // memory, reserve each bin's range once per chunk, then place.
  const int64_t chunk = (int64_t)blockDim.x * kScatterPer;
  for (int64_t start = (int64_t)blockIdx.x * chunk; start < N;
       start += (int64_t)gridDim.x * chunk) {
    for (int b = threadIdx.x; b < kSmallBins; b += blockDim.x) cnt[b] = 0;
    __syncthreads();
    int v[kScatterPer], rank[kScatterPer];
#pragma unroll
    for (int u = 0; u < kScatterPer; u++) {
      const int64_t p = start + (int64_t)u * blockDim.x + threadIdx.x;
      v[u] = p < N ? h[p] : -1;
      if (v[u] >= H) v[u] = -1;
    }
#pragma unroll
    for (int u = 0; u < kScatterPer; u++)
      rank[u] = (v[u] >= 0 && v[u] < kSmallBins) ? atomicAdd(&cnt[v[u]], 1) : 0;
    __syncthreads();
    for (int b = threadIdx.x; b < kSmallBins; b += blockDim.x)
      base[b] = cnt[b] ? atomicAdd(&cursor[b], cnt[b]) : 0;
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kScatterPer; u++) {
      const int64_t p = start + (int64_t)u * blockDim.x + threadIdx.x;
      const int hv = v[u];
      if (hv < 0) continue;
      int slot;
      if (hv < kSmallBins) {
        slot = base[hv] + rank[u];
      } else {
        const unsigned grp = __match_any_sync(__activemask(), hv);
        const int leader = __ffs(grp) - 1;
        const int lane = threadIdx.x & 31;
        int b0 = 0;
        if (lane == leader) b0 = atomicAdd(&cursor[hv], __popc(grp));
        b0 = __shfl_sync(grp, b0, leader);
        slot = b0 + __popc(grp & ((1u << lane) - 1));
      }
      node[off[hv] + slot] = (ptrdiff_t)p;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------
// Adjoint: root-ward path sums in float-float.
// ------------------------------------------------------------------
struct FF {
  float hi, lo;
};

__device__ __forceinline__ FF ff_add(FF a, FF b) {
  float s = __fadd_rn(a.hi, b.hi);
  float bb = __fsub_rn(s, a.hi);
  float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  float lo = __fadd_rn(__fadd_rn(err, a.lo), b.lo);
  float hi = __fadd_rn(s, lo);
  lo = __fsub_rn(lo, __fsub_rn(hi, s));
  return {hi, lo};
}

struct DownArgs {
  const uint8_t *dir;
  const float *g;  // grad_acc
  int64_t m, n;
  int tm, tn;
  unsigned order;
  int phase;     // 1: coarse inputs, 3: output
  float *clhi;   // per entry pixel: path sum to its in-tile end
  float *cllo;
  int *cx;       // per entry pixel: exit reached, or -1
  int *eidx;     // per exit: its index in elist
  int *elist;
  int *ecount;
  const float *Dhi;  // per exit index: sum from its receiver to the outlet
  const float *Dlo;
  float *out;
  int *err;
};

struct DownTile {
  uint8_t dir[kHalo][36];
  int16_t rl[kTileCells];
  float hi[2][kTileCells];
  float lo[2][kTileCells];
  int16_t nx[2][kTileCells];
  int16_t last[2][kTileCells];
};

constexpr int kDownThreads = 128;

__global__ void __launch_bounds__(kDownThreads) forest_down_kernel(DownArgs a) {
  __shared__ DownTile t;
  const int tid = threadIdx.x;
  const int T = a.tm * a.tn;
  for (int tile = blockIdx.x; tile < T; tile += gridDim.x) {
    const int ti = tile % a.tm, tj = tile / a.tm;
    const int64_t i0 = (int64_t)ti * kTile, j0 = (int64_t)tj * kTile;
    {  // stage the directions with every load in flight at once
      constexpr int kL = (kHalo * kHalo + kDownThreads - 1) / kDownThreads;
      uint8_t v[kL];
#pragma unroll
      for (int u = 0; u < kL; u++) {
        const int e = tid + u * kDownThreads;
        const int c = e / kHalo, r = e % kHalo;
        const int64_t i = i0 - 1 + r, j = j0 - 1 + c;
        v[u] = (e < kHalo * kHalo && i >= 0 && i < a.m && j >= 0 && j < a.n) ? a.dir[j * a.m + i] : 0;
      }
#pragma unroll
      for (int u = 0; u < kL; u++) {
        const int e = tid + u * kDownThreads;
        if (e < kHalo * kHalo) t.dir[e / kHalo][e % kHalo] = v[u];
      }
    }
    __syncthreads();
    int bad = 0;
    for (int e = tid; e < kTileCells; e += kDownThreads) {
      const int ii = e % kTile, jj = e / kTile;
      const int64_t i = i0 + ii, j = j0 + jj;
      const int rl = local_receiver(t.dir, ii, jj, i, j, a.m, a.n, a.order);
      bad |= rl == RL_BADDIR;
      t.rl[e] = (int16_t)rl;
      t.hi[0][e] = (rl != RL_NONE) ? a.g[j * a.m + i] : 0.0f;
      t.lo[0][e] = 0.0f;
      t.nx[0][e] = (int16_t)(rl >= 0 ? rl : -1);
      t.last[0][e] = (int16_t)e;
    }
    if (__syncthreads_or(bad) && tid == 0) atomicOr(a.err, ERR_BADDIR);
    // Synchronous pointer jumping (double buffered): sum of g from each pixel
    // to the end of its in-tile path, and that end pixel.
    int cur = 0;
    for (int round = 0; round < 10; round++) {
      int moved = 0;
      for (int e = tid; e < kTileCells; e += kDownThreads) {
        const int q = t.nx[cur][e];
        FF v{t.hi[cur][e], t.lo[cur][e]};
        int nq = -1, lq = t.last[cur][e];
        if (q >= 0) {
          v = ff_add(v, FF{t.hi[cur][q], t.lo[cur][q]});
          nq = t.nx[cur][q];
          lq = t.last[cur][q];
          moved |= nq >= 0;
        }
        t.hi[cur ^ 1][e] = v.hi;
        t.lo[cur ^ 1][e] = v.lo;
        t.nx[cur ^ 1][e] = (int16_t)nq;
        t.last[cur ^ 1][e] = (int16_t)lq;
      }
      cur ^= 1;
      if (!__syncthreads_or(moved)) break;
    }
    int cyc = 0;
    for (int e = tid; e < kTileCells; e += kDownThreads) cyc |= t.nx[cur][e] >= 0;
    if (__syncthreads_or(cyc) && tid == 0) atomicOr(a.err, ERR_CYCLE);
    for (int e = tid; e < kTileCells; e += kDownThreads) {
      const int ii = e % kTile, jj = e / kTile;
      const int64_t i = i0 + ii, j = j0 + jj;
      if (i >= a.m || j >= a.n) continue;
      const int64_t gp = j * a.m + i;
      const int x = t.last[cur][e];
      int64_t ge = -1;
      if (t.rl[x] == RL_EXIT) ge = (j0 + x / kTile) * a.m + (i0 + x % kTile);
      if (a.phase == 1) {
        if (t.rl[e] == RL_EXIT) {
          const int slot = append_slot(a.ecount);
          a.eidx[gp] = slot;
          a.elist[slot] = (int)gp;
        }
        // Entry pixel: some neighbour in another tile drains here.
        bool entry = false;
#pragma unroll
        for (int k = 0; k < 8; k++) {
          const int di = d8_di(k, a.order), dj = d8_dj(k, a.order);
          const int qr = ii + 1 - di, qc = jj + 1 - dj;
          if (qr >= 1 && qr <= kTile && qc >= 1 && qc <= kTile) continue;
          const unsigned dq = t.dir[qc][qr];
          if (dq && d8_bit(dq) == k) entry = true;
        }
        if (entry) {
          a.clhi[gp] = t.hi[cur][e];
          a.cllo[gp] = t.lo[cur][e];
          a.cx[gp] = (int)ge;
        }
      } else {
        FF v{t.hi[cur][e], t.lo[cur][e]};
        if (ge >= 0) {
          const int ex = a.eidx[ge];
          v = ff_add(v, FF{a.Dhi[ex], a.Dlo[ex]});
        }
        a.out[gp] = __fadd_rn(v.hi, v.lo);
      }
    }
    __syncthreads();
  }
}

// D(e) = path sum from receiver(e) to its outlet:
//   D(e) = lps(receiver(e)) + D(exit reached from receiver(e)).
__global__ void down_init_kernel(const int *__restrict__ elist,
                                 const int *__restrict__ ecount,
                                 const uint8_t *__restrict__ dir, int64_t m,
                                 unsigned order, const float *__restrict__ clhi,
                                 const float *__restrict__ cllo,
                                 const int *__restrict__ cx,
                                 const int *__restrict__ eidx,
                                 float *Dhi, float *Dlo, int *nx) {
  const int E = *ecount;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < E; a += gridDim.x * blockDim.x) {
    int e = elist[a];
    int64_t r = receiver_of(dir, e, m, order);
    Dhi[a] = clhi[r];
    Dlo[a] = cllo[r];
    int x = cx[r];
    nx[a] = x >= 0 ? eidx[x] : -1;
  }
}

__global__ void down_jump_kernel(const int *__restrict__ ecount,
                                 const float *__restrict__ Dhi0,
                                 const float *__restrict__ Dlo0,
                                 const int *__restrict__ nx0, float *Dhi1,
                                 float *Dlo1, int *nx1, int *active) {
  const int E = *ecount;
  int act = 0;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < E; a += gridDim.x * blockDim.x) {
    int q = nx0[a];
    FF v{Dhi0[a], Dlo0[a]};
    int nq = -1;
    if (q >= 0) {
      v = ff_add(v, FF{Dhi0[q], Dlo0[q]});
      nq = nx0[q];
    }
    Dhi1[a] = v.hi;
    Dlo1[a] = v.lo;
    nx1[a] = nq;
    act |= nq >= 0;
  }
  if (__any_sync(__activemask(), act) && (threadIdx.x & 31) == 0) atomicAdd(active, 1);
}

// out[0] = bits of the largest |w| (NaN/INF sort above every finite
// value), out[1] = bits of the smallest nonzero |w| (start: all ones).
__global__ void weight_range_kernel(const float *__restrict__ w, int64_t N,
                                    unsigned *__restrict__ out) {
  unsigned mx = 0, mn = 0xffffffffu;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    const unsigned b = __float_as_uint(w[p]) & 0x7fffffffu;
    mx = max(mx, b);
    if (b) mn = min(mn, b);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
    mn = min(mn, __shfl_down_sync(0xffffffffu, mn, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out, mx);
    atomicMin(out + 1, mn);
  }
}

// Two-sum of doubles (Knuth): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
  s = __dadd_rn(a, b);
  const double bb = __dsub_rn(s, a);
  e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}

// Adds the integer x * 2^-k to the double-double (hi, lo): x is split into
// 32-bit halves, each exact in a double.
__device__ __forceinline__ void dd_add_scaled(double &hi, double &lo, long long x, int k) {
  const double a = ldexp((double)(x >> 32), 32 - k);  // exact: |x >> 32| < 2^32
  const double b = ldexp((double)(unsigned)(x & 0xffffffffLL), -k);
  double s, e;
  two_sum(hi, a, s, e);
  lo = __dadd_rn(lo, e);
  two_sum(s, b, hi, e);
  lo = __dadd_rn(lo, e);
}

// Float totals from the fixed-point residues of `passes` contractions at
// scales k1, k1 + d, ...: X_1 = R_0 exactly, and pass i adds the
// correction delta_i = R_i - (R_(i-1) << d) (mod 2^64, signed) at scale
// 2^-(k1 + i d).
__global__ void combine_passes_kernel(float *__restrict__ acc, const long long *__restrict__ R,
                                      int passes, int64_t N, int k1, int d,
                                      const int *__restrict__ plan) {
  if (plan) {  // deferred: the plan is on the device; one pass wrote acc itself
    passes = plan[0];
    k1 = plan[1];
    d = plan[2];
    if (passes <= 1) return;
  }
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    long long prev = R[p];
    double hi = 0.0, lo = 0.0;
    dd_add_scaled(hi, lo, prev, k1);
    for (int i = 1; i < passes; i++) {
      const long long r = R[(int64_t)i * N + p];
      const long long delta = (long long)((unsigned long long)r -
                                          ((unsigned long long)prev << d));
      dd_add_scaled(hi, lo, delta, k1 + i * d);
      prev = r;
    }
    acc[p] = __double2float_rn(__dadd_rn(hi, lo));
  }
}

int list_grid(int64_t n) {
  int64_t b = (n + 255) / 256;
  int64_t cap = (int64_t)sm_count() * 16;
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}

struct UpWork {
  CoarseCell *ccell, *cell;
  void *lacc;  // long long per pixel (int for unit counts)
  int16_t *lrl;
  uint8_t *emask;
  int2 *link;
  int *xmap, *xsteps, *elist, *leaves, *h;
  long long *raw;  // passes * N fixed-point totals (multi-scale sums only)
  int *counters;  // [0] ecount, [1] lcount, [2] processed, [3] hmax, [4] err
  int *plan;      // [0..2] deferred weighted sums' {passes, k1, d}, [4..5] their range,
                  // [8] the maximum height, kept from the pass that computed it
};

// Later passes of a multi-scale sum reset the counters, so the maximum
// height that the node order reads is copied aside by the pass that
// computes the heights.
tt_cuda_status keep_hmax(UpWork &w, cudaStream_t st) {
  TT_CHECK(cudaMemcpyAsync(w.plan + 8, w.counters + 3, sizeof(int), cudaMemcpyDeviceToDevice, st));
  return TT_CUDA_SUCCESS;
}

tt_cuda_status up_alloc(const GridDims &g, bool want_acc, bool want_h,
                        UpWork &w, int raw_passes = 0) {
  const size_t N = (size_t)g.cells();
  Workspace &ws = workspace();
  // Exits are ring pixels: at most 124 per tile.
  const size_t E = std::min(N, (size_t)g.tiles() * kRing);
  size_t need = 512 + align_up(N * sizeof(CoarseCell)) + align_up(E * sizeof(CoarseCell)) +
                align_up(E * 8) + 2 * align_up(E * 4) + 2 * align_up(N * 4) +
                (want_acc ? align_up(N * 8) : 0) + (want_h ? align_up(N * 4) : 0) +
                align_up(N * 2) + align_up((size_t)g.tiles() * kRing) +
                (size_t)raw_passes * align_up(N * 8) + 4096;
  if (!ws.reserve(need)) return TT_CUDA_ERR_ALLOC;
  w.counters = (int *)ws.take(256);
  w.plan = (int *)ws.take(256);
  w.cell = (CoarseCell *)ws.take(N * sizeof(CoarseCell));
  w.ccell = (CoarseCell *)ws.take(E * sizeof(CoarseCell));
  w.link = (int2 *)ws.take(E * 8);
  w.lacc = want_acc ? ws.take(N * 8) : nullptr;
  w.lrl = (int16_t *)ws.take(N * 2);
  w.emask = (uint8_t *)ws.take((size_t)g.tiles() * kRing);
  w.h = want_h ? (int *)ws.take(N * 4) : nullptr;
  w.xmap = (int *)ws.take(N * 4);
  w.xsteps = (int *)ws.take(N * 4);
  w.elist = (int *)ws.take(E * 4);
  w.leaves = (int *)ws.take(E * 4);
  w.raw = raw_passes ? (long long *)ws.take((size_t)raw_passes * N * 8) : nullptr;
  return TT_CUDA_SUCCESS;
}

// Runs both tile passes and the coarse walk.
tt_cuda_status up_run(const uint8_t *dir, const float *weights, int wshift,
                      const GridDims &g, unsigned order, bool want_acc,
                      bool want_h, float *acc_out, UpWork &w, cudaStream_t st,
                      int *count_out = nullptr, long long *raw_out = nullptr,
                      const int *plan = nullptr, int pass = 0) {
  const int T = g.tiles();
  TT_CHECK(cudaMemsetAsync(w.counters, 0, 256, st));
  UpArgs a{};
  a.dir = dir;
  a.m = g.m;
  a.n = g.n;
  a.tm = g.tm;
  a.tn = g.tn;
  a.order = order;
  a.w = weights;
  a.wshift = wshift;
  a.phase = 1;
  a.want_acc = want_acc;
  a.want_h = want_h;
  a.ccell = w.ccell;
  a.cell = w.cell;
  a.lacc = w.lacc;
  a.lrl = w.lrl;
  a.emask = w.emask;
  a.xmap = w.xmap;
  a.xsteps = w.xsteps;
  a.elist = w.elist;
  a.ecount = w.counters + 0;
  a.acc_out = acc_out;
  a.raw_out = raw_out;
  a.plan = plan;
  a.pass = pass;
  a.count_out = count_out;
  a.h_out = w.h;
  a.hmax = w.counters + 3;
  a.err = w.counters + 4;
  // The first pass takes one tile per block, so the block scheduler evens
  // out tiles whose walks differ in length.  The final pass does the same
  // unless it carries heights: then it stays persistent, since each block
  // ends with an atomic on the shared maximum height (measured at 16384^2,
  // same box: pipeline 38.77 ms with both passes persistent, 38.55 ms with
  // this split, 39.0 ms with both one tile per block).
  const int tgrid = (int)std::min<int64_t>(T, INT_MAX);
  const int fgrid = want_h ? (int)std::min<int64_t>(T, (int64_t)sm_count() * kFinBlocks) : tgrid;
  void (*up)(UpArgs) = nullptr;
  void (*fin)(UpArgs) = nullptr;
  const bool u32 = !weights;  // unit weights: 32-bit counts in the tile passes
  if (want_acc && want_h && u32) {
    up = order ? forest_up_kernel<true, true, 1, true> : forest_up_kernel<true, true, 0, true>;
    fin = order ? forest_fin_kernel<true, true, 1, true> : forest_fin_kernel<true, true, 0, true>;
  } else if (want_acc && want_h) {
    up = order ? forest_up_kernel<true, true, 1, false> : forest_up_kernel<true, true, 0, false>;
    fin = order ? forest_fin_kernel<true, true, 1, false>
                : forest_fin_kernel<true, true, 0, false>;
  } else if (want_acc && u32) {
    up = order ? forest_up_kernel<true, false, 1, true> : forest_up_kernel<true, false, 0, true>;
    fin = order ? forest_fin_kernel<true, false, 1, true>
                : forest_fin_kernel<true, false, 0, true>;
  } else if (want_acc) {
    up = order ? forest_up_kernel<true, false, 1, false>
               : forest_up_kernel<true, false, 0, false>;
    fin = order ? forest_fin_kernel<true, false, 1, false>
                : forest_fin_kernel<true, false, 0, false>;
  } else {
    up = order ? forest_up_kernel<false, true, 1, false> : forest_up_kernel<false, true, 0, false>;
    fin = order ? forest_fin_kernel<false, true, 1, false>
                : forest_fin_kernel<false, true, 0, false>;
  }
  TT_LAUNCH(up, tgrid, kUpThreads, 0, st, a);
  const int lg = list_grid(g.cells() / 8 + 1);
  TT_LAUNCH(coarse_link_kernel, lg, 256, 0, st, w.elist, w.counters + 0, dir,
            g.m, order, w.xmap, w.xsteps, w.link, w.ccell);
  TT_LAUNCH(coarse_leaves_kernel, lg, 256, 0, st, w.counters + 0, w.ccell, w.link, w.leaves,
            w.counters + 1);
  // One walker per leaf (blocks beyond the leaf count exit at once): the
  // block scheduler hands freed SMs the next leaves, instead of each thread
  // walking a fixed share of them one after another.
  const int64_t exits = std::min<int64_t>(g.cells(), (int64_t)g.tiles() * kRing);
  const int wg = (int)std::max<int64_t>(1, std::min<int64_t>((exits + 255) / 256, INT_MAX));
  TT_LAUNCH(coarse_walk_kernel, wg, 256, 0, st, w.leaves, w.counters + 1, w.link,
            w.ccell, w.counters + 2, (int)std::min<int64_t>(g.cells(), INT_MAX));
  TT_LAUNCH(coarse_scatter_kernel, lg, 256, 0, st, w.counters + 0, w.elist, w.ccell,
            w.cell);
  a.phase = 3;
  TT_LAUNCH(fin, fgrid, kUpThreads, 0, st, a);
  TT_CHECK(cudaGetLastError());
  return TT_CUDA_SUCCESS;
}

// Reads the counters back and maps error bits to a status.
tt_cuda_status up_status(UpWork &w, cudaStream_t st, int *host6) {
  // deferred: ecount, processed and error bits go to the status sink (when
  // the sink is full, the status is read back here as usual)
  if (int *rec = status_sink() ? sink_record(REC_FOREST, st) : nullptr) {
    TT_CHECK(cudaMemcpyAsync(rec + 1, w.counters + 0, sizeof(int), cudaMemcpyDeviceToDevice, st));
    TT_CHECK(cudaMemcpyAsync(rec + 2, w.counters + 2, sizeof(int), cudaMemcpyDeviceToDevice, st));
    TT_CHECK(cudaMemcpyAsync(rec + 3, w.counters + 4, sizeof(int), cudaMemcpyDeviceToDevice, st));
    for (int k = 0; k < 6; k++) host6[k] = 0;
    return TT_CUDA_SUCCESS;
  }
  int *h = (int *)pinned_scratch();
  if (!h) return TT_CUDA_ERR_ALLOC;
  TT_CHECK(cudaMemcpyAsync(h, w.counters, 6 * sizeof(int), cudaMemcpyDeviceToHost, st));
  TT_CHECK(cudaStreamSynchronize(st));
  for (int k = 0; k < 6; k++) host6[k] = h[k];
  if (host6[2] != host6[0]) return TT_CUDA_ERR_CYCLE;  // coarse nodes not all reached
  if (host6[4] & ERR_CYCLE) return TT_CUDA_ERR_CYCLE;
  if (host6[4] & (ERR_BADDIR | ERR_WEIGHT)) return TT_CUDA_ERR_INVALID_ARGUMENT;
  return TT_CUDA_SUCCESS;
}

}  // namespace

// Exact pixel counts of every subtree (unit weights), as int: the number of
// pixels whose flow path passes through each pixel, itself included.
tt_cuda_status count_dev(int *count, const uint8_t *dir, const GridDims &g, cudaStream_t st) {
  UpWork w;
  {
    tt_cuda_status s = up_alloc(g, true, false, w);
    if (s != TT_CUDA_SUCCESS) return s;
  }
  {
    tt_cuda_status s = up_run(dir, nullptr, 0, g, 0, true, false, nullptr, w, st, count);
    if (s != TT_CUDA_SUCCESS) return s;
  }
  int h6[6];
  return up_status(w, st, h6);
}

namespace {

// Fixed-point scales of a weighted sum.  The first pass uses 2^k1 with
// max|w| * N * 2^k1 <= 2^62, so no partial sum overflows.  Rounding a weight
// to that grid costs at most 2^-(k1+1), so a total over weights of one sign
// is within 2^-(k1+1) / min|w| of exact, relative; when that exceeds
// kRelTarget the contraction is repeated at k1 + d, k1 + 2d, ... (at most
// kMaxPasses scales) with d = 61 - ceil(log2 N), which keeps every pass's
// total within 2^61 units of 2^d times the previous one.
constexpr double kRelTarget = 1e-7;
constexpr int kMaxPasses = 4;
struct WeightPlan {
  int k1 = 0;      // scale of the first pass
  int d = 0;       // scale step between passes
  int passes = 1;  // contractions to run
};

// ceil(log2(x)) of a positive finite double, exactly: x = f * 2^e with f in
// [0.5, 1), so the answer is e, or e - 1 when x is a power of two.
__host__ __device__ inline int ceil_log2(double x) {
  int e = 0;
  const double f = frexp(x, &e);
  return f == 0.5 ? e - 1 : e;
}

// The plan from the weights' largest and smallest nonzero magnitudes (as
// float bit patterns).  The host and the device run this same function, so
// the deferred form scales exactly like the synchronous one.
__host__ __device__ inline WeightPlan plan_from_range(unsigned mx_bits, unsigned mn_bits,
                                                      double N) {
  WeightPlan p;
  if (mx_bits >= 0x7f800000u) return p;  // non-finite: flagged per pixel
  if (mx_bits == 0) return p;            // all weights zero
  float mxv, mnv;
#ifdef __CUDA_ARCH__
  mxv = __uint_as_float(mx_bits);
  mnv = __uint_as_float(mn_bits);
#else
  std::memcpy(&mxv, &mx_bits, 4);
  std::memcpy(&mnv, &mn_bits, 4);
#endif
  p.k1 = 62 - ceil_log2((double)mxv * N);
  p.d = 61 - ceil_log2(N > 2.0 ? N : 2.0);
  const int need = ceil_log2(0.5 / ((double)mnv * kRelTarget));
  if (need > p.k1 && p.d > 0) {
    const int more = (need - p.k1 + p.d - 1) / p.d;
    p.passes = 1 + more < kMaxPasses ? 1 + more : kMaxPasses;
  }
  return p;
}

// One thread: the plan of the range found by weight_range_kernel, as
// {passes, k1, d}.
__global__ void weight_plan_kernel(const unsigned *__restrict__ rng, double N,
                                   int *__restrict__ plan) {
  const WeightPlan p = plan_from_range(rng[0], rng[1], N);
  plan[0] = p.passes;
  plan[1] = p.k1;
  plan[2] = p.d;
}

tt_cuda_status weight_plan(const float *weights, const GridDims &g, cudaStream_t st,
                           WeightPlan *plan) {
  *plan = WeightPlan{};
  if (!weights) return TT_CUDA_SUCCESS;
  Workspace &ws = workspace();
  if (!ws.reserve(256)) return TT_CUDA_ERR_ALLOC;
  unsigned *rng = (unsigned *)ws.take(256);
  TT_CHECK(cudaMemsetAsync(rng, 0, 4, st));
  TT_CHECK(cudaMemsetAsync(rng + 1, 0xff, 4, st));
  TT_LAUNCH(weight_range_kernel, list_grid(g.cells()), 256, 0, st, weights, g.cells(), rng);
  unsigned *h = (unsigned *)pinned_scratch();
  if (!h) return TT_CUDA_ERR_ALLOC;
  TT_CHECK(cudaMemcpyAsync(h, rng, 8, cudaMemcpyDeviceToHost, st));
  TT_CHECK(cudaStreamSynchronize(st));
  *plan = plan_from_range(h[0], h[1], (double)g.cells());
  return TT_CUDA_SUCCESS;
}

// Weighted (or unit) accumulation into `acc` following `plan`; `want_h`
// also leaves the subtree heights of the first pass in w.h and their
// maximum in h6[3].  w must come from up_alloc with plan.passes raw slots
// when plan.passes > 1.
tt_cuda_status accumulate_planned(float *acc, const uint8_t *dir, const float *weights,
                                  const WeightPlan &plan, const GridDims &g, bool want_h,
                                  UpWork &w, cudaStream_t st, int h6[6]) {
  if (plan.passes == 1) {
    TT_TRY_STATUS(up_run(dir, weights, plan.k1, g, 0, true, want_h, acc, w, st));
    if (want_h) TT_TRY_STATUS(keep_hmax(w, st));
    return up_status(w, st, h6);
  }
  const int64_t N = g.cells();
  tt_cuda_status first = TT_CUDA_SUCCESS;
  for (int p = 0; p < plan.passes; p++) {
    TT_TRY_STATUS(up_run(dir, weights, plan.k1 + p * plan.d, g, 0, true, want_h && p == 0,
                         nullptr, w, st, nullptr, w.raw + (size_t)p * N));
    if (p == 0) {  // later passes walk the same forest
      if (want_h) TT_TRY_STATUS(keep_hmax(w, st));
      first = up_status(w, st, h6);
      if (first == TT_CUDA_ERR_CYCLE) return first;
    }
  }
  TT_LAUNCH(combine_passes_kernel, list_grid(N), 256, 0, st, acc, w.raw, plan.passes, N,
            plan.k1, plan.d, (const int *)nullptr);
  TT_CHECK(cudaGetLastError());
  return first;
}

// Deferred weighted accumulation (a status sink is set): the weights'
// range and the plan stay on the device and every pass reads the plan, so
// nothing waits for the weights.  kMaxPasses passes are enqueued; those
// past the plan's count return at once, and a single-pass plan writes
// `acc` from the first pass as the synchronous form does.  w must come from
// up_alloc with kMaxPasses raw slots.
tt_cuda_status accumulate_deferred(float *acc, const uint8_t *dir, const float *weights,
                                   const GridDims &g, bool want_h, UpWork &w,
                                   cudaStream_t st, int h6[6]) {
  const int64_t N = g.cells();
  unsigned *rng = (unsigned *)(w.plan + 4);
  TT_CHECK(cudaMemsetAsync(rng, 0, 4, st));
  TT_CHECK(cudaMemsetAsync(rng + 1, 0xff, 4, st));
  TT_LAUNCH(weight_range_kernel, list_grid(N), 256, 0, st, weights, N, rng);
  TT_LAUNCH(weight_plan_kernel, 1, 1, 0, st, rng, (double)N, w.plan);
  tt_cuda_status first = TT_CUDA_SUCCESS;
  for (int p = 0; p < kMaxPasses; p++) {
    TT_TRY_STATUS(up_run(dir, weights, 0, g, 0, true, want_h && p == 0, acc, w, st, nullptr,
                         w.raw + (size_t)p * N, w.plan, p));
    if (p == 0) {
      if (want_h) TT_TRY_STATUS(keep_hmax(w, st));
      first = up_status(w, st, h6);
      if (first == TT_CUDA_ERR_CYCLE) return first;
    }
  }
  TT_LAUNCH(combine_passes_kernel, list_grid(N), 256, 0, st, acc, w.raw, kMaxPasses, N, 0, 0,
            (const int *)w.plan);
  TT_CHECK(cudaGetLastError());
  return first;
}

// Node order from the subtree heights of a finished up_run: pixels sorted
// by height (a donor's height is below its receiver's), stable within a
// height by a counting sort.  The number of heights is read on the device
// (the contraction's maximum height), so nothing waits for it.
tt_cuda_status node_scatter(ptrdiff_t *node, UpWork &w, const GridDims &g, cudaStream_t st) {
  // hist, off and cursor reuse the coarse arrays (N ints each, no longer needed).
  int *hist = w.xmap, *off = w.xsteps, *cursor = reinterpret_cast<int *>(w.cell);
  const int *hmax = w.plan + 8;
  const int64_t N = g.cells();
  const int eg = list_grid(N);
  TT_LAUNCH(clear_bins_kernel, eg, 256, 0, st, hist, cursor, hmax, N);
  TT_LAUNCH(h_hist_kernel, eg, 256, 0, st, w.h, N, hist, hmax);
  TT_LAUNCH(scan_kernel, 1, 1024, 0, st, hist, off, hmax, N);
  TT_LAUNCH(node_scatter_kernel, eg, 256, 0, st, w.h, N, off, cursor, node, hmax);
  TT_CHECK(cudaGetLastError());
  return TT_CUDA_SUCCESS;
}

}  // namespace

tt_cuda_status accumulate_dev(float *acc, const uint8_t *dir,
                              const float *weights, const GridDims &g,
                              cudaStream_t st) {
  UpWork w;
  int h6[6];
  if (weights && status_sink()) {
    TT_TRY_STATUS(up_alloc(g, true, false, w, kMaxPasses));
    return accumulate_deferred(acc, dir, weights, g, false, w, st, h6);
  }
  WeightPlan plan;
  TT_TRY_STATUS(weight_plan(weights, g, st, &plan));
  TT_TRY_STATUS(up_alloc(g, true, false, w, plan.passes > 1 ? plan.passes : 0));
  return accumulate_planned(acc, dir, weights, plan, g, false, w, st, h6);
}

tt_cuda_status node_order_dev(ptrdiff_t *node, const uint8_t *dir,
                              const GridDims &g, unsigned order,
                              cudaStream_t st) {
  UpWork w;
  TT_TRY_STATUS(up_alloc(g, false, true, w));
  TT_TRY_STATUS(up_run(dir, nullptr, 0, g, order, false, true, nullptr, w, st));
  TT_TRY_STATUS(keep_hmax(w, st));
  int h6[6];
  tt_cuda_status s = up_status(w, st, h6);
  if (s == TT_CUDA_ERR_CYCLE) return s;
  TT_TRY_STATUS(node_scatter(node, w, g, st));
  return s;
}

// Column-major node order and flow accumulation from one contraction of the
// receiver forest: the tile and coarse passes carry the subtree sums and the
// subtree heights together, so the pipeline walks the forest once for both.
tt_cuda_status node_order_acc_dev(ptrdiff_t *node, float *acc, const uint8_t *dir,
                                  const float *weights, const GridDims &g,
                                  cudaStream_t st, tt_cuda_status (*acc_done)(void *),
                                  void *ctx) {
  UpWork w;
  int h6[6];
  tt_cuda_status s;
  if (weights && status_sink()) {
    TT_TRY_STATUS(up_alloc(g, true, true, w, kMaxPasses));
    s = accumulate_deferred(acc, dir, weights, g, true, w, st, h6);
  } else {
    WeightPlan plan;
    TT_TRY_STATUS(weight_plan(weights, g, st, &plan));
    TT_TRY_STATUS(up_alloc(g, true, true, w, plan.passes > 1 ? plan.passes : 0));
    s = accumulate_planned(acc, dir, weights, plan, g, true, w, st, h6);
  }
  if (s == TT_CUDA_ERR_CYCLE) return s;
  if (acc_done) TT_TRY_STATUS(acc_done(ctx));  // acc is complete on `st` here
  TT_TRY_STATUS(node_scatter(node, w, g, st));
  return s;
}

tt_cuda_status accumulate_backward_dev(float *grad_w, const uint8_t *dir,
                                       const float *grad_acc, const GridDims &g,
                                       cudaStream_t st) {
  const size_t N = (size_t)g.cells();
  Workspace &ws = workspace();
  size_t need = 256 + 11 * align_up(N * 4) + 4096;
  if (!ws.reserve(need)) return TT_CUDA_ERR_ALLOC;
  int *counters = (int *)ws.take(256);
  float *clhi = (float *)ws.take(N * 4);
  float *cllo = (float *)ws.take(N * 4);
  int *cx = (int *)ws.take(N * 4);
  int *eidx = (int *)ws.take(N * 4);
  int *elist = (int *)ws.take(N * 4);
  float *D[2][2] = {{(float *)ws.take(N * 4), (float *)ws.take(N * 4)},
                    {(float *)ws.take(N * 4), (float *)ws.take(N * 4)}};
  int *nx[2] = {(int *)ws.take(N * 4), (int *)ws.take(N * 4)};
  TT_CHECK(cudaMemsetAsync(counters, 0, 256, st));
  DownArgs a{};
  a.dir = dir;
  a.g = grad_acc;
  a.m = g.m;
  a.n = g.n;
  a.tm = g.tm;
  a.tn = g.tn;
  a.order = 0;
  a.phase = 1;
  a.clhi = clhi;
  a.cllo = cllo;
  a.cx = cx;
  a.eidx = eidx;
  a.elist = elist;
  a.ecount = counters + 0;
  a.out = grad_w;
  a.err = counters + 4;
  const int T = g.tiles();
  const int tgrid = (int)std::min<int64_t>(T, INT_MAX);  // one tile per block
  TT_LAUNCH(forest_down_kernel, tgrid, kDownThreads, 0, st, a);
  const int lg = list_grid(g.cells() / 8 + 1);
  TT_LAUNCH(down_init_kernel, lg, 256, 0, st, elist, counters + 0, dir, g.m, 0u,
            clhi, cllo, cx, eidx, D[0][0], D[0][1], nx[0]);
  int *hcnt = (int *)pinned_scratch();
  if (!hcnt) return TT_CUDA_ERR_ALLOC;
  int cur = 0;
  for (int round = 0; round < 40; round += 4) {
    for (int b = 0; b < 4; b++) {
      TT_CHECK(cudaMemsetAsync(counters + 1, 0, 4, st));
      TT_LAUNCH(down_jump_kernel, lg, 256, 0, st, counters + 0, D[cur][0], D[cur][1],
                nx[cur], D[cur ^ 1][0], D[cur ^ 1][1], nx[cur ^ 1], counters + 1);
      cur ^= 1;
    }
    TT_CHECK(cudaMemcpyAsync(hcnt, counters + 1, 4, cudaMemcpyDeviceToHost, st));
    TT_CHECK(cudaStreamSynchronize(st));
    if (*hcnt == 0) break;
    if (round + 4 >= 40) return TT_CUDA_ERR_CYCLE;
  }
  a.phase = 3;
  a.Dhi = D[cur][0];
  a.Dlo = D[cur][1];
  TT_LAUNCH(forest_down_kernel, tgrid, kDownThreads, 0, st, a);
  TT_CHECK(cudaGetLastError());
  TT_CHECK(cudaMemcpyAsync(hcnt, counters + 4, 4, cudaMemcpyDeviceToHost, st));
  TT_CHECK(cudaStreamSynchronize(st));
  if (*hcnt & ERR_CYCLE) return TT_CUDA_ERR_CYCLE;
  if (*hcnt & ERR_BADDIR) return TT_CUDA_ERR_INVALID_ARGUMENT;
  return TT_CUDA_SUCCESS;
}

}  // namespace tt
