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
// Work decomposition: one warp relaxes one 32 x 32 tile at a time.  It stages
// the tile and a one-pixel halo in shared memory and runs directional
// Gauss-Seidel sweeps (down, up, right, left, each lane carrying one line)
// over the pixels marked for re-evaluation until none is marked.  Changed
// cells are written back with plain stores (a tile has one owner, so no
// other warp writes them meanwhile); a changed edge or corner marks the
// neighbouring tile dirty.
//
// Scheduling: one persistent launch.  Warp w of W owns the tiles
// w, w + W, w + 2W, ... and keeps scanning their "dirty" flags (32 at a time
// with a ballot); a warp that relaxes a tile and changes an edge marks the
// neighbouring tile dirty, so information crosses tile borders as soon as a
// tile finishes, with no host round trips and no shared queue to contend on.
// A tile has a single owner, so no two warps relax it at once.
//
// Termination: only a running warp sets flags.  A warp that finds none of
// its tiles dirty adds itself to an idle count (after its own flags are
// visible); a warp that finds a flag again leaves the count, and bumps a
// wake counter kept in the same 64-bit word, before it takes the flag.  The
// warp whose arrival makes every warp idle scans all flags and ends the run
// if none is set and the word is unchanged since its arrival (no warp woke,
// so none ran and none could set a flag behind the scan); otherwise the
// owners of the set flags wake up and the last one to go idle scans again.  Every wait is bounded: a warp that idles too
// long, or a run that exceeds its visit budget, raises an abort flag and all
// warps return with an error status.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <mutex>

#include "tt_internal.cuh"

namespace tt {
namespace {

constexpr int kWarps = 4;        // tiles per block
constexpr int kMaxSweeps = 256;  // per tile visit; a capped tile re-enqueues
constexpr float kSqrt2 = 1.41421356237309504880f;

// GWDT_HALF: gwdt over costs stored halved (the pipeline's own costs, at
// least 0.1, so halving is exact and every intermediate stays normal): a
// step's weights lose one multiplication and keep their bits, since
// RN(x / 2) = RN(x) / 2 for normal x.
enum Kind { FILL = 0, GWDT = 1, GWDT_HALF = 2 };

struct WarpTile {
  float s[kHalo][kPitch];  // state: f (fill) or dist (gwdt); [c][r]
  float a[kHalo][kPitch];  // aux: dem (fill) or costs (gwdt)
};

// Control block (device memory, zero-initialised).
struct QueueCtl {
  unsigned long long visits;  // tiles relaxed so far (flushed in batches)
  unsigned long long idle;    // wakes << 32 | warps that found nothing to do
  int done;                   // set once every warp is idle and no flag is set
  int abort;                  // ABORT_* bits
  int thresh;                 // ordered schedules: tiles with priority <= thresh run
};

enum : int { ABORT_SPIN = 1, ABORT_VISITS = 2 };

constexpr long long kSpinLimit = 1LL << 22;  // idle scans before giving up

struct RelaxArgs {
  float *state;
  const float *aux;
  int64_t m, n;
  int tm, tn;
  QueueCtl *ctl;
  int *dirty;  // per tile: nonzero while waiting to be relaxed
  unsigned long long max_visits;
  int visit_flush;  // a warp adds its visits to ctl->visits in batches of this
  int *prio;        // ordered schedules: per tile, the key of the lowest value
                    // published into it since it was last taken (kClean: none)
  int *wmin;        // ordered schedules: per warp, the lowest priority among
                    // its waiting tiles at its last pass (kClean: none)
};

// Order-preserving integer key of a float (key order == value order).
__device__ __forceinline__ int value_key(float x) {
  const int b = __float_as_int(x);
  return b >= 0 ? b : b ^ 0x7fffffff;
}
__device__ __forceinline__ float key_value(int k) {
  return __int_as_float(k >= 0 ? k : k ^ 0x7fffffff);
}
constexpr int kClean = 0x7f7f7f7f;        // no priority (above every finite key)
constexpr int kUrgent = (int)0x80000000;  // below every key: runs at any threshold

// Dirty flag bits: 1 = a halo pixel changed (re-evaluate the edge ring),
// 2 = evaluate every pixel (first visit, or a visit that hit its sweep cap).

// Release / acquire at device scope (lighter than a sequentially consistent
// fence): a writer fences before it sets a flag, a reader after it takes one.
__device__ __forceinline__ void fence_acq_rel_gpu() {
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
}

// 4-byte asynchronous copy global -> shared, cached in L1 (read-only inputs).
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  // No memory clobber: the copies may interleave with the other staging
  // loads; cp_async_wait_all() orders them before any use, and the warp
  // barriers before staging order them after the previous visit's reads.
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// Transpose of a 32 x 32 bit matrix held one row per lane.
__device__ __forceinline__ uint32_t transpose32(uint32_t x, int lane) {
  uint32_t y = 0;
#pragma unroll
  for (int k = 0; k < 32; k++) {
    const uint32_t b = __ballot_sync(0xffffffffu, (x >> k) & 1u);
    if (lane == k) y = b;
  }
  return y;
}

// One Gauss-Seidel sweep.  Each lane carries one line of the tile: a column
// (ALONG_C false: the sweep walks down or up the rows) or a row (ALONG_C
// true: it walks right or left along the columns).  `nd` marks the pixels of
// the lane's line whose neighbourhood changed since they were last evaluated
// against all eight neighbours, `dm` collects the pixels that changed; both
// live in registers, bit k = k-th pixel of the line.
//
// A step (one pixel per lane) evaluates every lane's pixel: in SIMT that
// costs the same as evaluating only the marked ones, and it keeps the
// per-step dependency chain down to the loads and the minimum.  After the
// sweep a pixel is marked again if a neighbour evaluated in the same step or
// a later one changed (neighbours of earlier steps were already final when
// it was evaluated), and unevaluated pixels keep their marks.  An unmarked
// pixel therefore cannot be lowered by any neighbour, and the tile is at its
// local fixpoint exactly when no pixel is marked.  Neighbour values may be
// old or new: every value is an upper bound of the fixpoint, so any mix
// gives a valid (and never higher) result.
//
// Both kinds run every step from the first marked one to the end of the
// line with no vote at all: a per-step vote would put a warp-wide round trip
// on the chain between steps.
__device__ __forceinline__ void remark(int lane, int dir, uint32_t dm, uint32_t evald,
                                       uint32_t &nd, uint32_t &dm_all) {
  const uint32_t from_prev = __shfl_up_sync(0xffffffffu, dm, 1);
  const uint32_t from_next = __shfl_down_sync(0xffffffffu, dm, 1);
  const uint32_t side = (lane > 0 ? from_prev : 0u) | (lane < 31 ? from_next : 0u);
  const uint32_t any3 = dm | side;
  const uint32_t later = dir > 0 ? (any3 >> 1) : (any3 << 1);
  nd = (nd & ~evald) | side | later;
  dm_all |= dm;
}

// Fill sweep.  A step reads what an evaluation after the previous step's
// stores would read, but carries part of it in registers: the lane's own
// pixel behind (its previous result), its own pixel and the adjacent lines'
// pixels at the current position (read one step ahead; only this step
// writes them).  It loads only the adjacent lines' pixels behind (written by
// the previous step) and the three pixels ahead: five state loads a step
// instead of nine, on the shared-memory pipe that all warps of an SM share.
template <bool ALONG_C>
__device__ __forceinline__ void sweep_fill(WarpTile &t, int lane, int dir, uint32_t &nd,
                                           uint32_t &dm_all) {
  const uint32_t steps = __reduce_or_sync(0xffffffffu, nd);
  if (!steps) return;
  const int first = dir > 0 ? __ffs(steps) - 1 : kTile - 1 - (31 - __clz(steps));
  // Pixel (line l, position p): t.s[l][p] in the column layout, t.s[p][l]
  // in the row layout.  The lane's line is l = lane + 1.
  constexpr int PS = ALONG_C ? kPitch : 1;  // between positions
  constexpr int LS = ALONG_C ? 1 : kPitch;  // between lines
  float *const sline = ALONG_C ? &t.s[0][lane + 1] : &t.s[lane + 1][0];
  const float *const aline = ALONG_C ? &t.a[0][lane + 1] : &t.a[lane + 1][0];
  const int D = dir * PS;  // to the next position of the sweep
  uint32_t dm = 0, evald = 0;
  float ob = 0.f, op = 0.f, lp = 0.f, rp = 0.f;  // own behind / here, adjacent here
  bool have = false;  // the registers hold the previous step's values
#pragma unroll 1
  for (int s = first; s < kTile; s++) {
    const int k = dir > 0 ? s : kTile - 1 - s;  // position along the line
    const uint32_t bit = 1u << k;
    evald |= bit;
    float *const sp = sline + (k + 1) * PS;
    if (!have) {
      ob = sp[-D];
      op = sp[0];
      lp = sp[-LS];
      rp = sp[LS];
    }
    const float lb = sp[-LS - D], rb = sp[LS - D];  // written by the previous step
    const float oa = sp[D], la = sp[-LS + D], ra = sp[LS + D];
    const float cur = op;
    const float z = aline[(k + 1) * PS];
    const float a0 = fminf(lb, lp), a1 = fminf(la, ob);
    const float a2 = fminf(oa, rb), a3 = fminf(rp, ra);
    const float lo = fminf(cur, fminf(fminf(a0, a1), fminf(a2, a3)));
    const float nv = (lo > z) ? lo : z;
    const bool ch = nv < cur;
    if (ch) {
      sp[0] = nv;
      dm |= bit;
    }
    ob = ch ? nv : cur;
    op = oa;
    lp = la;
    rp = ra;
    have = true;
    __syncwarp();
  }
  remark(lane, dir, dm, evald, nd, dm_all);
}

// Gwdt sweep in the fill's form: every step from the first marked one to
// the end of the line, no votes, with the values a step would re-read
// unchanged carried in registers (state of the lane's own pixel behind and
// here, adjacent lines here; costs of all three lines behind and here).
// Non-flat and off-grid pixels are staged with cost NaN (state 0 or +INF):
// every path through them evaluates to NaN, which never wins the minimum,
// and a non-flat centre (cost NaN) keeps its value.
template <bool ALONG_C, bool HALF>
__device__ __forceinline__ void sweep_gwdt_run(WarpTile &t, int lane, int dir, uint32_t &nd,
                                               uint32_t &dm_all) {
  const uint32_t steps = __reduce_or_sync(0xffffffffu, nd);
  if (!steps) return;
  const int first = dir > 0 ? __ffs(steps) - 1 : kTile - 1 - (31 - __clz(steps));
  constexpr int PS = ALONG_C ? kPitch : 1;
  constexpr int LS = ALONG_C ? 1 : kPitch;
  float *const sline = ALONG_C ? &t.s[0][lane + 1] : &t.s[lane + 1][0];
  const float *const aline = ALONG_C ? &t.a[0][lane + 1] : &t.a[lane + 1][0];
  const int D = dir * PS;
  uint32_t dm = 0, evald = 0;
  float ob = 0.f, op = 0.f, lp = 0.f, rp = 0.f;
  float cb0 = 0.f, cb1 = 0.f, cb2 = 0.f, cp0 = 0.f, cp1 = 0.f, cp2 = 0.f;
  bool have = false;
#pragma unroll 1
  for (int s = first; s < kTile; s++) {
    const int k = dir > 0 ? s : kTile - 1 - s;
    const uint32_t bit = 1u << k;
    evald |= bit;
    float *const sp = sline + (k + 1) * PS;
    const float *const ap = aline + (k + 1) * PS;
    if (!have) {
      ob = sp[-D];
      op = sp[0];
      lp = sp[-LS];
      rp = sp[LS];
      cb0 = ap[-LS - D];
      cb1 = ap[-D];
      cb2 = ap[LS - D];
      cp0 = ap[-LS];
      cp1 = ap[0];
      cp2 = ap[LS];
    }
    const float lb = sp[-LS - D], rb = sp[LS - D];  // written by the previous step
    const float oa = sp[D], la = sp[-LS + D], ra = sp[LS + D];
    const float ca0 = ap[-LS + D], ca1 = ap[D], ca2 = ap[LS + D];
    const float cur = op, cs = cp1;
    // d(u) + chamfer * (c(u) + c(v)) / 2; multiplying by 1 is exact (HALF:
    // the costs are already halved)
    auto side = [&](float d, float c) {
      return HALF ? __fadd_rn(d, __fadd_rn(cs, c))
                  : __fadd_rn(d, __fmul_rn(__fadd_rn(cs, c), 0.5f));
    };
    auto diag = [&](float d, float c) {
      return HALF ? __fadd_rn(d, __fmul_rn(kSqrt2, __fadd_rn(cs, c)))
                  : __fadd_rn(d, __fmul_rn(__fmul_rn(kSqrt2, __fadd_rn(cs, c)), 0.5f));
    };
    float best = fminf(cur, fminf(side(oa, ca1), side(lp, cp0)));
    best = fminf(best, fminf(side(rp, cp2), diag(la, ca0)));
    best = fminf(best, diag(ra, ca2));
    best = fminf(best, fminf(side(ob, cb1), fminf(diag(lb, cb0), diag(rb, cb2))));
    const float nv = best;
    const bool ch = nv < cur;
    if (ch) {
      sp[0] = nv;
      dm |= bit;
    }
    ob = ch ? nv : cur;
    op = oa;
    lp = la;
    rp = ra;
    cb0 = cp0;
    cb1 = cp1;
    cb2 = cp2;
    cp0 = ca0;
    cp1 = ca1;
    cp2 = ca2;
    have = true;
    __syncwarp();
  }
  remark(lane, dir, dm, evald, nd, dm_all);
}

template <int KIND, bool ALONG_C>
__device__ __forceinline__ void sweep(WarpTile &t, int lane, int dir, uint32_t &nd,
                                      uint32_t &dm_all) {
  if (KIND == FILL)
    sweep_fill<ALONG_C>(t, lane, dir, nd, dm_all);
  else
    sweep_gwdt_run<ALONG_C, KIND == GWDT_HALF>(t, lane, dir, nd, dm_all);
}

// Sweep schedules (a template parameter, picked at run time): bit 0 runs the
// row sweeps (right, left) of a round before the column sweeps (down, up);
// bit 1 caps a visit at kCapSweeps sweeps, after which the tile publishes
// what changed and queues itself again, so that neighbours see partial
// results sooner.  Schedules 4 and 5 order the visits by value (delta
// stepping over tiles): a tile carries the lowest value published into it,
// and only tiles at or below a global threshold run; when every warp is
// idle and some tile is still waiting, the threshold rises to the lowest
// waiting value plus a band (a fraction of that value, at least a fixed
// step: 1/8 and 1 for schedule 4, 1/2 and 4 for schedule 5).  Both updates
// only lower values and any order reaches the same fixpoint, so every
// schedule gives the same bits; ordering trades idle time at band
// boundaries for fewer repeated lowerings of the same pixels.
constexpr int kSchedules = 6;
constexpr int kCapSweeps = 8;
constexpr bool ordered_sched(int s) { return s >= 4; }
__device__ __forceinline__ int band_above(int key, int sched) {
  const float v = key_value(key);
  if (!(v > -INFINITY)) return value_key(-3.4028234663852886e38f);  // -INF or NaN
  const float rel = sched == 5 ? 0.5f : 0.125f, step = sched == 5 ? 4.0f : 1.0f;
  const float nv = v + fmaxf(fabsf(v) * rel, step);
  return value_key(nv);
}

template <int KIND, int SCHED>
__device__ void relax_tile(const RelaxArgs &a, WarpTile &t, int lane, int tile, int mode);

// Ordered schedules: with every warp idle, raise the threshold above the
// lowest priority any warp reported waiting.  Returns false when no warp
// reported waiting work.
template <int SCHED>
__device__ bool raise_threshold(const RelaxArgs &a, int lane, int W, int thr) {
  int g = kClean;
  for (int w = lane; w < W; w += 32) g = min(g, *(volatile int *)&a.wmin[w]);
  g = __reduce_min_sync(0xffffffffu, g);
  if (g == kClean) return false;
  const int nt = band_above(g, SCHED);
  if (lane == 0 && nt > thr) atomicMax(&a.ctl->thresh, nt);
  return true;
}

// The warp that made every warp idle (idle word `seen` after its arrival):
// finish the run if no flag is set and no warp has woken since.
__device__ void check_done(const RelaxArgs &a, int lane, int T, unsigned long long seen) {
  bool any = false;
  for (int t = lane; t < T; t += 32) any |= *(volatile int *)&a.dirty[t] != 0;
  if (__any_sync(0xffffffffu, any) || lane != 0) return;
  fence_acq_rel_gpu();
  if (*(volatile unsigned long long *)&a.ctl->idle == seen) atomicExch(&a.ctl->done, 1);
}

template <int KIND, int SCHED>
__global__ void __launch_bounds__(kWarps * 32)
relax_persistent_kernel(RelaxArgs a) {
  __shared__ WarpTile tiles[kWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpTile &t = tiles[warp];
  const int W = gridDim.x * kWarps;
  const int wid = blockIdx.x * kWarps + warp;
  const int T = a.tm * a.tn;
  long long spins = 0;
  bool idle = false;                 // counted in ctl->idle (warp-uniform)
  unsigned long long unflushed = 0;  // lane 0: visits not yet added to ctl
  int posted = kClean;               // ordered: this warp's last wmin entry
  int raised_at = kUrgent;           // ordered: threshold this warp last raised from
  for (;;) {
    if (*(volatile int *)&a.ctl->abort || *(volatile int *)&a.ctl->done) break;
    const int thr = ordered_sched(SCHED) ? *(volatile int *)&a.ctl->thresh : 0;
    int lane_wait = kClean;  // ordered: lowest priority of this lane's waiting tiles
    if (lane == 0) {
      if (unflushed >= (unsigned long long)a.visit_flush) {
        atomicAdd(&a.ctl->visits, unflushed);
        unflushed = 0;
      }
      if (*(volatile unsigned long long *)&a.ctl->visits >= a.max_visits)
        atomicOr(&a.ctl->abort, ABORT_VISITS);
    }
    bool did = false;
    for (int base = wid; base < T; base += W * 32) {
      const int mine = base + lane * W;
      int f = (mine < T) ? *(volatile int *)&a.dirty[mine] : 0;
      bool elig = f != 0;
      if (ordered_sched(SCHED) && elig) {
        const int pr = *(volatile int *)&a.prio[mine];
        elig = pr <= thr;
        // a flag whose priority was cleared by a take racing its publication
        // waits with the highest priority short of "none"
        if (!elig) lane_wait = min(lane_wait, pr == kClean ? kClean - 1 : pr);
      }
      unsigned mask = __ballot_sync(0xffffffffu, elig);
      if (mask && idle) {  // wake: leave the idle count before taking a flag
        if (lane == 0) {
          const unsigned long long before =
              atomicAdd(&a.ctl->idle, (1ULL << 32) - 1ULL);  // wakes + 1, idle - 1
          asm volatile("" ::"l"(before));
          fence_acq_rel_gpu();
        }
        idle = false;
        __syncwarp();
      }
      while (mask) {
        const int l = __ffs(mask) - 1;
        mask &= mask - 1;
        const int tile = base + l * W;
        int got = 0;
        if (lane == 0) {
          // ordered: clear the priority before taking the flag, so a value
          // published in between keeps a priority (at worst a stale one)
          if (ordered_sched(SCHED)) atomicExch(&a.prio[tile], kClean);
          got = atomicExch(&a.dirty[tile], 0);
          if (got) {
            unflushed++;
            fence_acq_rel_gpu();  // acquire: the writes published before the flag
          }
        }
        got = __shfl_sync(0xffffffffu, got, 0);
        if (!got) continue;
        did = true;
        relax_tile<KIND, SCHED>(a, t, lane, tile, got);
      }
    }
    int wait_min = kClean;
    if (ordered_sched(SCHED)) {  // report this warp's waiting work
      wait_min = __reduce_min_sync(0xffffffffu, lane_wait);
      if (lane == 0 && wait_min != posted) *(volatile int *)&a.wmin[wid] = wait_min;
      posted = wait_min;
    }
    if (did) {
      spins = 0;
      continue;
    }
    if (!idle) {
      idle = true;
      fence_acq_rel_gpu();  // every lane: its flags (and wait report) before the idle mark
      __syncwarp();
      unsigned long long seen = 0;
      if (lane == 0) {
        seen = atomicAdd(&a.ctl->idle, 1ULL) + 1ULL;
        if ((unsigned)seen == (unsigned)W) fence_acq_rel_gpu();  // all flags visible
      }
      seen = __shfl_sync(0xffffffffu, seen, 0);
      if ((unsigned)seen == (unsigned)W) {
        if (!ordered_sched(SCHED) || !raise_threshold<SCHED>(a, lane, W, thr))
          check_done(a, lane, T, seen);
        raised_at = thr;
      }
      continue;
    }
    if (ordered_sched(SCHED) && wait_min != kClean && raised_at != thr &&
        (unsigned)*(volatile unsigned long long *)&a.ctl->idle == (unsigned)W) {
      // every warp idle and this one still waiting: open the next band
      raise_threshold<SCHED>(a, lane, W, thr);
      raised_at = thr;
    }
    int stop = 0;
    if (lane == 0) {
      if (++spins > kSpinLimit) {
        atomicOr(&a.ctl->abort, ABORT_SPIN);
        stop = 1;
      } else {
        __nanosleep(spins < 64 ? 64 : 512);
      }
    }
    if (__shfl_sync(0xffffffffu, stop, 0)) break;
  }
  if (lane == 0 && unflushed) atomicAdd(&a.ctl->visits, unflushed);
}

// Relaxes one tile to its local fixpoint and marks changed neighbours dirty.
template <int KIND, int SCHED>
__device__ void relax_tile(const RelaxArgs &a, WarpTile &t, int lane, int tile, int mode) {
  const int ti = tile % a.tm, tj = tile / a.tm;
  const int64_t i0 = (int64_t)ti * kTile, j0 = (int64_t)tj * kTile;

  __syncwarp();  // the previous visit's reads of the tile are done
  // Stage tile + halo with every load in flight at once.  Lane l carries
  // halo row l (pixel row i0 - 1 + l) of all 34 columns; the two last halo
  // rows (32, 33) are spread over the warp, three columns per lane.  The
  // state (updated concurrently by other SMs) is read from L2 into
  // registers; the read-only aux goes straight to shared memory by
  // asynchronous copies.  Off-grid pixels are staged as state +INF with aux
  // +INF (fill: never lowered, never lowers) or NaN (gwdt: a NaN cost makes
  // every path through the pixel NaN, which never wins a minimum).  gwdt's
  // non-flat pixels arrive with cost NaN from global memory already (state
  // 0 during the run), so no flat flags are staged.
  constexpr float kOffAux = KIND == FILL ? INFINITY : NAN;
  float sv[kHalo], sx[3];
  const int64_t im = i0 - 1 + lane;
  const bool im_ok = im >= 0 && im < a.m;
  const int rx = kTile + (lane & 1);  // halo row 32 or 33
  const int64_t ix = i0 - 1 + rx;
  const bool ix_ok = ix < a.m;
#pragma unroll
  for (int c = 0; c < kHalo; c++) {
    const int64_t j = j0 - 1 + c;
    sv[c] = INFINITY;
    if (im_ok && j >= 0 && j < a.n) {
      const int64_t p = j * a.m + im;
      sv[c] = __ldcg(&a.state[p]);
      cp_async4(&t.a[c][lane], &a.aux[p]);
    } else {
      t.a[c][lane] = kOffAux;
    }
  }
#pragma unroll
  for (int u = 0; u < 3; u++) {
    const int c = (lane >> 1) + 16 * u;
    const int64_t j = j0 - 1 + c;
    sx[u] = INFINITY;
    if (c < kHalo) {
      if (ix_ok && j >= 0 && j < a.n) {
        const int64_t p = j * a.m + ix;
        sx[u] = __ldcg(&a.state[p]);
        cp_async4(&t.a[c][rx], &a.aux[p]);
      } else {
        t.a[c][rx] = kOffAux;
      }
    }
  }
#pragma unroll
  for (int c = 0; c < kHalo; c++) t.s[c][lane] = sv[c];
#pragma unroll
  for (int u = 0; u < 3; u++) {
    const int c = (lane >> 1) + 16 * u;
    if (c < kHalo) t.s[c][rx] = sx[u];
  }
  cp_async_wait_all();
  __syncwarp();

  // Marks in the column layout: lane l holds interior column l + 1, bit k =
  // interior row k + 1.  An edge visit starts from the ring next to the halo.
  uint32_t nd = ((mode & DIRTY_FULL) || lane == 0 || lane == kTile - 1) ? 0xffffffffu
                                                                       : 0x80000001u;
  uint32_t dm = 0;

  // Sweep until no pixel is marked for re-evaluation: the local fixpoint.
  // Down and up run in the column layout, right and left in the row layout
  // (the marks are transposed between the two).
  constexpr int kCap = (!ordered_sched(SCHED) && (SCHED & 2)) ? kCapSweeps : kMaxSweeps;
  bool done = false;
  int sweeps = 0;
  auto rows = [&]() {  // right and left in the row layout
    uint32_t ndr = transpose32(nd, lane), dmr = 0;
    sweep<KIND, true>(t, lane, +1, ndr, dmr);
    sweeps++;
    if (__any_sync(0xffffffffu, ndr != 0)) {
      sweep<KIND, true>(t, lane, -1, ndr, dmr);
      sweeps++;
    }
    nd = transpose32(ndr, lane);
    dm |= transpose32(dmr, lane);
  };
  while (sweeps < kCap) {
    if (!__any_sync(0xffffffffu, nd != 0)) {
      done = true;
      break;
    }
    if (!ordered_sched(SCHED) && (SCHED & 1)) {
      rows();
      if (!__any_sync(0xffffffffu, nd != 0)) {
        done = true;
        break;
      }
    }
    sweep<KIND, false>(t, lane, +1, nd, dm);
    sweeps++;
    if (!__any_sync(0xffffffffu, nd != 0)) {
      done = true;
      break;
    }
    sweep<KIND, false>(t, lane, -1, nd, dm);
    sweeps++;
    if (ordered_sched(SCHED) || !(SCHED & 1)) {
      if (!__any_sync(0xffffffffu, nd != 0)) {
        done = true;
        break;
      }
      rows();
    }
  }

  // Write back changed cells (coalesced per column: lane = row).
#pragma unroll 4
  for (int c = 0; c < kTile; c++) {
    const uint32_t d = __shfl_sync(0xffffffffu, dm, c);
    if (!d) continue;
    if ((d >> lane) & 1u) {
      const int64_t j = j0 + c, i = i0 + lane;
      if (j < a.n && i < a.m) a.state[j * a.m + i] = t.s[c + 1][lane + 1];
    }
  }
  const bool top = __any_sync(0xffffffffu, dm & 1u);
  const bool bottom = __any_sync(0xffffffffu, (dm >> 31) & 1u);
  const uint32_t left = __shfl_sync(0xffffffffu, dm, 0);
  const uint32_t right = __shfl_sync(0xffffffffu, dm, kTile - 1);

  // Lanes 0..8 mark one neighbour each with an atomic OR, after a release
  // fence.  A tile whose edges did not change publishes nothing: only its
  // owner reads its interior again.
  int tgt = -1, val = DIRTY_EDGE;
  switch (lane) {
    case 0: if (top) { tgt = 0; } break;
    case 1: if (bottom) { tgt = 1; } break;
    case 2: if (left) { tgt = 2; } break;
    case 3: if (right) { tgt = 3; } break;
    case 4: if (left & 1u) { tgt = 4; } break;
    case 5: if ((left >> 31) & 1u) { tgt = 5; } break;
    case 6: if (right & 1u) { tgt = 6; } break;
    case 7: if ((right >> 31) & 1u) { tgt = 7; } break;
    case 8: if (!done) { tgt = 8; val = DIRTY_FULL; } break;  // capped: revisit
    default: break;
  }
  if (tgt >= 0) {
    const int di = (tgt == 0 || tgt == 4 || tgt == 6) ? -1 : (tgt == 1 || tgt == 5 || tgt == 7) ? 1 : 0;
    const int dj = (tgt == 2 || tgt == 4 || tgt == 5) ? -1 : (tgt == 3 || tgt == 6 || tgt == 7) ? 1 : 0;
    const int ni = ti + di, nj = tj + dj;
    tgt = (ni < 0 || nj < 0 || ni >= a.tm || nj >= a.tn) ? -1 : nj * a.tm + ni;
  }
  // Every lane fences its own stores, then the warp barrier orders those
  // fences before the flag atomics (the fence-then-barrier publication
  // pattern): a warp that takes a flag and fences sees every store made
  // before it.
  if (!__any_sync(0xffffffffu, tgt >= 0)) return;
  int key = kUrgent;
  if (ordered_sched(SCHED)) {  // the lowest changed value on the tile's edges
    float v = INFINITY;
    if (dm & 1u) v = fminf(v, t.s[lane + 1][1]);
    if ((dm >> 31) & 1u) v = fminf(v, t.s[lane + 1][kTile]);
    if ((left >> lane) & 1u) v = fminf(v, t.s[1][lane + 1]);
    if ((right >> lane) & 1u) v = fminf(v, t.s[kTile][lane + 1]);
    key = __reduce_min_sync(0xffffffffu, value_key(v));
    if (tgt >= 0 && val == DIRTY_FULL) key = kUrgent;  // a capped visit resumes at once
  }
  fence_acq_rel_gpu();
  __syncwarp();
  if (tgt >= 0) {
    if (ordered_sched(SCHED)) atomicMin(&a.prio[tgt], key);
    atomicOr(&a.dirty[tgt], val);
  }
}

// f = dem where bc == 1 (and where dem is NaN), +INF elsewhere
// (src/fillsinks.c:24-37 in the un-negated space).  With `dirty`, the tiles
// whose pixels or halo hold such a seed start dirty: every other tile is
// +INF throughout and already at its local fixpoint until a neighbour
// publishes a change (plain stores: idempotent).
// Marks dirty the tiles whose pixels or halo hold pixel (i, j).
// (Ordered schedules: those tiles also get the most urgent priority.)
__device__ __forceinline__ void mark_tiles_around(int *dirty, int *prio, int tm, int64_t i,
                                                  int64_t j, int64_t m, int64_t n) {
  mark_tiles_near(dirty, tm, i, j, m, n);
  if (!prio) return;
  const int ti0 = (int)((i > 0 ? i - 1 : 0) / kTile), ti1 = (int)((i + 1 < m ? i + 1 : i) / kTile);
  const int tj0 = (int)((j > 0 ? j - 1 : 0) / kTile), tj1 = (int)((j + 1 < n ? j + 1 : j) / kTile);
  for (int tj = tj0; tj <= tj1; tj++)
    for (int ti = ti0; ti <= ti1; ti++) prio[tj * tm + ti] = kUrgent;
}

// Elements per thread and loop trip of the elementwise kernels: their loads
// are all issued before any is used.
constexpr int kEw = 4;

__global__ void fill_init_kernel(float *__restrict__ f, const float *__restrict__ dem,
                                 const uint8_t *__restrict__ bc, int64_t m, int64_t n,
                                 int *__restrict__ dirty, int *__restrict__ prio, int tm) {
  const int64_t N = m * n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p0 < N; p0 += kEw * stride) {
    float z[kEw];
    uint8_t b[kEw];
#pragma unroll
    for (int u = 0; u < kEw; u++) {
      const int64_t p = p0 + u * stride;
      z[u] = p < N ? dem[p] : 0.f;
      b[u] = p < N ? bc[p] : 0;
    }
#pragma unroll
    for (int u = 0; u < kEw; u++) {
      const int64_t p = p0 + u * stride;
      if (p >= N) continue;
      const bool seed = b[u] == 1 || isnan(z[u]);
      f[p] = seed ? z[u] : INFINITY;
      if (seed && dirty) mark_tiles_around(dirty, prio, tm, p % m, p / m, m, n);
    }
  }
}

// ------------------------------------------------------------------
// Sink filling from an upper bound.  The fill is the smallest value, over
// all paths from a pixel to a seed, of the highest pixel on the path; the
// relaxation lowers any start that lies between the fill and the seeded
// +INF start to the same fixpoint (every step keeps an upper bound, and the
// seeded start is the largest upper bound).  A start close to the fill
// needs far fewer tile visits than the flood from the seeds.
//
// The bound is the fill of the DEM max-pooled over kCoarse x kCoarse cells:
// along a path of 8-connected cells there is a path of 8-connected pixels
// through the same cells, from any pixel of the first to any pixel of the
// last, whose highest pixel is at most the largest cell maximum, so the
// coarse fill of a pixel's cell bounds the pixel's fill from above.  A cell
// holding a NaN pixel (a barrier) may be split by it: it gets +INF and is
// never a seed, so no coarse path passes it.
// ------------------------------------------------------------------
constexpr int kCoarse = 4;

// Coarse DEM and seeds; grid: x over coarse rows, y over coarse columns.
// bcc: 1 for a coarse seed, 2 for a cell whose seed pixels cannot make it
// one (it holds a NaN pixel), 0 for a cell without seed pixels.
__global__ void maxpool_kernel(float *__restrict__ dc, uint8_t *__restrict__ bcc,
                               const float *__restrict__ dem, const uint8_t *__restrict__ bc,
                               int64_t m, int64_t n, int64_t mc, int64_t nc) {
  for (int64_t jc = blockIdx.y; jc < nc; jc += gridDim.y)
    for (int64_t ic = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ic < mc;
         ic += (int64_t)gridDim.x * blockDim.x) {
      float mx = -INFINITY;
      bool nan = false, seed = false;
      for (int dj = 0; dj < kCoarse; dj++) {
        const int64_t j = jc * kCoarse + dj;
        if (j >= n) break;
        for (int di = 0; di < kCoarse; di++) {
          const int64_t i = ic * kCoarse + di;
          if (i >= m) break;
          const float v = dem[j * m + i];
          nan |= isnan(v);
          mx = fmaxf(mx, v);
          seed |= bc[j * m + i] == 1;
        }
      }
      dc[jc * mc + ic] = nan ? INFINITY : mx;
      bcc[jc * mc + ic] = !seed ? 0 : nan ? 2 : 1;
    }
}

// The same for grids whose rows come in whole cells (m a multiple of 4,
// so every column of a 16-byte aligned array starts 16-byte aligned): a
// thread takes one cell's four rows of a column with one 16-byte load.
__global__ void maxpool4_kernel(float *__restrict__ dc, uint8_t *__restrict__ bcc,
                                const float4 *__restrict__ dem,
                                const uint32_t *__restrict__ bc, int64_t m, int64_t n,
                                int64_t mc, int64_t nc) {
  const int64_t m4 = m / kCoarse;  // == mc
  for (int64_t jc = blockIdx.y; jc < nc; jc += gridDim.y)
    for (int64_t ic = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ic < mc;
         ic += (int64_t)gridDim.x * blockDim.x) {
      float mx = -INFINITY;
      bool nan = false, seed = false;
      float4 v[kCoarse];
      uint32_t b[kCoarse];
#pragma unroll
      for (int dj = 0; dj < kCoarse; dj++) {
        const int64_t j = jc * kCoarse + dj;
        const int64_t jj = j < n ? j : n - 1;  // a partial last cell repeats its last column
        v[dj] = dem[jj * m4 + ic];
        b[dj] = bc[jj * m4 + ic];
      }
#pragma unroll
      for (int dj = 0; dj < kCoarse; dj++) {
        nan |= isnan(v[dj].x) | isnan(v[dj].y) | isnan(v[dj].z) | isnan(v[dj].w);
        mx = fmaxf(mx, fmaxf(fmaxf(v[dj].x, v[dj].y), fmaxf(v[dj].z, v[dj].w)));
        // bc bytes are 0 or 1 on the path; a seed is a byte equal to 1
        const uint32_t w = b[dj];
        seed |= ((w & 0xffu) == 1u) | (((w >> 8) & 0xffu) == 1u) | (((w >> 16) & 0xffu) == 1u) |
                ((w >> 24) == 1u);
      }
      dc[jc * mc + ic] = nan ? INFINITY : mx;
      bcc[jc * mc + ic] = !seed ? 0 : nan ? 2 : 1;
    }
}

// f = dem at seeds and NaN pixels, max(dem, coarse fill of the pixel's cell)
// elsewhere.
__global__ void fill_bound_init_kernel(float *__restrict__ f, const float *__restrict__ dem,
                                       const uint8_t *__restrict__ bc,
                                       const float *__restrict__ fc, int64_t m, int64_t n,
                                       int64_t mc) {
  for (int64_t j = blockIdx.y; j < n; j += gridDim.y) {
    const float *const fcol = fc + (j / kCoarse) * mc;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
         i += (int64_t)gridDim.x * blockDim.x) {
      const int64_t p = j * m + i;
      const float z = dem[p];
      const bool seed = bc[p] == 1 || isnan(z);
      f[p] = seed ? z : fmaxf(z, fcol[i / kCoarse]);
    }
  }
}

// fill_bound_init_kernel for m a multiple of 4: a thread takes the four
// rows of one cell in one column (one coarse value, 16-byte loads and
// stores).
__global__ void fill_bound_init4_kernel(float4 *__restrict__ f, const float4 *__restrict__ dem,
                                        const uint32_t *__restrict__ bc,
                                        const float *__restrict__ fc, int64_t m, int64_t n,
                                        int64_t mc) {
  const int64_t m4 = m / kCoarse;
  for (int64_t j = blockIdx.y; j < n; j += gridDim.y) {
    const float *const fcol = fc + (j / kCoarse) * mc;
    for (int64_t i4 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i4 < m4;
         i4 += (int64_t)gridDim.x * blockDim.x) {
      const int64_t q = j * m4 + i4;
      const float4 z = dem[q];
      const uint32_t b = bc[q];
      const float c = fcol[i4];
      auto one = [&](float zv, uint32_t bv) {
        return (bv == 1u || isnan(zv)) ? zv : fmaxf(zv, c);
      };
      f[q] = make_float4(one(z.x, b & 0xffu), one(z.y, (b >> 8) & 0xffu),
                         one(z.z, (b >> 16) & 0xffu), one(z.w, b >> 24));
    }
  }
}

// The tiles that can change start dirty: a pixel at +INF is lowered only by
// a finite pixel beside it, and a finite non-seed pixel may lie above the
// fill.  So a tile starts dirty when a coarse cell over it or over its
// one-pixel halo (the ring of cells around it) has a finite bound or a
// seed pixel.  One thread per tile.
__global__ void dirty_bound_kernel(int *__restrict__ dirty, int *__restrict__ prio,
                                   const float *__restrict__ fc,
                                   const uint8_t *__restrict__ bcc, int64_t mc, int64_t nc,
                                   int tm, int T) {
  constexpr int kCells = kTile / kCoarse;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x) {
    const int64_t ic0 = (int64_t)(t % tm) * kCells, jc0 = (int64_t)(t / tm) * kCells;
    const int64_t ia = ic0 > 0 ? ic0 - 1 : 0, ib = ic0 + kCells + 1 < mc ? ic0 + kCells + 1 : mc;
    const int64_t ja = jc0 > 0 ? jc0 - 1 : 0, jb = jc0 + kCells + 1 < nc ? jc0 + kCells + 1 : nc;
    bool any = false;
    for (int64_t jc = ja; jc < jb && !any; jc++)
      for (int64_t ic = ia; ic < ib; ic++)
        if (fc[jc * mc + ic] < INFINITY || bcc[jc * mc + ic]) {
          any = true;
          break;
        }
    if (any) {
      dirty[t] = DIRTY_FULL;
      if (prio) prio[t] = kUrgent;
    }
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

// Mark every tile dirty (fill starts everywhere), most urgent.
__global__ void dirty_all_kernel(int *dirty, int *prio, int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    dirty[t] = DIRTY_FULL;
    if (prio) prio[t] = kUrgent;
  }
}

// gwdt working arrays: distance 1 at presills, +INF at other flats and 0
// at non-flat pixels, as src/gwdt.c:296-308 starts.  Non-flat pixels take
// cost NaN for the run: every path through one and every update of one
// evaluates to NaN, which never wins a minimum, so they keep their 0 and
// pass nothing on.  Tiles next to a presill start dirty.
__global__ void gwdt_init_kernel(float *__restrict__ dist, float *__restrict__ wcost,
                                 const float *__restrict__ costs,
                                 const int32_t *__restrict__ flats, int64_t m,
                                 int64_t n, RelaxArgs qa) {
  const int64_t N = m * n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p0 < N; p0 += kEw * stride) {
    int32_t fv[kEw];
    float cv[kEw];
#pragma unroll
    for (int u = 0; u < kEw; u++) {
      const int64_t p = p0 + u * stride;
      fv[u] = p < N ? flats[p] : 0;
      cv[u] = p < N ? costs[p] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < kEw; u++) {
      const int64_t p = p0 + u * stride;
      if (p >= N) continue;
      const int32_t f = fv[u];
      dist[p] = (f & 5) == 5 ? 1.0f : (f & 1) ? INFINITY : 0.0f;
      wcost[p] = (f & 1) ? cv[u] : NAN;
      if ((f & 5) == 5) mark_tiles_around(qa.dirty, qa.prio, qa.tm, p % m, p / m, m, n);
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

// Visits a warp counts locally before adding them to the shared counter: up
// to 32, fewer when the budget is small enough for the batching to matter.
int visit_flush(unsigned long long max_visits, int warps) {
  const unsigned long long f = max_visits / (64ULL * (unsigned long long)std::max(warps, 1));
  return (int)std::max(1ULL, std::min(32ULL, f));
}

int elementwise_grid(int64_t N) {
  int64_t b = (N + 255) / 256;
  int64_t cap = (int64_t)sm_count() * 16;
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}

// Grid of the column-wise kernels: x over rows (256 threads a block), y over
// columns, about 16 blocks per SM in all.
dim3 col_grid(int64_t rows, int64_t cols) {
  const int64_t bx = std::max<int64_t>(1, std::min<int64_t>((rows + 255) / 256, 8));
  const int64_t by = std::max<int64_t>(
      1, std::min<int64_t>(cols, std::min<int64_t>(65535, (int64_t)sm_count() * 16 / bx)));
  return dim3((unsigned)bx, (unsigned)by);
}

inline bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }
inline bool aligned4(const void *p) { return ((uintptr_t)p & 3u) == 0; }

// Smallest grid side that starts the fill from a coarse bound (0: never);
// TT_CUDA_FILL_BOUND_MIN overrides it.  Measured on the 16384² workload
// generator: 16384² 10.11 -> 9.45 ms (visits per tile 5 -> 3), 8192² no
// change, 4096² slower (1.13 -> 1.42 ms: the coarse run and the full first
// visit of every tile cost more than the visits saved).
int64_t fill_bound_min() {
  static const int64_t v = [] {
    const char *s = std::getenv("TT_CUDA_FILL_BOUND_MIN");
    return s ? (int64_t)std::atoll(s) : (int64_t)12288;
  }();
  return v;
}

// Launches the persistent relaxation as a cooperative kernel: every block
// of the grid is resident at once or the launch is refused
// (cudaErrorCooperativeLaunchTooLarge), so no warp waits for a block that
// cannot be scheduled -- for example while other work holds some SMs.  The
// grid never exceeds the occupancy bound computed for this kernel.
template <int KIND, int SCHED>
cudaError_t launch_relax(int grid, const RelaxArgs &ra, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(kWarps * 32);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  note_launch();
  return cudaLaunchKernelEx(&cfg, relax_persistent_kernel<KIND, SCHED>, ra);
}

// Host driver: mark the starting tiles, run one persistent launch, read the
// status.  `bc` (sink filling only) selects the seeded start: the fill's
// initial state is written here and only tiles next to a seed start dirty;
// without it every tile starts dirty on the caller's initial state.
template <int KIND>
tt_cuda_status run_queue(float *state, const float *aux, const int32_t *flats,
                         const GridDims &g, cudaStream_t st, const uint8_t *bc = nullptr,
                         const float *bound = nullptr, int64_t bound_mc = 0,
                         int64_t bound_nc = 0, bool report = true,
                         int *seeded_dirty = nullptr, const uint8_t *bound_seeds = nullptr) {
  const int T = g.tiles();
  const int sched = relax_schedule();
  const bool ordered = sched >= 4;
  // gwdt seeded by the costs pass: state, costs and flags are in place
  const bool seeded = KIND != FILL && seeded_dirty;
  if (seeded && ordered) return TT_CUDA_ERR_INVALID_ARGUMENT;  // no priorities seeded
  const int wmax = sm_count() * 32 * kWarps;  // more warp slots than any grid has warps
  Workspace &ws = workspace();
  size_t need = align_up(sizeof(QueueCtl)) + align_up((size_t)T * 4);
  if (KIND != FILL && !seeded) need += align_up((size_t)g.cells() * 4);
  if (ordered) need += align_up((size_t)T * 4) + align_up((size_t)wmax * 4);
  if (!ws.reserve(need)) return TT_CUDA_ERR_ALLOC;
  QueueCtl *ctl = (QueueCtl *)ws.take(sizeof(QueueCtl));
  int *dirty = seeded ? seeded_dirty : (int *)ws.take((size_t)T * 4);
  // gwdt relaxes over a copy of the costs with NaN at non-flat pixels (a
  // seeded run over the costs array itself, already in that form)
  float *wcost = KIND == FILL ? nullptr
                 : seeded    ? const_cast<float *>(aux)
                             : (float *)ws.take((size_t)g.cells() * 4);
  int *prio = ordered ? (int *)ws.take((size_t)T * 4) : nullptr;
  int *wmin = ordered ? (int *)ws.take((size_t)wmax * 4) : nullptr;
  QueueCtl *hctl = (QueueCtl *)pinned_scratch();
  if (!hctl) return TT_CUDA_ERR_ALLOC;

  RelaxArgs ra{state, KIND != FILL ? wcost : aux, g.m, g.n, g.tm, g.tn, ctl, dirty, 0, 1,
               prio, wmin};
  if (ordered) {  // no priorities, no waiting work (kClean = 0x7f7f7f7f)
    TT_CHECK(cudaMemsetAsync(prio, 0x7f, (size_t)T * 4, st));
    TT_CHECK(cudaMemsetAsync(wmin, 0x7f, (size_t)wmax * 4, st));
  }
  const int64_t cap_rounds = max_rounds();
  ra.max_visits = (unsigned long long)T * (unsigned long long)std::min<int64_t>(cap_rounds, 1LL << 20);
  TT_CHECK(cudaMemsetAsync(ctl, 0, sizeof(QueueCtl), st));
  const int tgrid = (T + 255) / 256;
  if (KIND == FILL && bc && bound) {
    TT_CHECK(cudaMemsetAsync(dirty, 0, (size_t)T * 4, st));
    if (g.m % kCoarse == 0 && aligned16(state) && aligned16(aux) && aligned4(bc))
      TT_LAUNCH(fill_bound_init4_kernel, col_grid(g.m / kCoarse, g.n), 256, 0, st,
                (float4 *)state, (const float4 *)aux, (const uint32_t *)bc, bound, g.m, g.n,
                bound_mc);
    else
      TT_LAUNCH(fill_bound_init_kernel, col_grid(g.m, g.n), 256, 0, st, state, aux, bc, bound,
                g.m, g.n, bound_mc);
    TT_LAUNCH(dirty_bound_kernel, tgrid, 256, 0, st, dirty, prio, bound, bound_seeds,
              bound_mc, bound_nc, g.tm, T);
  } else if (KIND == FILL && bc) {
    TT_CHECK(cudaMemsetAsync(dirty, 0, (size_t)T * 4, st));
    TT_LAUNCH(fill_init_kernel, elementwise_grid(g.cells()), 256, 0, st, state, aux, bc, g.m,
              g.n, dirty, prio, g.tm);
  } else if (KIND == FILL) {
    TT_LAUNCH(dirty_all_kernel, tgrid, 256, 0, st, dirty, prio, T);
  } else if (!seeded) {
    TT_CHECK(cudaMemsetAsync(dirty, 0, (size_t)T * 4, st));
    TT_LAUNCH(gwdt_init_kernel, elementwise_grid(g.cells()), 256, 0, st, state, wcost, aux,
              flats, g.m, g.n, ra);
  }
  TT_CHECK(cudaGetLastError());
  static int blocks_per_sm[3][kSchedules] = {};
  if (!blocks_per_sm[KIND][sched]) {
    int b = 0;
    switch (sched) {
      case 1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, relax_persistent_kernel<KIND, 1>, kWarps * 32, 0); break;
      case 2: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, relax_persistent_kernel<KIND, 2>, kWarps * 32, 0); break;
      case 3: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, relax_persistent_kernel<KIND, 3>, kWarps * 32, 0); break;
      case 4: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, relax_persistent_kernel<KIND, 4>, kWarps * 32, 0); break;
      case 5: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, relax_persistent_kernel<KIND, 5>, kWarps * 32, 0); break;
      default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, relax_persistent_kernel<KIND, 0>, kWarps * 32, 0); break;
    }
    blocks_per_sm[KIND][sched] = b > 0 ? b : 1;
  }
  // No more warps than tiles (each warp owns at least one tile).
  int grid = sm_count() * blocks_per_sm[KIND][sched];
  grid = std::max(1, std::min(grid, (T + kWarps - 1) / kWarps));
  ra.visit_flush = visit_flush(ra.max_visits, grid * kWarps);
  switch (sched) {
    case 1: TT_CHECK((launch_relax<KIND, 1>(grid, ra, st))); break;
    case 2: TT_CHECK((launch_relax<KIND, 2>(grid, ra, st))); break;
    case 3: TT_CHECK((launch_relax<KIND, 3>(grid, ra, st))); break;
    case 4: TT_CHECK((launch_relax<KIND, 4>(grid, ra, st))); break;
    case 5: TT_CHECK((launch_relax<KIND, 5>(grid, ra, st))); break;
    default: TT_CHECK((launch_relax<KIND, 0>(grid, ra, st))); break;
  }
  TT_CHECK(cudaGetLastError());
  // deferred: the abort word goes to the status sink, no round trip (when the
  // sink is full, the status is read back here as usual)
  if (status_sink() && !report) return TT_CUDA_SUCCESS;  // an intermediate run
  if (int *rec = status_sink() ? sink_record(REC_RELAX, st) : nullptr) {
    TT_CHECK(cudaMemcpyAsync(rec + 1, &ctl->abort, sizeof(int), cudaMemcpyDeviceToDevice, st));
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

namespace {
// `report`: whether this run's iteration cap counts in the call's status (a
// coarse run that stops at the cap still leaves an upper bound).
tt_cuda_status fill_impl(float *f, const float *dem, const uint8_t *bc, const GridDims &g,
                         cudaStream_t st, bool bounded, bool report) {
  const int64_t lim = fill_bound_min();
  if (!bounded || lim <= 0 || g.m < lim || g.n < lim)
    return run_queue<FILL>(f, dem, nullptr, g, st, bc, nullptr, 0, 0, report);
  // The coarse fill (itself started from a coarser bound while large enough).
  const int64_t mc = (g.m + kCoarse - 1) / kCoarse, nc = (g.n + kCoarse - 1) / kCoarse;
  const size_t Nc = (size_t)(mc * nc);
  char *buf = nullptr;
  TT_CHECK(cudaMallocAsync((void **)&buf, align_up(Nc * 4) * 2 + align_up(Nc), st));
  float *dc = (float *)buf, *fc = (float *)(buf + align_up(Nc * 4));
  uint8_t *bcc = (uint8_t *)(buf + 2 * align_up(Nc * 4));
  if (g.m % kCoarse == 0 && aligned16(dem) && aligned4(bc))
    TT_LAUNCH(maxpool4_kernel, col_grid(mc, nc), 256, 0, st, dc, bcc, (const float4 *)dem,
              (const uint32_t *)bc, g.m, g.n, mc, nc);
  else
    TT_LAUNCH(maxpool_kernel, col_grid(mc, nc), 256, 0, st, dc, bcc, dem, bc, g.m, g.n, mc, nc);
  const ptrdiff_t cd[2] = {(ptrdiff_t)mc, (ptrdiff_t)nc};
  tt_cuda_status s = fill_impl(fc, dc, bcc, make_dims(cd), st, true, false);
  // A coarse fill that reached the iteration cap is still an upper bound.
  if (s == TT_CUDA_SUCCESS || s == TT_CUDA_ERR_NOT_CONVERGED)
    s = run_queue<FILL>(f, dem, nullptr, g, st, bc, fc, mc, nc, report, nullptr, bcc);
  cudaFreeAsync(buf, st);
  return s;
}
}  // namespace

tt_cuda_status fill_dev(float *f, const float *dem, const uint8_t *bc,
                        const GridDims &g, cudaStream_t st, bool bounded) {
  return fill_impl(f, dem, bc, g, st, bounded, true);
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

tt_cuda_status gwdt_seeded_dev(float *dist, const float *costs, const int32_t *flats,
                               int *dirty, const GridDims &g, cudaStream_t st) {
  return run_queue<GWDT_HALF>(dist, costs, flats, g, st, nullptr, nullptr, 0, 0, true, dirty);
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
// start at zero, and calls that overlap on the GPU race on it.  The array's
// device address is looked up once per device and kept; a caller that
// resets the device (cudaDeviceReset, which unloads this module) must not
// call this entry point afterwards in the same process.
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
  TT_LAUNCH(fill_init_kernel, elementwise_grid(g.cells()), 256, 0, st, f, dem, bc, g.m,
            g.n, nullptr, nullptr, g.tm);
  TT_CHECK(cudaMemsetAsync(ctl, 0, sizeof(QueueCtl), st));
  TT_LAUNCH(dirty_all_kernel, (T + 255) / 256, 256, 0, st, dirty, (int *)nullptr, T);
  TT_CHECK(cudaGetLastError());
  RelaxArgs ra{f, dem, g.m, g.n, g.tm, g.tn, ctl, dirty, 0, 1, nullptr, nullptr};
  ra.max_visits = (unsigned long long)T *
                  (unsigned long long)std::min<int64_t>(max_rounds(), 1LL << 20);
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, relax_persistent_kernel<FILL, 0>,
                                                kWarps * 32, 0);
  int grid = sm_count() * (b > 0 ? b : 1);
  grid = std::max(1, std::min(grid, (T + kWarps - 1) / kWarps));
  ra.visit_flush = visit_flush(ra.max_visits, grid * kWarps);
  TT_CHECK((launch_relax<FILL, 0>(grid, ra, st)));
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
