// Sweeps over arbitrary edge lists:
//
//  * flow_accumulation_edgelist (src/flow_accumulation.c:10-30):
//      acc = weights (or 1); for e in list order: acc[tgt] += f[e] * acc[src]
//  * traverse_down_f32_add_mul (src/streamquad.c:171-180):
//      for e in list order: out[tgt] = out[tgt] + out[src] * in[e]
//  * traverse_down_u32_or_and (src/streamquad.c:49-60):
//      for e in list order: out[tgt] = out[tgt] | (out[src] & in[e])
//  * traverse_up_u32_or_and (src/streamquad.c:37-47):
//      for e in reverse list order: out[src] = out[src] | (out[tgt] & in[e]),
//      which is the downward sweep of the reversed list with source and
//      target exchanged (edge e of the reversed list is edge E - 1 - e).
//
// All are the same recurrence over the list order, in the (+, *) semiring
// (in FP64, rounded once) or the (|, &) one (exact).  For any order -- a
// topological one (every edge into a node listed before every edge out of
// it, as the routing functions produce) or not -- the value an edge e = (u, v)
// carries is
//      val(e) = f(e) * (w(u) + sum of val(e') over edges e' into u with e' < e)
// and the result is out(v) = w(v) + sum of val(e) over every edge into v
// (with | and & for + and * in the other semiring).
// val(e) depends only on edges listed before e, so the edges form a DAG by
// index and the recurrence has a unique value for every list.
//
// GPU form.  The edges are grouped by target and by source (radix sort of
// (node, edge) keys), so each node's in- and out-edges are in list order.
// pend(e) counts the in-edges of u listed before e.  Walks start at edges
// with pend 0; a walker computes val(e) by pulling the values of those
// in-edges in list order, then counts itself off every out-edge of v listed
// after e, and continues with each edge whose count it took to zero (a
// small private stack, spilling to a global work list that a further launch
// drains).  Every edge is computed exactly once, by the last contributor to
// arrive, and every sum is taken in list order in FP64: the result does not
// depend on thread timing and is rounded once to float32.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <climits>

#include "tt_internal.cuh"

namespace tt {
namespace {

constexpr int kWalkStack = 24;

enum : int { EF_BAD_INDEX = 1, EF_CYCLE = 2 };

struct FlowArgs {
  const ptrdiff_t *src;
  const ptrdiff_t *tgt;
  const void *frac;    // per edge: float (+, *) or uint32 (|, &)
  const void *w;       // per node start value, the output's type (nullptr: 1)
  int64_t N, E;
  bool rev;            // sweep the reversed list, source and target exchanged
  const int *in_off;   // N + 1: edges into each node ...
  const int *in_list;  // ... in list order
  const int *out_off;  // N + 1: edges out of each node ...
  const int *out_list;
  int *pend;      // per edge: earlier in-edges of its source not yet computed
  void *val;      // per edge, 8 bytes: double (+, *) or uint32 (|, &)
  int *work;      // spill list of ready edges (each edge enters at most once)
  int *ctl;       // [0] spill count, [1] edges computed, [2] error bits
};

// Edge e of the swept list: its source, target and list position.
__device__ __forceinline__ int64_t e_src(const FlowArgs &a, int64_t e) {
  return a.rev ? a.tgt[a.E - 1 - e] : a.src[e];
}
__device__ __forceinline__ int64_t e_tgt(const FlowArgs &a, int64_t e) {
  return a.rev ? a.src[a.E - 1 - e] : a.tgt[e];
}
__device__ __forceinline__ int64_t e_pos(const FlowArgs &a, int64_t e) {
  return a.rev ? a.E - 1 - e : e;
}

// The two semirings.
struct AddMul {  // (+, *) carried in FP64, float in and out
  using T = double;
  static __device__ T start(const FlowArgs &a, int64_t u) {
    return a.w ? (double)static_cast<const float *>(a.w)[u] : 1.0;
  }
  static __device__ T add(T s, T x) { return s + x; }
  static __device__ T mul(const FlowArgs &a, int64_t e, T s) {
    return (double)static_cast<const float *>(a.frac)[e_pos(a, e)] * s;
  }
  static __device__ void store(void *out, int64_t v, T s) {
    static_cast<float *>(out)[v] = (float)s;
  }
};
struct OrAnd {  // (|, &) on 32-bit words, exact
  using T = uint32_t;
  static __device__ T start(const FlowArgs &a, int64_t u) {
    return a.w ? static_cast<const uint32_t *>(a.w)[u] : 0xffffffffu;
  }
  static __device__ T add(T s, T x) { return s | x; }
  static __device__ T mul(const FlowArgs &a, int64_t e, T s) {
    return static_cast<const uint32_t *>(a.frac)[e_pos(a, e)] & s;
  }
  static __device__ void store(void *out, int64_t v, T s) {
    static_cast<uint32_t *>(out)[v] = s;
  }
};

int list_grid(int64_t n) {
  int64_t b = (n + 255) / 256;
  int64_t cap = (int64_t)sm_count() * 16;
  return (int)std::max<int64_t>(1, std::min(b, cap));
}

// Validates the indices, counts degrees and builds the sort keys
// (node << 32 | edge) of the swept list.
__global__ void ef_keys_kernel(FlowArgs a, unsigned long long *__restrict__ kin,
                               unsigned long long *__restrict__ kout, int *__restrict__ din,
                               int *__restrict__ dout, int *__restrict__ err) {
  const int64_t E = a.E, N = a.N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = e_src(a, e), v = e_tgt(a, e);
    if (u < 0 || u >= N || v < 0 || v >= N) {
      atomicOr(err, EF_BAD_INDEX);
      kin[e] = kout[e] = 0;
      continue;
    }
    kin[e] = ((unsigned long long)v << 32) | (unsigned long long)e;
    kout[e] = ((unsigned long long)u << 32) | (unsigned long long)e;
    atomicAdd(&din[v], 1);
    atomicAdd(&dout[u], 1);
  }
}

__global__ void ef_extract_kernel(const unsigned long long *__restrict__ sin,
                                  const unsigned long long *__restrict__ sout, int64_t E,
                                  int *__restrict__ in_list, int *__restrict__ out_list) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < E;
       i += (int64_t)gridDim.x * blockDim.x) {
    in_list[i] = (int)(unsigned)(sin[i] & 0xffffffffULL);
    out_list[i] = (int)(unsigned)(sout[i] & 0xffffffffULL);
  }
}

// First position in list[lo, hi) (ascending) holding a value > x.
__device__ __forceinline__ int first_after(const int *list, int lo, int hi, int x) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (list[mid] <= x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// pend(e) = in-edges of src(e) listed before e; edges with none start walks.
__global__ void ef_pend_kernel(FlowArgs a, int *__restrict__ starts, int *__restrict__ nstart) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < a.E;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = e_src(a, e);
    const int lo = a.in_off[u];
    const int p = first_after(a.in_list, lo, a.in_off[u + 1], (int)e - 1) - lo;
    a.pend[e] = p;
    if (p == 0) starts[append_slot(nstart)] = (int)e;
  }
}

// Value of node u just before edge x is applied: w(u) plus the values of
// its in-edges listed before x, in list order.
template <class S>
__device__ __forceinline__ typename S::T value_before(const FlowArgs &a, int64_t u, int x) {
  using T = typename S::T;
  T s = S::start(a, u);
  const T *val = static_cast<const T *>(a.val);
  const int hi = a.in_off[u + 1];
  for (int k = a.in_off[u]; k < hi; k++) {
    const int e2 = a.in_list[k];
    if (e2 >= x) break;
    s = S::add(s, __ldcg(&val[e2]));
  }
  return s;
}

// Walks from the ready edges list[base, base + n), n = *n_dev when n_dev is
// set (a count that no longer changes during this launch), else n_host.
template <class S>
__global__ void ef_walk_kernel(FlowArgs a, const int *__restrict__ list,
                               const int *__restrict__ n_dev, int n_host, int base) {
  const int n = n_dev ? *n_dev : n_host;
  int done = 0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    int stack[kWalkStack];
    int sp = 0;
    stack[sp++] = list[base + t];
    while (sp) {
      const int x = stack[--sp];
      const int64_t u = e_src(a, x), v = e_tgt(a, x);
      static_cast<typename S::T *>(a.val)[x] = S::mul(a, x, value_before<S>(a, u, x));
      done++;
      __threadfence();  // val(x) before the counts that announce it
      const int hi = a.out_off[v + 1];
      for (int k = first_after(a.out_list, a.out_off[v], hi, x); k < hi; k++) {
        const int o = a.out_list[k];
        if (atomicSub(&a.pend[o], 1) != 1) continue;
        __threadfence();  // every earlier in-edge of v is visible now
        if (sp < kWalkStack) stack[sp++] = o;
        else a.work[atomicAdd(&a.ctl[0], 1)] = o;
      }
    }
  }
  if (done) atomicAdd(&a.ctl[1], done);
}

// out(v) = w(v) + the values of every edge into v, in list order.
template <class S>
__global__ void ef_final_kernel(FlowArgs a, void *__restrict__ out) {
  using T = typename S::T;
  const T *val = static_cast<const T *>(a.val);
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < a.N;
       v += (int64_t)gridDim.x * blockDim.x) {
    T s = S::start(a, v);
    for (int k = a.in_off[v]; k < a.in_off[v + 1]; k++) s = S::add(s, val[a.in_list[k]]);
    S::store(out, v, s);
  }
}

__global__ void ef_max_index_kernel(const ptrdiff_t *__restrict__ src,
                                    const ptrdiff_t *__restrict__ tgt, int64_t E,
                                    unsigned long long *__restrict__ mx) {
  unsigned long long m = 0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
       e += (int64_t)gridDim.x * blockDim.x) {
    const ptrdiff_t u = src[e], v = tgt[e];
    // a negative index gives the largest count, which the caller refuses
    m = (u < 0 || v < 0) ? ~0ULL : max(m, (unsigned long long)max(u, v) + 1ULL);
  }
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m) atomicMax(mx, m);
}

int bits_for(int64_t n) {
  int b = 1;
  while (b < 31 && (1LL << b) < n) b++;
  return b;
}

template <class S>
tt_cuda_status edge_sweep_impl(void *out, const void *w, const ptrdiff_t *source,
                               const ptrdiff_t *target, const void *frac, int64_t E, int64_t N,
                               bool rev, cudaStream_t st) {
  if (N <= 0) return TT_CUDA_SUCCESS;
  const int64_t Em = std::max<int64_t>(E, 1);
  const int nbs = scan_blocks_for(N + 1);
  size_t sort_tmp = 0;
  cub::DeviceRadixSort::SortKeys(nullptr, sort_tmp, (unsigned long long *)nullptr,
                                 (unsigned long long *)nullptr, (int)Em, 0, 64, st);
  Workspace &ws = workspace();
  const size_t need = 256 + 4 * align_up((size_t)Em * 8) + 2 * align_up((size_t)(N + 1) * 4) +
                      2 * align_up((size_t)(N + 1) * 4) + 5 * align_up((size_t)Em * 4) +
                      2 * align_up((size_t)(nbs + 1) * 4) + align_up(sort_tmp) + 4096;
  if (!ws.reserve(need)) return TT_CUDA_ERR_ALLOC;
  int *ctl = (int *)ws.take(256);  // [0] spill, [1] computed, [2] errors, [3] starts
  unsigned long long *kin = (unsigned long long *)ws.take((size_t)Em * 8);
  unsigned long long *kout = (unsigned long long *)ws.take((size_t)Em * 8);
  unsigned long long *sin = (unsigned long long *)ws.take((size_t)Em * 8);
  unsigned long long *sout = (unsigned long long *)ws.take((size_t)Em * 8);
  int *din = (int *)ws.take((size_t)(N + 1) * 4);
  int *dout = (int *)ws.take((size_t)(N + 1) * 4);
  int *in_off = (int *)ws.take((size_t)(N + 1) * 4);
  int *out_off = (int *)ws.take((size_t)(N + 1) * 4);
  int *in_list = (int *)ws.take((size_t)Em * 4);
  int *out_list = (int *)ws.take((size_t)Em * 4);
  int *pend = (int *)ws.take((size_t)Em * 4);
  int *starts = (int *)ws.take((size_t)Em * 4);
  int *work = (int *)ws.take((size_t)Em * 4);
  int *cnt = (int *)ws.take((size_t)(nbs + 1) * 4);
  int *off = (int *)ws.take((size_t)(nbs + 1) * 4);
  void *tmp = ws.take(sort_tmp);
  // The values (8 bytes an edge at most) reuse the key buffers, which are
  // spent once the lists exist.
  void *val = kin;

  TT_CHECK(cudaMemsetAsync(ctl, 0, 256, st));
  TT_CHECK(cudaMemsetAsync(din, 0, (size_t)(N + 1) * 4, st));
  TT_CHECK(cudaMemsetAsync(dout, 0, (size_t)(N + 1) * 4, st));
  const int eg = list_grid(E);
  FlowArgs a{source, target, frac, w, N, E, rev, nullptr, nullptr, nullptr, nullptr,
             pend, val, work, ctl};
  if (E > 0) TT_LAUNCH(ef_keys_kernel, eg, 256, 0, st, a, kin, kout, din, dout, ctl + 2);
  int *h = (int *)pinned_scratch();
  if (!h) return TT_CUDA_ERR_ALLOC;
  TT_CHECK(cudaMemcpyAsync(h, ctl + 2, 4, cudaMemcpyDeviceToHost, st));
  TT_CHECK(cudaStreamSynchronize(st));
  if (h[0] & EF_BAD_INDEX) return TT_CUDA_ERR_INVALID_ARGUMENT;
  TT_TRY_STATUS(scan_exclusive_dev(din, N + 1, in_off, cnt, off, st));
  TT_TRY_STATUS(scan_exclusive_dev(dout, N + 1, out_off, cnt, off, st));
  a.in_off = in_off;
  a.in_list = in_list;
  a.out_off = out_off;
  a.out_list = out_list;
  if (E > 0) {
    const int end_bit = 32 + bits_for(N);
    size_t tb = sort_tmp;
    TT_CHECK(cub::DeviceRadixSort::SortKeys(tmp, tb, kin, sin, (int)E, 0, end_bit, st));
    tb = sort_tmp;
    TT_CHECK(cub::DeviceRadixSort::SortKeys(tmp, tb, kout, sout, (int)E, 0, end_bit, st));
    TT_LAUNCH(ef_extract_kernel, eg, 256, 0, st, sin, sout, E, in_list, out_list);
    TT_LAUNCH(ef_pend_kernel, eg, 256, 0, st, a, starts, ctl + 3);
    TT_LAUNCH(ef_walk_kernel<S>, eg, 256, 0, st, a, starts, ctl + 3, 0, 0);
    // Drain the spill list: each launch walks the edges spilled by the
    // previous one.  Every edge is spilled at most once, so this ends.
    int base = 0;
    for (int round = 0;; round++) {
      TT_CHECK(cudaMemcpyAsync(h, ctl, 8, cudaMemcpyDeviceToHost, st));
      TT_CHECK(cudaStreamSynchronize(st));
      const int spilled = h[0];
      if (spilled == base) break;
      if (round > E) return TT_CUDA_ERR_CYCLE;  // cannot happen: bounded by E
      TT_LAUNCH(ef_walk_kernel<S>, list_grid(spilled - base), 256, 0, st, a, work,
                (const int *)nullptr, spilled - base, base);
      base = spilled;
    }
    if (h[1] != (int)E) return TT_CUDA_ERR_CYCLE;  // an edge was never reached
  }
  TT_LAUNCH(ef_final_kernel<S>, list_grid(N), 256, 0, st, a, out);
  TT_CHECK(cudaGetLastError());
  return TT_CUDA_SUCCESS;
}

}  // namespace

tt_cuda_status edge_sweep_dev(float *out, const float *w, const ptrdiff_t *source,
                              const ptrdiff_t *target, const float *frac, int64_t E, int64_t N,
                              cudaStream_t st) {
  return edge_sweep_impl<AddMul>(out, w, source, target, frac, E, N, false, st);
}

tt_cuda_status edge_sweep_u32_dev(uint32_t *out, const uint32_t *w, const ptrdiff_t *source,
                                  const ptrdiff_t *target, const uint32_t *in, int64_t E,
                                  int64_t N, bool up, cudaStream_t st) {
  return edge_sweep_impl<OrAnd>(out, w, source, target, in, E, N, up, st);
}

// 1 + the largest node index in the edge list (0 for an empty list), read
// back to the host; negative indices come back as a huge count.
tt_cuda_status edge_node_count_dev(const ptrdiff_t *source, const ptrdiff_t *target, int64_t E,
                                   int64_t *count, cudaStream_t st) {
  *count = 0;
  if (E <= 0) return TT_CUDA_SUCCESS;
  Workspace &ws = workspace();
  if (!ws.reserve(256)) return TT_CUDA_ERR_ALLOC;
  unsigned long long *mx = (unsigned long long *)ws.take(256);
  TT_CHECK(cudaMemsetAsync(mx, 0, 8, st));
  TT_LAUNCH(ef_max_index_kernel, list_grid(E), 256, 0, st, source, target, E, mx);
  unsigned long long *h = (unsigned long long *)pinned_scratch();
  if (!h) return TT_CUDA_ERR_ALLOC;
  TT_CHECK(cudaMemcpyAsync(h, mx, 8, cudaMemcpyDeviceToHost, st));
  TT_CHECK(cudaStreamSynchronize(st));
  *count = *h > (unsigned long long)INT64_MAX ? INT64_MAX : (int64_t)*h;
  return TT_CUDA_SUCCESS;
}

}  // namespace tt
