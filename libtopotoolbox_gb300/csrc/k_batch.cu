// Batched form: many independent DEMs through the whole D8 pipeline with one
// launch per stage, captured once in a CUDA graph and replayed.
//
// The DEMs are packed into one mosaic grid ("canvas") by shelf packing, each
// separated from its neighbours by a one-pixel gutter of NaN.  Every stage is
// exact on the mosaic because a NaN neighbour behaves exactly like a missing
// (off-grid) neighbour on this path:
//  * fill: fminf ignores NaN, and NaN pixels stay NaN (src/reconstruct.c:178);
//  * identifyflats: a NaN neighbour counts as -INF, so a DEM's outer ring is
//    never flat (the reference skips it, src/identifyflats.c:46-49), and NaN
//    never compares equal in the sill/presill test;
//  * directions: the slope to a NaN neighbour is NaN and never selected;
//    flats, the only pixels that compare the auxiliary topography, are never
//    on a DEM's outer ring;
//  * accumulation: no receiver points into a gutter.
// (A DEM whose outer ring holds -INF is the one exception: such a pixel
// would see a NaN gutter as an equal -INF neighbour.  The batch is meant for
// finite DEMs.)
//
// The canvas width is the tuning parameter (python: libtopotoolbox_gb300.batch
// measures candidates and caches the fastest per batch signature).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "tt_internal.cuh"

using namespace tt;

struct tt_cuda_batch {
  int device = 0;
  int count = 0;
  int64_t Mc = 0, Nc = 0;               // canvas rows (fast) and columns
  std::vector<int64_t> m, n, i0, j0;     // per DEM
  std::vector<int64_t> off;              // prefix of m*n, size count+1
  int64_t *d_tab = nullptr;              // device: m, n, i0, j0, off (5 x count, off count+1)
  void **d_ptr = nullptr;                // device pointer table, 7 x count
  std::vector<const void *> cap_ptr;     // pointers the graph was captured with
  float *dem = nullptr, *filled = nullptr, *costs = nullptr, *dist = nullptr, *acc = nullptr;
  int32_t *flats = nullptr;
  uint8_t *bc = nullptr, *dir = nullptr;
  int *d_sink = nullptr;
  int *h_sink = nullptr;
  int sink_cap = 16;
  Workspace ws;
  cudaStream_t st = nullptr;
  cudaEvent_t ev_in = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t graph_nodes = 0;
};

namespace {

enum { P_DEM = 0, P_BC, P_FILLED, P_FLATS, P_DIST, P_DIR, P_ACC, P_COUNT };

__device__ __forceinline__ int find_dem(const int64_t *off, int count, int64_t q) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= q) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// canvas <- DEMs and boundary conditions
__global__ void pack_kernel(const int64_t *__restrict__ tab, void *const *__restrict__ ptr,
                            int count, int64_t total, int64_t Mc, float *cdem, uint8_t *cbc) {
  const int64_t *m = tab, *i0 = tab + 2 * count, *j0 = tab + 3 * count, *off = tab + 4 * count;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int b = find_dem(off, count, q);
    const int64_t l = q - off[b], i = l % m[b], j = l / m[b];
    const int64_t p = (j0[b] + j) * Mc + (i0[b] + i);
    cdem[p] = ((const float *)ptr[P_DEM * count + b])[l];
    cbc[p] = ((const uint8_t *)ptr[P_BC * count + b])[l];
  }
}

// DEM outputs <- canvas (an output family with a NULL table entry is skipped)
__global__ void unpack_kernel(const int64_t *__restrict__ tab, void *const *__restrict__ ptr,
                              int count, int64_t total, int64_t Mc, const float *filled,
                              const int32_t *flats, const float *dist, const uint8_t *dir,
                              const float *acc) {
  const int64_t *m = tab, *i0 = tab + 2 * count, *j0 = tab + 3 * count, *off = tab + 4 * count;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int b = find_dem(off, count, q);
    const int64_t l = q - off[b], i = l % m[b], j = l / m[b];
    const int64_t p = (j0[b] + j) * Mc + (i0[b] + i);
    if (void *o = ptr[P_FILLED * count + b]) ((float *)o)[l] = filled[p];
    if (void *o = ptr[P_FLATS * count + b]) ((int32_t *)o)[l] = flats[p];
    if (void *o = ptr[P_DIST * count + b]) ((float *)o)[l] = dist[p];
    if (void *o = ptr[P_DIR * count + b]) ((uint8_t *)o)[l] = dir[p];
    if (void *o = ptr[P_ACC * count + b]) ((float *)o)[l] = acc[p];
  }
}

int ew_grid(int64_t N) {
  int64_t b = (N + 255) / 256;
  int64_t cap = (int64_t)sm_count() * 16;
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}

// Shelf packing: DEMs by decreasing height; a shelf is a band of rows whose
// height is its tallest DEM; DEMs go left to right with one gutter column.
void plan(tt_cuda_batch *b, int64_t canvas_cols) {
  const int B = b->count;
  std::vector<int> idx(B);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return b->m[x] > b->m[y]; });
  int64_t widest = 0;
  for (int k = 0; k < B; k++) widest = std::max(widest, b->n[k]);
  const int64_t Nc = std::max(canvas_cols, widest + 2);
  int64_t row = 1, col = 1, shelf_h = 0;
  for (int k : idx) {
    if (col + b->n[k] + 1 > Nc) {  // next shelf
      row += shelf_h + 1;
      col = 1;
      shelf_h = 0;
    }
    b->i0[k] = row;
    b->j0[k] = col;
    col += b->n[k] + 1;
    shelf_h = std::max(shelf_h, b->m[k]);
  }
  b->Mc = row + shelf_h + 1;
  b->Nc = Nc;
}

// Every stage of the pipeline on the canvas, without host round trips.
tt_cuda_status enqueue(tt_cuda_batch *b, cudaStream_t st) {
  const int64_t N = b->Mc * b->Nc;
  const ptrdiff_t dims[2] = {(ptrdiff_t)b->Mc, (ptrdiff_t)b->Nc};
  const GridDims g = make_dims(dims);
  const int64_t total = b->off[b->count];
  TT_CHECK(cudaMemsetAsync(b->d_sink, 0, (size_t)b->sink_cap * kRecordInts * 4, st));
  TT_CHECK(cudaMemsetAsync(b->dem, 0xff, (size_t)N * 4, st));  // NaN gutters
  TT_CHECK(cudaMemsetAsync(b->bc, 0, (size_t)N, st));
  TT_LAUNCH(pack_kernel, ew_grid(total), 256, 0, st, b->d_tab, b->d_ptr, b->count, total,
            b->Mc, b->dem, b->bc);
  TT_CHECK(cudaGetLastError());
  tt_cuda_status s;
  if ((s = fill_dev(b->filled, b->dem, b->bc, g, st, false)) != TT_CUDA_SUCCESS) return s;
  if ((s = identifyflats_dev(b->flats, b->filled, g, nullptr, st)) != TT_CUDA_SUCCESS) return s;
  if ((s = costs_dev(b->costs, nullptr, b->flats, b->dem, b->filled, g, st)) != TT_CUDA_SUCCESS)
    return s;
  if ((s = gwdt_dev(b->dist, nullptr, b->costs, b->flats, g, st)) != TT_CUDA_SUCCESS) return s;
  if ((s = directions_dev(b->dir, b->filled, b->dist, b->flats, g, 0, st)) != TT_CUDA_SUCCESS)
    return s;
  if ((s = accumulate_dev(b->acc, b->dir, nullptr, g, st)) != TT_CUDA_SUCCESS) return s;
  TT_LAUNCH(unpack_kernel, ew_grid(total), 256, 0, st, b->d_tab, b->d_ptr, b->count, total,
            b->Mc, b->filled, b->flats, b->dist, b->dir, b->acc);
  TT_CHECK(cudaGetLastError());
  return TT_CUDA_SUCCESS;
}

// Status recorded by the deferred stages.
tt_cuda_status read_sink(tt_cuda_batch *b, int records) {
  return sink_status(b->h_sink, records);
}

void free_batch(tt_cuda_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->ev_in) cudaEventDestroy(b->ev_in);
  if (b->st) cudaStreamDestroy(b->st);
  cudaFree(b->d_tab);
  cudaFree(b->d_ptr);
  cudaFree(b->dem);
  cudaFree(b->filled);
  cudaFree(b->costs);
  cudaFree(b->dist);
  cudaFree(b->acc);
  cudaFree(b->flats);
  cudaFree(b->bc);
  cudaFree(b->dir);
  cudaFree(b->d_sink);
  if (b->h_sink) cudaFreeHost(b->h_sink);
  b->ws.release();
  delete b;
}

}  // namespace

extern "C" {

tt_cuda_status tt_cuda_batch_create(int count, const ptrdiff_t *dims, int64_t canvas_cols,
                                    tt_cuda_batch **out) {
  if (!out || !dims || count <= 0) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return TT_CUDA_ERR_INVALID_ARGUMENT;
  }
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_status(TT_CUDA_ERR_NO_DEVICE);
    return TT_CUDA_ERR_NO_DEVICE;
  }
  tt_cuda_batch *b = new tt_cuda_batch();
  cudaGetDevice(&b->device);
  b->count = count;
  b->m.resize(count);
  b->n.resize(count);
  b->i0.resize(count);
  b->j0.resize(count);
  b->off.assign(count + 1, 0);
  double area = 0;
  for (int k = 0; k < count; k++) {
    b->m[k] = dims[2 * k];
    b->n[k] = dims[2 * k + 1];
    if (b->m[k] <= 0 || b->n[k] <= 0) {
      delete b;
      set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
      return TT_CUDA_ERR_INVALID_ARGUMENT;
    }
    b->off[k + 1] = b->off[k] + b->m[k] * b->n[k];
    area += (double)(b->m[k] + 1) * (double)(b->n[k] + 1);
  }
  if (canvas_cols <= 0) canvas_cols = (int64_t)std::ceil(std::sqrt(area * 1.15));
  plan(b, canvas_cols);
  const int64_t N = b->Mc * b->Nc;
  if (N >= (1LL << 31)) {
    delete b;
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return TT_CUDA_ERR_INVALID_ARGUMENT;
  }
  std::vector<int64_t> tab;
  for (auto *v : {&b->m, &b->n, &b->i0, &b->j0}) tab.insert(tab.end(), v->begin(), v->end());
  tab.insert(tab.end(), b->off.begin(), b->off.end());
  bool ok = cudaMalloc(&b->d_tab, tab.size() * 8) == cudaSuccess &&
            cudaMalloc(&b->d_ptr, (size_t)P_COUNT * count * sizeof(void *)) == cudaSuccess &&
            cudaMalloc(&b->dem, N * 4) == cudaSuccess &&
            cudaMalloc(&b->filled, N * 4) == cudaSuccess &&
            cudaMalloc(&b->costs, N * 4) == cudaSuccess &&
            cudaMalloc(&b->dist, N * 4) == cudaSuccess &&
            cudaMalloc(&b->acc, N * 4) == cudaSuccess &&
            cudaMalloc(&b->flats, N * 4) == cudaSuccess &&
            cudaMalloc(&b->bc, N) == cudaSuccess && cudaMalloc(&b->dir, N) == cudaSuccess &&
            cudaMalloc(&b->d_sink, (size_t)b->sink_cap * kRecordInts * 4) == cudaSuccess &&
            cudaMallocHost(&b->h_sink, (size_t)b->sink_cap * kRecordInts * 4) == cudaSuccess &&
            cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming) == cudaSuccess &&
            cudaMemcpy(b->d_tab, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    free_batch(b);
    set_status(TT_CUDA_ERR_ALLOC);
    return TT_CUDA_ERR_ALLOC;
  }
  *out = b;
  set_status(TT_CUDA_SUCCESS);
  return TT_CUDA_SUCCESS;
}

tt_cuda_status tt_cuda_batch_info(const tt_cuda_batch *b, int64_t *info) {
  if (!b || !info) return TT_CUDA_ERR_INVALID_ARGUMENT;
  info[0] = b->Mc;
  info[1] = b->Nc;
  info[2] = b->off[b->count];
  info[3] = b->graph_nodes;
  return TT_CUDA_SUCCESS;
}

tt_cuda_status tt_cuda_batch_run(tt_cuda_batch *b, const float *const *dem,
                                 const uint8_t *const *bc, float *const *filled,
                                 int32_t *const *flats, float *const *dist,
                                 uint8_t *const *direction, float *const *acc,
                                 void *stream) {
  if (!b || !dem || !bc) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return TT_CUDA_ERR_INVALID_ARGUMENT;
  }
  cudaSetDevice(b->device);
  DeviceLock lock;
  const int B = b->count;
  std::vector<const void *> ptrs((size_t)P_COUNT * B, nullptr);
  for (int k = 0; k < B; k++) {
    ptrs[P_DEM * B + k] = dem[k];
    ptrs[P_BC * B + k] = bc[k];
    if (filled) ptrs[P_FILLED * B + k] = filled[k];
    if (flats) ptrs[P_FLATS * B + k] = flats[k];
    if (dist) ptrs[P_DIST * B + k] = dist[k];
    if (direction) ptrs[P_DIR * B + k] = direction[k];
    if (acc) ptrs[P_ACC * B + k] = acc[k];
  }
  // Order this work after the caller's stream.
  cudaStream_t user = (cudaStream_t)stream;
  tt_cuda_status s = TT_CUDA_SUCCESS;
  if (cudaEventRecord(b->ev_in, user) != cudaSuccess ||
      cudaStreamWaitEvent(b->st, b->ev_in, 0) != cudaSuccess) {
    cudaGetLastError();
    set_status(TT_CUDA_ERR_CUDA);
    return TT_CUDA_ERR_CUDA;
  }
  StatusSink sink{b->d_sink, b->sink_cap, 0};
  {
    SinkScope scope(&sink, &b->ws);
    if (!b->exec || ptrs != b->cap_ptr) {
      // A plain run sizes the private workspace and produces this call's
      // result; the same sequence is then captured for later calls.
      if (cudaMemcpyAsync(b->d_ptr, ptrs.data(), ptrs.size() * sizeof(void *),
                          cudaMemcpyHostToDevice, b->st) != cudaSuccess) s = TT_CUDA_ERR_CUDA;
      if (s == TT_CUDA_SUCCESS) s = enqueue(b, b->st);
      const int records = sink.next;
      if (s == TT_CUDA_SUCCESS &&
          cudaMemcpyAsync(b->h_sink, b->d_sink, (size_t)records * kRecordInts * 4,
                          cudaMemcpyDeviceToHost, b->st) != cudaSuccess)
        s = TT_CUDA_ERR_CUDA;
      if (cudaStreamSynchronize(b->st) != cudaSuccess) s = TT_CUDA_ERR_CUDA;
      if (s == TT_CUDA_SUCCESS) s = read_sink(b, records);
      if (s == TT_CUDA_SUCCESS || s == TT_CUDA_ERR_NOT_CONVERGED || s == TT_CUDA_ERR_CYCLE) {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
        cudaGraph_t graph = nullptr;
        sink.next = 0;
        tt_cuda_status cs = TT_CUDA_SUCCESS;
        if (cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
          cs = TT_CUDA_ERR_CUDA;
        if (cs == TT_CUDA_SUCCESS) {
          cs = enqueue(b, b->st);
          cudaMemcpyAsync(b->h_sink, b->d_sink, (size_t)sink.next * kRecordInts * 4,
                          cudaMemcpyDeviceToHost, b->st);
          if (cudaStreamEndCapture(b->st, &graph) != cudaSuccess) cs = TT_CUDA_ERR_CUDA;
        }
        if (cs == TT_CUDA_SUCCESS &&
            cudaGraphInstantiate(&b->exec, graph, 0) != cudaSuccess) cs = TT_CUDA_ERR_CUDA;
        if (graph) {
          size_t nn = 0;
          cudaGraphGetNodes(graph, nullptr, &nn);
          b->graph_nodes = (int64_t)nn;
          cudaGraphDestroy(graph);
        }
        if (cs == TT_CUDA_SUCCESS) {
          b->cap_ptr = ptrs;
        } else {
          cudaGetLastError();
          b->exec = nullptr;
          b->cap_ptr.clear();
        }
      }
    } else {
      if (cudaGraphLaunch(b->exec, b->st) != cudaSuccess) s = TT_CUDA_ERR_CUDA;
      if (cudaStreamSynchronize(b->st) != cudaSuccess) s = TT_CUDA_ERR_CUDA;
      if (s == TT_CUDA_SUCCESS) s = read_sink(b, b->sink_cap);
    }
  }  // scope
  if (s == TT_CUDA_ERR_CUDA) cudaGetLastError();
  set_status(s);
  return s;
}

void tt_cuda_batch_destroy(tt_cuda_batch *b) {
  if (!b) return;
  cudaSetDevice(b->device);
  DeviceLock lock;
  cudaStreamSynchronize(b->st);
  free_batch(b);
}

}  // extern "C"
