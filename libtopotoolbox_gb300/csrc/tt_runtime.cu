// Runtime and C ABI of libtt_cuda: per-thread status, per-device
// workspaces and call locks, and the public entry points of
// include/tt_cuda.h.  Host-pointer entry points stage their arrays through
// device buffers and call the device-pointer stage functions.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "tt_internal.cuh"

namespace tt {

namespace {
thread_local tt_cuda_status g_status = TT_CUDA_SUCCESS;
thread_local int64_t g_launches = 0;
thread_local int64_t g_last_rounds = 0;
thread_local StatusSink *g_sink = nullptr;
thread_local Workspace *g_ws_override = nullptr;
thread_local Workspace *g_io_override = nullptr;
thread_local int g_relax_schedule = -1;  // -1: the environment's or 0
int64_t g_max_rounds_override = 0;

constexpr int kMaxDevices = 64;
constexpr int kCopyEvents = 24;

struct DeviceState {
  std::mutex mu;
  Workspace scratch;
  Workspace io;
  void *pinned = nullptr;
  int sms = 0;
  // side streams and events for host-device copies that overlap the
  // kernels of a host-pointer call
  cudaStream_t copy = nullptr, copy2 = nullptr;
  cudaEvent_t ready[kCopyEvents] = {};
};

DeviceState g_dev[kMaxDevices];

// Deferred status of one thread's device-pointer calls
// (tt_cuda_defer_begin / tt_cuda_defer_end).  Deferred calls take their
// scratch from private workspaces, because their work is still in flight
// when the call returns and the device's shared workspaces are reused by
// the next call of any thread.
struct Deferral {
  int device = -1;
  bool active = false;
  cudaStream_t stream = nullptr;
  Workspace ws, io;
  int *d_rec = nullptr, *h_rec = nullptr;  // kDeferRecords status records
  StatusSink sink{nullptr, 0, 0};
};
constexpr int kDeferRecords = 4096;
thread_local Deferral *g_defer = nullptr;

void release_deferral(Deferral &d) {
  d.ws.release();
  d.io.release();
  if (d.d_rec) cudaFree(d.d_rec);
  if (d.h_rec) cudaFreeHost(d.h_rec);
  d.d_rec = d.h_rec = nullptr;
  d.device = -1;
}

int current_device() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess) d = 0;
  return (d >= 0 && d < kMaxDevices) ? d : 0;
}
}  // namespace

void set_status(tt_cuda_status s) { g_status = s; }
tt_cuda_status get_status() { return g_status; }
void note_launch(int count) { g_launches += count; }
void set_last_rounds(int64_t r) { g_last_rounds = r; }
int relax_schedule() {
  if (g_relax_schedule >= 0) return g_relax_schedule;
  static const int env = [] {
    const char *s = std::getenv("TT_CUDA_RELAX_SCHEDULE");
    const int v = s ? std::atoi(s) : 0;
    return (v >= 0 && v < 6) ? v : 0;
  }();
  return env;
}

StatusSink *status_sink() { return g_sink; }

SinkScope::SinkScope(StatusSink *sink, Workspace *ws, Workspace *io)
    : sink_(g_sink), ws_(g_ws_override), io_(g_io_override) {
  g_sink = sink;
  g_ws_override = ws;
  g_io_override = io;
}
SinkScope::~SinkScope() {
  g_sink = sink_;
  g_ws_override = ws_;
  g_io_override = io_;
}

tt_cuda_status sink_status(const int *records, int count) {
  for (int r = 0; r < count; r++) {
    const int *rec = records + (size_t)r * kRecordInts;
    if (rec[0] == REC_RELAX && rec[1] != 0) return TT_CUDA_ERR_NOT_CONVERGED;
    if (rec[0] == REC_FOREST) {
      if (rec[1] != rec[2] || (rec[3] & 1)) return TT_CUDA_ERR_CYCLE;  // unreached exits
      if (rec[3] & 6) return TT_CUDA_ERR_INVALID_ARGUMENT;  // bad direction or weight
    }
  }
  return TT_CUDA_SUCCESS;
}

int *sink_record(int kind, cudaStream_t st) {
  StatusSink *s = g_sink;
  if (!s || s->next >= s->capacity) return nullptr;
  int *rec = s->dev + (size_t)s->next * kRecordInts;
  s->next++;
  // the kind word is written by a kernel-free memset of its low byte
  cudaMemsetAsync(rec, 0, kRecordInts * sizeof(int), st);
  cudaMemsetAsync(rec, kind, 1, st);
  return rec;
}

bool cuda_ok(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return true;
  if (std::getenv("TT_CUDA_VERBOSE"))
    std::fprintf(stderr, "tt_cuda: %s failed: %s\n", what, cudaGetErrorString(e));
  return false;
}

int64_t max_rounds() {
  if (g_max_rounds_override > 0) return g_max_rounds_override;
  static int64_t env = [] {
    const char *s = std::getenv("TT_CUDA_MAX_ROUNDS");
    return s ? std::atoll(s) : 0LL;
  }();
  return env > 0 ? env : 1000000;
}

void *Workspace::take(size_t bytes) {
  size_t need = align_up(used_) + align_up(bytes);
  if (need > cap_) return nullptr;
  void *p = base_ + align_up(used_);
  used_ = need;
  return p;
}

bool Workspace::reserve(size_t bytes) {
  used_ = 0;
  if (bytes <= cap_) return true;
  if (base_) cudaFree(base_);
  base_ = nullptr;
  cap_ = 0;
  size_t want = align_up(bytes, 1 << 20);
  if (std::getenv("TT_CUDA_FAIL_ALLOC")) return false;  // fault injection
  if (cudaMalloc(&base_, want) != cudaSuccess) {
    cudaGetLastError();
    base_ = nullptr;
    return false;
  }
  cap_ = want;
  return true;
}

void Workspace::release() {
  if (base_) cudaFree(base_);
  base_ = nullptr;
  cap_ = used_ = 0;
}

Workspace &workspace() {
  return g_ws_override ? *g_ws_override : g_dev[current_device()].scratch;
}
static Workspace &io_workspace() {
  return g_io_override ? *g_io_override : g_dev[current_device()].io;
}

void *pinned_scratch() {
  DeviceState &d = g_dev[current_device()];
  if (!d.pinned) {
    if (cudaMallocHost(&d.pinned, 4096) != cudaSuccess) {
      cudaGetLastError();
      d.pinned = nullptr;
    }
  }
  return d.pinned;
}

// The per-device copy streams and their events, created on first use.
static bool copy_lanes(cudaStream_t *cs, cudaStream_t *cs2, cudaEvent_t **ev) {
  DeviceState &d = g_dev[current_device()];
  for (cudaStream_t *p : {&d.copy, &d.copy2})
    if (!*p && cudaStreamCreateWithFlags(p, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      *p = nullptr;
      return false;
    }
  for (auto &e : d.ready)
    if (!e && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      e = nullptr;
      return false;
    }
  *cs = d.copy;
  if (cs2) *cs2 = d.copy2;
  *ev = d.ready;
  return true;
}

int sm_count() {
  DeviceState &d = g_dev[current_device()];
  if (d.sms == 0) {
    int dev = current_device(), v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    d.sms = v > 0 ? v : 1;
  }
  return d.sms;
}

DeviceLock::DeviceLock() : dev_(current_device()) { g_dev[dev_].mu.lock(); }
DeviceLock::~DeviceLock() { g_dev[dev_].mu.unlock(); }

void sun_vector(float azimuth, float altitude, float *sx, float *sy,
                float *sz) {
  double zen = 1.57079632679489661923132169163975 - (double)altitude;
  *sx = (float)(std::sin(zen) * std::cos((double)azimuth));
  *sy = (float)(std::sin(zen) * std::sin((double)azimuth));
  *sz = (float)std::cos(zen);
}

}  // namespace tt

using namespace tt;

// ------------------------------------------------------------------
// Helpers for the host-pointer entry points
// ------------------------------------------------------------------
namespace {

bool dims_ok(const ptrdiff_t dims[2]) {
  return dims && dims[0] > 0 && dims[1] > 0 && dims[0] < (1LL << 31) &&
         dims[1] < (1LL << 31) && dims[0] * dims[1] < (1LL << 31);
}

bool have_device() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return n > 0;
}

// Device staging for one host-pointer call.
struct Staging {
  std::vector<std::pair<void *, size_t>> plan;
  Workspace &ws = io_workspace();
  size_t total = 0;
  void add(size_t bytes) { total += align_up(bytes); }
  bool reserve() { return ws.reserve(total); }
  void *take(size_t bytes) { return ws.take(bytes); }
};

tt_cuda_status h2d(void *dst, const void *src, size_t bytes, cudaStream_t st) {
  TT_CHECK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
  return TT_CUDA_SUCCESS;
}
tt_cuda_status d2h(void *dst, const void *src, size_t bytes, cudaStream_t st) {
  TT_CHECK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
  return TT_CUDA_SUCCESS;
}

tt_cuda_status finish(tt_cuda_status s, cudaStream_t st) {
  if (s == TT_CUDA_SUCCESS || s == TT_CUDA_ERR_NOT_CONVERGED ||
      s == TT_CUDA_ERR_CYCLE) {
    if (!cuda_ok(cudaStreamSynchronize(st), "cudaStreamSynchronize"))
      s = TT_CUDA_ERR_CUDA;
  }
  if (s == TT_CUDA_ERR_CUDA) cudaGetLastError();
  set_status(s);
  return s;
}

#define TT_TRY(expr)                                  \
  do {                                                \
    tt_cuda_status _s = (expr);                       \
    if (_s != TT_CUDA_SUCCESS) return _s;             \
  } while (0)

#define TT_TRY_SOFT(expr, keep)                                            \
  do {                                                                     \
    tt_cuda_status _s = (expr);                                            \
    if (_s == TT_CUDA_ERR_NOT_CONVERGED || _s == TT_CUDA_ERR_CYCLE)        \
      keep = _s;                                                           \
    else if (_s != TT_CUDA_SUCCESS)                                        \
      return _s;                                                           \
  } while (0)

}  // namespace

// ------------------------------------------------------------------
// Library state
// ------------------------------------------------------------------
extern "C" {

int tt_cuda_has_gpu(void) { return have_device() ? 1 : 0; }
tt_cuda_status tt_cuda_last_error(void) { return get_status(); }

const char *tt_cuda_status_string(tt_cuda_status s) {
  switch (s) {
    case TT_CUDA_SUCCESS: return "success";
    case TT_CUDA_ERR_INVALID_ARGUMENT: return "invalid argument";
    case TT_CUDA_ERR_ALLOC: return "allocation failed";
    case TT_CUDA_ERR_CUDA: return "CUDA runtime error";
    case TT_CUDA_ERR_NOT_CONVERGED: return "iteration cap reached";
    case TT_CUDA_ERR_CYCLE: return "direction grid contains a cycle";
    case TT_CUDA_ERR_NO_DEVICE: return "no CUDA device";
    case TT_CUDA_ERR_IO: return "file input/output failed";
  }
  return "unknown status";
}

void tt_cuda_set_max_rounds(int64_t rounds) {
  g_max_rounds_override = rounds > 0 ? rounds : 0;
}

void tt_cuda_release_workspace(void) {
  if (!have_device()) return;
  DeviceLock lock;
  workspace().release();
  io_workspace().release();
  if (g_defer && !g_defer->active) release_deferral(*g_defer);
}

int64_t tt_cuda_launch_count(int reset) {
  int64_t v = g_launches;
  if (reset) g_launches = 0;
  return v;
}

int64_t tt_cuda_last_rounds(void) { return g_last_rounds; }

void tt_cuda_set_relax_schedule(int schedule) {
  g_relax_schedule = (schedule >= 0 && schedule < 6) ? schedule : -1;
}

}  // extern "C"

// ------------------------------------------------------------------
// Device-pointer entry points
// ------------------------------------------------------------------
namespace {

Deferral *active_deferral() {
  return (g_defer && g_defer->active && g_defer->device == current_device()) ? g_defer
                                                                             : nullptr;
}

template <class F>
tt_cuda_status dev_call(const ptrdiff_t dims[2], void *stream, F &&body) {
  if (!dims_ok(dims)) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return TT_CUDA_ERR_INVALID_ARGUMENT;
  }
  if (!have_device()) {
    set_status(TT_CUDA_ERR_NO_DEVICE);
    return TT_CUDA_ERR_NO_DEVICE;
  }
  DeviceLock lock;
  cudaStream_t st = (cudaStream_t)stream;
  GridDims g = make_dims(dims);
  if (Deferral *d = active_deferral()) {
    if (st != d->stream) {  // the private workspaces are ordered by one stream
      set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
      return TT_CUDA_ERR_INVALID_ARGUMENT;
    }
    tt_cuda_status s;
    {
      SinkScope scope(&d->sink, &d->ws, &d->io);
      s = body(g, st);
    }
    // no synchronisation: the stages' status words wait in the sink
    if (s == TT_CUDA_ERR_CUDA) cudaGetLastError();
    set_status(s);
    return s;
  }
  tt_cuda_status s = body(g, st);
  return finish(s, st);
}

}  // namespace

extern "C" {

tt_cuda_status tt_cuda_defer_begin(void *stream) {
  if (!have_device()) {
    set_status(TT_CUDA_ERR_NO_DEVICE);
    return TT_CUDA_ERR_NO_DEVICE;
  }
  if (g_defer && g_defer->active) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return TT_CUDA_ERR_INVALID_ARGUMENT;
  }
  const int dev = current_device();
  if (!g_defer) g_defer = new Deferral;
  Deferral &d = *g_defer;
  if (d.device != dev) release_deferral(d);  // buffers of another device
  if (!d.d_rec) {
    const size_t bytes = (size_t)kDeferRecords * kRecordInts * sizeof(int);
    if (std::getenv("TT_CUDA_FAIL_ALLOC") || cudaMalloc(&d.d_rec, bytes) != cudaSuccess ||
        cudaMallocHost(&d.h_rec, bytes) != cudaSuccess) {
      cudaGetLastError();
      release_deferral(d);
      set_status(TT_CUDA_ERR_ALLOC);
      return TT_CUDA_ERR_ALLOC;
    }
  }
  d.device = dev;
  d.stream = (cudaStream_t)stream;
  d.sink = StatusSink{d.d_rec, kDeferRecords, 0};
  d.active = true;
  set_status(TT_CUDA_SUCCESS);
  return TT_CUDA_SUCCESS;
}

tt_cuda_status tt_cuda_defer_end(void) {
  if (!g_defer || !g_defer->active) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return TT_CUDA_ERR_INVALID_ARGUMENT;
  }
  Deferral &d = *g_defer;
  d.active = false;
  int prev = -1;
  const bool other = cudaGetDevice(&prev) == cudaSuccess && prev != d.device;
  if (other && cudaSetDevice(d.device) != cudaSuccess) {
    cudaGetLastError();
    set_status(TT_CUDA_ERR_CUDA);
    return TT_CUDA_ERR_CUDA;
  }
  tt_cuda_status s = TT_CUDA_SUCCESS;
  const int n = d.sink.next;
  if (n > 0 && cudaMemcpyAsync(d.h_rec, d.d_rec, (size_t)n * kRecordInts * sizeof(int),
                               cudaMemcpyDeviceToHost, d.stream) != cudaSuccess)
    s = TT_CUDA_ERR_CUDA;
  if (cudaStreamSynchronize(d.stream) != cudaSuccess) s = TT_CUDA_ERR_CUDA;
  if (s == TT_CUDA_SUCCESS) s = sink_status(d.h_rec, n);
  if (s == TT_CUDA_ERR_CUDA) cudaGetLastError();
  if (other) cudaSetDevice(prev);
  set_status(s);
  return s;
}

tt_cuda_status tt_cuda_fillsinks_dev(float *output, const float *dem,
                                     const uint8_t *bc, const ptrdiff_t dims[2],
                                     void *stream) {
  if (!output || !dem || !bc) return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(dims, stream, [&](const GridDims &g, cudaStream_t st) {
    return fill_dev(output, dem, bc, g, st);
  });
}

tt_cuda_status tt_cuda_reconstruct_dev(float *marker, const float *mask,
                                       const ptrdiff_t dims[2], void *stream) {
  if (!marker || !mask) return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(dims, stream, [&](const GridDims &g, cudaStream_t st) {
    return reconstruct_dev(marker, mask, g, st);
  });
}

tt_cuda_status tt_cuda_identifyflats_dev(int32_t *output, const float *dem,
                                         const ptrdiff_t dims[2],
                                         int64_t *count_dev, void *stream) {
  if (!output || !dem) return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(dims, stream, [&](const GridDims &g, cudaStream_t st) {
    return identifyflats_dev(output, dem, g, (unsigned long long *)count_dev, st);
  });
}

tt_cuda_status tt_cuda_gwdt_computecosts_dev(float *costs, ptrdiff_t *conncomps,
                                             const int32_t *flats,
                                             const float *original_dem,
                                             const float *filled_dem,
                                             const ptrdiff_t dims[2],
                                             void *stream) {
  if (!costs || !conncomps || !flats || !original_dem || !filled_dem)
    return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(dims, stream, [&](const GridDims &g, cudaStream_t st) {
    return costs_dev(costs, conncomps, flats, original_dem, filled_dem, g, st);
  });
}

tt_cuda_status tt_cuda_gwdt_dev(float *dist, ptrdiff_t *prev, const float *costs,
                                const int32_t *flats, const ptrdiff_t dims[2],
                                void *stream) {
  if (!dist || !costs || !flats) return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(dims, stream, [&](const GridDims &g, cudaStream_t st) {
    return gwdt_dev(dist, prev, costs, flats, g, st);
  });
}

tt_cuda_status tt_cuda_flow_routing_d8_carve_dev(ptrdiff_t *node,
                                                 uint8_t *direction,
                                                 const float *dem,
                                                 const float *dist,
                                                 const int32_t *flats,
                                                 const ptrdiff_t dims[2],
                                                 unsigned int order,
                                                 void *stream) {
  if (!direction || !dem || !dist || !flats || order > 1)
    return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(dims, stream, [&](const GridDims &g, cudaStream_t st) {
    TT_TRY(directions_dev(direction, dem, dist, flats, g, order, st));
    if (!node) return TT_CUDA_SUCCESS;
    return node_order_dev(node, direction, g, order, st);
  });
}

tt_cuda_status tt_cuda_flow_accumulation_dev(float *acc,
                                             const uint8_t *direction,
                                             const float *weights,
                                             const ptrdiff_t dims[2],
                                             void *stream) {
  if (!acc || !direction) return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(dims, stream, [&](const GridDims &g, cudaStream_t st) {
    return accumulate_dev(acc, direction, weights, g, st);
  });
}

// Edge-list forms (device pointers).
static bool edges_ok(ptrdiff_t E) { return E >= 0 && E < (1LL << 31); }

tt_cuda_status tt_cuda_flow_routing_d8_edgelist_dev(ptrdiff_t *source, ptrdiff_t *target,
                                                    ptrdiff_t *edge_count,
                                                    const ptrdiff_t *node,
                                                    const uint8_t *direction,
                                                    const ptrdiff_t dims[2],
                                                    unsigned int order, void *stream) {
  if (!source || !target || !edge_count || !node || !direction)
    return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(dims, stream, [&](const GridDims &g, cudaStream_t st) {
    int64_t c = 0;
    tt_cuda_status s = edgelist_dev(source, target, &c, node, direction, g, order, st);
    *edge_count = (ptrdiff_t)c;
    return s;
  });
}

tt_cuda_status tt_cuda_flow_accumulation_edgelist_dev(float *acc, const ptrdiff_t *source,
                                                      const ptrdiff_t *target,
                                                      const float *fraction,
                                                      const float *weights,
                                                      ptrdiff_t edge_count,
                                                      const ptrdiff_t dims[2], void *stream) {
  if (!acc || (edge_count > 0 && (!source || !target || !fraction)) || !edges_ok(edge_count))
    return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(dims, stream, [&](const GridDims &g, cudaStream_t st) {
    return accumulate_edgelist_dev(acc, source, target, fraction, weights, edge_count, g, st);
  });
}

tt_cuda_status tt_cuda_traverse_down_f32_add_mul_dev(float *output, const float *input,
                                                     const ptrdiff_t *source,
                                                     const ptrdiff_t *target,
                                                     ptrdiff_t edge_count, ptrdiff_t node_count,
                                                     void *stream) {
  if (!output || (edge_count > 0 && (!source || !target || !input)) ||
      !edges_ok(edge_count) || node_count <= 0 || node_count >= (1LL << 31))
    return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  const ptrdiff_t nd[2] = {node_count, 1};
  return dev_call(nd, stream, [&](const GridDims &g, cudaStream_t st) {
    return edge_sweep_dev(output, output, source, target, input, edge_count, g.cells(), st);
  });
}

static tt_cuda_status traverse_u32_dev(uint32_t *output, const uint32_t *input,
                                       const ptrdiff_t *source, const ptrdiff_t *target,
                                       ptrdiff_t edge_count, ptrdiff_t node_count, bool up,
                                       void *stream) {
  if (!output || (edge_count > 0 && (!source || !target || !input)) ||
      !edges_ok(edge_count) || node_count <= 0 || node_count >= (1LL << 31))
    return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  const ptrdiff_t nd[2] = {node_count, 1};
  return dev_call(nd, stream, [&](const GridDims &g, cudaStream_t st) {
    return edge_sweep_u32_dev(output, output, source, target, input, edge_count, g.cells(),
                              up, st);
  });
}

tt_cuda_status tt_cuda_traverse_down_u32_or_and_dev(uint32_t *output, const uint32_t *input,
                                                    const ptrdiff_t *source,
                                                    const ptrdiff_t *target,
                                                    ptrdiff_t edge_count, ptrdiff_t node_count,
                                                    void *stream) {
  return traverse_u32_dev(output, input, source, target, edge_count, node_count, false, stream);
}

tt_cuda_status tt_cuda_traverse_up_u32_or_and_dev(uint32_t *output, const uint32_t *weights,
                                                  const ptrdiff_t *source,
                                                  const ptrdiff_t *target,
                                                  ptrdiff_t edge_count, ptrdiff_t node_count,
                                                  void *stream) {
  return traverse_u32_dev(output, weights, source, target, edge_count, node_count, true,
                          stream);
}

tt_cuda_status tt_cuda_drainagebasins_dev(ptrdiff_t *basins, const ptrdiff_t *source,
                                          const ptrdiff_t *target, ptrdiff_t edge_count,
                                          const ptrdiff_t dims[2], void *stream) {
  if (!basins || (edge_count > 0 && (!source || !target)) || !edges_ok(edge_count))
    return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(dims, stream, [&](const GridDims &g, cudaStream_t st) {
    return drainagebasins_dev(basins, source, target, edge_count, g, st);
  });
}

tt_cuda_status tt_cuda_edgelist_degree_dev(uint8_t *indegree, uint8_t *outdegree,
                                           const ptrdiff_t *source, const ptrdiff_t *target,
                                           ptrdiff_t node_count, ptrdiff_t edge_count,
                                           void *stream) {
  if (!indegree || !outdegree || (edge_count > 0 && (!source || !target)) ||
      !edges_ok(edge_count))
    return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  const ptrdiff_t nd[2] = {node_count, 1};
  return dev_call(nd, stream, [&](const GridDims &g, cudaStream_t st) {
    return degree_dev(indegree, outdegree, source, target, g.cells(), edge_count, st);
  });
}

// Graphflood single-flow graph (device pointers; dim = {rows, cols}).
static bool gf_dim_ok(const size_t dim[2], ptrdiff_t pd[2]) {
  if (!dim) return false;
  pd[0] = (ptrdiff_t)dim[1];
  pd[1] = (ptrdiff_t)dim[0];
  return dim[0] > 0 && dim[1] > 0 && dim[0] < (1ULL << 31) && dim[1] < (1ULL << 31);
}

tt_cuda_status tt_cuda_compute_sfgraph_dev(const double *topo, size_t *Sreceivers,
                                           double *distToReceivers, size_t *Sdonors,
                                           uint8_t *NSdonors, size_t *Stack, const uint8_t *BCs,
                                           const size_t dim[2], double dx, bool D8,
                                           void *stream) {
  ptrdiff_t pd[2] = {0, 0};
  if (!topo || !Sreceivers || !distToReceivers || !Sdonors || !NSdonors || !Stack || !BCs ||
      !gf_dim_ok(dim, pd))
    return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(pd, stream, [&](const GridDims &g, cudaStream_t st) {
    return sfgraph_dev(topo, Sreceivers, distToReceivers, Sdonors, NSdonors, Stack, BCs, g.n,
                       g.m, dx, D8, st);
  });
}

tt_cuda_status tt_cuda_compute_drainage_area_single_flow_dev(double *output,
                                                             const size_t *Sreceivers,
                                                             const size_t dim[2], double dx,
                                                             void *stream) {
  ptrdiff_t pd[2] = {0, 0};
  if (!output || !Sreceivers || !gf_dim_ok(dim, pd))
    return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(pd, stream, [&](const GridDims &g, cudaStream_t st) {
    return sf_drainage_area_dev(output, Sreceivers, g.n, g.m, dx, st);
  });
}

tt_cuda_status tt_cuda_flow_accumulation_backward_dev(float *grad_weights,
                                                      const uint8_t *direction,
                                                      const float *grad_acc,
                                                      const ptrdiff_t dims[2],
                                                      void *stream) {
  if (!grad_weights || !direction || !grad_acc)
    return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(dims, stream, [&](const GridDims &g, cudaStream_t st) {
    return accumulate_backward_dev(grad_weights, direction, grad_acc, g, st);
  });
}

tt_cuda_status tt_cuda_gradient_secondorder_dev(float *p0, float *p1,
                                                const float *dem, float cellsize,
                                                const ptrdiff_t dims[2],
                                                void *stream) {
  if (!p0 || !p1 || !dem || !dims || dims[0] < 3 || dims[1] < 3)
    return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(dims, stream, [&](const GridDims &g, cudaStream_t st) {
    return gradient2_dev(p0, p1, dem, cellsize, g, st);
  });
}

tt_cuda_status tt_cuda_hillshade_fused_dev(float *output, const float *dem,
                                           float azimuth, float altitude,
                                           float cellsize,
                                           const ptrdiff_t dims[2],
                                           void *stream) {
  if (!output || !dem || !dims || dims[0] < 3 || dims[1] < 3)
    return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(dims, stream, [&](const GridDims &g, cudaStream_t st) {
    return hillshade_dev(output, dem, azimuth, altitude, cellsize, g, st);
  });
}

tt_cuda_status tt_cuda_hillshade_backward_dev(float *grad_dem, const float *dem,
                                              const float *grad_output,
                                              float azimuth, float altitude,
                                              float cellsize,
                                              const ptrdiff_t dims[2],
                                              void *stream) {
  if (!grad_dem || !dem || !grad_output || !dims || dims[0] < 3 || dims[1] < 3)
    return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(dims, stream, [&](const GridDims &g, cudaStream_t st) {
    return hillshade_backward_dev(grad_dem, dem, grad_output, azimuth, altitude,
                                  cellsize, g, st);
  });
}

}  // extern "C"

// The pipeline body shared by the device and host forms.  Missing
// intermediates are carved from the io workspace by the caller.
// True for page-locked (pinned or registered) host memory.
static bool host_pinned(const void *p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

// Device-to-host copies of a host-pointer pipeline's outputs.  A copy into
// page-locked memory is issued as soon as the stage that writes its array
// has been enqueued: it runs on a side stream after an event on the compute
// stream, so it overlaps the later stages.  No later stage writes an array
// once its copy is issued.  A copy into pageable memory blocks the calling
// thread until it is done, so those are deferred to the end of the call and
// issued on the compute stream, after every kernel has been enqueued.
struct EarlyOut {
  void *filled = nullptr, *flats = nullptr, *dist = nullptr;
  void *node = nullptr, *direction = nullptr, *acc = nullptr;
  cudaStream_t cs = nullptr;
  cudaEvent_t *ev = nullptr;
  int used = 0;
  struct Late {
    void *host;
    const void *dev;
    size_t bytes;
  } late[6];
  int nlate = 0;

  tt_cuda_status send(void *host, const void *dev, size_t bytes, cudaStream_t st) {
    if (!host) return TT_CUDA_SUCCESS;
    if (!cs || !host_pinned(host)) {
      late[nlate++] = {host, dev, bytes};
      return TT_CUDA_SUCCESS;
    }
    TT_CHECK(cudaEventRecord(ev[used], st));
    TT_CHECK(cudaStreamWaitEvent(cs, ev[used], 0));
    used++;
    TT_CHECK(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, cs));
    return TT_CUDA_SUCCESS;
  }
  // the compute stream waits for every early copy, so a sync on it covers
  // them; the deferred copies follow on the compute stream
  tt_cuda_status join(cudaStream_t st) {
    if (cs && used) {
      TT_CHECK(cudaEventRecord(ev[used], cs));
      TT_CHECK(cudaStreamWaitEvent(st, ev[used], 0));
    }
    for (int k = 0; k < nlate; k++) TT_TRY(d2h(late[k].host, late[k].dev, late[k].bytes, st));
    return TT_CUDA_SUCCESS;
  }
};

static tt_cuda_status pipeline_body(float *filled, int32_t *flats, float *dist,
                                    ptrdiff_t *node, uint8_t *direction,
                                    float *acc, float *hill, const float *dem,
                                    const uint8_t *bc, const float *weights,
                                    float az, float alt, float cs,
                                    float *costs, ptrdiff_t *conncomps,
                                    const GridDims &g, cudaStream_t st,
                                    EarlyOut *out = nullptr) {
  tt_cuda_status soft = TT_CUDA_SUCCESS;
  const size_t n = (size_t)g.m * (size_t)g.n;
  TT_TRY_SOFT(fill_dev(filled, dem, bc, g, st), soft);
  if (out) TT_TRY(out->send(out->filled, filled, n * 4, st));
  TT_TRY(identifyflats_dev(flats, filled, g, nullptr, st));
  if (out) TT_TRY(out->send(out->flats, flats, n * 4, st));
  // The costs pass writes the gwdt start directly (the pipeline does not
  // return the costs), except under the ordered schedules, whose tile
  // priorities the start would have to set as well.
  if (relax_schedule() < 4) {
    const size_t tb = (size_t)g.tiles() * 4;
    int *gdirty = nullptr;
    TT_CHECK(cudaMallocAsync((void **)&gdirty, tb, st));
    struct Free {
      void *p;
      cudaStream_t st;
      ~Free() { cudaFreeAsync(p, st); }
    } free_dirty{gdirty, st};
    TT_CHECK(cudaMemsetAsync(gdirty, 0, tb, st));
    const GwdtSeed seed{dist, gdirty};
    TT_TRY(costs_dev(costs, conncomps, flats, dem, filled, g, st, &seed));
    TT_TRY_SOFT(gwdt_seeded_dev(dist, costs, flats, gdirty, g, st), soft);
  } else {
    TT_TRY(costs_dev(costs, conncomps, flats, dem, filled, g, st));  // conncomps may be null
    TT_TRY_SOFT(gwdt_dev(dist, nullptr, costs, flats, g, st), soft);
  }
  if (out) TT_TRY(out->send(out->dist, dist, n * 4, st));
  TT_TRY(directions_dev(direction, filled, dist, flats, g, 0, st));
  if (out) TT_TRY(out->send(out->direction, direction, n, st));
  if (node && acc) {  // one forest contraction for both
    struct AccCopy {
      EarlyOut *out;
      float *acc;
      size_t bytes;
      cudaStream_t st;
      bool sent;
    } ac{out, acc, n * 4, st, false};
    auto send_acc = [](void *c) -> tt_cuda_status {  // overlaps the node sort
      AccCopy *a = static_cast<AccCopy *>(c);
      a->sent = true;
      return a->out->send(a->out->acc, a->acc, a->bytes, a->st);
    };
    TT_TRY_SOFT(node_order_acc_dev(node, acc, direction, weights, g, st,
                                   out ? +send_acc : nullptr, &ac),
                soft);
    if (out && !ac.sent) TT_TRY(out->send(out->acc, acc, n * 4, st));
    if (out) TT_TRY(out->send(out->node, node, n * 8, st));
  } else {
    if (node) TT_TRY_SOFT(node_order_dev(node, direction, g, 0, st), soft);
    if (out && node) TT_TRY(out->send(out->node, node, n * 8, st));
    if (acc) TT_TRY_SOFT(accumulate_dev(acc, direction, weights, g, st), soft);
    if (out && acc) TT_TRY(out->send(out->acc, acc, n * 4, st));
  }
  if (hill) TT_TRY(hillshade_dev(hill, dem, az, alt, cs, g, st));
  if (out) TT_TRY(out->join(st));
  return soft;
}

extern "C" tt_cuda_status tt_cuda_d8_pipeline_dev(
    float *filled, int32_t *flats, float *dist, ptrdiff_t *node,
    uint8_t *direction, float *acc, float *hillshade, const float *dem,
    const uint8_t *bc, const float *weights, float azimuth, float altitude,
    float cellsize, const ptrdiff_t dims[2], void *stream) {
  if (!dem || !bc) return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  if (hillshade && (dims[0] < 3 || dims[1] < 3))
    return set_status(TT_CUDA_ERR_INVALID_ARGUMENT), TT_CUDA_ERR_INVALID_ARGUMENT;
  return dev_call(dims, stream, [&](const GridDims &g, cudaStream_t st) {
    int64_t N = g.cells();
    Staging sg;
    sg.add(N * 4);  // costs
    if (!filled) sg.add(N * 4);
    if (!flats) sg.add(N * 4);
    if (!dist) sg.add(N * 4);
    if (!direction) sg.add(N);
    if (!sg.reserve()) return TT_CUDA_ERR_ALLOC;
    float *costs = (float *)sg.take(N * 4);
    if (!filled) filled = (float *)sg.take(N * 4);
    if (!flats) flats = (int32_t *)sg.take(N * 4);
    if (!dist) dist = (float *)sg.take(N * 4);
    if (!direction) direction = (uint8_t *)sg.take(N);
    return pipeline_body(filled, flats, dist, node, direction, acc, hillshade,
                         dem, bc, weights, azimuth, altitude, cellsize, costs,
                         nullptr, g, st);
  });
}

// ------------------------------------------------------------------
// Host-pointer (drop-in) entry points
// ------------------------------------------------------------------
namespace {

// Runs `body` with device copies of host arrays.  `ins` are copied H2D,
// `outs` are copied D2H after the body; an array may appear in both.
struct HostArg {
  void *host;
  size_t bytes;
  bool in;
  bool out;
  void *dev = nullptr;
};

template <class F>
tt_cuda_status host_call(const ptrdiff_t dims[2], std::vector<HostArg> args,
                         F &&body) {
  if (!dims_ok(dims)) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return TT_CUDA_ERR_INVALID_ARGUMENT;
  }
  for (auto &a : args)
    if (!a.host && (a.in || a.out)) {
      set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
      return TT_CUDA_ERR_INVALID_ARGUMENT;
    }
  if (!have_device()) {
    set_status(TT_CUDA_ERR_NO_DEVICE);
    return TT_CUDA_ERR_NO_DEVICE;
  }
  DeviceLock lock;
  cudaStream_t st = 0;
  GridDims g = make_dims(dims);
  Staging sg;
  for (auto &a : args) sg.add(a.bytes);
  if (!sg.reserve()) return finish(TT_CUDA_ERR_ALLOC, st);
  for (auto &a : args) {
    a.dev = sg.take(a.bytes);
    if (a.in) {
      tt_cuda_status s = h2d(a.dev, a.host, a.bytes, st);
      if (s != TT_CUDA_SUCCESS) return finish(s, st);
    }
  }
  tt_cuda_status s = body(g, st, args);
  if (s == TT_CUDA_SUCCESS || s == TT_CUDA_ERR_NOT_CONVERGED || s == TT_CUDA_ERR_CYCLE) {
    for (auto &a : args)
      if (a.out) {
        tt_cuda_status c = d2h(a.host, a.dev, a.bytes, st);
        if (c != TT_CUDA_SUCCESS) return finish(c, st);
      }
  }
  return finish(s, st);
}

// Host-pointer hillshade in bands of tile columns: the DEM goes up on one
// copy stream band by band, each band's kernel starts once its columns and
// the next band's first columns (the stencil's halo) are in place, and its
// output goes down on a second copy stream while later bands still copy
// and compute.  Copies into or out of pageable memory block the calling
// thread, so those calls keep the plain upload, kernel, download sequence.
tt_cuda_status hillshade_banded(float *hout, const float *hdem, float *dout, float *ddem,
                                float az, float alt, float cs, const GridDims &g,
                                cudaStream_t st) {
  const size_t N = (size_t)g.m * (size_t)g.n;
  cudaStream_t cin = nullptr, cout = nullptr;
  cudaEvent_t *ev = nullptr;
  const int B = (int)std::min<int64_t>(8, g.tn);  // bands
  if (B < 2 || !host_pinned(hdem) || !host_pinned(hout) || !copy_lanes(&cin, &cout, &ev)) {
    TT_TRY(h2d(ddem, hdem, N * 4, st));
    TT_TRY(hillshade_dev(dout, ddem, az, alt, cs, g, st));
    return d2h(hout, dout, N * 4, st);
  }
  auto tile_of = [&](int b) { return (int)((int64_t)b * g.tn / B); };  // first tile column
  auto col_of = [&](int t) { return std::min<int64_t>((int64_t)t * kTile, g.n); };
  auto body = [&]() -> tt_cuda_status {
    TT_CHECK(cudaEventRecord(ev[0], st));  // after earlier work on the staging buffers
    TT_CHECK(cudaStreamWaitEvent(cin, ev[0], 0));
    for (int b = 0; b < B; b++) {
      const int64_t c0 = col_of(tile_of(b)), c1 = col_of(tile_of(b + 1));
      TT_CHECK(cudaMemcpyAsync(ddem + c0 * g.m, hdem + c0 * g.m, (size_t)((c1 - c0) * g.m) * 4,
                               cudaMemcpyHostToDevice, cin));
      TT_CHECK(cudaEventRecord(ev[1 + b], cin));
    }
    for (int b = 0; b < B; b++) {
      TT_CHECK(cudaStreamWaitEvent(st, ev[1 + std::min(b + 1, B - 1)], 0));  // band and halo
      TT_TRY(hillshade_cols_dev(dout, ddem, az, alt, cs, g, tile_of(b), tile_of(b + 1), st));
      TT_CHECK(cudaEventRecord(ev[1 + B + b], st));
      TT_CHECK(cudaStreamWaitEvent(cout, ev[1 + B + b], 0));
      const int64_t c0 = col_of(tile_of(b)), c1 = col_of(tile_of(b + 1));
      TT_CHECK(cudaMemcpyAsync(hout + c0 * g.m, dout + c0 * g.m, (size_t)((c1 - c0) * g.m) * 4,
                               cudaMemcpyDeviceToHost, cout));
    }
    TT_CHECK(cudaEventRecord(ev[1 + 2 * B], cout));
    TT_CHECK(cudaStreamWaitEvent(st, ev[1 + 2 * B], 0));
    return TT_CUDA_SUCCESS;
  };
  tt_cuda_status s = body();
  // nothing issued may still run into the caller's buffers after return
  if (cudaStreamSynchronize(cin) != cudaSuccess || cudaStreamSynchronize(cout) != cudaSuccess) {
    cudaGetLastError();
    if (s == TT_CUDA_SUCCESS) s = TT_CUDA_ERR_CUDA;
  }
  return s;
}

}  // namespace

extern "C" {

void tt_cuda_fillsinks(float *output, float *dem, uint8_t *bc,
                       ptrdiff_t dims[2]) {
  size_t N = dims ? (size_t)(dims[0] * dims[1]) : 0;
  host_call(dims, {{output, N * 4, false, true}, {dem, N * 4, true, false}, {bc, N, true, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              return fill_dev((float *)a[0].dev, (const float *)a[1].dev,
                              (const uint8_t *)a[2].dev, g, st);
            });
}

void tt_cuda_fillsinks_hybrid(float *output, ptrdiff_t *queue, float *dem,
                              uint8_t *bc, ptrdiff_t dims[2]) {
  (void)queue;
  tt_cuda_fillsinks(output, dem, bc, dims);
}

void tt_cuda_reconstruct(float *marker, float *mask, ptrdiff_t dims[2]) {
  size_t N = dims ? (size_t)(dims[0] * dims[1]) : 0;
  host_call(dims, {{marker, N * 4, true, true}, {mask, N * 4, true, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              return reconstruct_dev((float *)a[0].dev, (const float *)a[1].dev, g, st);
            });
}

int tt_cuda_reconstruct_hybrid(float *marker, ptrdiff_t *queue, float *mask,
                               ptrdiff_t dims[2]) {
  (void)queue;
  tt_cuda_reconstruct(marker, mask, dims);
  return get_status() == TT_CUDA_ERR_NOT_CONVERGED ? 1 : 0;
}

ptrdiff_t tt_cuda_identifyflats(int32_t *output, float *dem, ptrdiff_t dims[2]) {
  size_t N = dims ? (size_t)(dims[0] * dims[1]) : 0;
  int64_t count = 0;
  host_call(dims, {{output, N * 4, false, true}, {dem, N * 4, true, false}, {&count, 8, false, true}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              return identifyflats_dev((int32_t *)a[0].dev, (const float *)a[1].dev, g,
                                       (unsigned long long *)a[2].dev, st);
            });
  return get_status() == TT_CUDA_SUCCESS ? (ptrdiff_t)count : 0;
}

void tt_cuda_gwdt_computecosts(float *costs, ptrdiff_t *conncomps,
                               int32_t *flats, float *original_dem,
                               float *filled_dem, ptrdiff_t dims[2]) {
  size_t N = dims ? (size_t)(dims[0] * dims[1]) : 0;
  host_call(dims,
            {{costs, N * 4, false, true}, {conncomps, N * 8, false, true},
             {flats, N * 4, true, false}, {original_dem, N * 4, true, false},
             {filled_dem, N * 4, true, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              return costs_dev((float *)a[0].dev, (ptrdiff_t *)a[1].dev,
                               (const int32_t *)a[2].dev, (const float *)a[3].dev,
                               (const float *)a[4].dev, g, st);
            });
}

void tt_cuda_gwdt(float *dist, ptrdiff_t *prev, float *costs, int32_t *flats,
                  ptrdiff_t *heap, ptrdiff_t *back, ptrdiff_t dims[2]) {
  (void)heap;
  (void)back;
  size_t N = dims ? (size_t)(dims[0] * dims[1]) : 0;
  host_call(dims,
            {{dist, N * 4, false, true}, {prev, prev ? N * 8 : 0, false, prev != nullptr},
             {costs, N * 4, true, false}, {flats, N * 4, true, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              return gwdt_dev((float *)a[0].dev, prev ? (ptrdiff_t *)a[1].dev : nullptr,
                              (const float *)a[2].dev, (const int32_t *)a[3].dev, g, st);
            });
}

void tt_cuda_flow_routing_d8_carve(ptrdiff_t *node, uint8_t *direction,
                                   float *dem, float *dist, int32_t *flats,
                                   ptrdiff_t dims[2], unsigned int order) {
  if (order > 1) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return;
  }
  size_t N = dims ? (size_t)(dims[0] * dims[1]) : 0;
  host_call(dims,
            {{node, N * 8, false, true}, {direction, N, false, true},
             {dem, N * 4, true, false}, {dist, N * 4, true, false},
             {flats, N * 4, true, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              TT_TRY(directions_dev((uint8_t *)a[1].dev, (const float *)a[2].dev,
                                    (const float *)a[3].dev, (const int32_t *)a[4].dev,
                                    g, order, st));
              return node_order_dev((ptrdiff_t *)a[0].dev, (const uint8_t *)a[1].dev,
                                    g, order, st);
            });
}

void tt_cuda_flow_accumulation(float *acc, ptrdiff_t *source,
                               uint8_t *direction, float *weights,
                               ptrdiff_t dims[2]) {
  (void)source;
  size_t N = dims ? (size_t)(dims[0] * dims[1]) : 0;
  host_call(dims,
            {{acc, N * 4, false, true}, {direction, N, true, false},
             {weights, weights ? N * 4 : 0, weights != nullptr, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              return accumulate_dev((float *)a[0].dev, (const uint8_t *)a[1].dev,
                                    weights ? (const float *)a[2].dev : nullptr, g, st);
            });
}

ptrdiff_t tt_cuda_flow_routing_d8_edgelist(ptrdiff_t *source, ptrdiff_t *target,
                                           ptrdiff_t *node, uint8_t *direction,
                                           ptrdiff_t dims[2], unsigned int order) {
  size_t N = dims ? (size_t)(dims[0] * dims[1]) : 0;
  if (!source || !target) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return 0;
  }
  int64_t count = 0;
  host_call(dims,
            {{node, N * 8, true, false}, {direction, N, true, false},
             {source, N * 8, false, false}, {target, N * 8, false, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              tt_cuda_status s = edgelist_dev((ptrdiff_t *)a[2].dev, (ptrdiff_t *)a[3].dev,
                                              &count, (const ptrdiff_t *)a[0].dev,
                                              (const uint8_t *)a[1].dev, g, order, st);
              if (s != TT_CUDA_SUCCESS) return s;
              // only the edges found are copied back
              TT_TRY(d2h(source, a[2].dev, (size_t)count * 8, st));
              TT_TRY(d2h(target, a[3].dev, (size_t)count * 8, st));
              return TT_CUDA_SUCCESS;
            });
  return get_status() == TT_CUDA_SUCCESS ? (ptrdiff_t)count : 0;
}

void tt_cuda_flow_accumulation_edgelist(float *acc, ptrdiff_t *source, ptrdiff_t *target,
                                        float *fraction, float *weights,
                                        ptrdiff_t edge_count, ptrdiff_t dims[2]) {
  size_t N = dims ? (size_t)(dims[0] * dims[1]) : 0;
  if (!edges_ok(edge_count)) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return;
  }
  const size_t E = (size_t)edge_count;
  host_call(dims,
            {{acc, N * 4, false, true}, {source, E * 8, E > 0, false},
             {target, E * 8, E > 0, false}, {fraction, E * 4, E > 0, false},
             {weights, weights ? N * 4 : 0, weights != nullptr, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              return accumulate_edgelist_dev(
                  (float *)a[0].dev, (const ptrdiff_t *)a[1].dev, (const ptrdiff_t *)a[2].dev,
                  (const float *)a[3].dev, weights ? (const float *)a[4].dev : nullptr,
                  edge_count, g, st);
            });
}

void tt_cuda_drainagebasins(ptrdiff_t *basins, ptrdiff_t *source, ptrdiff_t *target,
                            ptrdiff_t edge_count, ptrdiff_t dims[2]) {
  size_t N = dims ? (size_t)(dims[0] * dims[1]) : 0;
  if (!edges_ok(edge_count)) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return;
  }
  const size_t E = (size_t)edge_count;
  host_call(dims,
            {{basins, N * 8, false, true}, {source, E * 8, E > 0, false},
             {target, E * 8, E > 0, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              return drainagebasins_dev((ptrdiff_t *)a[0].dev, (const ptrdiff_t *)a[1].dev,
                                        (const ptrdiff_t *)a[2].dev, edge_count, g, st);
            });
}

}  // extern "C"

namespace {
// Host-pointer sweeps over an edge list.  The reference's signatures carry
// no node count: `output` spans the nodes the edges name.  V is the node
// and edge value type; sweep(out, in, src, tgt, E, N, st) runs on device
// copies, `out` holding the start values.
template <class V, class Sweep>
void host_edge_sweep(V *output, const V *input, const ptrdiff_t *source,
                     const ptrdiff_t *target, ptrdiff_t edge_count, Sweep sweep) {
  if (!edges_ok(edge_count) ||
      (edge_count > 0 && (!output || !input || !source || !target))) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return;
  }
  if (edge_count == 0) {  // no edge: `output` is unchanged
    set_status(TT_CUDA_SUCCESS);
    return;
  }
  if (!have_device()) {
    set_status(TT_CUDA_ERR_NO_DEVICE);
    return;
  }
  DeviceLock lock;
  cudaStream_t st = 0;
  const size_t E = (size_t)edge_count;
  Staging sg;
  sg.add(E * 8);
  sg.add(E * 8);
  sg.add(E * sizeof(V));
  if (!sg.reserve()) {
    finish(TT_CUDA_ERR_ALLOC, st);
    return;
  }
  auto *dsrc = (ptrdiff_t *)sg.take(E * 8);
  auto *dtgt = (ptrdiff_t *)sg.take(E * 8);
  auto *din = (V *)sg.take(E * sizeof(V));
  tt_cuda_status s = h2d(dsrc, source, E * 8, st);
  if (s == TT_CUDA_SUCCESS) s = h2d(dtgt, target, E * 8, st);
  if (s == TT_CUDA_SUCCESS) s = h2d(din, input, E * sizeof(V), st);
  int64_t N = 0;
  if (s == TT_CUDA_SUCCESS) s = edge_node_count_dev(dsrc, dtgt, edge_count, &N, st);
  if (s == TT_CUDA_SUCCESS && N >= (1LL << 31)) s = TT_CUDA_ERR_INVALID_ARGUMENT;
  V *dout = nullptr;
  if (s == TT_CUDA_SUCCESS &&
      cudaMallocAsync((void **)&dout, (size_t)N * sizeof(V), st) != cudaSuccess) {
    cudaGetLastError();
    s = TT_CUDA_ERR_ALLOC;
    dout = nullptr;
  }
  if (s == TT_CUDA_SUCCESS) s = h2d(dout, output, (size_t)N * sizeof(V), st);
  if (s == TT_CUDA_SUCCESS) s = sweep(dout, din, dsrc, dtgt, edge_count, N, st);
  if (s == TT_CUDA_SUCCESS) s = d2h(output, dout, (size_t)N * sizeof(V), st);
  if (dout) cudaFreeAsync(dout, st);
  finish(s, st);
}
}  // namespace

extern "C" {

void tt_cuda_traverse_down_f32_add_mul(float *output, float *input, ptrdiff_t *source,
                                       ptrdiff_t *target, ptrdiff_t edge_count) {
  host_edge_sweep(output, input, source, target, edge_count,
                  [](float *o, const float *in, const ptrdiff_t *src, const ptrdiff_t *tgt,
                     int64_t E, int64_t N, cudaStream_t st) {
                    return edge_sweep_dev(o, o, src, tgt, in, E, N, st);
                  });
}

void tt_cuda_traverse_down_u32_or_and(uint32_t *output, uint32_t *input, ptrdiff_t *source,
                                      ptrdiff_t *target, ptrdiff_t edge_count) {
  host_edge_sweep(output, input, source, target, edge_count,
                  [](uint32_t *o, const uint32_t *in, const ptrdiff_t *src,
                     const ptrdiff_t *tgt, int64_t E, int64_t N, cudaStream_t st) {
                    return edge_sweep_u32_dev(o, o, src, tgt, in, E, N, false, st);
                  });
}

void tt_cuda_traverse_up_u32_or_and(uint32_t *output, uint32_t *weights, ptrdiff_t *source,
                                    ptrdiff_t *target, ptrdiff_t edge_count) {
  host_edge_sweep(output, weights, source, target, edge_count,
                  [](uint32_t *o, const uint32_t *in, const ptrdiff_t *src,
                     const ptrdiff_t *tgt, int64_t E, int64_t N, cudaStream_t st) {
                    return edge_sweep_u32_dev(o, o, src, tgt, in, E, N, true, st);
                  });
}

void tt_cuda_edgelist_degree(uint8_t *indegree, uint8_t *outdegree, ptrdiff_t *source,
                             ptrdiff_t *target, ptrdiff_t node_count, ptrdiff_t edge_count) {
  if (!edges_ok(edge_count)) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return;
  }
  const size_t E = (size_t)edge_count, N = node_count > 0 ? (size_t)node_count : 0;
  ptrdiff_t nd[2] = {node_count, 1};
  host_call(nd,
            {{indegree, N, false, true}, {outdegree, N, false, true},
             {source, E * 8, E > 0, false}, {target, E * 8, E > 0, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              return degree_dev((uint8_t *)a[0].dev, (uint8_t *)a[1].dev,
                                (const ptrdiff_t *)a[2].dev, (const ptrdiff_t *)a[3].dev,
                                g.cells(), edge_count, st);
            });
}

void tt_cuda_compute_sfgraph(double *topo, size_t *Sreceivers, double *distToReceivers,
                             size_t *Sdonors, uint8_t *NSdonors, size_t *Stack, uint8_t *BCs,
                             size_t *dim, double dx, bool D8) {
  ptrdiff_t pd[2] = {0, 0};
  if (!gf_dim_ok(dim, pd)) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return;
  }
  const size_t N = (size_t)(pd[0] * pd[1]), K = D8 ? 8 : 4;
  // Sdonors goes both ways: slots past each count keep the caller's bytes.
  host_call(pd,
            {{topo, N * 8, true, false}, {Sreceivers, N * 8, false, true},
             {distToReceivers, N * 8, false, true}, {Sdonors, N * K * 8, true, true},
             {NSdonors, N, false, true}, {Stack, N * 8, false, true}, {BCs, N, true, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              return sfgraph_dev((const double *)a[0].dev, (size_t *)a[1].dev,
                                 (double *)a[2].dev, (size_t *)a[3].dev, (uint8_t *)a[4].dev,
                                 (size_t *)a[5].dev, (const uint8_t *)a[6].dev, g.n, g.m, dx,
                                 D8, st);
            });
}

void tt_cuda_compute_drainage_area_single_flow(double *output, size_t *Sreceivers,
                                               size_t *Stack, size_t *dim, double dx) {
  (void)Stack;
  ptrdiff_t pd[2] = {0, 0};
  if (!gf_dim_ok(dim, pd)) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return;
  }
  const size_t N = (size_t)(pd[0] * pd[1]);
  host_call(pd, {{output, N * 8, false, true}, {Sreceivers, N * 8, true, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              return sf_drainage_area_dev((double *)a[0].dev, (const size_t *)a[1].dev, g.n,
                                          g.m, dx, st);
            });
}

void tt_cuda_flow_accumulation_backward(float *grad_weights, ptrdiff_t *source,
                                        uint8_t *direction, float *grad_acc,
                                        ptrdiff_t dims[2]) {
  (void)source;
  size_t N = dims ? (size_t)(dims[0] * dims[1]) : 0;
  host_call(dims,
            {{grad_weights, N * 4, false, true}, {direction, N, true, false},
             {grad_acc, N * 4, true, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              return accumulate_backward_dev((float *)a[0].dev, (const uint8_t *)a[1].dev,
                                             (const float *)a[2].dev, g, st);
            });
}

void tt_cuda_gradient_secondorder(float *p0, float *p1, float *dem,
                                  float cellsize, ptrdiff_t dims[2]) {
  if (!dims || dims[0] < 3 || dims[1] < 3) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return;
  }
  size_t N = (size_t)(dims[0] * dims[1]);
  host_call(dims,
            {{p0, N * 4, false, true}, {p1, N * 4, false, true}, {dem, N * 4, true, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              return gradient2_dev((float *)a[0].dev, (float *)a[1].dev,
                                   (const float *)a[2].dev, cellsize, g, st);
            });
}

void tt_cuda_hillshade(float *output, float *dx, float *dy, float *dem,
                       float azimuth, float altitude, float cellsize,
                       ptrdiff_t dims[2]) {
  if (!dims || dims[0] < 3 || dims[1] < 3) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return;
  }
  size_t N = (size_t)(dims[0] * dims[1]);
  host_call(dims,
            {{output, N * 4, false, true}, {dx, N * 4, false, true},
             {dy, N * 4, false, true}, {dem, N * 4, true, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              TT_TRY(gradient2_dev((float *)a[1].dev, (float *)a[2].dev,
                                   (const float *)a[3].dev, cellsize, g, st));
              return hillshade_dev((float *)a[0].dev, (const float *)a[3].dev, azimuth,
                                   altitude, cellsize, g, st);
            });
}

void tt_cuda_hillshade_fused(float *output, float *dem, float azimuth,
                             float altitude, float cellsize, ptrdiff_t dims[2]) {
  if (!dims || dims[0] < 3 || dims[1] < 3) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return;
  }
  size_t N = (size_t)(dims[0] * dims[1]);
  host_call(dims, {{output, N * 4, false, false}, {dem, N * 4, false, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              return hillshade_banded(output, dem, (float *)a[0].dev, (float *)a[1].dev,
                                      azimuth, altitude, cellsize, g, st);
            });
}

void tt_cuda_hillshade_backward(float *grad_dem, float *dem, float *grad_output,
                                float azimuth, float altitude, float cellsize,
                                ptrdiff_t dims[2]) {
  if (!dims || dims[0] < 3 || dims[1] < 3) {
    set_status(TT_CUDA_ERR_INVALID_ARGUMENT);
    return;
  }
  size_t N = (size_t)(dims[0] * dims[1]);
  host_call(dims,
            {{grad_dem, N * 4, false, true}, {dem, N * 4, true, false},
             {grad_output, N * 4, true, false}},
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              return hillshade_backward_dev((float *)a[0].dev, (const float *)a[1].dev,
                                            (const float *)a[2].dev, azimuth, altitude,
                                            cellsize, g, st);
            });
}

void tt_cuda_d8_pipeline(float *filled, int32_t *flats, float *dist,
                         ptrdiff_t *node, uint8_t *direction, float *acc,
                         float *dem, uint8_t *bc, float *weights,
                         ptrdiff_t dims[2]) {
  size_t N = dims ? (size_t)(dims[0] * dims[1]) : 0;
  host_call(dims,
            {{dem, N * 4, true, false}, {bc, N, true, false},
             {weights, weights ? N * 4 : 0, weights != nullptr, false},
             // outputs: copied back by EarlyOut as their stages finish
             {nullptr, N * 4, false, false},
             {nullptr, N * 4, false, false},
             {nullptr, N * 4, false, false},
             {nullptr, node ? N * 8 : 0, false, false},
             {nullptr, N, false, false},
             {nullptr, acc ? N * 4 : 0, false, false},
             {nullptr, N * 4, false, false}},  // costs
            [&](const GridDims &g, cudaStream_t st, std::vector<HostArg> &a) {
              EarlyOut out;
              out.filled = filled;
              out.flats = flats;
              out.dist = dist;
              out.node = node;
              out.direction = direction;
              out.acc = acc;
              if (!copy_lanes(&out.cs, nullptr, &out.ev)) out.cs = nullptr;
              tt_cuda_status s = pipeline_body(
                  (float *)a[3].dev, (int32_t *)a[4].dev, (float *)a[5].dev,
                  node ? (ptrdiff_t *)a[6].dev : nullptr, (uint8_t *)a[7].dev,
                  acc ? (float *)a[8].dev : nullptr, nullptr, (const float *)a[0].dev,
                  (const uint8_t *)a[1].dev, weights ? (const float *)a[2].dev : nullptr,
                  0.f, 0.f, 1.f, (float *)a[9].dev, nullptr, g, st, &out);
              // copies already issued end before the call returns, even when
              // a later stage failed
              if (out.cs && out.used && cudaStreamSynchronize(out.cs) != cudaSuccess) {
                cudaGetLastError();
                if (s == TT_CUDA_SUCCESS) s = TT_CUDA_ERR_CUDA;
              }
              return s;
            });
}

}  // extern "C"
