/**
 * @file tt_cuda.h
 * @brief GB300 (sm_103a) implementation of libtopotoolbox's D8 flow pipeline.
 *
 * Drop-in C ABI.  Every `tt_cuda_<name>` below with host pointers has exactly
 * the parameter list of `<name>` in libtopotoolbox's public header
 * include/topotoolbox.h (line numbers cited per function), so a caller swaps
 * `fillsinks(...)` for `tt_cuda_fillsinks(...)` and nothing else changes:
 *
 *  - arrays are column-major with `dims = {nrows, ncols}` (fastest dimension
 *    first, include/topotoolbox.h:284-290);
 *  - DEMs are float32, boundary-condition and direction grids uint8, flat
 *    flags int32, node lists and labels ptrdiff_t;
 *  - the caller owns every buffer; nothing is retained after return.
 *
 * Unlike the reference, no call mutates its inputs (the reference's
 * fillsinks negates `dem` in place while it runs, src/fillsinks.c:14-16).
 * The reference reports no errors; these functions keep its return types and
 * record a status per calling thread, read with tt_cuda_last_error().
 *
 * Scratch parameters of the reference (`queue`, `heap`, `back`) are accepted
 * and ignored: the GPU algorithms keep their scratch in a per-device
 * workspace owned by this library.
 *
 * The `_dev` variants take DEVICE pointers and a `cudaStream_t` (passed as
 * `void *`, NULL = legacy default stream), enqueue their work on that stream
 * and return a status.  They synchronise the stream before they return, to
 * report an iteration cap or a cycle, unless the caller defers their status
 * (tt_cuda_defer_begin / tt_cuda_defer_end below).
 *
 * Calls are serialised per device by an internal mutex.
 */
#ifndef TT_CUDA_H
#define TT_CUDA_H

#include <stddef.h>
#include <stdint.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define TT_CUDA_API __declspec(dllexport)
#else
#define TT_CUDA_API __attribute__((visibility("default")))
#endif

/** Status codes recorded by every call. */
typedef enum {
  TT_CUDA_SUCCESS = 0,
  TT_CUDA_ERR_INVALID_ARGUMENT = 1, /**< bad dims, NULL pointer, bad order */
  TT_CUDA_ERR_ALLOC = 2,            /**< device or pinned allocation failed */
  TT_CUDA_ERR_CUDA = 3,             /**< a CUDA runtime call failed */
  TT_CUDA_ERR_NOT_CONVERGED = 4,    /**< an iteration cap was reached */
  TT_CUDA_ERR_CYCLE = 5,            /**< the direction grid contains a cycle */
  TT_CUDA_ERR_NO_DEVICE = 6,        /**< no CUDA device is visible */
  TT_CUDA_ERR_IO = 7                /**< a file could not be opened, read or written */
} tt_cuda_status;

/* ------------------------------------------------------------------ */
/* Library state                                                        */
/* ------------------------------------------------------------------ */

/** 1 when a CUDA device is usable.  Counterpart of has_topotoolbox()
 *  (include/topotoolbox.h:41, src/topotoolbox.c:4). */
TT_CUDA_API int tt_cuda_has_gpu(void);
/** Status of the last tt_cuda_* call made by this thread. */
TT_CUDA_API tt_cuda_status tt_cuda_last_error(void);
/** Human-readable text of a status code. */
TT_CUDA_API const char *tt_cuda_status_string(tt_cuda_status status);
/** Iteration caps (0 restores the default).  `sweeps` caps the device
 *  rounds of the iterative stages (fill, gwdt); the environment variable
 *  TT_CUDA_MAX_ROUNDS sets the same cap at load time. */
TT_CUDA_API void tt_cuda_set_max_rounds(int64_t rounds);
/** Release the per-device workspace of the current device. */
TT_CUDA_API void tt_cuda_release_workspace(void);
/** Number of kernel launches this library has issued on this thread since
 *  the last reset (for launch accounting in benchmarks). */
TT_CUDA_API int64_t tt_cuda_launch_count(int reset);
/** Device rounds used by the last fill / gwdt call on this thread. */
TT_CUDA_API int64_t tt_cuda_last_rounds(void);
/** Sweep schedule of the tile relaxations (fill, reconstruct, gwdt) for this
 *  thread's later calls; no counterpart in the reference.  0..3: bit 0 runs
 *  each round's row sweeps before its column sweeps, bit 1 ends a tile
 *  visit after 8 sweeps (the tile publishes what changed and queues itself
 *  again).  4 and 5 order tile visits by value: only tiles whose lowest
 *  incoming value is at or below a global threshold run, and the threshold
 *  rises band by band (bands of 1/8 and 1/2 of the value, at least 1 and 4
 *  units) when every warp has run out of eligible tiles.  Results are
 *  identical for every schedule; only the time differs.  A value outside
 *  0..5 restores the default (the environment variable
 *  TT_CUDA_RELAX_SCHEDULE, else 0).  A batch takes the schedule in effect
 *  when its graph is captured (its first run). */
TT_CUDA_API void tt_cuda_set_relax_schedule(int schedule);
/** Deferred status for this thread's device-pointer calls; no counterpart
 *  in the reference.  Without it, every tt_cuda_*_dev call synchronises its
 *  stream before it returns, to report the iteration cap, a cycle or an
 *  invalid direction or weight.  Between tt_cuda_defer_begin(stream) and
 *  tt_cuda_defer_end(), the calls of the D8 path on this thread
 *  (fillsinks, reconstruct, identifyflats, gwdt_computecosts, gwdt,
 *  flow_routing_d8_carve, flow_accumulation with or without weights,
 *  gradient_secondorder, hillshade_fused, hillshade_backward, d8_pipeline)
 *  only enqueue their work on `stream`: each stage's status words are copied
 *  into a device record, and the call returns TT_CUDA_SUCCESS unless a check
 *  on the host fails (arguments, allocation, a launch).  The results are the
 *  same bits as without deferral.  tt_cuda_defer_end() copies the records
 *  back, synchronises the stream once and returns the first failure
 *  recorded (TT_CUDA_ERR_NOT_CONVERGED, TT_CUDA_ERR_CYCLE,
 *  TT_CUDA_ERR_INVALID_ARGUMENT) or TT_CUDA_SUCCESS.
 *   - A device-pointer call on this thread with another stream, while
 *     deferral is on, returns TT_CUDA_ERR_INVALID_ARGUMENT (deferred calls
 *     share private scratch ordered by that one stream).  Calls on another
 *     device, and host-pointer calls, run as usual.
 *   - The edge-list, drainage-basin, graphflood, file and adjoint
 *     (flow_accumulation_backward) forms still wait for their own results
 *     (they size outputs or test convergence on the host), and so for the
 *     deferred work before them on the stream.
 *   - Weighted accumulation under deferral computes its scales on the
 *     device and keeps scratch for four passes (32 bytes per cell).
 *   - tt_cuda_last_rounds() is not updated by deferred calls.
 *   - 4096 stage records per deferral (a pipeline call takes three); a stage
 *     past that reads its status back and synchronises as usual.
 *  tt_cuda_defer_begin returns TT_CUDA_ERR_INVALID_ARGUMENT when deferral
 *  is already on; tt_cuda_defer_end when it is not. */
TT_CUDA_API tt_cuda_status tt_cuda_defer_begin(void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_defer_end(void);
/* ------------------------------------------------------------------ */
/* Drop-in host-pointer entry points                                    */
/* ------------------------------------------------------------------ */

/** include/topotoolbox.h:293 fillsinks (src/fillsinks.c:23-48).  Grids of
 *  12288 pixels a side and more start from the fill of the DEM max-pooled
 *  over 4 x 4 cells, an upper bound of the result (the same bits, fewer
 *  iterations); the environment variable TT_CUDA_FILL_BOUND_MIN sets that
 *  side at load time (0: never). */
TT_CUDA_API void tt_cuda_fillsinks(float *output, float *dem, uint8_t *bc,
                                   ptrdiff_t dims[2]);
/** include/topotoolbox.h:351 fillsinks_hybrid (src/fillsinks.c:51-77).
 *  `queue` is not used. */
TT_CUDA_API void tt_cuda_fillsinks_hybrid(float *output, ptrdiff_t *queue,
                                          float *dem, uint8_t *bc,
                                          ptrdiff_t dims[2]);
/** include/topotoolbox.h:1056 reconstruct (src/reconstruct.c:270-278):
 *  grayscale reconstruction by dilation of `marker` under `mask`, in place. */
TT_CUDA_API void tt_cuda_reconstruct(float *marker, float *mask,
                                     ptrdiff_t dims[2]);
/** include/topotoolbox.h:1070 reconstruct_hybrid (src/reconstruct.c:291-312).
 *  Returns 0 on convergence, 1 if the round cap was hit. */
TT_CUDA_API int tt_cuda_reconstruct_hybrid(float *marker, ptrdiff_t *queue,
                                           float *mask, ptrdiff_t dims[2]);
/** include/topotoolbox.h:405 identifyflats (src/identifyflats.c:33-121).
 *  Returns the number of flat pixels. */
TT_CUDA_API ptrdiff_t tt_cuda_identifyflats(int32_t *output, float *dem,
                                            ptrdiff_t dims[2]);
/** include/topotoolbox.h:464 gwdt_computecosts (src/gwdt.c:167-278).
 *  `costs` are bit-identical to the reference.  `conncomps` holds, for every
 *  flat, the linear index of a pixel of maximal depth in its component (the
 *  smallest such index; the reference's choice among equal depths follows
 *  its scan order), 0 elsewhere. */
TT_CUDA_API void tt_cuda_gwdt_computecosts(float *costs, ptrdiff_t *conncomps,
                                           int32_t *flats, float *original_dem,
                                           float *filled_dem,
                                           ptrdiff_t dims[2]);
/** include/topotoolbox.h:533 gwdt (src/gwdt.c:290-351).  `dist` is
 *  bit-identical to the reference; `prev` (may be NULL) holds a valid
 *  back-link for every reached flat (dist[v] == dist[prev[v]] + edge
 *  weight), self elsewhere.  `heap` and `back` are not used. */
TT_CUDA_API void tt_cuda_gwdt(float *dist, ptrdiff_t *prev, float *costs,
                              int32_t *flats, ptrdiff_t *heap, ptrdiff_t *back,
                              ptrdiff_t dims[2]);
/** include/topotoolbox.h:860 flow_routing_d8_carve
 *  (src/flow_routing.c:135-256).  `direction` is bit-identical; `node` is a
 *  topological order (every donor before its receiver). */
TT_CUDA_API void tt_cuda_flow_routing_d8_carve(ptrdiff_t *node,
                                               uint8_t *direction, float *dem,
                                               float *dist, int32_t *flats,
                                               ptrdiff_t dims[2],
                                               unsigned int order);
/** include/topotoolbox.h:962 flow_accumulation
 *  (src/flow_accumulation.c:32-80).  The sum is exact in 64-bit fixed point
 *  and rounded once to float32, so it does not depend on the order in
 *  `source`; `source` is accepted and not read. */
TT_CUDA_API void tt_cuda_flow_accumulation(float *acc, ptrdiff_t *source,
                                           uint8_t *direction, float *weights,
                                           ptrdiff_t dims[2]);
/** include/topotoolbox.h:2347 gradient_secondorder (src/hillshade.c:23-76). */
TT_CUDA_API void tt_cuda_gradient_secondorder(float *p0, float *p1, float *dem,
                                              float cellsize,
                                              ptrdiff_t dims[2]);
/** include/topotoolbox.h:2400 hillshade (src/hillshade.c:79-97). */
TT_CUDA_API void tt_cuda_hillshade(float *output, float *dx, float *dy,
                                   float *dem, float azimuth, float altitude,
                                   float cellsize, ptrdiff_t dims[2]);
/** include/topotoolbox.h:2449 hillshade_fused (src/hillshade.c:102-213). */
TT_CUDA_API void tt_cuda_hillshade_fused(float *output, float *dem,
                                         float azimuth, float altitude,
                                         float cellsize, ptrdiff_t dims[2]);

/* ------------------------------------------------------------------ */
/* Edge-list forms (the callers of the path's outputs)                  */
/* ------------------------------------------------------------------ */

/** include/topotoolbox.h:912 flow_routing_d8_edgelist
 *  (src/flow_routing.c:258-312).  One edge (u, receiver(u)) per pixel with a
 *  direction, in `node` order, bit-identical to the reference for the same
 *  `node` and `direction`.  `source` and `target` need room for every pixel;
 *  only the first (returned) count entries are written. */
TT_CUDA_API ptrdiff_t tt_cuda_flow_routing_d8_edgelist(ptrdiff_t *source,
                                                       ptrdiff_t *target,
                                                       ptrdiff_t *node,
                                                       uint8_t *direction,
                                                       ptrdiff_t dims[2],
                                                       unsigned int order);
/** include/topotoolbox.h:1019 flow_accumulation_edgelist
 *  (src/flow_accumulation.c:10-30): acc = weights (or 1), then
 *  acc[target] += fraction * acc[source] for every edge in list order, for
 *  any edge list: fractional and multi-target (several edges out of a
 *  pixel), in any order, with the reference's list-order semantics.  Sums
 *  are taken in list order in FP64 and rounded once to float32, so the
 *  result is run-to-run identical and within float32 rounding of an FP64
 *  sweep.  The edge list of a D8 forest with unit fractions in topological
 *  order (as flow_routing_d8_edgelist produces) takes the exact forest sum
 *  of tt_cuda_flow_accumulation instead.  An index outside the grid gives
 *  TT_CUDA_ERR_INVALID_ARGUMENT. */
TT_CUDA_API void tt_cuda_flow_accumulation_edgelist(float *acc, ptrdiff_t *source,
                                                    ptrdiff_t *target,
                                                    float *fraction, float *weights,
                                                    ptrdiff_t edge_count,
                                                    ptrdiff_t dims[2]);
/** include/topotoolbox.h:1755 traverse_down_f32_add_mul
 *  (src/streamquad.c:171-180): output[target] = output[target] +
 *  output[source] * input[e] for every edge e in list order, any order,
 *  FP64 sums in list order rounded once to float32 (run-to-run identical).
 *  `output` spans nodes 0 .. the largest index the edges name, as in the
 *  reference. */
TT_CUDA_API void tt_cuda_traverse_down_f32_add_mul(float *output, float *input,
                                                   ptrdiff_t *source, ptrdiff_t *target,
                                                   ptrdiff_t edge_count);
/** include/topotoolbox.h:1235 traverse_down_u32_or_and
 *  (src/streamquad.c:49-60): output[target] |= output[source] & input[e]
 *  for every edge e in list order, any order, exact. */
TT_CUDA_API void tt_cuda_traverse_down_u32_or_and(uint32_t *output, uint32_t *input,
                                                  ptrdiff_t *source, ptrdiff_t *target,
                                                  ptrdiff_t edge_count);
/** include/topotoolbox.h:1186 traverse_up_u32_or_and
 *  (src/streamquad.c:37-47): output[source] |= output[target] & weights[e]
 *  for every edge e in reverse list order, any order, exact.  With
 *  `output` holding a distinct bit pattern at each outlet and zero elsewhere
 *  and all-ones weights, this labels drainage basins on a D8 edge list
 *  (test/random_dem.cpp:550-580).  Both or/and sweeps: `output` spans nodes
 *  0 .. the largest index the edges name, as in the reference. */
TT_CUDA_API void tt_cuda_traverse_up_u32_or_and(uint32_t *output, uint32_t *weights,
                                                ptrdiff_t *source, ptrdiff_t *target,
                                                ptrdiff_t edge_count);
/** include/topotoolbox.h:2304 drainagebasins (src/drainagebasins.c:6-27).
 *  For a topologically ordered edge list (as flow_routing_d8_edgelist
 *  produces) the labels equal the reference's on the same list. */
TT_CUDA_API void tt_cuda_drainagebasins(ptrdiff_t *basins, ptrdiff_t *source,
                                        ptrdiff_t *target, ptrdiff_t edge_count,
                                        ptrdiff_t dims[2]);
/** include/topotoolbox.h:1853 edgelist_degree (src/streamquad.c:209-224).
 *  uint8 degrees, wrapping modulo 256 as the reference's counters do. */
TT_CUDA_API void tt_cuda_edgelist_degree(uint8_t *indegree, uint8_t *outdegree,
                                         ptrdiff_t *source, ptrdiff_t *target,
                                         ptrdiff_t node_count, ptrdiff_t edge_count);

/* ------------------------------------------------------------------ */
/* Graphflood single-flow graph (row-major dim = {rows, cols}, FP64)     */
/* ------------------------------------------------------------------ */

/** include/topotoolbox.h:2053 compute_sfgraph (src/graphflood/sfgraph.c:27-113).
 *  Receivers, distances, donor lists and the Braun-Willett stack, all
 *  bit-identical to the reference.  Donor slots past NSdonors are left as the
 *  caller passed them, as in the reference. */
TT_CUDA_API void tt_cuda_compute_sfgraph(double *topo, size_t *Sreceivers,
                                         double *distToReceivers, size_t *Sdonors,
                                         uint8_t *NSdonors, size_t *Stack, uint8_t *BCs,
                                         size_t *dim, double dx, bool D8);
/** include/topotoolbox.h:2122 compute_drainage_area_single_flow
 *  (src/graphflood/gf_flowacc.c:19-35): cell area times the exact subtree
 *  pixel count (the node itself left out at roots).  `Stack` is accepted and
 *  not read: the count does not depend on the order. */
TT_CUDA_API void tt_cuda_compute_drainage_area_single_flow(double *output, size_t *Sreceivers,
                                                           size_t *Stack, size_t *dim,
                                                           double dx);

/* ------------------------------------------------------------------ */
/* Adjoints (no counterpart in the reference)                           */
/* ------------------------------------------------------------------ */

/** Adjoint of weighted flow_accumulation with the receivers held fixed:
 *  grad_weights[u] = sum of grad_acc over the flow path from u to its
 *  outlet, u included.  `source` is accepted and not read. */
TT_CUDA_API void tt_cuda_flow_accumulation_backward(float *grad_weights,
                                                    ptrdiff_t *source,
                                                    uint8_t *direction,
                                                    float *grad_acc,
                                                    ptrdiff_t dims[2]);
/** Adjoint of hillshade_fused with respect to the DEM:
 *  grad_dem = J^T grad_output.  Cells whose hillshade is NaN contribute
 *  nothing. */
TT_CUDA_API void tt_cuda_hillshade_backward(float *grad_dem, float *dem,
                                            float *grad_output, float azimuth,
                                            float altitude, float cellsize,
                                            ptrdiff_t dims[2]);

/* ------------------------------------------------------------------ */
/* Whole pipeline (composition of the calls above, no single reference  */
/* counterpart).  Host pointers.  Any output may be NULL to skip it.    */
/* ------------------------------------------------------------------ */

/** fillsinks -> identifyflats -> gwdt_computecosts -> gwdt ->
 *  flow_routing_d8_carve (order 0) -> flow_accumulation (the call sequence of
 *  test/random_dem.cpp:682-724).  `dem` follows the caller's NaN convention:
 *  NaN cells stay NaN (barriers); callers that want the reference test
 *  harness's behaviour pass -INF with bc = 1 there.  `weights` may be NULL
 *  (unit weights). */
TT_CUDA_API void tt_cuda_d8_pipeline(float *filled, int32_t *flats,
                                     float *dist, ptrdiff_t *node,
                                     uint8_t *direction, float *acc,
                                     float *dem, uint8_t *bc, float *weights,
                                     ptrdiff_t dims[2]);

/* ------------------------------------------------------------------ */
/* Device-pointer entry points                                          */
/* ------------------------------------------------------------------ */

TT_CUDA_API tt_cuda_status tt_cuda_fillsinks_dev(float *output,
                                                 const float *dem,
                                                 const uint8_t *bc,
                                                 const ptrdiff_t dims[2],
                                                 void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_reconstruct_dev(float *marker,
                                                   const float *mask,
                                                   const ptrdiff_t dims[2],
                                                   void *stream);
/** `count` (may be NULL) receives the number of flats (device int64). */
TT_CUDA_API tt_cuda_status tt_cuda_identifyflats_dev(int32_t *output,
                                                     const float *dem,
                                                     const ptrdiff_t dims[2],
                                                     int64_t *count_dev,
                                                     void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_gwdt_computecosts_dev(
    float *costs, ptrdiff_t *conncomps, const int32_t *flats,
    const float *original_dem, const float *filled_dem,
    const ptrdiff_t dims[2], void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_gwdt_dev(float *dist, ptrdiff_t *prev,
                                            const float *costs,
                                            const int32_t *flats,
                                            const ptrdiff_t dims[2],
                                            void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_flow_routing_d8_carve_dev(
    ptrdiff_t *node, uint8_t *direction, const float *dem, const float *dist,
    const int32_t *flats, const ptrdiff_t dims[2], unsigned int order,
    void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_flow_accumulation_dev(
    float *acc, const uint8_t *direction, const float *weights,
    const ptrdiff_t dims[2], void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_flow_accumulation_backward_dev(
    float *grad_weights, const uint8_t *direction, const float *grad_acc,
    const ptrdiff_t dims[2], void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_gradient_secondorder_dev(
    float *p0, float *p1, const float *dem, float cellsize,
    const ptrdiff_t dims[2], void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_hillshade_fused_dev(
    float *output, const float *dem, float azimuth, float altitude,
    float cellsize, const ptrdiff_t dims[2], void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_hillshade_backward_dev(
    float *grad_dem, const float *dem, const float *grad_output, float azimuth,
    float altitude, float cellsize, const ptrdiff_t dims[2], void *stream);
/** Device-pointer forms of the edge-list functions above; the edge count of
 *  tt_cuda_flow_routing_d8_edgelist_dev is written to *edge_count (host). */
TT_CUDA_API tt_cuda_status tt_cuda_flow_routing_d8_edgelist_dev(
    ptrdiff_t *source, ptrdiff_t *target, ptrdiff_t *edge_count,
    const ptrdiff_t *node, const uint8_t *direction, const ptrdiff_t dims[2],
    unsigned int order, void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_flow_accumulation_edgelist_dev(
    float *acc, const ptrdiff_t *source, const ptrdiff_t *target,
    const float *fraction, const float *weights, ptrdiff_t edge_count,
    const ptrdiff_t dims[2], void *stream);
/** Device form of tt_cuda_traverse_down_f32_add_mul; `node_count` is the
 *  length of `output` (every index in the edge list must be below it). */
TT_CUDA_API tt_cuda_status tt_cuda_traverse_down_f32_add_mul_dev(
    float *output, const float *input, const ptrdiff_t *source, const ptrdiff_t *target,
    ptrdiff_t edge_count, ptrdiff_t node_count, void *stream);
/** Device forms of the or/and sweeps, `node_count` as above. */
TT_CUDA_API tt_cuda_status tt_cuda_traverse_down_u32_or_and_dev(
    uint32_t *output, const uint32_t *input, const ptrdiff_t *source,
    const ptrdiff_t *target, ptrdiff_t edge_count, ptrdiff_t node_count, void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_traverse_up_u32_or_and_dev(
    uint32_t *output, const uint32_t *weights, const ptrdiff_t *source,
    const ptrdiff_t *target, ptrdiff_t edge_count, ptrdiff_t node_count, void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_drainagebasins_dev(
    ptrdiff_t *basins, const ptrdiff_t *source, const ptrdiff_t *target,
    ptrdiff_t edge_count, const ptrdiff_t dims[2], void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_edgelist_degree_dev(
    uint8_t *indegree, uint8_t *outdegree, const ptrdiff_t *source,
    const ptrdiff_t *target, ptrdiff_t node_count, ptrdiff_t edge_count,
    void *stream);
/** Device-pointer forms of the graphflood functions above. */
TT_CUDA_API tt_cuda_status tt_cuda_compute_sfgraph_dev(
    const double *topo, size_t *Sreceivers, double *distToReceivers, size_t *Sdonors,
    uint8_t *NSdonors, size_t *Stack, const uint8_t *BCs, const size_t dim[2], double dx,
    bool D8, void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_compute_drainage_area_single_flow_dev(
    double *output, const size_t *Sreceivers, const size_t dim[2], double dx, void *stream);
/** Raster I/O before and after the path (no counterpart in the reference,
 *  whose callers read DEMs with GDAL): `bytes` bytes of the file at `path`
 *  from byte `offset` into device memory at `dst`, or from `src` into the
 *  file at byte `offset` (the file is created if missing, not truncated), in
 *  chunks staged through two pinned host buffers so that disk transfers and
 *  host-device copies overlap.  Returns when the data has arrived.
 *  TT_CUDA_ERR_IO if the file cannot be opened or is short. */
TT_CUDA_API tt_cuda_status tt_cuda_read_file_dev(void *dst, const char *path, int64_t offset,
                                                 int64_t bytes, void *stream);
TT_CUDA_API tt_cuda_status tt_cuda_write_file_dev(const char *path, int64_t offset,
                                                  const void *src, int64_t bytes, void *stream);
/** fillsinks on device pointers without allocating anything.  No
 *  counterpart in the reference.  For callers that cannot call cudaMalloc
 *  while they run -- a framework whose own memory pool already owns the
 *  device, or a loop that must not pay for cudaMalloc/cudaFree, which can
 *  synchronise the whole device.  The fill's scratch (a control block and
 *  one flag per 32 x 32 tile) lives in a static device array sized for
 *  65536 tiles (for example 8192 x 8192 pixels); each device that loads the
 *  library keeps it until the process exits.  Larger grids are rejected with
 *  TT_CUDA_ERR_INVALID_ARGUMENT.  The first call on a device looks up the
 *  array's device address (cudaGetSymbolAddress) with that device current;
 *  make that first call before any stream capture.  All calls share the
 *  array: each call re-initialises it, and calls that overlap on the GPU
 *  (other streams, other threads on the same device) race on it.  The
 *  address looked up on the first call is kept for the life of the process:
 *  do not call this after a cudaDeviceReset of that device.  The fill's
 *  persistent kernel is a cooperative launch, so all of its blocks run at
 *  once even beside other work on the device.  The call synchronises
 *  `stream` before it returns. */
TT_CUDA_API tt_cuda_status tt_cuda_fillsinks_noalloc_dev(
    float *output, const float *dem, const uint8_t *bc,
    const ptrdiff_t dims[2], void *stream);
/** Device form of tt_cuda_d8_pipeline.  `hillshade` (may be NULL) adds the
 *  hillshade of the input DEM with the given angles. */
TT_CUDA_API tt_cuda_status tt_cuda_d8_pipeline_dev(
    float *filled, int32_t *flats, float *dist, ptrdiff_t *node,
    uint8_t *direction, float *acc, float *hillshade, const float *dem,
    const uint8_t *bc, const float *weights, float azimuth, float altitude,
    float cellsize, const ptrdiff_t dims[2], void *stream);

/* ------------------------------------------------------------------ */
/* Batched form (no counterpart in the reference)                       */
/* ------------------------------------------------------------------ */

/** A batch of independent DEMs run through fillsinks -> identifyflats ->
 *  gwdt_computecosts -> gwdt -> flow_routing_d8_carve (directions) ->
 *  flow_accumulation (unit weights) with one launch per stage over the whole
 *  batch.  The DEMs are packed into one mosaic with NaN gutters, which every
 *  stage treats exactly like the grid edge, so each DEM's results equal a
 *  separate call (finite DEMs).  The first run with a given set of pointers
 *  executes the sequence and captures it in a CUDA graph; later runs with
 *  the same pointers replay the graph. */
typedef struct tt_cuda_batch tt_cuda_batch;
/** `dims` holds count pairs {nrows, ncols}.  `canvas_cols` is the mosaic
 *  width in columns (0 picks one from the total area). */
TT_CUDA_API tt_cuda_status tt_cuda_batch_create(int count, const ptrdiff_t *dims,
                                                int64_t canvas_cols,
                                                tt_cuda_batch **out);
/** info[0..3] = canvas rows, canvas columns, DEM pixels, graph nodes. */
TT_CUDA_API tt_cuda_status tt_cuda_batch_info(const tt_cuda_batch *batch,
                                              int64_t *info);
/** Device pointers, one per DEM, in host arrays of length count; an output
 *  array may be NULL to skip that output.  Runs on an internal stream
 *  ordered after `stream` and returns when the results are written. */
TT_CUDA_API tt_cuda_status tt_cuda_batch_run(
    tt_cuda_batch *batch, const float *const *dem, const uint8_t *const *bc,
    float *const *filled, int32_t *const *flats, float *const *dist,
    uint8_t *const *direction, float *const *acc, void *stream);
TT_CUDA_API void tt_cuda_batch_destroy(tt_cuda_batch *batch);

#ifdef __cplusplus
}
#endif
#endif /* TT_CUDA_H */
