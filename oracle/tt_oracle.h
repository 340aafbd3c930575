/*
 * tt_oracle.h -- CPU oracle for the D8 flow pipeline (TEST INFRASTRUCTURE).
 *
 * This library is the checker, never the product: only tests/, the smoke
 * check in __graft_entry__.py and the CPU-baseline leg of bench.py load it.
 * It restates, in plain C, the reference algorithms of libtopotoolbox for
 * the hot path (fillsinks, identifyflats, gwdt_computecosts, gwdt,
 * flow_routing_d8_carve, flow_accumulation, hillshade) plus FP64 versions of
 * accumulation and hillshade and FP64 adjoints of both.  Each function names
 * the reference file:line it follows.  Arrays are column-major with
 * dims = {nrows, ncols} (fastest dimension first), exactly as in the
 * reference header include/topotoolbox.h.
 */
#ifndef TT_ORACLE_H
#define TT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* src/fillsinks.c:23-48 + src/reconstruct.c:68-114,134-205,270-278 */
void orc_fillsinks(float *output, const float *dem, const uint8_t *bc,
                   const ptrdiff_t dims[2]);
/* src/fillsinks.c:51-77 + src/reconstruct.c:13-45,207-251,291-312.
 * Returns 1 when the queue overflowed on the last allowed scan. */
int orc_fillsinks_hybrid(float *output, ptrdiff_t *queue, const float *dem,
                         const uint8_t *bc, const ptrdiff_t dims[2]);
/* src/reconstruct.c:270-278: `marker` reconstructed under `mask` in place. */
void orc_reconstruct(float *marker, const float *mask, const ptrdiff_t dims[2]);
/* src/reconstruct.c:291-312; returns 1 if the queue overflowed twice. */
int orc_reconstruct_hybrid(float *marker, ptrdiff_t *queue, const float *mask,
                           const ptrdiff_t dims[2]);
/* src/identifyflats.c:33-121 */
ptrdiff_t orc_identifyflats(int32_t *output, const float *dem,
                            const ptrdiff_t dims[2]);
/* src/gwdt.c:87-278 */
void orc_gwdt_computecosts(float *costs, ptrdiff_t *conncomps,
                           const int32_t *flats, const float *original_dem,
                           const float *filled_dem, const ptrdiff_t dims[2]);
/* src/gwdt.c:290-351 + src/helpers/priority_queue.c:52-133 */
void orc_gwdt(float *dist, ptrdiff_t *prev, const float *costs,
              const int32_t *flats, ptrdiff_t *heap, ptrdiff_t *back,
              const ptrdiff_t dims[2]);
/* src/flow_routing.c:15-76,135-256 */
void orc_flow_routing_d8_carve(ptrdiff_t *node, uint8_t *direction,
                               const float *dem, const float *dist,
                               const int32_t *flats, const ptrdiff_t dims[2],
                               unsigned int order);
/* src/flow_accumulation.c:32-80 (float32, node order) */
void orc_flow_accumulation(float *acc, const ptrdiff_t *source,
                           const uint8_t *direction, const float *weights,
                           const ptrdiff_t dims[2]);
/* FP64 restatement of src/flow_accumulation.c:32-80 */
void orc_flow_accumulation_f64(double *acc, const ptrdiff_t *source,
                               const uint8_t *direction, const float *weights,
                               const ptrdiff_t dims[2]);
/* As orc_flow_accumulation_f64 with float64 weights (for finite
 * differences of the adjoint). */
void orc_flow_accumulation_f64w(double *acc, const ptrdiff_t *source,
                                const uint8_t *direction, const double *weights,
                                const ptrdiff_t dims[2]);
/* FP64 adjoint: grad_w[u] = sum of grad_acc over the flow path from u to its
 * outlet (u included).  No counterpart in the reference. */
void orc_flow_accumulation_backward_f64(double *grad_w, const ptrdiff_t *source,
                                        const uint8_t *direction,
                                        const double *grad_acc,
                                        const ptrdiff_t dims[2]);
/* src/hillshade.c:11-20,102-213 (float32) */
void orc_hillshade_fused(float *output, const float *dem, float azimuth,
                         float altitude, float cellsize,
                         const ptrdiff_t dims[2]);
/* src/hillshade.c:23-97 (float32, materialised gradients) */
void orc_hillshade(float *output, float *dx, float *dy, const float *dem,
                   float azimuth, float altitude, float cellsize,
                   const ptrdiff_t dims[2]);
/* FP64 restatement of src/hillshade.c:11-20,102-213; sun vector in double */
void orc_hillshade_f64(double *output, const double *dem, double azimuth,
                       double altitude, double cellsize,
                       const ptrdiff_t dims[2]);
/* FP64 adjoint of orc_hillshade_f64 with respect to dem: grad_dem =
 * J^T grad_out.  Cells whose hillshade is NaN contribute nothing.  No
 * counterpart in the reference. */
void orc_hillshade_backward_f64(double *grad_dem, const double *dem,
                                const double *grad_out, double azimuth,
                                double altitude, double cellsize,
                                const ptrdiff_t dims[2]);

/* ---- Edge-list forms (the callers of the path's outputs) ---- */

/* src/flow_routing.c:258-312: one edge (u, receiver(u)) per pixel u with a
 * direction, listed in `node` order; neighbour offsets from the memory
 * order (order & 1: row-major).  Returns the edge count. */
ptrdiff_t orc_flow_routing_d8_edgelist(ptrdiff_t *source, ptrdiff_t *target,
                                       const ptrdiff_t *node,
                                       const uint8_t *direction,
                                       const ptrdiff_t dims[2], unsigned order);
/* src/flow_accumulation.c:10-30: acc = weights (or 1), then
 * acc[target] += fraction * acc[source] edge by edge in list order. */
void orc_flow_accumulation_edgelist(float *acc, const ptrdiff_t *source,
                                    const ptrdiff_t *target,
                                    const float *fraction, const float *weights,
                                    ptrdiff_t edge_count, const ptrdiff_t dims[2]);
/* The same sweep in FP64 (fractions and weights widened).  No counterpart in
 * the reference; the tolerance oracle for the float32 results. */
void orc_flow_accumulation_edgelist_f64(double *acc, const ptrdiff_t *source,
                                        const ptrdiff_t *target,
                                        const float *fraction,
                                        const float *weights,
                                        ptrdiff_t edge_count,
                                        const ptrdiff_t dims[2]);
/* src/drainagebasins.c:6-27: labels 1, 2, ... assigned in reverse edge
 * order to the first unlabelled target met; every source takes its
 * target's label; pixels on no edge stay 0. */
void orc_drainagebasins(ptrdiff_t *basins, const ptrdiff_t *source,
                        const ptrdiff_t *target, ptrdiff_t edge_count,
                        const ptrdiff_t dims[2]);
/* src/streamquad.c:209-224: in- and out-degree of every node (uint8,
 * wrapping as the reference's counters do). */
/* src/streamquad.c:171-180 */
void orc_traverse_down_f32_add_mul(float *output, const float *input,
                                   const ptrdiff_t *source, const ptrdiff_t *target,
                                   ptrdiff_t edge_count);
/* src/streamquad.c:49-60 and 37-47 */
void orc_traverse_down_u32_or_and(uint32_t *output, const uint32_t *input,
                                  const ptrdiff_t *source, const ptrdiff_t *target,
                                  ptrdiff_t edge_count);
void orc_traverse_up_u32_or_and(uint32_t *output, const uint32_t *input,
                                const ptrdiff_t *source, const ptrdiff_t *target,
                                ptrdiff_t edge_count);
/* the same sweep in FP64 (start values and edge weights given as float32) */
void orc_traverse_down_f64_from_f32(double *output, const float *input,
                                    const ptrdiff_t *source, const ptrdiff_t *target,
                                    ptrdiff_t edge_count);
void orc_edgelist_degree(uint8_t *indegree, uint8_t *outdegree,
                         const ptrdiff_t *source, const ptrdiff_t *target,
                         ptrdiff_t node_count, ptrdiff_t edge_count);

/* ---- Graphflood single-flow graph (FP64, row-major `dim`, own BC codes) ---- */

/* src/graphflood/sfgraph.c:27-113: steepest-descent receiver of every node
 * that can give (BC 1, 3, 6, 7, 8, 9) among the neighbours that can receive
 * (BC 1, 3, 4, 5, 6, 7, 9), slope (z - z_n) / distance in double, first
 * strict maximum in neighbour order; donors listed per receiver in node
 * order (8 or 4 slots per node); the Braun-Willett stack: a depth-first
 * preorder from every root in node order, donors in listed order.  The
 * restatement walks the tree with an explicit stack (same order). */
void orc_compute_sfgraph(double *topo, size_t *Sreceivers, double *distToReceivers,
                         size_t *Sdonors, uint8_t *NSdonors, size_t *Stack,
                         const uint8_t *BCs, const size_t dim[2], double dx, int D8);
/* src/graphflood/gf_flowacc.c:19-35 (and :41-57 with weights): drainage
 * area in reverse stack order; roots add their donors' areas only. */
void orc_compute_drainage_area_single_flow(double *output, const size_t *Sreceivers,
                                           const size_t *Stack, const size_t dim[2],
                                           double dx);
void orc_compute_weighted_drainage_area_single_flow(double *output, const double *weights,
                                                    const size_t *Sreceivers,
                                                    const size_t *Stack,
                                                    const size_t dim[2], double dx);

#ifdef __cplusplus
}
#endif
#endif
