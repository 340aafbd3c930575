/*
 * tt_oracle.c -- CPU oracle for the D8 flow pipeline (TEST INFRASTRUCTURE).
 *
 * A plain-C restatement of libtopotoolbox's algorithms on the D8 path.  It is
 * the checker for the CUDA library and the "port" CPU baseline in bench.py;
 * product code never links it.  Parity of this restatement with the
 * reference is pinned by tests/test_oracle_pins.py (bit-exact comparison
 * against the reference sources compiled by `make -C oracle ref`) and by the
 * golden fixtures in tests/golden/, which were produced by the compiled
 * reference.
 *
 * Conventions (include/topotoolbox.h:284-290): column-major arrays,
 * dims = {nrows, ncols}, linear index p = j * dims[0] + i.
 *
 * Sink filling is stated in the original (un-negated) elevation space:
 * the reference fills -reconstruct(-dem), which is f = max(dem, min of the
 * 3x3 neighbourhood of f) iterated from f = dem on bc==1 cells and +INF
 * elsewhere.  The fixpoint is identical; only the sign of a zero result may
 * differ, which the parity rule treats as equal.
 */
#include "tt_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_SQRT2F 1.41421356237309504880f

/* ------------------------------------------------------------------ */
/* Sink filling                                                        */
/* ------------------------------------------------------------------ */

/* One raster scan over the causal half-neighbourhood.  Follows
 * src/reconstruct.c:68-114 (forward) and :134-205 (backward).  `dir` is +1
 * for the forward scan and -1 for the backward scan.  When `q` is non-NULL
 * the backward scan records pixels that can still lower a neighbour
 * (src/reconstruct.c:179-196).  Returns the number of lowered pixels, or -1
 * when the queue overflowed. */
typedef struct {
  ptrdiff_t *buf;
  ptrdiff_t len;
  ptrdiff_t head;
  ptrdiff_t tail;
} orc_fifo; /* src/reconstruct.c:13-45: holds at most len-1 entries */

static int fifo_push(orc_fifo *q, ptrdiff_t v) {
  ptrdiff_t nxt = (q->tail + 1) % q->len;
  if (nxt == q->head) return 0;
  q->buf[q->tail] = v;
  q->tail = nxt;
  return 1;
}

static int fifo_pop(orc_fifo *q, ptrdiff_t *v) {
  if (q->head == q->tail) return 0;
  *v = q->buf[q->head];
  q->head = (q->head + 1) % q->len;
  return 1;
}

static ptrdiff_t fill_scan(float *f, const float *dem, const ptrdiff_t dims[2],
                           int dir, orc_fifo *q) {
  const ptrdiff_t m = dims[0], n = dims[1];
  /* causal neighbours of the forward scan: (i+1,j-1) (i,j-1) (i-1,j-1) (i-1,j);
     the backward scan mirrors them. */
  const ptrdiff_t di[4] = {1, 0, -1, -1};
  const ptrdiff_t dj[4] = {-1, -1, -1, 0};
  ptrdiff_t changed = 0;
  for (ptrdiff_t jj = 0; jj < n; jj++) {
    ptrdiff_t j = dir > 0 ? jj : n - 1 - jj;
    for (ptrdiff_t ii = 0; ii < m; ii++) {
      ptrdiff_t i = dir > 0 ? ii : m - 1 - ii;
      ptrdiff_t p = j * m + i;
      float lo = f[p];
      for (int k = 0; k < 4; k++) {
        ptrdiff_t ni = i + dir * di[k], nj = j + dir * dj[k];
        if (ni < 0 || ni >= m || nj < 0 || nj >= n) continue;
        lo = fminf(lo, f[nj * m + ni]);
      }
      float z = (lo > dem[p]) ? lo : dem[p];
      if (z < f[p]) changed++;
      f[p] = z;
      if (q) {
        for (int k = 0; k < 4; k++) {
          ptrdiff_t ni = i + dir * di[k], nj = j + dir * dj[k];
          if (ni < 0 || ni >= m || nj < 0 || nj >= n) continue;
          ptrdiff_t r = nj * m + ni;
          if (f[r] > f[p] && f[r] > dem[r]) {
            if (!fifo_push(q, p)) return -1;
          }
        }
      }
    }
  }
  return changed;
}

static void fill_init(float *f, const float *dem, const uint8_t *bc,
                      ptrdiff_t n) {
  /* src/fillsinks.c:24-37: fixed pixels keep the DEM, the rest start at the
     top of the lattice (+INF in the original elevation space). */
  for (ptrdiff_t p = 0; p < n; p++) f[p] = (bc[p] == 1) ? dem[p] : INFINITY;
}

void orc_fillsinks(float *output, const float *dem, const uint8_t *bc,
                   const ptrdiff_t dims[2]) {
  ptrdiff_t n = dims[0] * dims[1];
  fill_init(output, dem, bc, n);
  /* src/reconstruct.c:270-278: alternate scans until nothing changes, at
     most 1000 forward/backward pairs. */
  ptrdiff_t changed = n;
  for (int it = 0; it < 1000 && changed > 0; it++) {
    changed = fill_scan(output, dem, dims, +1, NULL);
    changed += fill_scan(output, dem, dims, -1, NULL);
  }
}

/* src/reconstruct.c:207-251: breadth-first propagation from queued pixels. */
static int fill_propagate(float *f, const float *dem, const ptrdiff_t dims[2],
                          orc_fifo *q) {
  const ptrdiff_t m = dims[0], n = dims[1];
  const ptrdiff_t di[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
  const ptrdiff_t dj[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
  int overflow = 0;
  ptrdiff_t p;
  while (fifo_pop(q, &p)) {
    ptrdiff_t i = p % m, j = p / m;
    float fp = f[p];
    for (int k = 0; k < 8; k++) {
      ptrdiff_t ni = i + di[k], nj = j + dj[k];
      if (ni < 0 || ni >= m || nj < 0 || nj >= n) continue;
      ptrdiff_t r = nj * m + ni;
      if (f[r] > fp && f[r] > dem[r]) {
        f[r] = fmaxf(fp, dem[r]);
        if (!fifo_push(q, r)) overflow = 1;
      }
    }
  }
  return overflow;
}

int orc_fillsinks_hybrid(float *output, ptrdiff_t *queue, const float *dem,
                         const uint8_t *bc, const ptrdiff_t dims[2]) {
  ptrdiff_t n = dims[0] * dims[1];
  fill_init(output, dem, bc, n);
  orc_fifo q = {queue, n, 0, 0};
  /* src/reconstruct.c:291-312: forward scan, backward scan that enqueues,
     FIFO propagation; repeat once if the queue overflowed. */
  int scans = 0, repeat = 0;
  do {
    fill_scan(output, dem, dims, +1, NULL);
    repeat = (fill_scan(output, dem, dims, -1, &q) == -1);
    repeat |= fill_propagate(output, dem, dims, &q);
    scans++;
  } while (repeat && scans < 2);
  return (scans == 2) && repeat;
}

/* Grayscale reconstruction by dilation, src/reconstruct.c:270-278 and
 * :291-312.  Its update marker = min(mask, max(marker, causal neighbours))
 * is the negation of the fill's update above with f = -marker and
 * dem = -mask, NaN comparisons included (fminf/fmaxf and `<` are symmetric
 * under negation), and so are the queue tests of the backward scan
 * (:179-196) and of the propagation (:207-251).  The scans therefore run on
 * negated copies; only the sign of a zero may differ. */
static void negate_copy(float *dst, const float *src, ptrdiff_t n) {
  for (ptrdiff_t p = 0; p < n; p++) dst[p] = -src[p];
}

void orc_reconstruct(float *marker, const float *mask, const ptrdiff_t dims[2]) {
  const ptrdiff_t n = dims[0] * dims[1];
  float *z = (float *)malloc((size_t)(n > 0 ? n : 1) * sizeof(float));
  negate_copy(z, mask, n);
  negate_copy(marker, marker, n);
  ptrdiff_t changed = n;
  for (int it = 0; it < 1000 && changed > 0; it++) {
    changed = fill_scan(marker, z, dims, +1, NULL);
    changed += fill_scan(marker, z, dims, -1, NULL);
  }
  negate_copy(marker, marker, n);
  free(z);
}

int orc_reconstruct_hybrid(float *marker, ptrdiff_t *queue, const float *mask,
                           const ptrdiff_t dims[2]) {
  const ptrdiff_t n = dims[0] * dims[1];
  float *z = (float *)malloc((size_t)(n > 0 ? n : 1) * sizeof(float));
  negate_copy(z, mask, n);
  negate_copy(marker, marker, n);
  orc_fifo q = {queue, n, 0, 0};
  int scans = 0, repeat = 0;
  do {
    fill_scan(marker, z, dims, +1, NULL);
    repeat = (fill_scan(marker, z, dims, -1, &q) == -1);
    repeat |= fill_propagate(marker, z, dims, &q);
    scans++;
  } while (repeat && scans < 2);
  negate_copy(marker, marker, n);
  free(z);
  return (scans == 2) && repeat;
}

/* ------------------------------------------------------------------ */
/* Flats, sills and presills (src/identifyflats.c:33-121)              */
/* ------------------------------------------------------------------ */

ptrdiff_t orc_identifyflats(int32_t *out, const float *dem,
                            const ptrdiff_t dims[2]) {
  const ptrdiff_t m = dims[0], n = dims[1];
  const ptrdiff_t di[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
  const ptrdiff_t dj[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
  ptrdiff_t nflats = 0;
  for (ptrdiff_t j = 0; j < n; j++) {
    for (ptrdiff_t i = 0; i < m; i++) {
      ptrdiff_t p = j * m + i;
      out[p] = 0;
      if (i == 0 || j == 0 || i == m - 1 || j == n - 1) continue;
      float z = dem[p], lo = z;
      for (int k = 0; k < 8; k++) {
        float zn = dem[(j + dj[k]) * m + i + di[k]];
        lo = fminf(lo, isnan(zn) ? -INFINITY : zn);
      }
      if (z == lo) { /* false for NaN */
        out[p] |= 1;
        nflats++;
      }
    }
  }
  for (ptrdiff_t j = 0; j < n; j++) {
    for (ptrdiff_t i = 0; i < m; i++) {
      ptrdiff_t p = j * m + i;
      if (out[p] & 1) continue;
      for (int k = 0; k < 8; k++) {
        ptrdiff_t ni = i + di[k], nj = j + dj[k];
        if (ni < 0 || ni >= m || nj < 0 || nj >= n) continue;
        ptrdiff_t r = nj * m + ni;
        if ((out[r] & 1) && dem[r] == dem[p]) {
          out[p] |= 2;
          out[r] |= 4;
        }
      }
    }
  }
  return nflats;
}

/* ------------------------------------------------------------------ */
/* GWDT costs: union-find labelling of flat components                 */
/* (src/gwdt.c:87-153 data structure, :167-278 driver)                 */
/* ------------------------------------------------------------------ */

static ptrdiff_t uf_root(const ptrdiff_t *lab, ptrdiff_t p) {
  while (lab[p] != p) p = lab[p];
  return p;
}

static void uf_compress(ptrdiff_t *lab, float *w, ptrdiff_t p, ptrdiff_t root,
                        float rw) {
  while (lab[p] != p) {
    ptrdiff_t nxt = lab[p];
    lab[p] = root;
    w[p] = rw;
    p = nxt;
  }
  lab[p] = root;
  w[p] = rw;
}

/* Merge the sets of `a` (an earlier flat neighbour) and `b` (the current
   pixel).  The surviving root is the one with the larger weight; on a tie
   the neighbour's root survives (src/gwdt.c:141-153). */
static void uf_merge(ptrdiff_t *lab, float *w, ptrdiff_t a, ptrdiff_t b) {
  ptrdiff_t ra = uf_root(lab, a);
  float wa = w[ra];
  if (ra != b) {
    ptrdiff_t rb = uf_root(lab, b);
    if (wa < w[rb]) {
      ra = rb;
      wa = w[rb];
    }
    uf_compress(lab, w, b, ra, wa);
  }
  uf_compress(lab, w, a, ra, wa);
}

void orc_gwdt_computecosts(float *costs, ptrdiff_t *conncomps,
                           const int32_t *flats, const float *orig,
                           const float *filled, const ptrdiff_t dims[2]) {
  const ptrdiff_t m = dims[0], n = dims[1];
  const ptrdiff_t dj[4] = {-1, -1, -1, 0};
  const ptrdiff_t di[4] = {-1, 0, 1, -1};
  for (ptrdiff_t j = 0; j < n; j++) {
    for (ptrdiff_t i = 0; i < m; i++) {
      ptrdiff_t p = j * m + i;
      if (!(flats[p] & 1)) {
        costs[p] = 0.0f;
        conncomps[p] = 0;
        continue;
      }
      conncomps[p] = p;
      costs[p] = filled[p] - orig[p];
      for (int k = 0; k < 4; k++) {
        ptrdiff_t ni = i + di[k], nj = j + dj[k];
        if (ni < 0 || ni >= m || nj < 0 || nj >= n) continue;
        ptrdiff_t r = nj * m + ni;
        if (flats[r] & 1) uf_merge(conncomps, costs, r, p);
      }
    }
  }
  for (ptrdiff_t j = 1; j < n - 1; j++) {
    for (ptrdiff_t i = 1; i < m - 1; i++) {
      ptrdiff_t p = j * m + i;
      if (!(flats[p] & 1)) continue;
      ptrdiff_t r = uf_root(conncomps, p);
      conncomps[p] = r;
      costs[p] = costs[r];
    }
  }
  /* src/gwdt.c:247-277: the difference is taken in float, the 0.1 offset is
     added in double and the sum rounded back to float. */
  for (ptrdiff_t j = 1; j < n - 1; j++) {
    for (ptrdiff_t i = 1; i < m - 1; i++) {
      ptrdiff_t p = j * m + i;
      if (!(flats[p] & 1)) continue;
      float depth = filled[p] - orig[p];
      float diff = costs[p] - depth;
      costs[p] = (float)((double)diff + 0.1);
    }
  }
}

/* ------------------------------------------------------------------ */
/* GWDT: Dijkstra over flat pixels (src/gwdt.c:290-351)                */
/* Indexed binary min-heap with the tie behaviour of                   */
/* src/helpers/priority_queue.c:52-133 (ties move towards the root).   */
/* ------------------------------------------------------------------ */

typedef struct {
  ptrdiff_t *heap;
  ptrdiff_t *back;
  float *key;
  ptrdiff_t count;
} orc_heap;

static void hp_swap(orc_heap *h, ptrdiff_t a, ptrdiff_t b) {
  ptrdiff_t ka = h->heap[a], kb = h->heap[b];
  h->back[ka] = b;
  h->back[kb] = a;
  h->heap[a] = kb;
  h->heap[b] = ka;
}

static void hp_up(orc_heap *h, ptrdiff_t pos) {
  while (pos > 0) {
    ptrdiff_t par = (pos - 1) / 2;
    float me = h->key[h->heap[pos]];
    if (isnan(me) || h->key[h->heap[par]] < me) return;
    hp_swap(h, pos, par);
    pos = par;
  }
}

static void hp_down(orc_heap *h, ptrdiff_t pos) {
  for (;;) {
    if (pos >= h->count / 2) return; /* leaf */
    ptrdiff_t c = 2 * pos + 1;
    if (c + 1 < h->count &&
        (isnan(h->key[h->heap[c]]) ||
         h->key[h->heap[c + 1]] < h->key[h->heap[c]]))
      c++;
    if (isnan(h->key[h->heap[c]]) ||
        h->key[h->heap[c]] > h->key[h->heap[pos]])
      return;
    hp_swap(h, pos, c);
    pos = c;
  }
}

void orc_gwdt(float *dist, ptrdiff_t *prev, const float *costs,
              const int32_t *flats, ptrdiff_t *heap, ptrdiff_t *back,
              const ptrdiff_t dims[2]) {
  const ptrdiff_t m = dims[0], n = dims[1];
  orc_heap h = {heap, back, dist, 0};
  for (ptrdiff_t p = 0; p < m * n; p++) {
    if (prev) prev[p] = p;
    dist[p] = 0.0f;
    if (flats[p] & 1) {
      back[p] = h.count;
      heap[h.count] = p;
      dist[p] = (flats[p] & 4) ? 1.0f : INFINITY;
      hp_up(&h, h.count++);
    }
  }
  /* neighbour order and chamfer weights of src/gwdt.c:318-320 */
  const ptrdiff_t di[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
  const ptrdiff_t dj[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
  const float ch[8] = {ORC_SQRT2F, 1.0f, ORC_SQRT2F, 1.0f,
                       1.0f,       ORC_SQRT2F, 1.0f, ORC_SQRT2F};
  while (h.count > 0) {
    ptrdiff_t u = heap[0];
    h.count--;
    if (h.count > 0) {
      hp_swap(&h, 0, h.count);
      hp_down(&h, 0);
    }
    back[u] = -1;
    float du = dist[u];
    ptrdiff_t i = u % m, j = u / m;
    for (int k = 0; k < 8; k++) {
      ptrdiff_t ni = i + di[k], nj = j + dj[k];
      if (ni < 0 || ni >= m || nj < 0 || nj >= n) continue;
      ptrdiff_t v = nj * m + ni;
      if (!(flats[v] & 1)) continue;
      float w = ch[k] * (costs[v] + costs[u]);
      float prop = du + w / 2;
      if (prop < dist[v]) {
        dist[v] = prop;
        hp_up(&h, back[v]);
        if (prev) prev[v] = u;
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* D8 carve routing (src/flow_routing.c:15-76, 135-256)                */
/* ------------------------------------------------------------------ */

/* Steepest descent over the 8 neighbours in the bit order of
   include/topotoolbox.h:807-816; flats compare the auxiliary topography. */
static uint8_t carve_direction(ptrdiff_t i, ptrdiff_t j, const float *dem,
                               const float *dist, const int32_t *flats,
                               const ptrdiff_t dims[2], unsigned order) {
  static const ptrdiff_t off[2][8] = {{0, 1, 1, 1, 0, -1, -1, -1},
                                      {1, 1, 0, -1, -1, -1, 0, 1}};
  const float sq2 = sqrtf(2.0f);
  const ptrdiff_t m = dims[0];
  ptrdiff_t p = j * m + i;
  int flat = flats[p] & 1;
  float z = flat ? dist[p] : dem[p];
  float best = 0.0f;
  uint8_t d = 0;
  for (int k = 0; k < 8; k++) {
    ptrdiff_t ni = i + off[order & 1][k];
    ptrdiff_t nj = j + off[(order ^ 1) & 1][k];
    if (ni < 0 || ni >= dims[0] || nj < 0 || nj >= dims[1]) continue;
    ptrdiff_t r = nj * m + ni;
    if (dem[r] > dem[p]) continue;
    float zn = flat ? dist[r] : dem[r];
    float g = (z - zn) / ((k & 1) ? sq2 : 1.0f);
    if (g > best) {
      best = g;
      d = (uint8_t)(1u << k);
    }
  }
  return d;
}

static int bit_index(uint8_t d) {
  int r = 0;
  while (d >>= 1) r++;
  return r;
}

void orc_flow_routing_d8_carve(ptrdiff_t *node, uint8_t *direction,
                               const float *dem, const float *dist,
                               const int32_t *flats, const ptrdiff_t dims[2],
                               unsigned int order) {
  const ptrdiff_t m = dims[0], n = dims[1];
  ptrdiff_t s0 = (order & 1) ? m : 1, s1 = (order & 1) ? 1 : m;
  const ptrdiff_t offs[8] = {s1, s0 + s1, s0, s0 - s1, -s1, -s0 - s1, -s0, -s0 + s1};
  memset(direction, 0xff, (size_t)(m * n));
  /* Iterative depth-first search; `node` doubles as the stack (bottom) and
     as the output list filled from the top in reverse postorder. */
  ptrdiff_t top = 0, next = m * n;
  for (ptrdiff_t j = 0; j < n; j++) {
    for (ptrdiff_t i = 0; i < m; i++) {
      ptrdiff_t start = j * m + i;
      if (direction[start] != 0xff) continue;
      node[top++] = start;
      while (top > 0) {
        ptrdiff_t u = node[--top];
        if (direction[u] != 0xff) continue; /* cycle: reference asserts */
        uint8_t d = carve_direction(u % m, u / m, dem, dist, flats, dims, order);
        if (d == 0) {
          direction[u] = 0;
          node[--next] = u;
          continue;
        }
        ptrdiff_t v = u + offs[bit_index(d)];
        if (direction[v] == 0xff) {
          node[top++] = u;
          node[top++] = v;
        } else {
          direction[u] = d;
          node[--next] = u;
        }
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* Flow accumulation (src/flow_accumulation.c:32-80)                   */
/* ------------------------------------------------------------------ */

static const ptrdiff_t ACC_DI[8] = {0, 1, 1, 1, 0, -1, -1, -1};
static const ptrdiff_t ACC_DJ[8] = {1, 1, 0, -1, -1, -1, 0, 1};

void orc_flow_accumulation(float *acc, const ptrdiff_t *source,
                           const uint8_t *direction, const float *weights,
                           const ptrdiff_t dims[2]) {
  const ptrdiff_t m = dims[0], n = m * dims[1];
  for (ptrdiff_t p = 0; p < n; p++) acc[p] = weights ? weights[p] : 1.0f;
  for (ptrdiff_t k = 0; k < n; k++) {
    ptrdiff_t u = source[k];
    uint8_t d = direction[u];
    if (d == 0) continue;
    int r = bit_index(d);
    ptrdiff_t v = (u / m + ACC_DJ[r]) * m + (u % m + ACC_DI[r]);
    acc[v] += acc[u];
  }
}

void orc_flow_accumulation_f64(double *acc, const ptrdiff_t *source,
                               const uint8_t *direction, const float *weights,
                               const ptrdiff_t dims[2]) {
  const ptrdiff_t m = dims[0], n = m * dims[1];
  for (ptrdiff_t p = 0; p < n; p++) acc[p] = weights ? (double)weights[p] : 1.0;
  for (ptrdiff_t k = 0; k < n; k++) {
    ptrdiff_t u = source[k];
    uint8_t d = direction[u];
    if (d == 0) continue;
    int r = bit_index(d);
    ptrdiff_t v = (u / m + ACC_DJ[r]) * m + (u % m + ACC_DI[r]);
    acc[v] += acc[u];
  }
}

void orc_flow_accumulation_f64w(double *acc, const ptrdiff_t *source,
                                const uint8_t *direction, const double *weights,
                                const ptrdiff_t dims[2]) {
  const ptrdiff_t m = dims[0], n = m * dims[1];
  for (ptrdiff_t p = 0; p < n; p++) acc[p] = weights[p];
  for (ptrdiff_t k = 0; k < n; k++) {
    ptrdiff_t u = source[k];
    uint8_t d = direction[u];
    if (d == 0) continue;
    int r = bit_index(d);
    ptrdiff_t v = (u / m + ACC_DJ[r]) * m + (u % m + ACC_DI[r]);
    acc[v] += acc[u];
  }
}

void orc_flow_accumulation_backward_f64(double *grad_w, const ptrdiff_t *source,
                                        const uint8_t *direction,
                                        const double *grad_acc,
                                        const ptrdiff_t dims[2]) {
  const ptrdiff_t m = dims[0], n = m * dims[1];
  /* Receivers follow their donors in `source`, so a reverse sweep sees every
     receiver's path sum before its donors need it. */
  for (ptrdiff_t k = n - 1; k >= 0; k--) {
    ptrdiff_t u = source[k];
    uint8_t d = direction[u];
    double g = grad_acc[u];
    if (d != 0) {
      int r = bit_index(d);
      ptrdiff_t v = (u / m + ACC_DJ[r]) * m + (u % m + ACC_DI[r]);
      g += grad_w[v];
    }
    grad_w[u] = g;
  }
}

/* ------------------------------------------------------------------ */
/* Hillshade (src/hillshade.c:11-213)                                  */
/* ------------------------------------------------------------------ */

#define ORC_PI_2F 1.57079632679489661923f

static float shade_f32(float dx, float dy, float sx, float sy, float sz) {
  float inv = 1.0f / sqrtf(dx * dx + dy * dy + 1.0f);
  return (-dx * inv) * sx + (-dy * inv) * sy + inv * sz;
}

/* Second-order gradient along one axis: one-sided [-3 4 -1]/(2h) and
   [1 -4 3]/(2h) at the ends, central [-1 0 1]/(2h) inside, NaN where the
   centre is NaN inside (src/hillshade.c:23-76). `s` is the stride along the
   axis, `k` the position along it and `len` its length. */
static float grad_axis_f32(const float *z, ptrdiff_t p, ptrdiff_t s,
                           ptrdiff_t k, ptrdiff_t len, float cs) {
  if (k == 0) return (-z[p + 2 * s] + 4 * z[p + s] - 3 * z[p]) / (2 * cs);
  if (k == len - 1) return (z[p - 2 * s] - 4 * z[p - s] + 3 * z[p]) / (2 * cs);
  return isnan(z[p]) ? NAN : (z[p + s] - z[p - s]) / (2 * cs);
}

void orc_hillshade_fused(float *out, const float *dem, float az, float alt,
                         float cs, const ptrdiff_t dims[2]) {
  const ptrdiff_t m = dims[0], n = dims[1];
  float sx = sinf(ORC_PI_2F - alt) * cosf(az);
  float sy = sinf(ORC_PI_2F - alt) * sinf(az);
  float sz = cosf(ORC_PI_2F - alt);
  for (ptrdiff_t j = 0; j < n; j++)
    for (ptrdiff_t i = 0; i < m; i++) {
      ptrdiff_t p = j * m + i;
      float dx = grad_axis_f32(dem, p, 1, i, m, cs);
      float dy = grad_axis_f32(dem, p, m, j, n, cs);
      out[p] = shade_f32(dx, dy, sx, sy, sz);
    }
}

void orc_hillshade(float *out, float *dxo, float *dyo, const float *dem,
                   float az, float alt, float cs, const ptrdiff_t dims[2]) {
  const ptrdiff_t m = dims[0], n = dims[1];
  float sx = sinf(ORC_PI_2F - alt) * cosf(az);
  float sy = sinf(ORC_PI_2F - alt) * sinf(az);
  float sz = cosf(ORC_PI_2F - alt);
  for (ptrdiff_t j = 0; j < n; j++)
    for (ptrdiff_t i = 0; i < m; i++) {
      ptrdiff_t p = j * m + i;
      dxo[p] = grad_axis_f32(dem, p, 1, i, m, cs);
      dyo[p] = grad_axis_f32(dem, p, m, j, n, cs);
      out[p] = shade_f32(dxo[p], dyo[p], sx, sy, sz);
    }
}

static double grad_axis_f64(const double *z, ptrdiff_t p, ptrdiff_t s,
                            ptrdiff_t k, ptrdiff_t len, double cs) {
  if (k == 0) return (-z[p + 2 * s] + 4 * z[p + s] - 3 * z[p]) / (2 * cs);
  if (k == len - 1) return (z[p - 2 * s] - 4 * z[p - s] + 3 * z[p]) / (2 * cs);
  return isnan(z[p]) ? NAN : (z[p + s] - z[p - s]) / (2 * cs);
}

static void sun_f64(double az, double alt, double *sx, double *sy, double *sz) {
  double zen = 1.57079632679489661923132169163975 - alt;
  *sx = sin(zen) * cos(az);
  *sy = sin(zen) * sin(az);
  *sz = cos(zen);
}

void orc_hillshade_f64(double *out, const double *dem, double az, double alt,
                       double cs, const ptrdiff_t dims[2]) {
  const ptrdiff_t m = dims[0], n = dims[1];
  double sx, sy, sz;
  sun_f64(az, alt, &sx, &sy, &sz);
  for (ptrdiff_t j = 0; j < n; j++)
    for (ptrdiff_t i = 0; i < m; i++) {
      ptrdiff_t p = j * m + i;
      double dx = grad_axis_f64(dem, p, 1, i, m, cs);
      double dy = grad_axis_f64(dem, p, m, j, n, cs);
      double inv = 1.0 / sqrt(dx * dx + dy * dy + 1.0);
      out[p] = (-dx * sx - dy * sy + sz) * inv;
    }
}

/* Adjoint of the one-axis stencil: scatter `g` (dH/d gradient at position k)
   onto the DEM samples that the stencil at k reads. */
static void grad_axis_adj(double *gd, ptrdiff_t p, ptrdiff_t s, ptrdiff_t k,
                          ptrdiff_t len, double cs, double g) {
  double c = g / (2 * cs);
  if (k == 0) {
    gd[p + 2 * s] -= c;
    gd[p + s] += 4 * c;
    gd[p] -= 3 * c;
  } else if (k == len - 1) {
    gd[p - 2 * s] += c;
    gd[p - s] -= 4 * c;
    gd[p] += 3 * c;
  } else {
    gd[p + s] += c;
    gd[p - s] -= c;
  }
}

void orc_hillshade_backward_f64(double *grad_dem, const double *dem,
                                const double *grad_out, double az, double alt,
                                double cs, const ptrdiff_t dims[2]) {
  const ptrdiff_t m = dims[0], n = dims[1];
  double sx, sy, sz;
  sun_f64(az, alt, &sx, &sy, &sz);
  for (ptrdiff_t p = 0; p < m * n; p++) grad_dem[p] = 0.0;
  for (ptrdiff_t j = 0; j < n; j++)
    for (ptrdiff_t i = 0; i < m; i++) {
      ptrdiff_t p = j * m + i;
      double dx = grad_axis_f64(dem, p, 1, i, m, cs);
      double dy = grad_axis_f64(dem, p, m, j, n, cs);
      double q = dx * dx + dy * dy + 1.0;
      double inv = 1.0 / sqrt(q);
      double num = -dx * sx - dy * sy + sz;
      if (isnan(num * inv)) continue;
      /* H = num * q^{-1/2}:  dH/ddx = -sx*inv - num*dx*inv^3 */
      double inv3 = inv * inv * inv;
      double hx = -sx * inv - num * dx * inv3;
      double hy = -sy * inv - num * dy * inv3;
      double g = grad_out[p];
      grad_axis_adj(grad_dem, p, 1, i, m, cs, g * hx);
      grad_axis_adj(grad_dem, p, m, j, n, cs, g * hy);
    }
}

/* ------------------------------------------------------------------
 * Edge-list forms.
 * ------------------------------------------------------------------ */

/* src/flow_routing.c:258-312.  With strides s0 (between rows) and s1
 * (between columns) of the given memory order, bit r of a direction byte
 * points at linear offset {s1, s0+s1, s0, s0-s1, -s1, -s0-s1, -s0, -s0+s1}[r]. */
ptrdiff_t orc_flow_routing_d8_edgelist(ptrdiff_t *source, ptrdiff_t *target,
                                       const ptrdiff_t *node,
                                       const uint8_t *direction,
                                       const ptrdiff_t dims[2], unsigned order) {
  const ptrdiff_t s0 = (order & 1) ? dims[0] : 1;
  const ptrdiff_t s1 = (order & 1) ? 1 : dims[0];
  const ptrdiff_t off[8] = {s1, s0 + s1, s0, s0 - s1, -s1, -s0 - s1, -s0, -s0 + s1};
  const ptrdiff_t n = dims[0] * dims[1];
  ptrdiff_t count = 0;
  for (ptrdiff_t k = 0; k < n; k++) {
    const ptrdiff_t u = node[k];
    const uint8_t d = direction[u];
    if (!d) continue;
    source[count] = u;
    target[count] = u + off[bit_index(d)];
    count++;
  }
  return count;
}

/* src/flow_accumulation.c:10-30 */
void orc_flow_accumulation_edgelist(float *acc, const ptrdiff_t *source,
                                    const ptrdiff_t *target,
                                    const float *fraction, const float *weights,
                                    ptrdiff_t edge_count, const ptrdiff_t dims[2]) {
  const ptrdiff_t n = dims[0] * dims[1];
  for (ptrdiff_t p = 0; p < n; p++) acc[p] = weights ? weights[p] : 1.0f;
  for (ptrdiff_t e = 0; e < edge_count; e++) {
    const float add = fraction[e] * acc[source[e]];
    acc[target[e]] = acc[target[e]] + add;
  }
}

void orc_flow_accumulation_edgelist_f64(double *acc, const ptrdiff_t *source,
                                        const ptrdiff_t *target,
                                        const float *fraction,
                                        const float *weights,
                                        ptrdiff_t edge_count,
                                        const ptrdiff_t dims[2]) {
  const ptrdiff_t n = dims[0] * dims[1];
  for (ptrdiff_t p = 0; p < n; p++) acc[p] = weights ? (double)weights[p] : 1.0;
  for (ptrdiff_t e = 0; e < edge_count; e++)
    acc[target[e]] += (double)fraction[e] * acc[source[e]];
}

/* src/streamquad.c:171-180: out[v] = out[v] + out[u] * in[e] in list order. */
void orc_traverse_down_f32_add_mul(float *output, const float *input,
                                   const ptrdiff_t *source, const ptrdiff_t *target,
                                   ptrdiff_t edge_count) {
  for (ptrdiff_t e = 0; e < edge_count; e++) {
    const float add = output[source[e]] * input[e];
    output[target[e]] = output[target[e]] + add;
  }
}

/* src/streamquad.c:49-60: in list order, out[target] |= out[source] & in[e]. */
void orc_traverse_down_u32_or_and(uint32_t *output, const uint32_t *input,
                                  const ptrdiff_t *source, const ptrdiff_t *target,
                                  ptrdiff_t edge_count) {
  for (ptrdiff_t e = 0; e < edge_count; e++)
    output[target[e]] = output[target[e]] | (output[source[e]] & input[e]);
}

/* src/streamquad.c:37-47: in reverse list order, out[source] |= out[target] & in[e]. */
void orc_traverse_up_u32_or_and(uint32_t *output, const uint32_t *input,
                                const ptrdiff_t *source, const ptrdiff_t *target,
                                ptrdiff_t edge_count) {
  for (ptrdiff_t e = edge_count - 1; e >= 0; e--)
    output[source[e]] = output[source[e]] | (output[target[e]] & input[e]);
}

/* The same sweep in FP64 over a float32 start and float32 edge weights. */
void orc_traverse_down_f64_from_f32(double *output, const float *input,
                                    const ptrdiff_t *source, const ptrdiff_t *target,
                                    ptrdiff_t edge_count) {
  for (ptrdiff_t e = 0; e < edge_count; e++)
    output[target[e]] += output[source[e]] * (double)input[e];
}

/* src/drainagebasins.c:6-27 */
void orc_drainagebasins(ptrdiff_t *basins, const ptrdiff_t *source,
                        const ptrdiff_t *target, ptrdiff_t edge_count,
                        const ptrdiff_t dims[2]) {
  const ptrdiff_t n = dims[0] * dims[1];
  for (ptrdiff_t p = 0; p < n; p++) basins[p] = 0;
  ptrdiff_t next = 1;
  for (ptrdiff_t e = edge_count - 1; e >= 0; e--) {
    if (basins[target[e]] == 0) basins[target[e]] = next++;
    basins[source[e]] = basins[target[e]];
  }
}

/* src/streamquad.c:209-224 */
void orc_edgelist_degree(uint8_t *indegree, uint8_t *outdegree,
                         const ptrdiff_t *source, const ptrdiff_t *target,
                         ptrdiff_t node_count, ptrdiff_t edge_count) {
  for (ptrdiff_t v = 0; v < node_count; v++) indegree[v] = outdegree[v] = 0;
  for (ptrdiff_t e = 0; e < edge_count; e++) {
    indegree[target[e]]++;
    outdegree[source[e]]++;
  }
}

/* ------------------------------------------------------------------
 * Graphflood single-flow graph.
 * ------------------------------------------------------------------ */

static int gf_can_give(uint8_t b) {
  return b == 1 || b == 3 || b == 6 || b == 7 || b == 8 || b == 9;
}
static int gf_can_receive(uint8_t b) {
  return b == 1 || b == 3 || b == 4 || b == 5 || b == 6 || b == 7 || b == 9;
}

/* Neighbour n of `node` exists (no wrap across the first/last row or
 * column; src/graphflood/gf_utils.c:202-253). */
static int gf_neighbour_ok(size_t node, int n, const size_t dim[2], int D8) {
  const size_t N = dim[0] * dim[1], c = node % dim[1];
  if (node < dim[1] && (D8 ? n < 3 : n == 0)) return 0;
  if (node >= N - dim[1] && (D8 ? n >= 5 : n == 3)) return 0;
  if (c == 0 && (D8 ? (n == 0 || n == 3 || n == 5) : n == 1)) return 0;
  if (c == dim[1] - 1 && (D8 ? (n == 2 || n == 4 || n == 7) : n == 2)) return 0;
  return 1;
}

void orc_compute_sfgraph(double *topo, size_t *Sreceivers, double *distToReceivers,
                         size_t *Sdonors, uint8_t *NSdonors, size_t *Stack,
                         const uint8_t *BCs, const size_t dim[2], double dx, int D8) {
  const size_t N = dim[0] * dim[1];
  const ptrdiff_t w = (ptrdiff_t)dim[1];
  const ptrdiff_t off8[8] = {-w - 1, -w, -w + 1, -1, 1, w - 1, w, w + 1};
  const ptrdiff_t off4[4] = {-w, -1, 1, w};
  const double diag = (double)sqrt(2) * dx;
  const double dx8[8] = {diag, dx, diag, dx, dx, diag, dx, diag};
  const int K = D8 ? 8 : 4;
  for (size_t node = 0; node < N; node++) {
    Sreceivers[node] = node;
    distToReceivers[node] = 0.;
    NSdonors[node] = 0;
    if (!gf_can_give(BCs[node])) continue;
    size_t best = node;
    double bestdx = 0., slope = 0.;
    for (int n = 0; n < K; n++) {
      if (!gf_neighbour_ok(node, n, dim, D8)) continue;
      const size_t q = (size_t)((ptrdiff_t)node + (D8 ? off8[n] : off4[n]));
      if (!gf_can_receive(BCs[q])) continue;
      const double d = D8 ? dx8[n] : dx;
      const double s = (topo[node] - topo[q]) / d;
      if (s > slope) {
        best = q;
        bestdx = d;
        slope = s;
      }
    }
    Sreceivers[node] = best;
    distToReceivers[node] = bestdx;
  }
  for (size_t node = 0; node < N; node++) {
    const size_t r = Sreceivers[node];
    if (r != node) Sdonors[r * K + NSdonors[r]++] = node;
  }
  /* preorder from each root, donors in listed order */
  size_t *todo = (size_t *)malloc(N * sizeof(size_t));
  size_t top = 0, pos = 0;
  for (size_t root = 0; root < N; root++) {
    if (Sreceivers[root] != root) continue;
    todo[top++] = root;
    while (top) {
      const size_t v = todo[--top];
      Stack[pos++] = v;
      for (int k = NSdonors[v] - 1; k >= 0; k--) todo[top++] = Sdonors[v * K + k];
    }
  }
  free(todo);
}

void orc_compute_drainage_area_single_flow(double *output, const size_t *Sreceivers,
                                           const size_t *Stack, const size_t dim[2],
                                           double dx) {
  const size_t N = dim[0] * dim[1];
  const double area = dx * dx;
  for (size_t i = 0; i < N; i++) output[i] = 0.;
  for (size_t i = N; i-- > 0;) {
    const size_t v = Stack[i];
    if (v == Sreceivers[v]) continue;
    output[v] += area;
    output[Sreceivers[v]] += output[v];
  }
}

void orc_compute_weighted_drainage_area_single_flow(double *output, const double *weights,
                                                    const size_t *Sreceivers,
                                                    const size_t *Stack,
                                                    const size_t dim[2], double dx) {
  const size_t N = dim[0] * dim[1];
  const double area = dx * dx;
  for (size_t i = 0; i < N; i++) output[i] = 0.;
  for (size_t i = N; i-- > 0;) {
    const size_t v = Stack[i];
    if (v == Sreceivers[v]) continue;
    output[v] += area * weights[v];
    output[Sreceivers[v]] += output[v];
  }
}
