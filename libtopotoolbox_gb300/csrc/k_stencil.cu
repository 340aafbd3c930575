// 3x3 stencil kernels: flat/sill/presill labelling, D8 carve directions,
// second-order gradients, hillshade and the hillshade adjoint.
//
// Every kernel is HBM-bound.  Tiles of 32 x 32 pixels (plus a halo) are
// staged in shared memory with coalesced 128-byte column segments, so each
// input byte is read from DRAM about once.
#include <algorithm>
#include <cmath>

#include "tt_internal.cuh"

namespace tt {
namespace {

constexpr int kBlockX = 32;  // along i
constexpr int kBlockY = 8;   // along j

// ------------------------------------------------------------------
// identifyflats (src/identifyflats.c:33-121)
//
// flat(p)    = interior pixel, not NaN, and no neighbour lower, a NaN
//              neighbour counting as -INF (src/identifyflats.c:64)
// sill(s)    = !flat(s) && exists flat neighbour f with z_f == z_s
// presill(f) =  flat(f) && exists non-flat neighbour s with z_s == z_f
// (the scatter at src/identifyflats.c:83-119 restated as a gather).
//
// One 32 x 32 output tile per block of 32 x 8 threads: the DEM is staged
// with a two-pixel halo (NaN off the grid).  Thread (tx, ty) takes column
// tx, rows 4 ty .. 4 ty + 3, and reads the 3 x 6 neighbourhood of that strip
// once into registers: it serves both the flat test of the four pixels and
// their sill / presill gather.  The flat bits of the one-pixel ring around
// the tile (132 pixels) are computed one per thread.  A strip with no flat
// pixel in its neighbourhood is all zeros (a non-flat pixel needs a flat
// neighbour to be a sill).  The flags go out through shared memory in
// coalesced columns, and each block adds its flat count to one of
// kCountSlots counters (spread so that blocks do not queue on one address),
// which a last step sums.
// ------------------------------------------------------------------
constexpr int kFz = kTile + 4;  // staged DEM side (two-pixel halo)
constexpr int kFr = 4;          // flat-bit row r of the tile is stored at r + kFr
constexpr int kFp = 44;         // flat-bit column pitch (bytes): rows -1 .. 32 at 3 .. 36,
                                // conflict-free 32-bit reads (44 / 4 = 11 is odd)
constexpr int kCountSlots = 64;

// Flat test of the pixel whose 3 x 3 neighbourhood is (a0 a1 a2 | b0 b1 b2 |
// c0 c1 c2), centre b1: not NaN and no neighbour lower, a NaN neighbour
// counting as -INF.  A neighbour x passes when (NaN ? -INF : x) >= b1: for
// b1 = -INF every neighbour passes, otherwise x passes exactly when
// x >= b1 (false for NaN), one compare per neighbour.
__device__ __forceinline__ bool is_flat(float a0, float a1, float a2, float b0, float b1,
                                        float b2, float c0, float c1, float c2) {
  const bool ge = (a0 >= b1) & (a1 >= b1) & (a2 >= b1) & (b0 >= b1) & (b2 >= b1) &
                  (c0 >= b1) & (c1 >= b1) & (c2 >= b1);
  return b1 == b1 && (ge || b1 == -INFINITY);
}

__global__ void __launch_bounds__(kBlockX * kBlockY)
identifyflats_kernel(int32_t *__restrict__ out, const float *__restrict__ dem, int64_t m,
                     int64_t n, unsigned long long *slots) {
  __shared__ float zs[kFz][kFz + 1];                   // [c][r]: dem at (i0 - 2 + r, j0 - 2 + c)
  __shared__ __align__(4) uint8_t fs[kTile + 2][kFp];  // [c + 1][r + kFr]: flat at (i0 + r, j0 + c)
  __shared__ int32_t os[kTile][kTile + 1];
  __shared__ unsigned wsum[kBlockY];
  const int tx = threadIdx.x, ty = threadIdx.y;
  constexpr int kC = (kFz + kBlockY - 1) / kBlockY;  // 5
  const int64_t i0 = (int64_t)blockIdx.x * kTile, j0 = (int64_t)blockIdx.y * kTile;
  const bool inner = i0 >= 2 && j0 >= 2 && i0 + kTile + 2 <= m && j0 + kTile + 2 <= n;
  {
    float v[kC][2];
    if (inner) {
      const float *base = dem + (j0 - 2) * m + (i0 - 2);
#pragma unroll
      for (int k = 0; k < kC; k++) {
        const int c = ty + k * kBlockY;
        const int64_t co = (int64_t)(c < kFz ? c : 0) * m;
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int r = tx + h * kBlockX;
          v[k][h] = base[co + (r < kFz ? r : 0)];
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < kC; k++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int c = ty + k * kBlockY, r = tx + h * kBlockX;
          const int64_t i = i0 - 2 + r, j = j0 - 2 + c;
          v[k][h] = (c < kFz && r < kFz && i >= 0 && i < m && j >= 0 && j < n) ? dem[j * m + i]
                                                                             : NAN;
        }
    }
#pragma unroll
    for (int k = 0; k < kC; k++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int c = ty + k * kBlockY, r = tx + h * kBlockX;
        if (c < kFz && r < kFz) zs[c][r] = v[k][h];
      }
  }
  __syncthreads();
  // interior pixels may be flat: global row 1 .. m - 2, column 1 .. n - 2
  auto interior = [&](int r, int c) {  // tile coordinates
    const int64_t i = i0 + r, j = j0 + c;
    return i >= 1 && i < m - 1 && j >= 1 && j < n - 1;
  };
  const int c = tx, r0 = 4 * ty;
  float z[3][6];  // tile columns c - 1 .. c + 1, rows r0 - 1 .. r0 + 4
#pragma unroll
  for (int dc = 0; dc < 3; dc++)
#pragma unroll
    for (int u = 0; u < 6; u++) z[dc][u] = zs[c + 1 + dc][r0 + 1 + u];
  {  // flat bits of the strip, one aligned word
    uint32_t w = 0;
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (interior(r0 + u, c) && is_flat(z[0][u], z[0][u + 1], z[0][u + 2], z[1][u], z[1][u + 1],
                                         z[1][u + 2], z[2][u], z[2][u + 1], z[2][u + 2]))
        w |= 1u << (8 * u);
    *reinterpret_cast<uint32_t *>(&fs[c + 1][r0 + kFr]) = w;
  }
  {  // flat bits of the ring: rows -1 and 32 (columns -1 .. 32), columns -1
     // and 32 (rows 0 .. 31)
    const int k = ty * kBlockX + tx;
    if (k < 2 * (kTile + 2) + 2 * kTile) {
      int rr, cc;
      if (k < kTile + 2) { rr = -1; cc = k - 1; }
      else if (k < 2 * (kTile + 2)) { rr = kTile; cc = k - (kTile + 2) - 1; }
      else if (k < 2 * (kTile + 2) + kTile) { cc = -1; rr = k - 2 * (kTile + 2); }
      else { cc = kTile; rr = k - 2 * (kTile + 2) - kTile; }
      const int zc = cc + 2, zr = rr + 2;  // staged coordinates of the pixel
      const bool f = interior(rr, cc) &&
                     is_flat(zs[zc - 1][zr - 1], zs[zc - 1][zr], zs[zc - 1][zr + 1],
                             zs[zc][zr - 1], zs[zc][zr], zs[zc][zr + 1], zs[zc + 1][zr - 1],
                             zs[zc + 1][zr], zs[zc + 1][zr + 1]);
      fs[cc + 1][rr + kFr] = (uint8_t)f;
    }
  }
  __syncthreads();
  // sill / presill: a neighbour of the other kind at the same elevation
  unsigned cnt = 0;
  {
    uint32_t fb[3];  // flat bits of rows r0 - 1 .. r0 + 4 (bit u) of the three columns
#pragma unroll
    for (int dc = 0; dc < 3; dc++) {
      const uint8_t *col = fs[c + dc];
      const uint32_t w0 = *reinterpret_cast<const uint32_t *>(col + r0);
      const uint32_t w1 = *reinterpret_cast<const uint32_t *>(col + r0 + 4);
      const uint32_t w2 = *reinterpret_cast<const uint32_t *>(col + r0 + 8);
      fb[dc] = ((w0 >> 24) & 1u) | ((w1 & 1u) << 1) | (((w1 >> 8) & 1u) << 2) |
               (((w1 >> 16) & 1u) << 3) | (((w1 >> 24) & 1u) << 4) | ((w2 & 1u) << 5);
    }
    if (fb[0] | fb[1] | fb[2]) {
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int uc = u + 1;
        const unsigned fc = (fb[1] >> uc) & 1u;
        const float z1 = z[1][uc];
        bool hit = false;
#pragma unroll
        for (int dc = 0; dc < 3; dc++)
#pragma unroll
          for (int du = -1; du <= 1; du++) {
            if (dc == 1 && du == 0) continue;
            hit |= (((fb[dc] >> (uc + du)) & 1u) != fc) & (z[dc][uc + du] == z1);
          }
        os[c][r0 + u] = (int32_t)(fc | (hit ? (fc ? 4u : 2u) : 0u));
        cnt += fc;
      }
    } else {
#pragma unroll
      for (int u = 0; u < 4; u++) os[c][r0 + u] = 0;
    }
  }
  __syncthreads();
  {
    const int64_t i = i0 + tx;
    if (i < m)
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const int cc = ty + k * kBlockY;
        const int64_t j = j0 + cc;
        if (j < n) out[j * m + i] = os[cc][tx];
      }
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  if (tx == 0) wsum[ty] = cnt;
  __syncthreads();
  if (tx == 0 && ty == 0) {
    unsigned long long tot = 0;
    for (int w = 0; w < kBlockY; w++) tot += wsum[w];
    if (tot) atomicAdd(&slots[(blockIdx.x + blockIdx.y * 7) % kCountSlots], tot);
  }
}

__global__ void sum_slots_kernel(const unsigned long long *__restrict__ slots,
                                 unsigned long long *__restrict__ count) {
  unsigned long long v = slots[threadIdx.x] + slots[threadIdx.x + 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (threadIdx.x == 0) *count = v;
}

// ------------------------------------------------------------------
// D8 carve directions (src/flow_routing.c:15-76)
//
// z = flat ? dist : dem; neighbours higher than the centre (in dem) are
// skipped; g = (z - z_n) / chamfer with chamfer = sqrtf(2) on odd bits; the
// first strictly largest positive g wins.  The subtraction and the IEEE
// division are written with explicit round-to-nearest intrinsics so that no
// contraction changes a bit.
// ------------------------------------------------------------------
//
// One 32 x 32 tile per block of 32 x 8 threads.  Staging: dem and dist with
// a one-pixel halo (NaN off the grid) and the centre flat bits.  Compute:
// thread (tx, ty) takes column tx, rows 4 ty .. 4 ty + 3, reading the 3 x 6
// neighbourhood of its strip once into registers.  The neighbour order is a
// template parameter, so every offset is a compile-time constant; the IEEE
// division of a diagonal difference by sqrt(2) runs only when the
// difference itself beats the best slope so far (fl(diff / sqrt(2)) <= diff,
// so otherwise it cannot win).
// The direction bytes go out through shared memory in coalesced rows.
// Directions of a 4-pixel column strip from its 3 x 6 window (dem z,
// auxiliary topography d), one byte per pixel.  FLATS: whether the strip
// may hold flats (bit 8u of fl4: pixel u is flat and compares d).
template <unsigned ORDER, bool FLATS>
__device__ __forceinline__ uint32_t strip_directions(const float (&z)[3][6],
                                                     const float (&d)[3][6], uint32_t fl4,
                                                     float sq2) {
  uint32_t out4 = 0;
#pragma unroll
  for (int u = 0; u < 4; u++) {
    const bool fl = FLATS && ((fl4 >> (8 * u)) & 1u);
    const float zc = z[1][u + 1];
    const float zz0 = fl ? d[1][u + 1] : zc;
    float best = 0.0f;
    unsigned dv = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      constexpr unsigned A = ORDER ? kD8B : kD8A, B = ORDER ? kD8A : kD8B;
      const int di = (int)((A >> (2 * k)) & 3u) - 1, dj = (int)((B >> (2 * k)) & 3u) - 1;
      const float zn = z[1 + dj][u + 1 + di];
      const float zz = fl ? d[1 + dj][u + 1 + di] : zn;
      const float diff = __fsub_rn(zz0, zz);
      // skip higher neighbours; a difference that does not beat the best
      // (or is NaN) cannot win, since a diagonal's quotient is <= diff
      if (zn > zc || !(diff > best)) continue;
      const float g = (k & 1) ? __fdiv_rn(diff, sq2) : diff;
      if (g > best) {
        best = g;
        dv = 1u << k;
      }
    }
    out4 |= dv << (8 * u);
  }
  return out4;
}

template <unsigned ORDER>
__global__ void __launch_bounds__(kBlockX * kBlockY)
directions_kernel(uint8_t *__restrict__ dir, const float *__restrict__ dem,
                  const float *__restrict__ dist,
                  const int32_t *__restrict__ flats, int64_t m, int64_t n) {
  __shared__ float zs[kTile + 2][kTile + 3];
  __shared__ float ds[kTile + 2][kTile + 3];
  __shared__ __align__(4) uint8_t fs[kTile][kTile + 4];
  __shared__ __align__(4) uint8_t os[kTile][kTile + 4];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t i0 = (int64_t)blockIdx.x * kTile;
  const int64_t j0 = (int64_t)blockIdx.y * kTile;
  constexpr int kH = kTile + 2;
  constexpr int kC = (kH + kBlockY - 1) / kBlockY;  // 5 halo columns per thread row
  const bool inner = i0 >= 1 && j0 >= 1 && i0 + kTile + 1 <= m && j0 + kTile + 1 <= n;
  {  // every load in flight at once
    float va[kC][2], vb[kC][2];
    int vf[4];
    if (inner) {
      const float *pd = dem + (j0 - 1) * m + (i0 - 1);
      const float *pt = dist + (j0 - 1) * m + (i0 - 1);
#pragma unroll
      for (int k = 0; k < kC; k++) {
        const int c = ty + k * kBlockY;
        const int64_t co = (int64_t)(c < kH ? c : 0) * m;
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int r = tx + h * kBlockX;
          const int rr = r < kH ? r : 0;
          va[k][h] = pd[co + rr];
          vb[k][h] = pt[co + rr];
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < kC; k++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int c = ty + k * kBlockY, r = tx + h * kBlockX;
          const int64_t i = i0 - 1 + r, j = j0 - 1 + c;
          va[k][h] = NAN;
          vb[k][h] = NAN;
          if (c < kH && r < kH && i >= 0 && i < m && j >= 0 && j < n) {
            const int64_t p = j * m + i;
            va[k][h] = dem[p];
            vb[k][h] = dist[p];
          }
        }
    }
    const bool row_ok = i0 + tx < m;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int64_t j = j0 + ty + k * kBlockY;
      vf[k] = (row_ok && j < n) ? flats[j * m + i0 + tx] : 0;
    }
#pragma unroll
    for (int k = 0; k < kC; k++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int c = ty + k * kBlockY, r = tx + h * kBlockX;
        if (c < kH && r < kH) {
          zs[c][r] = va[k][h];
          ds[c][r] = vb[k][h];
        }
      }
#pragma unroll
    for (int k = 0; k < 4; k++) fs[ty + k * kBlockY][tx] = (uint8_t)(vf[k] & 1);
  }
  __syncthreads();
  // Off-grid neighbours hold NaN: their slope is NaN and never selected,
  // exactly as the reference skips them, so no bounds checks are needed.
  const float sq2 = 1.41421353816986083984375f;  // sqrtf(2.0f) = 0x3FB504F3
  {
    const int c = tx, r0 = 4 * ty;  // centre (c + 1, r0 + 1 + u) in halo coordinates
    float z[3][6], d[3][6];
#pragma unroll
    for (int dc = 0; dc < 3; dc++)
#pragma unroll
      for (int u = 0; u < 6; u++) {
        z[dc][u] = zs[c + dc][r0 + u];
        d[dc][u] = ds[c + dc][r0 + u];
      }
    const uint32_t fl4 = *reinterpret_cast<const uint32_t *>(&fs[c][r0]);
    // One code path for every strip: a second one without the flat selects
    // measured slower (warps whose strips differ run both).
    const uint32_t out4 = strip_directions<ORDER, true>(z, d, fl4, sq2);
    *reinterpret_cast<uint32_t *>(&os[c][r0]) = out4;
  }
  __syncthreads();
  const int64_t i = i0 + tx;
  if (i < m)
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int c = ty + k * kBlockY;
      const int64_t j = j0 + c;
      if (j < n) dir[j * m + i] = os[c][tx];
    }
}

// ------------------------------------------------------------------
// Second-order gradient and hillshade (src/hillshade.c:11-213)
// ------------------------------------------------------------------
struct Grad {
  float dx, dy;
};

// Gradient along one axis at position k of len, reading the stencil values
// a(-2..2) around the centre.  Mirrors src/hillshade.c:113-155.
__device__ __forceinline__ float axis_grad(float zm2, float zm1, float z0,
                                           float zp1, float zp2, int64_t k,
                                           int64_t len, float twoh) {
  if (k == 0) return (-zp2 + 4 * zp1 - 3 * z0) / twoh;
  if (k == len - 1) return (zm2 - 4 * zm1 + 3 * z0) / twoh;
  return isnan(z0) ? NAN : (zp1 - zm1) / twoh;
}

__device__ __forceinline__ float shade(float dx, float dy, float sx, float sy,
                                       float sz) {
  float inv = 1.0f / sqrtf(dx * dx + dy * dy + 1.0f);
  return (-dx * inv) * sx + (-dy * inv) * sy + inv * sz;
}

// ------------------------------------------------------------------
// Float-float (unevaluated sum hi + lo) arithmetic for the shading.  The
// cancellation in -dx*sx - dy*sy + sz would otherwise cost up to ~1e-5 of
// relative accuracy where the shade is near zero on steep terrain; carrying
// ~44 bits keeps the result within a few float32 ulps of the FP64 formula.
// Error-free transformations: TwoSum (Knuth) and TwoProduct via FMA.
// ------------------------------------------------------------------
struct F2 {
  float hi, lo;
};

__device__ __forceinline__ F2 two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ F2 two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ F2 f2_norm(float hi, float lo) {
  float s = __fadd_rn(hi, lo);
  return {s, __fsub_rn(lo, __fsub_rn(s, hi))};
}
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  F2 s = two_sum(a.hi, b.hi);
  return f2_norm(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
  F2 p = two_prod(a.hi, b.hi);
  float t = __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi));
  return f2_norm(p.hi, __fadd_rn(p.lo, t));
}

// Exact stencil sums: the one-sided [-3 4 -1] / [1 -4 3] and central
// [-1 0 1] combinations of float32 samples, as float-float.
__device__ __forceinline__ F2 axis_diff_f2(float zm2, float zm1, float z0,
                                           float zp1, float zp2, int64_t k,
                                           int64_t len) {
  if (k == 0) {
    F2 t = f2_add(two_prod(4.0f, zp1), two_prod(-3.0f, z0));
    return f2_add(t, F2{-zp2, 0.0f});
  }
  if (k == len - 1) {
    F2 t = f2_add(two_prod(-4.0f, zm1), two_prod(3.0f, z0));
    return f2_add(t, F2{zm2, 0.0f});
  }
  return two_sum(zp1, -zm1);
}

struct Sun2 {
  float sxh, sxl, syh, syl, szh, szl;
  float rh, rl;  // 1 / (2 * cellsize) as float-float
};


constexpr int kHS = kTile + 4;  // 2-pixel halo for one-sided borders

// Block (x, y) computes tile (x, y + jt0): a launch may cover a band of tile
// columns, whose DEM columns (plus two on each side) must be in place.
template <int MODE>  // 0: hillshade, 1: gradients
__global__ void __launch_bounds__(kBlockX * kBlockY)
hillshade_kernel(float *__restrict__ out0, float *__restrict__ out1,
                 const float *__restrict__ dem, const float *__restrict__ gout,
                 int64_t m, int64_t n, float twoh, float sx, float sy, float sz,
                 Sun2 s2, int jt0) {
  __shared__ float z[kHS][kHS + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t i0 = (int64_t)blockIdx.x * kTile;
  const int64_t j0 = (int64_t)(blockIdx.y + jt0) * kTile;
  {  // stage the DEM with every load in flight at once
    constexpr int kC = (kHS + kBlockY - 1) / kBlockY;
    float v[kC][2];
#pragma unroll
    for (int k = 0; k < kC; k++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int c = ty + k * kBlockY, r = tx + h * kBlockX;
        const int64_t i = i0 - 2 + r, j = j0 - 2 + c;
        v[k][h] = (c < kHS && r < kHS && i >= 0 && i < m && j >= 0 && j < n) ? dem[j * m + i] : 0.0f;
      }
#pragma unroll
    for (int k = 0; k < kC; k++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int c = ty + k * kBlockY, r = tx + h * kBlockX;
        if (c < kHS && r < kHS) z[c][r] = v[k][h];
      }
  }
  __syncthreads();
  // Tiles at least two pixels away from every grid edge use central
  // differences only: no per-pixel border tests, and the float gradients
  // dx, dy are formed only where the float-float path is not finite.
  const bool deep = MODE == 0 && i0 >= 2 && i0 + kTile + 2 <= m && j0 >= 2 && j0 + kTile + 2 <= n;
  if (deep) {
    for (int c = ty; c < kTile; c += kBlockY) {
      const int r = tx + 2, cc = c + 2;
      const float zc0 = z[cc][r];
      const F2 ex = f2_mul(two_sum(z[cc][r + 1], -z[cc][r - 1]), F2{s2.rh, s2.rl});
      const F2 ey = f2_mul(two_sum(z[cc + 1][r], -z[cc - 1][r]), F2{s2.rh, s2.rl});
      float h = NAN;
      if (zc0 == zc0 && isfinite(ex.hi) && isfinite(ey.hi)) {
        const F2 num = f2_add(f2_add(f2_mul(ex, F2{-s2.sxh, -s2.sxl}),
                                     f2_mul(ey, F2{-s2.syh, -s2.syl})),
                              F2{s2.szh, s2.szl});
        const float q = __fmaf_rn(ex.hi, ex.hi, __fmaf_rn(ey.hi, ey.hi, 1.0f));
        h = __fdiv_rn(__fadd_rn(num.hi, num.lo), __fsqrt_rn(q));
      }
      if (!isfinite(h)) {  // NaN / INF exactly as the reference
        const float dx = isnan(zc0) ? NAN : __fdiv_rn(__fsub_rn(z[cc][r + 1], z[cc][r - 1]), twoh);
        const float dy = isnan(zc0) ? NAN : __fdiv_rn(__fsub_rn(z[cc + 1][r], z[cc - 1][r]), twoh);
        h = shade(dx, dy, sx, sy, sz);
      }
      out0[(j0 + c) * m + i0 + tx] = h;
    }
    return;
  }
  for (int c = ty; c < kTile; c += kBlockY) {
    int64_t j = j0 + c;
    int64_t i = i0 + tx;
    if (j >= n || i >= m) continue;
    int r = tx + 2, cc = c + 2;
    int64_t p = j * m + i;
    {
      float dx = axis_grad(z[cc][r - 2], z[cc][r - 1], z[cc][r], z[cc][r + 1],
                           z[cc][r + 2], i, m, twoh);
      float dy = axis_grad(z[cc - 2][r], z[cc - 1][r], z[cc][r], z[cc + 1][r],
                           z[cc + 2][r], j, n, twoh);
      if (MODE == 0) {
        float h;
        if (isfinite(dx) && isfinite(dy)) {
          // Only the numerator -dx*sx - dy*sy + sz cancels; it is carried in
          // float-float from the exact stencil differences.  The rest is one
          // rounded square root and one division (a few ulps, no
          // cancellation).
          const F2 ex = f2_mul(axis_diff_f2(z[cc][r - 2], z[cc][r - 1], z[cc][r], z[cc][r + 1],
                                            z[cc][r + 2], i, m), F2{s2.rh, s2.rl});
          const F2 ey = f2_mul(axis_diff_f2(z[cc - 2][r], z[cc - 1][r], z[cc][r], z[cc + 1][r],
                                            z[cc + 2][r], j, n), F2{s2.rh, s2.rl});
          const F2 num = f2_add(f2_add(f2_mul(ex, F2{-s2.sxh, -s2.sxl}),
                                       f2_mul(ey, F2{-s2.syh, -s2.syl})),
                                F2{s2.szh, s2.szl});
          const float q = __fmaf_rn(ex.hi, ex.hi, __fmaf_rn(ey.hi, ey.hi, 1.0f));
          h = __fdiv_rn(__fadd_rn(num.hi, num.lo), __fsqrt_rn(q));
          if (!isfinite(h)) h = shade(dx, dy, sx, sy, sz);
        } else {
          h = shade(dx, dy, sx, sy, sz);  // NaN / INF exactly as the reference
        }
        out0[p] = h;
      } else {
        out0[p] = dx;
        out1[p] = dy;
      }
    }
  }
}

// Weight with which the stencil centred at k (axis length len) reads the
// sample at k + off (src/hillshade.c:23-76: central differences inside,
// second-order one-sided differences on the first and last sample).
__device__ __forceinline__ float stencil_weight(int64_t k, int64_t len, int off) {
  if (k == 0) return (off == 0) ? -3.f : (off == 1) ? 4.f : (off == 2) ? -1.f : 0.f;
  if (k == len - 1) return (off == 0) ? 3.f : (off == -1) ? -4.f : (off == -2) ? 1.f : 0.f;
  return (off == 1) ? 1.f : (off == -1) ? -1.f : 0.f;
}

// Adjoint of hillshade w.r.t. the DEM: grad_dem = S^T (dH/d(dx) * g, dH/d(dy)
// * g), S the gradient stencils.  A 32 x 32 output tile needs dH/d(dx),
// dH/d(dy) at centres up to two pixels away, whose stencils read the DEM up
// to four pixels away: the block stages the DEM with a 4-pixel halo and the
// upstream gradient with a 2-pixel halo, evaluates the 36 x 36 centres from
// shared memory, then applies the transposed stencils.
constexpr int kHB = kTile + 8;  // DEM tile with a 4-pixel halo
constexpr int kHG = kTile + 4;  // centres with a 2-pixel halo

__global__ void __launch_bounds__(kBlockX * kBlockY)
hillshade_bwd_kernel(float *__restrict__ gdem, const float *__restrict__ dem,
                     const float *__restrict__ gout, int64_t m, int64_t n,
                     float twoh, float sx, float sy, float sz) {
  __shared__ float z[kHB][kHB + 1];
  __shared__ float gx[kHG][kHG + 1];  // upstream gradient, then dL/d(dx)
  __shared__ float gy[kHG][kHG + 1];  // dL/d(dy)
  constexpr int kThreads = kBlockX * kBlockY;
  const int tid = threadIdx.y * kBlockX + threadIdx.x;
  const int64_t i0 = (int64_t)blockIdx.x * kTile;
  const int64_t j0 = (int64_t)blockIdx.y * kTile;
  {  // stage the DEM and the upstream gradient, every load in flight at once
    constexpr int kZ = (kHB * kHB + kThreads - 1) / kThreads;
    constexpr int kG = (kHG * kHG + kThreads - 1) / kThreads;
    float vz[kZ], vg[kG];
#pragma unroll
    for (int u = 0; u < kZ; u++) {
      const int e = tid + u * kThreads;
      const int c = e / kHB, r = e % kHB;
      const int64_t i = i0 - 4 + r, j = j0 - 4 + c;
      vz[u] = (e < kHB * kHB && i >= 0 && i < m && j >= 0 && j < n) ? dem[j * m + i] : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < kG; u++) {
      const int e = tid + u * kThreads;
      const int c = e / kHG, r = e % kHG;
      const int64_t i = i0 - 2 + r, j = j0 - 2 + c;
      vg[u] = (e < kHG * kHG && i >= 0 && i < m && j >= 0 && j < n) ? gout[j * m + i] : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < kZ; u++) {
      const int e = tid + u * kThreads;
      if (e < kHB * kHB) z[e / kHB][e % kHB] = vz[u];
    }
#pragma unroll
    for (int u = 0; u < kG; u++) {
      const int e = tid + u * kThreads;
      if (e < kHG * kHG) gx[e / kHG][e % kHG] = vg[u];
    }
  }
  __syncthreads();
  // Tiles whose centres and samples all lie at least two pixels inside the
  // grid take a fast path: central differences only, multiplication by
  // 1 / (2h) and rsqrtf (each within an ulp or two of the exact path, far
  // inside the adjoint's 1e-5 tolerance), no per-pixel border tests.
  const bool deep = i0 >= 4 && i0 + kTile + 4 <= m && j0 >= 4 && j0 + kTile + 4 <= n;
  if (deep) {
    const float r2h = 1.0f / twoh;
    for (int e = tid; e < kHG * kHG; e += kThreads) {
      const int c = e / kHG, r = e % kHG;
      const int zc = c + 2, zr = r + 2;
      const float z0 = z[zc][zr];
      const float dx = (z[zc][zr + 1] - z[zc][zr - 1]) * r2h;
      const float dy = (z[zc + 1][zr] - z[zc - 1][zr]) * r2h;
      const float inv = rsqrtf(fmaf(dx, dx, fmaf(dy, dy, 1.0f)));
      const float num = fmaf(-dx, sx, fmaf(-dy, sy, sz));
      float ax = 0.f, ay = 0.f;
      if (z0 == z0 && !isnan(num * inv)) {
        const float tt = num * (inv * inv * inv);
        const float g = gx[c][r];
        ax = g * (-sx * inv - dx * tt);
        ay = g * (-sy * inv - dy * tt);
      }
      gx[c][r] = ax;  // this thread alone read gx[c][r]
      gy[c][r] = ay;
    }
    __syncthreads();
    for (int cy = threadIdx.y; cy < kTile; cy += kBlockY) {
      const int r = threadIdx.x + 2, cc = cy + 2;
      const float acc = ((gx[cc][r - 1] - gx[cc][r + 1]) + gy[cc - 1][r]) - gy[cc + 1][r];
      gdem[(j0 + cy) * m + i0 + threadIdx.x] = acc * r2h;
    }
    return;
  }
  // dH/d(dx) * g and dH/d(dy) * g at the 36 x 36 centres.
  for (int e = tid; e < kHG * kHG; e += kThreads) {
    const int c = e / kHG, r = e % kHG;
    const int64_t i = i0 - 2 + r, j = j0 - 2 + c;
    float ax = 0.f, ay = 0.f;
    if (i >= 0 && i < m && j >= 0 && j < n) {
      const int zc = c + 2, zr = r + 2;
      const float dx = axis_grad(z[zc][zr - 2], z[zc][zr - 1], z[zc][zr], z[zc][zr + 1],
                                 z[zc][zr + 2], i, m, twoh);
      const float dy = axis_grad(z[zc - 2][zr], z[zc - 1][zr], z[zc][zr], z[zc + 1][zr],
                                 z[zc + 2][zr], j, n, twoh);
      const float q = dx * dx + dy * dy + 1.0f;
      const float inv = 1.0f / sqrtf(q);
      const float num = -dx * sx - dy * sy + sz;
      if (!isnan(num * inv)) {
        const float inv3 = inv * inv * inv;
        const float g = gx[c][r];
        ax = g * (-sx * inv - num * dx * inv3);
        ay = g * (-sy * inv - num * dy * inv3);
      }
    }
    gx[c][r] = ax;  // this thread alone read gx[c][r]
    gy[c][r] = ay;
  }
  __syncthreads();
  // Transposed stencils: sample (i, j) receives from the centres whose
  // stencil reads it.  Away from the borders only the two central neighbours
  // along each axis contribute.
  const int tx = threadIdx.x;
  const int64_t i = i0 + tx;
  for (int cy = threadIdx.y; cy < kTile; cy += kBlockY) {
    const int64_t j = j0 + cy;
    if (j >= n || i >= m) continue;
    const int r = tx + 2, cc = cy + 2;
    float acc;
    if (i >= 3 && i <= m - 4 && j >= 3 && j <= n - 4) {
      acc = gx[cc][r - 1] - gx[cc][r + 1];
      acc = acc + gy[cc - 1][r];
      acc = acc - gy[cc + 1][r];
    } else {
      acc = 0.0f;
#pragma unroll
      for (int d = -2; d <= 2; d++) {
        const int64_t k = i + d;  // centre position along i
        if (k < 0 || k >= m) continue;
        const float w = stencil_weight(k, m, (int)(i - k));
        if (w != 0.f) acc += w * gx[cc][r + d];
      }
#pragma unroll
      for (int d = -2; d <= 2; d++) {
        const int64_t k = j + d;
        if (k < 0 || k >= n) continue;
        const float w = stencil_weight(k, n, (int)(j - k));
        if (w != 0.f) acc += w * gy[cc + d][r];
      }
    }
    gdem[j * m + i] = acc / twoh;
  }
}

dim3 tile_grid(const GridDims &g) { return dim3(g.tm, g.tn); }

}  // namespace

tt_cuda_status identifyflats_dev(int32_t *flags, const float *dem,
                                 const GridDims &g,
                                 unsigned long long *count_dev,
                                 cudaStream_t st) {
  Workspace &ws = workspace();
  if (!ws.reserve(1024)) return TT_CUDA_ERR_ALLOC;
  unsigned long long *slots = (unsigned long long *)ws.take(kCountSlots * 8);
  unsigned long long *cnt = count_dev ? count_dev : (unsigned long long *)ws.take(8);
  TT_CHECK(cudaMemsetAsync(slots, 0, kCountSlots * 8, st));
  TT_LAUNCH(identifyflats_kernel, tile_grid(g), dim3(kBlockX, kBlockY), 0, st, flags, dem, g.m,
            g.n, slots);
  TT_LAUNCH(sum_slots_kernel, 1, 32, 0, st, slots, cnt);
  TT_CHECK(cudaGetLastError());
  return TT_CUDA_SUCCESS;
}

tt_cuda_status directions_dev(uint8_t *dir, const float *dem, const float *dist,
                              const int32_t *flats, const GridDims &g,
                              unsigned order, cudaStream_t st) {
  if (order & 1)
    TT_LAUNCH(directions_kernel<1>, tile_grid(g), dim3(kBlockX, kBlockY), 0, st, dir, dem,
              dist, flats, g.m, g.n);
  else
    TT_LAUNCH(directions_kernel<0>, tile_grid(g), dim3(kBlockX, kBlockY), 0, st, dir, dem,
              dist, flats, g.m, g.n);
  TT_CHECK(cudaGetLastError());
  return TT_CUDA_SUCCESS;
}

tt_cuda_status gradient2_dev(float *p0, float *p1, const float *dem,
                             float cellsize, const GridDims &g,
                             cudaStream_t st) {
  TT_LAUNCH(hillshade_kernel<1>, tile_grid(g), dim3(kBlockX, kBlockY), 0, st,
            p0, p1, dem, nullptr, g.m, g.n, 2 * cellsize, 0.f, 0.f, 0.f, Sun2{}, 0);
  TT_CHECK(cudaGetLastError());
  return TT_CUDA_SUCCESS;
}

tt_cuda_status hillshade_cols_dev(float *out, const float *dem, float azimuth,
                                  float altitude, float cellsize, const GridDims &g,
                                  int jt0, int jt1, cudaStream_t st) {
  if (jt1 <= jt0) return TT_CUDA_SUCCESS;
  float sx, sy, sz;
  sun_vector(azimuth, altitude, &sx, &sy, &sz);
  double zen = 1.57079632679489661923132169163975 - (double)altitude;
  double dsx = std::sin(zen) * std::cos((double)azimuth);
  double dsy = std::sin(zen) * std::sin((double)azimuth);
  double dsz = std::cos(zen);
  const double rinv = 1.0 / (2.0 * (double)cellsize);
  const float rh = (float)rinv;
  Sun2 s2{sx, (float)(dsx - (double)sx), sy, (float)(dsy - (double)sy),
          sz, (float)(dsz - (double)sz), rh, (float)(rinv - (double)rh)};
  TT_LAUNCH(hillshade_kernel<0>, dim3(g.tm, jt1 - jt0), dim3(kBlockX, kBlockY), 0, st,
            out, nullptr, dem, nullptr, g.m, g.n, 2 * cellsize, sx, sy, sz, s2, jt0);
  TT_CHECK(cudaGetLastError());
  return TT_CUDA_SUCCESS;
}

tt_cuda_status hillshade_dev(float *out, const float *dem, float azimuth,
                             float altitude, float cellsize, const GridDims &g,
                             cudaStream_t st) {
  return hillshade_cols_dev(out, dem, azimuth, altitude, cellsize, g, 0, g.tn, st);
}

tt_cuda_status hillshade_backward_dev(float *grad_dem, const float *dem,
                                      const float *grad_out, float azimuth,
                                      float altitude, float cellsize,
                                      const GridDims &g, cudaStream_t st) {
  float sx, sy, sz;
  sun_vector(azimuth, altitude, &sx, &sy, &sz);
  TT_LAUNCH(hillshade_bwd_kernel, tile_grid(g), dim3(kBlockX, kBlockY), 0, st,
            grad_dem, dem, grad_out, g.m, g.n, 2 * cellsize, sx, sy, sz);
  TT_CHECK(cudaGetLastError());
  return TT_CUDA_SUCCESS;
}

}  // namespace tt
