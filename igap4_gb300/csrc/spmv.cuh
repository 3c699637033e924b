// One row of the CSR multiply y = A x by a group of SPMV_G = 4 lanes (8 rows
// per warp; rows hold 108-375 entries).  On this GPU the multiply is bound by
// the FP64 pipe (one FMA per nonzero), not by HBM, so the cross-lane sum is
// kept short: two shuffle steps per row instead of five for a warp per row.
//
// The assembled pattern is the full structured stencil (setnz_iga,
// src/assmcore_iga.c:1054-1087): row 3*cp + d lists the clipped neighbour
// control points of cp, x-major and z fastest, three columns each.  With the
// lattice dimensions given (nb0 > 0) the column of entry 3*q + e is computed
// from k instead of read, so a multiply streams 8 instead of 12 bytes per
// nonzero; the lanes of a group take consecutive entries, as with the stored
// columns.  nb0 = 0 (a batch's block-diagonal matrix) reads the stored column
// indices, with the same entry-to-lane map and summation order.  Every lane
// of the warp must call this (the shuffles are warp-wide); `valid` = false
// for a group past the last row.
#pragma once
#include "common.cuh"
#include "element.cuh"
#include "df32.cuh"

namespace igap {

constexpr int SPMV_G = 4;  // lanes per row

// DF = true (split and FP64-quality modes, structured columns): every
// product and the row sum on float pairs (the value and x split on the
// integer pipe, compensated Dot2 accumulation), so that the multiply runs
// on the FP32 pipe instead of the FP64 pipe (~1e-15 relative to FP64).
template <bool DF = false>
__device__ __forceinline__ double spmv_row(const int64_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
                                           const double *__restrict__ vals, const double *__restrict__ x,
                                           int64_t row, bool valid, int sub, int nb0, int nb1, int nb2)
{
  double s = 0.0;
  float ps = 0.f, pc = 0.f;  // Dot2 accumulator (DF)
  if (valid) {
    const int64_t s0 = __ldg(rowptr + row);
    if (nb0 > 0) {
      const int64_t cp = row / 3;
      const int iz = (int)(cp % nb2);
      const int64_t t = cp / nb2;
      const int iy = (int)(t % nb1), ix = (int)(t / nb1);
      const int lox = max(ix - P, 0), loy = max(iy - P, 0), loz = max(iz - P, 0);
      const int cx = min(ix + P, nb0 - 1) - lox + 1, cy = min(iy + P, nb1 - 1) - loy + 1,
                cz = min(iz + P, nb2 - 1) - loz + 1;
      const int len = 3 * cx * cy * cz;
      // lane `sub` handles entries k = sub, sub + 4, ...; k = 3 (((a cy) + b) cz + c) + e,
      // advanced by 4 = 3 * 1 + 1 per step
      int e = sub % 3, q = sub / 3;
      int c = q % cz, bq = q / cz;
      int bb = bq % cy, a = bq / cy;
      const double *v = vals + s0;
      for (int k = sub; k < len; k += SPMV_G) {
        const int64_t col = 3 * (((int64_t)(lox + a) * nb1 + (loy + bb)) * nb2 + (loz + c)) + e;
        if constexpr (DF) dot2(ps, pc, f64_to_pair(__ldg(v + k)), f64_to_pair(__ldg(x + col)));
        else s = fma(__ldg(v + k), __ldg(x + col), s);
        int dq = 1;
        if (++e == 3) {
          e = 0;
          dq = 2;
        }
        c += dq;
        while (c >= cz) {
          c -= cz;
          if (++bb == cy) {
            bb = 0;
            ++a;
          }
        }
      }
    } else {
      const int64_t s1 = __ldg(rowptr + row + 1);
      for (int64_t k = s0 + sub; k < s1; k += SPMV_G) {
        if constexpr (DF) dot2(ps, pc, f64_to_pair(__ldg(vals + k)), f64_to_pair(__ldg(x + __ldg(cols + k))));
        else s = fma(__ldg(vals + k), __ldg(x + __ldg(cols + k)), s);
      }
    }
  }
  if constexpr (DF) {
    float2 r = dot2_pair(ps, pc);
#pragma unroll
    for (int o = 1; o < SPMV_G; o <<= 1) {
      const float2 t = make_float2(__shfl_xor_sync(0xffffffffu, r.x, o), __shfl_xor_sync(0xffffffffu, r.y, o));
      r = df_add(r, t);
    }
    return (double)r.x + (double)r.y;
  } else {
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    return s;
  }
}

}  // namespace igap

namespace igap {

// Point-block Jacobi: the 3x3 diagonal block of every control point (rows and
// columns 3 cp .. 3 cp + 2; a control point's columns are consecutive in its
// rows), inverted in FP64.  A block with zero or non-finite determinant falls
// back to the inverse of its diagonal (1 where that is zero).
static __global__ void bdiag_invert_kernel(const int64_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
                                    const double *__restrict__ vals, double *__restrict__ inv, int64_t ncp)
{
  const int64_t cp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cp >= ncp) return;
  double a[9];
  for (int d = 0; d < 3; d++) {
    const int64_t r = 3 * cp + d;
    int64_t lo = rowptr[r], hi = rowptr[r + 1];
    const int64_t target = 3 * cp;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (cols[mid] < target) lo = mid + 1;
      else hi = mid;
    }
    const bool ok = lo + 2 < rowptr[r + 1] && cols[lo] == target;
    for (int e = 0; e < 3; e++) a[3 * d + e] = ok ? vals[lo + e] : (d == e ? 1.0 : 0.0);
  }
  const double c0 = a[4] * a[8] - a[5] * a[7], c1 = a[2] * a[7] - a[1] * a[8], c2 = a[1] * a[5] - a[2] * a[4];
  const double c3 = a[5] * a[6] - a[3] * a[8], c4 = a[0] * a[8] - a[2] * a[6], c5 = a[2] * a[3] - a[0] * a[5];
  const double c6 = a[3] * a[7] - a[4] * a[6], c7 = a[1] * a[6] - a[0] * a[7], c8 = a[0] * a[4] - a[1] * a[3];
  const double det = a[0] * c0 + a[1] * c3 + a[2] * c6;
  double *o = inv + 9 * cp;
  if (det != 0.0 && isfinite(det)) {
    const double id = 1.0 / det;
    o[0] = c0 * id; o[1] = c1 * id; o[2] = c2 * id;
    o[3] = c3 * id; o[4] = c4 * id; o[5] = c5 * id;
    o[6] = c6 * id; o[7] = c7 * id; o[8] = c8 * id;
  } else {
    for (int i = 0; i < 9; i++) o[i] = 0.0;
    for (int d = 0; d < 3; d++) o[4 * d] = a[4 * d] != 0.0 ? 1.0 / a[4 * d] : 1.0;
  }
}

// Cell-block Jacobi: the diagonal blocks of the 2 x 2 x 2 control-point cells
// of the lattice (cells clipped at the far faces; up to 24 x 24, the cell's
// DOFs in DOF order), inverted in FP64 by Gauss-Jordan elimination with
// partial pivoting, one warp per cell.  A block whose pivot vanishes or is not
// finite falls back to the inverse of its diagonal (1 where that is zero).
// Entries are found from the structured stencil (the cell's control points
// are within one of each other, so every entry exists in the pattern).
constexpr int CBS = 24;  // largest block (8 control points x 3 DOFs)

struct CellGeom {
  int nb[3];     // control points per direction
  int nc[3];     // cells per direction
};

__host__ __device__ inline int64_t cell_count(const CellGeom &g)
{
  return (int64_t)g.nc[0] * g.nc[1] * g.nc[2];
}

// Control points of cell `cell` (x-major, z fastest) and their count.
__device__ __forceinline__ int cell_points(const CellGeom &g, int64_t cell, int64_t cps[8])
{
  const int gz = (int)(cell % g.nc[2]);
  const int64_t t = cell / g.nc[2];
  const int gy = (int)(t % g.nc[1]), gx = (int)(t / g.nc[1]);
  int n = 0;
  for (int jx = 2 * gx; jx < 2 * gx + 2 && jx < g.nb[0]; jx++)
    for (int jy = 2 * gy; jy < 2 * gy + 2 && jy < g.nb[1]; jy++)
      for (int jz = 2 * gz; jz < 2 * gz + 2 && jz < g.nb[2]; jz++)
        cps[n++] = ((int64_t)jx * g.nb[1] + jy) * g.nb[2] + jz;
  return n;
}

constexpr int CB_WARPS = 4;  // cells per block of the inversion

static __global__ void __launch_bounds__(32 * CB_WARPS) cblock_invert_kernel(const int64_t *__restrict__ rowptr,
                                                                             const double *__restrict__ vals,
                                                                             double *__restrict__ inv, CellGeom g,
                                                                             int64_t ncell)
{
  __shared__ double Aug[CB_WARPS][CBS][2 * CBS + 1];  // per warp [A | I], padded row
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t cell = (int64_t)blockIdx.x * CB_WARPS + warp;
  if (cell >= ncell) return;  // whole warp
  double(*A)[2 * CBS + 1] = Aug[warp];
  int64_t cps[8];
  const int np = cell_points(g, cell, cps);
  const int bs = 3 * np;
  for (int t = lane; t < CBS * 2 * CBS; t += 32) {
    const int a = t / (2 * CBS), b = t % (2 * CBS);
    double v = 0.0;
    if (a < bs && b < bs) {
      const int p = a / 3, d = a % 3, q = b / 3, e = b % 3;
      int ix, iy, iz, jx, jy, jz;
      cp_coords(cps[p], g.nb, ix, iy, iz);
      cp_coords(cps[q], g.nb, jx, jy, jz);
      const int64_t r = 3 * cps[p] + d;
      v = vals[rowptr[r] + 3 * stencil_pos(ix, iy, iz, jx, jy, jz, g.nb) + e];
    } else if (b >= CBS) {
      v = (b - CBS == a) ? 1.0 : 0.0;
    }
    A[a][b] = v;
  }
  __syncwarp();
  bool ok = true;
  for (int k = 0; k < bs && ok; k++) {
    // pivot: the largest |A[i][k]|, i >= k
    double best = (lane >= k && lane < bs) ? fabs(A[lane][k]) : -1.0;
    int arg = lane;
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
      if (ob > best || (ob == best && oa < arg)) {
        best = ob;
        arg = oa;
      }
    }
    if (!(best > 0.0) || !isfinite(best)) {
      ok = false;
      break;
    }
    if (arg != k)
      for (int c = lane; c < 2 * CBS; c += 32) {
        const double tmp = A[k][c];
        A[k][c] = A[arg][c];
        A[arg][c] = tmp;
      }
    __syncwarp();
    const double piv = A[k][k];
    double f[CBS];
#pragma unroll
    for (int i = 0; i < CBS; i++) f[i] = A[i][k];
    __syncwarp();
    for (int c = lane; c < 2 * CBS; c += 32) {
      const double rk = A[k][c] / piv;
      A[k][c] = rk;
#pragma unroll
      for (int i = 0; i < CBS; i++)
        if (i != k && i < bs) A[i][c] -= f[i] * rk;
    }
    __syncwarp();
  }
  double *o = inv + (size_t)cell * CBS * CBS;
  for (int t = lane; t < CBS * CBS; t += 32) {
    const int a = t / CBS, b = t % CBS;
    double v = 0.0;
    if (a < bs && b < bs) {
      if (ok) {
        v = A[a][CBS + b];
      } else if (a == b) {  // fallback: inverse of the diagonal
        const int p = a / 3, d = a % 3;
        int ix, iy, iz;
        cp_coords(cps[p], g.nb, ix, iy, iz);
        const int64_t r = 3 * cps[p] + d;
        const double dg = vals[rowptr[r] + 3 * stencil_pos(ix, iy, iz, ix, iy, iz, g.nb) + d];
        v = dg != 0.0 ? 1.0 / dg : 1.0;
      }
    }
    o[t] = v;
  }
}

// z = B^-1 v with the inverted cell blocks: a warp per cell, lane a < bs
// computes the cell's DOF a (grid-stride over cells).
__device__ __forceinline__ void cblock_apply(double *__restrict__ z, const double *__restrict__ v,
                                             const double *__restrict__ inv, const CellGeom &g, int64_t ncell)
{
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t cell = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); cell < ncell; cell += nw) {
    int64_t cps[8];
    const int np = cell_points(g, cell, cps);
    const int bs = 3 * np;
    if (lane < bs) {
      const double *row = inv + (size_t)cell * CBS * CBS + (size_t)lane * CBS;
      double s = 0.0;
      for (int b = 0; b < bs; b++) s = fma(row[b], v[3 * cps[b / 3] + b % 3], s);
      z[3 * cps[lane / 3] + lane % 3] = s;
    }
  }
}

// z = B^-1 v with the inverted blocks
__device__ __forceinline__ void bdiag_apply(double *__restrict__ z, const double *__restrict__ v,
                                            const double *__restrict__ inv, int64_t ncp)
{
  for (int64_t cp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; cp < ncp;
       cp += (int64_t)gridDim.x * blockDim.x) {
    const double *b = inv + 9 * cp;
    const double v0 = v[3 * cp], v1 = v[3 * cp + 1], v2 = v[3 * cp + 2];
    z[3 * cp] = b[0] * v0 + b[1] * v1 + b[2] * v2;
    z[3 * cp + 1] = b[3] * v0 + b[4] * v1 + b[5] * v2;
    z[3 * cp + 2] = b[6] * v0 + b[7] * v1 + b[8] * v2;
  }
}

}  // namespace igap
