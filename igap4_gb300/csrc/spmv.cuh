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

namespace igap {

constexpr int SPMV_G = 4;  // lanes per row

__device__ __forceinline__ double spmv_row(const int64_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
                                           const double *__restrict__ vals, const double *__restrict__ x,
                                           int64_t row, bool valid, int sub, int nb0, int nb1, int nb2)
{
  double s = 0.0;
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
        s = fma(__ldg(v + k), __ldg(x + col), s);
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
      for (int64_t k = s0 + sub; k < s1; k += SPMV_G) s = fma(__ldg(vals + k), __ldg(x + __ldg(cols + k)), s);
    }
  }
  s += __shfl_xor_sync(0xffffffffu, s, 1);
  s += __shfl_xor_sync(0xffffffffu, s, 2);
  return s;
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
