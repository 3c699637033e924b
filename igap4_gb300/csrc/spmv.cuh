// One row of the CSR multiply y = A x, by one warp (rows hold 108-375 entries).
//
// The assembled pattern is the full structured stencil (setnz_iga,
// src/assmcore_iga.c:1054-1087): row 3*cp + d lists the clipped neighbour
// control points of cp, x-major and z fastest, three columns each.  With the
// lattice dimensions given (nb0 > 0) the column of entry 3*q + e is computed
// from k instead of read, so a multiply streams 8 instead of 12 bytes per
// nonzero; lanes take consecutive entries, as with the stored columns.  nb0 = 0
// (a batch's block-diagonal matrix) reads the stored column indices.
#pragma once
#include "common.cuh"

namespace igap {

__device__ __forceinline__ double spmv_row(const int64_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
                                           const double *__restrict__ vals, const double *__restrict__ x,
                                           int64_t row, int lane, int nb0, int nb1, int nb2)
{
  const int64_t s0 = __ldg(rowptr + row);
  double s = 0.0;
  if (nb0 > 0) {
    const int64_t cp = row / 3;
    const int iz = (int)(cp % nb2);
    const int64_t t = cp / nb2;
    const int iy = (int)(t % nb1), ix = (int)(t / nb1);
    const int lox = max(ix - P, 0), loy = max(iy - P, 0), loz = max(iz - P, 0);
    const int cx = min(ix + P, nb0 - 1) - lox + 1, cy = min(iy + P, nb1 - 1) - loy + 1,
              cz = min(iz + P, nb2 - 1) - loz + 1;
    const int len = 3 * cx * cy * cz;
    // lane handles entries k = lane, lane + 32, ... (coalesced, as the stored
    // CSR); k = 3 (((a cy) + b) cz + c) + e, advanced by 32 = 3 * 10 + 2 per step
    int e = lane % 3, q = lane / 3;
    int c = q % cz, bq = q / cz;
    int bb = bq % cy, a = bq / cy;
    const double *v = vals + s0;
    for (int k = lane; k < len; k += 32) {
      const int64_t col = 3 * (((int64_t)(lox + a) * nb1 + (loy + bb)) * nb2 + (loz + c)) + e;
      s = fma(__ldg(v + k), __ldg(x + col), s);
      e += 2;
      int dq = 10;
      if (e >= 3) {
        e -= 3;
        dq = 11;
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
    for (int64_t k = s0 + lane; k < s1; k += 32) s = fma(__ldg(vals + k), __ldg(x + __ldg(cols + k)), s);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

}  // namespace igap
