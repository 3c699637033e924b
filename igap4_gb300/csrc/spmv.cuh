// One row of the CSR multiply y = A x, by one warp (rows hold 108-375 entries).
//
// The assembled pattern is the full structured stencil (setnz_iga,
// src/assmcore_iga.c:1054-1087): row 3*cp + d lists the clipped neighbour
// control points of cp, x-major and z fastest, three columns each.  With the
// lattice dimensions given (nb0 > 0) the column of entry 3*q + e is computed
// from q instead of read, so a multiply streams 8 instead of 12 bytes per
// nonzero; each lane takes whole neighbour control points.  nb0 = 0 (a batch's
// block-diagonal matrix) reads the stored column indices.
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
    const int cyz = cy * cz, ncp = cx * cyz;
    for (int q = lane; q < ncp; q += 32) {
      const int jx = lox + q / cyz, r = q % cyz;
      const int jy = loy + r / cz, jz = loz + r % cz;
      const double *v = vals + s0 + 3 * q;
      const double *xx = x + 3 * (((int64_t)jx * nb1 + jy) * nb2 + jz);
      s = fma(__ldcs(v), __ldg(xx), s);
      s = fma(__ldcs(v + 1), __ldg(xx + 1), s);
      s = fma(__ldcs(v + 2), __ldg(xx + 2), s);
    }
  } else {
    const int64_t s1 = __ldg(rowptr + row + 1);
    for (int64_t k = s0 + lane; k < s1; k += 32) s = fma(__ldcs(vals + k), __ldg(x + __ldg(cols + k)), s);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

}  // namespace igap
