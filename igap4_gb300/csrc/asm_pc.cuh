// Restricted additive Schwarz (ASM, restrict) preconditioner on the
// control-point lattice: the device counterpart of the reference's default
// PCASM with PC_ASM_RESTRICT (src/interface.c:240-241).
//
// Subdomains: the 2 x 2 x 2 control-point cells of the cell-block Jacobi
// (spmv.cuh), each extended by one control-point layer on every side (up to
// 4 x 4 x 4 control points, 192 DOFs).  Set-up, one CTA per subdomain: the
// subdomain matrix A_i (rows and columns of its extended DOFs) is gathered
// from the CSR values through the structured stencil, and the rows of A_i^-1
// that belong to the cell's own DOFs are computed by Gaussian elimination
// with partial pivoting on A_i^T X = E (E: the identity columns of the cell's
// DOFs), in FP32 in shared memory (a preconditioner needs no FP64 inverse;
// GMRES stays FP64).  Apply: z on the cell's DOFs = (A_i^-1 restricted to
// them) . v on the extended DOFs, so every DOF is written by exactly one
// subdomain (the "restrict" variant: no overlap in the prolongation).  A
// subdomain whose elimination meets a zero pivot falls back to the inverse
// diagonal on its DOFs.
#pragma once
#include "spmv.cuh"

namespace igap {

constexpr int AS_N = 192;    // largest extended subdomain: 64 control points x 3 DOFs
constexpr int AS_NC = 24;    // DOFs of the cell itself: 8 control points x 3
constexpr int AS_LD = AS_N + 1;
constexpr int AS_THREADS = 256;

struct AsmSmem {
  float M[AS_N * AS_LD];     // A_i^T, eliminated in place
  float E[AS_N * AS_NC];     // right-hand sides, then the solution X
  int64_t cps[64];           // extended control points (x-major, z fastest)
  int core[8];               // positions of the cell's control points among them
  int ne, nc, piv;
  int fail;
};

// Extended control points of subdomain `cell` (cells of 2 x 2 x 2 control
// points, x-major, z fastest), and where the cell's own points sit among them.
__device__ __forceinline__ void asm_points(const CellGeom &g, int64_t cell, int64_t *cps, int *core, int &ne,
                                           int &nc)
{
  const int gz = (int)(cell % g.nc[2]);
  const int64_t t = cell / g.nc[2];
  const int gy = (int)(t % g.nc[1]), gx = (int)(t / g.nc[1]);
  ne = 0;
  nc = 0;
  for (int jx = 2 * gx - 1; jx < 2 * gx + 3; jx++) {
    if (jx < 0 || jx >= g.nb[0]) continue;
    for (int jy = 2 * gy - 1; jy < 2 * gy + 3; jy++) {
      if (jy < 0 || jy >= g.nb[1]) continue;
      for (int jz = 2 * gz - 1; jz < 2 * gz + 3; jz++) {
        if (jz < 0 || jz >= g.nb[2]) continue;
        if (jx >= 2 * gx && jx < 2 * gx + 2 && jy >= 2 * gy && jy < 2 * gy + 2 && jz >= 2 * gz && jz < 2 * gz + 2)
          core[nc++] = ne;
        cps[ne++] = ((int64_t)jx * g.nb[1] + jy) * g.nb[2] + jz;
      }
    }
  }
}

// Z[cell][c][b] (FP32, AS_NC x AS_N per cell): row c of A_i^-1 for the cell's
// DOF c, over the extended DOFs b.
static __global__ void __launch_bounds__(AS_THREADS) asm_setup_kernel(const int64_t *__restrict__ rowptr,
                                                                      const double *__restrict__ vals,
                                                                      float *__restrict__ Z, CellGeom g)
{
  extern __shared__ __align__(16) unsigned char asm_smem_raw[];
  AsmSmem &S = *reinterpret_cast<AsmSmem *>(asm_smem_raw);
  const int64_t cell = blockIdx.x;
  const int tid = threadIdx.x;
  if (tid == 0) {
    int ne, nc;
    asm_points(g, cell, S.cps, S.core, ne, nc);
    S.ne = ne;
    S.nc = nc;
    S.fail = 0;
  }
  __syncthreads();
  const int n = 3 * S.ne, ncd = 3 * S.nc;
  // M = A_i^T: M[a][b] = A[dof b][dof a]; entries outside the stencil are zero
  for (int t = tid; t < n * n; t += AS_THREADS) {
    const int a = t / n, b = t % n;
    const int p = b / 3, d = b % 3, q = a / 3, e = a % 3;  // row dof b = (p, d), column dof a = (q, e)
    int ix, iy, iz, jx, jy, jz;
    cp_coords(S.cps[p], g.nb, ix, iy, iz);
    cp_coords(S.cps[q], g.nb, jx, jy, jz);
    float v = 0.f;
    if (abs(ix - jx) <= P && abs(iy - jy) <= P && abs(iz - jz) <= P) {
      const int64_t r = 3 * S.cps[p] + d;
      v = (float)vals[rowptr[r] + 3 * stencil_pos(ix, iy, iz, jx, jy, jz, g.nb) + e];
    }
    S.M[a * AS_LD + b] = v;
  }
  for (int t = tid; t < n * AS_NC; t += AS_THREADS) {
    const int a = t / AS_NC, c = t % AS_NC;
    S.E[t] = (c < ncd && a == 3 * S.core[c / 3] + c % 3) ? 1.f : 0.f;
  }
  __syncthreads();
  // Gaussian elimination with partial pivoting on [M | E]
  for (int k = 0; k < n; k++) {
    if (tid < 32) {
      float best = -1.f;
      int arg = k;
      for (int i = k + tid; i < n; i += 32) {
        const float v = fabsf(S.M[i * AS_LD + k]);
        if (v > best) { best = v; arg = i; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
        if (ob > best || (ob == best && oa < arg)) { best = ob; arg = oa; }
      }
      if (tid == 0) {
        S.piv = arg;
        if (!(best > 0.f) || !isfinite(best)) S.fail = 1;
      }
    }
    __syncthreads();
    if (S.fail) break;
    const int pr = S.piv;
    if (pr != k) {
      for (int j = k + tid; j < n; j += AS_THREADS) {
        const float tmp = S.M[k * AS_LD + j];
        S.M[k * AS_LD + j] = S.M[pr * AS_LD + j];
        S.M[pr * AS_LD + j] = tmp;
      }
      for (int c = tid; c < AS_NC; c += AS_THREADS) {
        const float tmp = S.E[k * AS_NC + c];
        S.E[k * AS_NC + c] = S.E[pr * AS_NC + c];
        S.E[pr * AS_NC + c] = tmp;
      }
    }
    __syncthreads();
    const float inv = 1.f / S.M[k * AS_LD + k];
    for (int i = k + 1 + tid; i < n; i += AS_THREADS) S.M[i * AS_LD + k] *= inv;  // multipliers
    __syncthreads();
    const int rows = n - k - 1, cols = n - k - 1 + AS_NC;
    for (int t = tid; t < rows * cols; t += AS_THREADS) {
      const int i = k + 1 + t / cols, jj = t % cols;
      const float f = S.M[i * AS_LD + k];
      if (jj < n - k - 1) {
        const int j = k + 1 + jj;
        S.M[i * AS_LD + j] -= f * S.M[k * AS_LD + j];
      } else {
        const int c = jj - (n - k - 1);
        S.E[i * AS_NC + c] -= f * S.E[k * AS_NC + c];
      }
    }
    __syncthreads();
  }
  // back substitution (upper triangle), X overwrites E
  if (!S.fail) {
    for (int k = n - 1; k >= 0; k--) {
      if (tid < AS_NC) S.E[k * AS_NC + tid] /= S.M[k * AS_LD + k];
      __syncthreads();
      for (int t = tid; t < k * AS_NC; t += AS_THREADS) {
        const int i = t / AS_NC, c = t % AS_NC;
        S.E[i * AS_NC + c] -= S.M[i * AS_LD + k] * S.E[k * AS_NC + c];
      }
      __syncthreads();
    }
  }
  float *o = Z + (size_t)cell * AS_NC * AS_N;
  for (int t = tid; t < AS_NC * AS_N; t += AS_THREADS) {
    const int c = t / AS_N, b = t % AS_N;
    float v = 0.f;
    if (c < ncd && b < n) {
      if (!S.fail) {
        v = S.E[b * AS_NC + c];
      } else if (b == 3 * S.core[c / 3] + c % 3) {  // fallback: the inverse diagonal
        const int64_t cp = S.cps[b / 3];
        int ix, iy, iz;
        cp_coords(cp, g.nb, ix, iy, iz);
        const double dg = vals[rowptr[3 * cp + b % 3] + 3 * stencil_pos(ix, iy, iz, ix, iy, iz, g.nb) + b % 3];
        v = dg != 0.0 ? (float)(1.0 / dg) : 1.f;
      }
    }
    o[t] = v;
  }
}

// z = restricted additive Schwarz applied to v: a warp per subdomain (grid
// stride), lane c < 3 (cell points) computes the cell's DOF c in FP64 from
// the FP32 rows.
__device__ __forceinline__ void asm_apply(double *__restrict__ z, const double *__restrict__ v,
                                          const float *__restrict__ Z, const CellGeom &g, int64_t ncell)
{
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t cell = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); cell < ncell; cell += nw) {
    int64_t cps[64];
    int core[8], ne, nc;
    asm_points(g, cell, cps, core, ne, nc);
    if (lane < 3 * nc) {
      const float *row = Z + (size_t)cell * AS_NC * AS_N + (size_t)lane * AS_N;
      double s = 0.0;
      for (int b = 0; b < 3 * ne; b++) s = fma((double)row[b], v[3 * cps[b / 3] + b % 3], s);
      z[3 * cps[core[lane / 3]] + lane % 3] = s;
    }
  }
}

inline size_t asm_smem_bytes() { return sizeof(AsmSmem); }

}  // namespace igap
