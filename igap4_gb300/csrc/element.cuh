// Per-element data and the per-quadrature-point set-up (phase A) shared by
// the FP64 element kernel and the tensor-core split-precision kernel.
// Mesh, tables, geometry cache, state and law constants are read-only during
// an assembly and are loaded through the read-only path (__ldg), also in the
// batched kernels whose queue atomics would otherwise hide that from the
// compiler.
#pragma once
#include "common.cuh"
#include "laws.cuh"

namespace igap {

constexpr int PW = 8;  // points per chunk (one warp each)
constexpr int GEO_STRIDE = NB * NDD + 2;  // cached R (270), weight, pad

// Element data in shared memory: weights, control points, state levels.
struct ElemData {
  double XV[NB * 3];
  double wV[NB];
  double U[3 * NE];  // [nhist][27][3]
};

// Per-warp scratch of one point.
struct PointScratch {
  double W[NDD];
  double Xg[3 * NDD];
  double u[90];
  double wt;  // quadrature weight x |span| x detG of the point
};

template <int LAWK>
struct LawSmem {
  LawScratch<1> s[1];
};
template <>
struct LawSmem<1> {
  LawScratch<1> s[PW];
};
template <>
struct LawSmem<2> {
  LawScratch<4> s[PW];
};

// One entry of a 1-D basis table at knot coordinate x of the span whose
// local knots are kv[0..2P+1] (Cox-de Boor with derivatives, every knot-span
// denominator shifted by mt; the 1-D factor of eval_Bspline,
// src/meshcore_iga.c:243-310): o[0..2] N, o[3..5] dN, o[6..8] ddN of the
// span's three functions, o[9] = x, o[10] = the span length.
__device__ inline void basis_1d(const double *kv, double x, double mt, double *o)
{
  double lev[P + 1][2 * P + 1], dlev[P + 1][2 * P + 1];
  for (int i = 0; i < 2 * P + 1; i++) { lev[0][i] = 0.0; dlev[0][i] = 0.0; }
  lev[0][P] = 1.0;
  for (int q = 1; q <= P; q++)
    for (int i = 0; i < 2 * P + 1 - q; i++) {
      double dl = kv[i + q] - kv[i] + mt, dr = kv[i + q + 1] - kv[i + 1] + mt;
      double a = (dl != 0.0) ? (x - kv[i]) / dl * lev[q - 1][i] : 0.0;
      double b = (dr != 0.0) ? (kv[i + q + 1] - x) / dr * lev[q - 1][i + 1] : 0.0;
      lev[q][i] = a + b;
      double da = (dl != 0.0) ? (double)q / dl * lev[q - 1][i] : 0.0;
      double db = (dr != 0.0) ? (double)q / dr * lev[q - 1][i + 1] : 0.0;
      dlev[q][i] = da - db;
    }
  for (int i = 0; i <= P; i++) {
    o[i] = lev[P][i];
    o[P1 + i] = dlev[P][i];
    double dl = kv[i + P] - kv[i] + mt, dr = kv[i + P + 1] - kv[i + 1] + mt;
    double a = (dl != 0.0) ? (double)P / dl * dlev[P - 1][i] : 0.0;
    double b = (dr != 0.0) ? (double)P / dr * dlev[P - 1][i + 1] : 0.0;
    o[2 * P1 + i] = a - b;
  }
  o[3 * P1] = x;
  o[3 * P1 + 1] = kv[P + 1] - kv[P];
}

__device__ __forceinline__ void load_element(ElemData &E, const DevMesh &m, int nh,
                                             const double *__restrict__ Uhist, int ex, int ey,
                                             int ez, int tid, int nthreads)
{
  const int nb1 = m.nbasis[1], nb2 = m.nbasis[2];
  for (int t = tid; t < NB; t += nthreads) {
    const int i = t / 9, j = (t / 3) % 3, l = t % 3;
    const int64_t cp = ((int64_t)(ex + i) * nb1 + (ey + j)) * nb2 + (ez + l);
    E.wV[t] = __ldg(m.w + cp);
    for (int d = 0; d < 3; d++) E.XV[3 * t + d] = __ldg(m.X + 3 * cp + d);
    for (int h = 0; h < nh; h++)
      for (int d = 0; d < 3; d++)
        E.U[h * NE + 3 * t + d] = __ldg(Uhist + (int64_t)h * m.ndof + m.dof_off + 3 * cp + d);
  }
}

__device__ __forceinline__ void cp_coords(int64_t cp, const int nb[3], int &ix, int &iy, int &iz)
{
  iz = (int)(cp % nb[2]);
  int64_t t = cp / nb[2];
  iy = (int)(t % nb[1]);
  ix = (int)(t / nb[1]);
}

// Position of column control point (jx,jy,jz) in the row of (ix,iy,iz).
__device__ __forceinline__ int64_t stencil_pos(int ix, int iy, int iz, int jx, int jy, int jz,
                                               const int nb[3])
{
  int lox = max(ix - P, 0), loy = max(iy - P, 0), loz = max(iz - P, 0);
  int cy = min(iy + P, nb[1] - 1) - loy + 1;
  int cz = min(iz + P, nb[2] - 1) - loz + 1;
  return ((int64_t)(jx - lox) * cy + (jy - loy)) * cz + (jz - loz);
}

// Phase A for one point, executed by one warp.
// Geometry of one quadrature point q (< npts) of element (ex,ey,ez), by one
// warp: physical basis R[27*10] (value, gradient, Hessian of every rational
// basis function) and the returned quadrature weight w_q * |span| * detG.
__device__ inline double point_geometry(const ElemData &E, PointScratch &P, const DevMesh &m, int ex,
                                        int ey, int ez, int q, int lane, double *R)
{
  const int nq = m.nquad;
  const int qx = q / (nq * nq), qy = (q / nq) % nq, qz = q % nq;
  const double *tx = m.tab[0] + ((size_t)ex * nq + qx) * TAB;
  const double *ty = m.tab[1] + ((size_t)ey * nq + qy) * TAB;
  const double *tz = m.tab[2] + ((size_t)ez * nq + qz) * TAB;
  // (a) tensor-product basis, src/meshcore_iga.c:311-326
  if (lane < NB) {
    const int i = lane / 9, j = (lane / 3) % 3, l = lane % 3;
    const double nx = __ldg(tx + i), dx = __ldg(tx + P1 + i), ddx = __ldg(tx + 2 * P1 + i);
    const double ny = __ldg(ty + j), dy = __ldg(ty + P1 + j), ddy = __ldg(ty + 2 * P1 + j);
    const double nz = __ldg(tz + l), dz = __ldg(tz + P1 + l), ddz = __ldg(tz + 2 * P1 + l);
    double *o = R + NDD * lane;
    o[0] = nx * ny * nz;
    o[1] = dx * ny * nz;
    o[2] = nx * dy * nz;
    o[3] = nx * ny * dz;
    o[4] = ddx * ny * nz;
    o[5] = dx * dy * nz;
    o[6] = dx * ny * dz;
    o[7] = nx * ddy * nz;
    o[8] = nx * dy * dz;
    o[9] = nx * ny * ddz;
  }
  __syncwarp();
  // (b) weight function W and its derivatives
  if (lane < NDD) {
    double s = 0.0;
    for (int b = 0; b < NB; b++) s += E.wV[b] * R[NDD * b + lane];
    P.W[lane] = s;
  }
  __syncwarp();
  // (c) rational basis by the quotient rule, src/assmcore_iga.c:155-165
  if (lane < NB) {
    double *r = R + NDD * lane;
    const double *W = P.W;
    const double wb = E.wV[lane];
    for (int k = 0; k < NDD; k++) r[k] = r[k] * wb / W[0];
    for (int k = 1; k < NDD; k++) r[k] -= r[0] * W[k] / W[0];
    int a = 4;
    for (int i = 1; i < 4; i++)
      for (int j = i; j < 4; j++) { r[a] -= (r[j] * W[i] + r[i] * W[j]) / W[0]; a++; }
  }
  __syncwarp();
  // (d) geometry X and its derivatives, src/assmcore_iga.c:166-174
  if (lane < 30) {
    const int d = lane / NDD, k = lane % NDD;
    double s = 0.0;
    for (int b = 0; b < NB; b++) s += E.XV[3 * b + d] * R[NDD * b + k];
    P.Xg[lane] = s;
  }
  __syncwarp();
  // (e) Jacobian, its determinant and inverse
  const double *Xg = P.Xg;
  double G[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) G[3 * i + j] = Xg[NDD * i + 1 + j];
  const double detG = G[0] * (G[4] * G[8] - G[5] * G[7]) - G[1] * (G[3] * G[8] - G[5] * G[6]) +
                      G[2] * (G[3] * G[7] - G[4] * G[6]);
  double Gi[9];
  {
    double c0 = G[4] * G[8] - G[5] * G[7], c1 = G[2] * G[7] - G[1] * G[8], c2 = G[1] * G[5] - G[2] * G[4];
    double c3 = G[5] * G[6] - G[3] * G[8], c4 = G[0] * G[8] - G[2] * G[6], c5 = G[2] * G[3] - G[0] * G[5];
    double c6 = G[3] * G[7] - G[4] * G[6], c7 = G[1] * G[6] - G[0] * G[7], c8 = G[0] * G[4] - G[1] * G[3];
    double id = 1.0 / (G[0] * c0 + G[1] * c3 + G[2] * c6);
    Gi[0] = c0 * id; Gi[1] = c1 * id; Gi[2] = c2 * id;
    Gi[3] = c3 * id; Gi[4] = c4 * id; Gi[5] = c5 * id;
    Gi[6] = c6 * id; Gi[7] = c7 * id; Gi[8] = c8 * id;
  }
  // (f) physical first and second derivatives, src/assmcore_iga.c:179-208
  if (lane < NB) {
    double *r = R + NDD * lane;
    double n[NDD];
    for (int k = 0; k < NDD; k++) n[k] = r[k];
    for (int i = 0; i < 3; i++) {
      double s = 0.0;
      for (int j = 0; j < 3; j++) s += n[1 + j] * Gi[3 * j + i];
      r[1 + i] = s;
    }
    for (int k = 4; k < NDD; k++)
      for (int i = 0; i < 3; i++) n[k] -= r[1 + i] * Xg[NDD * i + k];
    const double Hs[3][3] = {{n[4], n[5], n[6]}, {n[5], n[7], n[8]}, {n[6], n[8], n[9]}};
    int a = 4;
    for (int i = 0; i < 3; i++)
      for (int j = i; j < 3; j++) {
        double s = 0.0;
        for (int mm = 0; mm < 3; mm++) {
          double t = 0.0;
          for (int l = 0; l < 3; l++) t += Hs[mm][l] * Gi[3 * l + j];
          s += Gi[3 * mm + i] * t;
        }
        r[a++] = s;
      }
  }
  __syncwarp();
  return __ldg(m.wq + qx) * __ldg(m.wq + qy) * __ldg(m.wq + qz) * __ldg(tx + 3 * P1 + 1) * __ldg(ty + 3 * P1 + 1) *
         __ldg(tz + 3 * P1 + 1) * detG;
}

// Outputs: R[27*10] physical basis, rr[30] weighted residual integrand,
// D[900] weighted tangent integrand (DT = double, or float for the split mode).
// With a geometry cache (m.geo) R and the weight are read, not recomputed.
// fill_D = false (constant-tangent law only): D is not written; the caller
// contracts with the sparse constant tangent and the weight P.wt.
template <int LAWK, bool RES, bool TAN, typename DT>
__device__ void point_setup(const ElemData &E, PointScratch &P, LawSmem<LAWK> &LS, const DevMesh &m,
                            const DevLaw &L, int ex, int ey, int ez, int w, int q, int lane,
                            double *R, double *rr, DT *D, bool fill_D = true)
{
  const double *__restrict__ Dconst = L.Dconst;
  if (q >= m.npts) {  // padding point of an incomplete chunk: no contribution
    for (int i = lane; i < NB * NDD; i += 32) R[i] = 0.0;
    if (RES) for (int i = lane; i < 30; i += 32) rr[i] = 0.0;
    if (TAN && fill_D) for (int i = lane; i < 900; i += 32) D[i] = (DT)0;
    if (lane == 0) P.wt = 0.0;
    __syncwarp();
    return;
  }
  double wt;
  if (m.geo) {
    const int64_t e = ((int64_t)ex * m.nelem[1] + ey) * m.nelem[2] + ez;
    const double *g = m.geo + (e * m.npts + q) * GEO_STRIDE;
    for (int i = lane; i < NB * NDD; i += 32) R[i] = __ldg(g + i);
    wt = __ldg(g + NB * NDD);
    __syncwarp();
  } else {
    wt = point_geometry(E, P, m, ex, ey, ez, q, lane, R);
  }
  if (lane == 0) P.wt = wt;
  if constexpr (LAWK != 0) {
    if (L.preR) {  // law outputs of every point computed beforehand (law_points_kernel)
      // point-minor layout [element][entry][point]
      const int64_t e = ((int64_t)ex * m.nelem[1] + ey) * m.nelem[2] + ez;
      if (RES)
        for (int i = lane; i < 30; i += 32) rr[i] = __ldg(L.preR + (e * 30 + i) * m.npts + q);
      if (TAN && fill_D) {
        if (L.preDf)
          for (int i = lane; i < 900; i += 32) D[i] = (DT)__ldg(L.preDf + (e * 900 + i) * m.npts + q);
        else
          for (int i = lane; i < 900; i += 32) D[i] = (DT)__ldg(L.preD + (e * 900 + i) * m.npts + q);
      }
      __syncwarp();
      return;
    }
  }
  // (g) interpolated state of every history level, src/assmcore_iga.c:209-229
  const int nh = L.nhist;
  constexpr bool NEED_U = RES || LAWK != 0;
  // the linear law's tangent has no value column: its value slots (k = 0) are
  // set to zero instead of interpolated
  if (LAWK == 0 && NEED_U && lane < 30 && lane % NDD == 0)
    for (int h = 0; h < L.nhist; h++) P.u[30 * h + lane] = 0.0;
  if (NEED_U && lane < 30 && (LAWK != 0 || lane % NDD != 0)) {
    const int d = lane / NDD, k = lane % NDD;
    for (int h = 0; h < nh; h++) {
      double s = 0.0;
      for (int b = 0; b < NB; b++) s += R[NDD * b + k] * E.U[h * NE + 3 * b + d];
      P.u[30 * h + lane] = s;
    }
  }
  __syncwarp();
  // (h) law
  if constexpr (LAWK == 0) {
    const double *u = P.u;
    if (RES && lane < 30) {
      double s = 0.0;
      if (L.dptr) {  // sparse constant tangent
        const int j1 = __ldg(L.dptr + lane + 1);
        for (int j = __ldg(L.dptr + lane); j < j1; j++) s += __ldg(L.dval + j) * u[__ldg(L.dcol + j)];
      } else {
        for (int j = 0; j < 30; j++) s += __ldg(Dconst + 30 * lane + j) * u[j];
      }
      rr[lane] = wt * s;
    }
    if (TAN && fill_D)
      for (int i = lane; i < 900; i += 32) D[i] = (DT)(wt * __ldg(Dconst + i));
    __syncwarp();
  } else if constexpr (LAWK == 1) {
    gradelast_warp<1, RES, TAN, DT>(P.u, L.par, false, wt, rr, D, LS.s[w], lane);
  } else {
    gradelast_warp<4, RES, TAN, DT>(P.u, L.par, true, wt, rr, D, LS.s[w], lane);
  }
}


}  // namespace igap
