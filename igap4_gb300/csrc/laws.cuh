// Device constitutive laws, evaluated by one warp per quadrature point.
//
// Per-point ABI of the reference (include/physimpl.h:6-7): u[10 d + k] with
// k = 0 value, 1..3 first, 4..9 second derivatives (xx,xy,xz,yy,yz,zz) of
// displacement component d; rr[10 d + k] = dpsi/du[10 d + k];
// D[30 row + col] = d rr[row] / d u[col] (current level only).
//
// gradelast (phys/gradelast.c) and gradelasttime (phys/gradelasttime.c) are
// evaluated from the stored energy through 15 strain measures
//   q = (E00,E11,E22,E01,E02,E12, E_aa,m  a,m = 0..2),
// each quadratic in u, with sparse gradients (<= 6 entries each):
//   rr = sum_c psi_c grad q_c,
//   D  = sum_cd psi_cd grad q_c grad q_d^T + sum_c psi_c hess q_c.
// The transient law is the average-vector-field force along the segment
// m + s delta, m = (u_n + u_{n-1})/2, delta = (u - u_{n-1})/2, truncated at
// third order in delta:  rr = sum_k r_k/(k+1),  D = 1/2 sum_k T_k/(k+2),
// r_k / T_k the s^k Taylor coefficients of the static residual / tangent on
// the segment.  Every s-polynomial is carried as a truncated Taylor jet.
//
// lingrad (no reference counterpart): psi = lam/2 tr(eps)^2 + mu eps:eps
//   + ell^2 (lam/2 |grad tr eps|^2 + mu |grad eps|^2); its constant tangent is
// built once on the device (lingrad_dconst_kernel) and rr = D u.
#pragma once
#include "common.cuh"

namespace igap {

// Truncated power series (s-jets) c[0] + c[1] s + ... in the scalar type T.
template <int N, typename T = double>
struct Jet {
  T c[N];
};
template <int N, typename T = double>
__device__ __forceinline__ Jet<N, T> jzero()
{
  Jet<N, T> r;
#pragma unroll
  for (int i = 0; i < N; i++) r.c[i] = T(0);
  return r;
}
template <int N, typename T = double, typename S>
__device__ __forceinline__ Jet<N, T> jconst(S a)
{
  Jet<N, T> r = jzero<N, T>();
  r.c[0] = T(a);
  return r;
}
template <int N, typename T>
__device__ __forceinline__ Jet<N, T> jadd(const Jet<N, T> &a, const Jet<N, T> &b)
{
  Jet<N, T> r;
#pragma unroll
  for (int i = 0; i < N; i++) r.c[i] = a.c[i] + b.c[i];
  return r;
}
template <int N, typename T, typename S>
__device__ __forceinline__ Jet<N, T> jscale(const Jet<N, T> &a, S s)
{
  Jet<N, T> r;
  const T st = T(s);
#pragma unroll
  for (int i = 0; i < N; i++) r.c[i] = a.c[i] * st;
  return r;
}
template <int N, typename T>
__device__ __forceinline__ Jet<N, T> jmul(const Jet<N, T> &a, const Jet<N, T> &b)
{
  Jet<N, T> r;
#pragma unroll
  for (int i = 0; i < N; i++) {
    T s = T(0);
#pragma unroll
    for (int j = 0; j <= i; j++) s = fma(a.c[j], b.c[i - j], s);
    r.c[i] = s;
  }
  return r;
}

__device__ __forceinline__ int sym6(int j, int m)
{
  int lo = j < m ? j : m, hi = j < m ? m : j;
  return lo == 0 ? hi : (lo == 1 ? 2 + hi : 5);
}

constexpr int NQM = 15;  // strain measures
constexpr int NQE = 6;   // max gradient entries per measure

// Per-warp scratch of the energy-based laws (shared memory).
template <int NJ>
struct LawScratch {
  double F[9], H[27], dF[9], dH[27];
  double m[30], delta[30];
  int idx[NQM][NQE];
  int cnt[NQM];
  double g0[NQM][NQE], g1[NQM][NQE];
  Jet<NJ> q[NQM];
  Jet<NJ> d1[NQM];
  Jet<NJ> d2b[3][3];  // block of (E00,E11,E22)
  double cs2, grad2[3][3];
};

__device__ __forceinline__ void landau(const double *par, double &A, double &B, double &C)
{
  double r = par[0], cv = par[1];
  double den = r * r - 2.0 * r * r * cv - r * (4.0 / 3.0 * r - 4.0 / 3.0 * r * cv);
  B = -(4.0 / 3.0 * r - 4.0 / 3.0 * r * cv) / (r * r * den);
  A = 2.0 * cv / den;
  C = -1.0 / (r * r * den);
}

// Finite-strain gradient elasticity, NJ = 1 (static point) or 4 (transient
// segment jets).  u: nhist*30 (smem), rr/D outputs scaled by wt.
template <int NJ, bool RES, bool TAN, typename DT = double>
__device__ void gradelast_warp(const double *u, const double *par, bool transient, double wt,
                               double *rr, DT *D, LawScratch<NJ> &S, int lane)
{
  // segment: static -> m = u, delta = 0
  if (lane < 30) {
    if (transient) {
      S.m[lane] = 0.5 * (u[30 + lane] + u[60 + lane]);
      S.delta[lane] = 0.5 * (u[lane] - u[60 + lane]);
    } else {
      S.m[lane] = u[lane];
      S.delta[lane] = 0.0;
    }
  }
  __syncwarp();
  if (lane < 9) {
    int i = lane / 3, j = lane % 3;
    S.F[lane] = (i == j ? 1.0 : 0.0) + S.m[10 * i + 1 + j];
    S.dF[lane] = S.delta[10 * i + 1 + j];
    for (int mm = 0; mm < 3; mm++) {
      S.H[9 * i + 3 * j + mm] = S.m[10 * i + 4 + sym6(j, mm)];
      S.dH[9 * i + 3 * j + mm] = S.delta[10 * i + 4 + sym6(j, mm)];
    }
  }
  __syncwarp();
  // measures and their sparse gradients: lane c
  if (lane < NQM) {
    const int c = lane;
    double q0 = 0.0, q2 = 0.0;
    int n = 0;
    if (c < 6) {
      const int PA[6] = {0, 1, 2, 0, 0, 1}, PB[6] = {0, 1, 2, 1, 2, 2};
      int a = PA[c], b = PB[c];
      for (int k = 0; k < 3; k++) {
        q0 += S.F[3 * k + a] * S.F[3 * k + b];
        q2 += S.dF[3 * k + a] * S.dF[3 * k + b];
      }
      q0 = 0.5 * (q0 - (a == b ? 1.0 : 0.0));
      q2 = 0.5 * q2;
      for (int k = 0; k < 3; k++) {
        if (a == b) {
          S.idx[c][n] = 10 * k + 1 + a; S.g0[c][n] = S.F[3 * k + a]; S.g1[c][n] = S.dF[3 * k + a]; n++;
        } else {
          S.idx[c][n] = 10 * k + 1 + a; S.g0[c][n] = 0.5 * S.F[3 * k + b]; S.g1[c][n] = 0.5 * S.dF[3 * k + b]; n++;
          S.idx[c][n] = 10 * k + 1 + b; S.g0[c][n] = 0.5 * S.F[3 * k + a]; S.g1[c][n] = 0.5 * S.dF[3 * k + a]; n++;
        }
      }
    } else {
      int a = (c - 6) / 3, mm = (c - 6) % 3;
      for (int k = 0; k < 3; k++) {
        q0 += S.F[3 * k + a] * S.H[9 * k + 3 * a + mm];
        q2 += S.dF[3 * k + a] * S.dH[9 * k + 3 * a + mm];
        S.idx[c][n] = 10 * k + 1 + a; S.g0[c][n] = S.H[9 * k + 3 * a + mm]; S.g1[c][n] = S.dH[9 * k + 3 * a + mm]; n++;
        S.idx[c][n] = 10 * k + 4 + sym6(a, mm); S.g0[c][n] = S.F[3 * k + a]; S.g1[c][n] = S.dF[3 * k + a]; n++;
      }
    }
    S.cnt[c] = n;
    double q1 = 0.0;
    for (int e = 0; e < n; e++) q1 += S.g0[c][e] * S.delta[S.idx[c][e]];
    Jet<NJ> qj = jconst<NJ>(q0);
    if constexpr (NJ > 1) qj.c[1] = q1;
    if constexpr (NJ > 2) qj.c[2] = q2;
    S.q[c] = qj;
  }
  __syncwarp();
  // energy derivatives: lane 0
  if (lane == 0) {
    const double s2 = sqrt(2.0), s3 = sqrt(3.0), s6 = sqrt(6.0);
    double A, B, C;
    landau(par, A, B, C);
    double cvol = par[2], cs = par[3], l2 = par[4] * par[4];
    const double Lv[3] = {1 / s3, 1 / s3, 1 / s3};
    const double L1[3] = {1 / s2, -1 / s2, 0.0};
    const double L2[3] = {1 / s6, 1 / s6, -2 / s6};
    Jet<NJ> ev = jzero<NJ>(), e1 = jzero<NJ>(), e2 = jzero<NJ>();
    for (int i = 0; i < 3; i++) {
      ev = jadd(ev, jscale(S.q[i], Lv[i]));
      e1 = jadd(e1, jscale(S.q[i], L1[i]));
      e2 = jadd(e2, jscale(S.q[i], L2[i]));
    }
    Jet<NJ> e11 = jmul(e1, e1), e22 = jmul(e2, e2), e12 = jmul(e1, e2);
    Jet<NJ> rho = jadd(e11, e22);
    Jet<NJ> p_v = jscale(ev, 2.0 * cvol);
    Jet<NJ> p_1 = jadd(jadd(jscale(e1, 2.0 * A), jscale(e12, -6.0 * B)), jscale(jmul(e1, rho), 4.0 * C));
    Jet<NJ> p_2 = jadd(jadd(jscale(e2, 2.0 * A), jscale(jadd(e22, jscale(e11, -1.0)), 3.0 * B)),
                       jscale(jmul(e2, rho), 4.0 * C));
    Jet<NJ> p_11 = jadd(jadd(jconst<NJ>(2.0 * A), jscale(e2, -6.0 * B)),
                        jadd(jscale(rho, 4.0 * C), jscale(e11, 8.0 * C)));
    Jet<NJ> p_12 = jadd(jscale(e1, -6.0 * B), jscale(e12, 8.0 * C));
    Jet<NJ> p_22 = jadd(jadd(jconst<NJ>(2.0 * A), jscale(e2, 6.0 * B)),
                        jadd(jscale(rho, 4.0 * C), jscale(e22, 8.0 * C)));
    for (int i = 0; i < 3; i++) {
      S.d1[i] = jadd(jadd(jscale(p_v, Lv[i]), jscale(p_1, L1[i])), jscale(p_2, L2[i]));
      for (int j = 0; j < 3; j++)
        S.d2b[i][j] = jadd(jadd(jconst<NJ>(2.0 * cvol * Lv[i] * Lv[j]), jscale(p_11, L1[i] * L1[j])),
                           jadd(jscale(p_12, L1[i] * L2[j] + L2[i] * L1[j]), jscale(p_22, L2[i] * L2[j])));
    }
    for (int c = 3; c < 6; c++) S.d1[c] = jscale(S.q[c], 2.0 * cs);
    S.cs2 = 2.0 * cs;
    for (int mm = 0; mm < 3; mm++) {
      Jet<NJ> g1 = jzero<NJ>(), g2 = jzero<NJ>();
      for (int a = 0; a < 3; a++) {
        g1 = jadd(g1, jscale(S.q[6 + 3 * a + mm], L1[a]));
        g2 = jadd(g2, jscale(S.q[6 + 3 * a + mm], L2[a]));
      }
      for (int a = 0; a < 3; a++)
        S.d1[6 + 3 * a + mm] = jscale(jadd(jscale(g1, L1[a]), jscale(g2, L2[a])), 2.0 * l2);
    }
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) S.grad2[a][b] = 2.0 * l2 * (L1[a] * L1[b] + L2[a] * L2[b]);
  }
  __syncwarp();
  const double rho_m = par[5], damp = par[6], dt = par[7];
  // residual: lane i
  if (RES && lane < 30) {
    const int i = lane;
    Jet<NJ> r = jzero<NJ>();
    for (int c = 0; c < NQM; c++)
      for (int e = 0; e < S.cnt[c]; e++)
        if (S.idx[c][e] == i) {
          Jet<NJ> g = jconst<NJ>(S.g0[c][e]);
          if constexpr (NJ > 1) g.c[1] = S.g1[c][e];
          r = jadd(r, jmul(S.d1[c], g));
        }
    double v = r.c[0];
    if constexpr (NJ > 3) v = r.c[0] + r.c[1] / 2.0 + r.c[2] / 3.0 + r.c[3] / 4.0;
    if (transient && (i % 10) == 0)
      v += damp * (u[i] - u[60 + i]) / (2.0 * dt) + rho_m * (u[i] + u[60 + i] - 2.0 * u[30 + i]) / (dt * dt);
    rr[i] = wt * v;
  }
  // tangent rows: lane i owns row i of D
  if (TAN && lane < 30) {
    const int i = lane;
    DT *row = D + 30 * i;
    for (int j = 0; j < 30; j++) row[j] = (DT)0;
    // collapse of an s-jet of the static tangent to the discrete-gradient Jacobian
    auto collapse = [&](const Jet<NJ> &t) -> double {
      if constexpr (NJ == 1) return t.c[0];
      else return 0.5 * (t.c[0] / 2.0 + t.c[1] / 3.0 + t.c[2] / 4.0);
    };
    for (int c = 0; c < NQM; c++)
      for (int e = 0; e < S.cnt[c]; e++) {
        if (S.idx[c][e] != i) continue;
        Jet<NJ> gci = jconst<NJ>(S.g0[c][e]);
        if constexpr (NJ > 1) gci.c[1] = S.g1[c][e];
        // psi_cd grad q_c[i] grad q_d
        int dlist[3];
        Jet<NJ> dcoef[3];
        int nd = 0;
        if (c < 3) {
          for (int d = 0; d < 3; d++) { dlist[nd] = d; dcoef[nd] = jmul(gci, S.d2b[c][d]); nd++; }
        } else if (c < 6) {
          dlist[0] = c; dcoef[0] = jscale(gci, S.cs2); nd = 1;
        } else {
          int a = (c - 6) / 3, mm = (c - 6) % 3;
          for (int b = 0; b < 3; b++) { dlist[nd] = 6 + 3 * b + mm; dcoef[nd] = jscale(gci, S.grad2[a][b]); nd++; }
        }
        for (int t = 0; t < nd; t++) {
          int d = dlist[t];
          for (int e2 = 0; e2 < S.cnt[d]; e2++) {
            Jet<NJ> gd = jconst<NJ>(S.g0[d][e2]);
            if constexpr (NJ > 1) gd.c[1] = S.g1[d][e2];
            row[S.idx[d][e2]] += (DT)collapse(jmul(dcoef[t], gd));
          }
        }
      }
    // psi_c hess q_c (constant Hessians of the measures)
    for (int c = 0; c < 6; c++) {
      const int PA[6] = {0, 1, 2, 0, 0, 1}, PB[6] = {0, 1, 2, 1, 2, 2};
      int a = PA[c], b = PB[c];
      if (i % 10 == 0 || i % 10 > 3) continue;
      int k = i / 10, col = i % 10 - 1;
      double h = collapse(S.d1[c]);
      if (col == a) row[10 * k + 1 + b] += (DT)(0.5 * h);
      if (col == b) row[10 * k + 1 + a] += (DT)(0.5 * h);
    }
    for (int c = 6; c < NQM; c++) {
      int a = (c - 6) / 3, mm = (c - 6) % 3;
      double h = collapse(S.d1[c]);
      int k = i / 10, r10 = i % 10;
      if (r10 == 1 + a) row[10 * k + 4 + sym6(a, mm)] += (DT)h;
      if (r10 == 4 + sym6(a, mm)) row[10 * k + 1 + a] += (DT)h;
    }
    if (transient && (i % 10) == 0) row[i] += (DT)(damp / (2.0 * dt) + rho_m / (dt * dt));
    for (int j = 0; j < 30; j++) row[j] = (DT)(row[j] * wt);
  }
  __syncwarp();
}

// Linear law residual at one state (device restatement of the project law;
// used to build its constant tangent column by column).
__device__ inline void lingrad_residual_dev(const double *u, const double *par, double *rr)
{
  const double lam = par[0], mu = par[1], ell = par[2];
  double g[3][3], h[3][3][3];
  for (int i = 0; i < 3; i++) {
    for (int j = 0; j < 3; j++) g[i][j] = u[10 * i + 1 + j];
    for (int j = 0; j < 3; j++)
      for (int m = 0; m < 3; m++) h[i][j][m] = u[10 * i + 4 + sym6(j, m)];
  }
  double eps[3][3], kap[3][3][3], tr = 0.0, trk[3] = {0, 0, 0};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      eps[i][j] = 0.5 * (g[i][j] + g[j][i]);
      for (int m = 0; m < 3; m++) kap[i][j][m] = 0.5 * (h[i][j][m] + h[j][i][m]);
    }
  for (int i = 0; i < 3; i++) {
    tr += eps[i][i];
    for (int m = 0; m < 3; m++) trk[m] += kap[i][i][m];
  }
  for (int d = 0; d < 3; d++) {
    rr[10 * d] = 0.0;
    for (int j = 0; j < 3; j++) rr[10 * d + 1 + j] = 2.0 * mu * eps[d][j] + (d == j ? lam * tr : 0.0);
    const int SJ[6] = {0, 0, 0, 1, 1, 2}, SM[6] = {0, 1, 2, 1, 2, 2};
    for (int s = 0; s < 6; s++) {
      int j = SJ[s], m = SM[s];
      double t1 = ell * ell * (2.0 * mu * kap[d][j][m] + (d == j ? lam * trk[m] : 0.0));
      double t2 = ell * ell * (2.0 * mu * kap[d][m][j] + (d == m ? lam * trk[j] : 0.0));
      rr[10 * d + 4 + s] = (j == m) ? t1 : t1 + t2;
    }
  }
}

}  // namespace igap
