// The gradient laws gradelast (phys/gradelast.c:7-1023) and gradelasttime
// (phys/gradelasttime.c:7-9181) at one quadrature point per thread.
//
// Same energy and the same strain-measure restatement as gradelast_warp
// (laws.cuh): 15 measures q_c, quadratic in the point state, whose gradients
// g_c = dq_c/du have a fixed sparsity (<= 6 slots each).  Here every index of
// that sparsity is a compile-time constant, so a thread evaluates its point's
// law with no divergence and no per-slot searching:
//
//   rr[i]   = sum_{c : i in g_c} collapse_R(d1_c * g_c[i])
//   D[i][j] = sum_{c,d} collapse_T(psi_cd * g_c[i] * g_d[j])
//             + sum_c collapse_T(d1_c) hess(q_c)[i][j]  (+ inertia, damping)
//
// On the transient segment every g_c[i] is linear in s (g0 + g1 s) and
// collapse_T is linear with weights w = (1/4, 1/6, 1/8) on the s^0..s^2
// coefficients, so a coupling jet x = psi_cd contributes
//   collapse_T(x g_ci g_dj) = (X0 a_i + X1 b_i) a_j + (X1 a_i + X2 b_i) b_j,
//   X0 = w0 x0 + w1 x1 + w2 x2,  X1 = w1 x0 + w2 x1,  X2 = w2 x0,
// (a, b) = (g0, g1); the static law is the case w = (1, 0, 0), b = 0.
// Terms of degree >= 3 in s never reach the collapse, so the truncation of the
// s-jets at degree 3 is the one gradelast_warp makes.
//
// Inputs per point (shared memory, column t, leading dimension ld):
//   sm[slot]  m at the gradient and Hessian slots (m = u for the static law,
//             (u_n + u_{n-1})/2 for the transient one); at the value slots of
//             the transient law the inertia + damping residual term;
//   sd[slot]  delta = (u - u_{n-1})/2 (transient law only).
// Outputs: rr[30] and D[900] (row-major, row = test slot) scaled by wt,
// written to out_r[i * ostride] and out_d[(30 i + j) * ostride].
#pragma once
#include "laws.cuh"

namespace igap {

namespace lawpt {

__device__ __forceinline__ constexpr int slot(int k, int f) { return 10 * k + f; }
__device__ __forceinline__ constexpr int symi(int j, int m)
{
  return (j < m ? j : m) == 0 ? (j < m ? m : j) : ((j < m ? j : m) == 1 ? 2 + (j < m ? m : j) : 5);
}
// the shear measure of the pair (a, b), a != b: c = 3, 4, 5 for (0,1), (0,2), (1,2)
__device__ __forceinline__ constexpr int shear(int a, int b)
{
  return (a + b == 1) ? 3 : ((a + b == 2) ? 4 : 5);
}

}  // namespace lawpt

template <int NJ, bool RES, bool TAN>
__device__ __forceinline__ void gradelast_point(const double *__restrict__ sm, const double *__restrict__ sd,
                                                int ld, const double *par, double wt,
                                                double *__restrict__ out_r, double *__restrict__ out_d,
                                                int64_t ostride)
{
  using namespace lawpt;
  constexpr bool TR = NJ > 1;
#define LP_F(k, a) (((k) == (a) ? 1.0 : 0.0) + sm[slot(k, 1 + (a)) * ld])
#define LP_DF(k, a) (TR ? sd[slot(k, 1 + (a)) * ld] : 0.0)
#define LP_H(k, s) (sm[slot(k, 4 + (s)) * ld])
#define LP_DH(k, s) (TR ? sd[slot(k, 4 + (s)) * ld] : 0.0)
  const double s2 = sqrt(2.0), s3 = sqrt(3.0), s6 = sqrt(6.0);
  const double Lv[3] = {1 / s3, 1 / s3, 1 / s3};
  const double L1[3] = {1 / s2, -1 / s2, 0.0};
  const double L2[3] = {1 / s6, 1 / s6, -2 / s6};
  double A, B, C;
  landau(par, A, B, C);
  const double cvol = par[2], cs = par[3], l2 = par[4] * par[4];
  // ---- measures (s-jets q0 + q1 s + q2 s^2) and the energy derivatives
  Jet<NJ> qn[3], qs[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    double q0 = 0.0, q1 = 0.0, q2 = 0.0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      q0 += LP_F(k, a) * LP_F(k, a);
      q2 += LP_DF(k, a) * LP_DF(k, a);
      q1 += LP_F(k, a) * LP_DF(k, a);
    }
    qn[a] = jconst<NJ>(0.5 * (q0 - 1.0));
    if constexpr (NJ > 1) qn[a].c[1] = q1;
    if constexpr (NJ > 2) qn[a].c[2] = 0.5 * q2;
  }
#pragma unroll
  for (int c = 3; c < 6; c++) {
    const int a = c == 5 ? 1 : 0, b = c == 3 ? 1 : 2;
    double q0 = 0.0, q1 = 0.0, q2 = 0.0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      q0 += LP_F(k, a) * LP_F(k, b);
      q2 += LP_DF(k, a) * LP_DF(k, b);
      q1 += 0.5 * LP_F(k, b) * LP_DF(k, a);
      q1 += 0.5 * LP_F(k, a) * LP_DF(k, b);
    }
    qs[c - 3] = jconst<NJ>(0.5 * q0);
    if constexpr (NJ > 1) qs[c - 3].c[1] = q1;
    if constexpr (NJ > 2) qs[c - 3].c[2] = 0.5 * q2;
  }
  // gradient measures only enter through G1[mm] = sum_a L1[a] q_(a,mm), G2 likewise
  Jet<NJ> G1[3], G2[3];
#pragma unroll
  for (int mm = 0; mm < 3; mm++) {
    G1[mm] = jzero<NJ>();
    G2[mm] = jzero<NJ>();
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const int s = symi(a, mm);
      double q0 = 0.0, q1 = 0.0, q2 = 0.0;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        q0 += LP_F(k, a) * LP_H(k, s);
        q2 += LP_DF(k, a) * LP_DH(k, s);
        q1 += LP_H(k, s) * LP_DF(k, a);
        q1 += LP_F(k, a) * LP_DH(k, s);
      }
      Jet<NJ> q = jconst<NJ>(q0);
      if constexpr (NJ > 1) q.c[1] = q1;
      if constexpr (NJ > 2) q.c[2] = q2;
      G1[mm] = jadd(G1[mm], jscale(q, L1[a]));
      G2[mm] = jadd(G2[mm], jscale(q, L2[a]));
    }
  }
  Jet<NJ> ev = jzero<NJ>(), e1 = jzero<NJ>(), e2 = jzero<NJ>();
#pragma unroll
  for (int i = 0; i < 3; i++) {
    ev = jadd(ev, jscale(qn[i], Lv[i]));
    e1 = jadd(e1, jscale(qn[i], L1[i]));
    e2 = jadd(e2, jscale(qn[i], L2[i]));
  }
  const Jet<NJ> e11 = jmul(e1, e1), e22 = jmul(e2, e2), e12 = jmul(e1, e2);
  const Jet<NJ> rho = jadd(e11, e22);
  const Jet<NJ> p_v = jscale(ev, 2.0 * cvol);
  const Jet<NJ> p_1 = jadd(jadd(jscale(e1, 2.0 * A), jscale(e12, -6.0 * B)), jscale(jmul(e1, rho), 4.0 * C));
  const Jet<NJ> p_2 = jadd(jadd(jscale(e2, 2.0 * A), jscale(jadd(e22, jscale(e11, -1.0)), 3.0 * B)),
                           jscale(jmul(e2, rho), 4.0 * C));
  // collapse weights: residual (sum_k t_k/(k+1), and the g1 part sum_k t_k/(k+2));
  // tangent (w0, w1, w2)
  auto colR0 = [](const Jet<NJ> &t) -> double {
    if constexpr (NJ == 1) return t.c[0];
    else return t.c[0] + t.c[1] / 2.0 + t.c[2] / 3.0 + t.c[3] / 4.0;
  };
  auto colR1 = [](const Jet<NJ> &t) -> double {
    if constexpr (NJ == 1) return 0.0;
    else return t.c[0] / 2.0 + t.c[1] / 3.0 + t.c[2] / 4.0;
  };
  auto colT = [](const Jet<NJ> &t) -> double {
    if constexpr (NJ == 1) return t.c[0];
    else return 0.5 * (t.c[0] / 2.0 + t.c[1] / 3.0 + t.c[2] / 4.0);
  };
  // d1 of the normal strains
  Jet<NJ> d1n[3];
#pragma unroll
  for (int i = 0; i < 3; i++) d1n[i] = jadd(jadd(jscale(p_v, Lv[i]), jscale(p_1, L1[i])), jscale(p_2, L2[i]));
  // d1 of the gradient measures: 2 l2 (L1[a] G1 + L2[a] G2)
  auto d1g = [&](int a, int mm) -> Jet<NJ> {
    return jscale(jadd(jscale(G1[mm], L1[a]), jscale(G2[mm], L2[a])), 2.0 * l2);
  };
  const double rho_m = par[5], damp = par[6], dt = par[7];
  (void)rho_m; (void)damp; (void)dt;

  if constexpr (RES) {
    double Rn0[3], Rn1[3], Rs0[3], Rs1[3], Rg0[3][3], Rg1[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      Rn0[i] = colR0(d1n[i]); Rn1[i] = colR1(d1n[i]);
      const Jet<NJ> d = jscale(qs[i], 2.0 * cs);
      Rs0[i] = colR0(d); Rs1[i] = colR1(d);
    }
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int mm = 0; mm < 3; mm++) {
        const Jet<NJ> d = d1g(a, mm);
        Rg0[a][mm] = colR0(d); Rg1[a][mm] = colR1(d);
      }
#pragma unroll
    for (int k = 0; k < 3; k++) {
      // value slot: inertia and damping of the transient law
      out_r[slot(k, 0) * ostride] = TR ? wt * sm[slot(k, 0) * ld] : 0.0;
#pragma unroll
      for (int a = 0; a < 3; a++) {
        double v = Rn0[a] * LP_F(k, a) + Rn1[a] * LP_DF(k, a);
#pragma unroll
        for (int b = 0; b < 3; b++) {
          if (b == a) continue;
          const int c = shear(a, b) - 3;
          v += Rs0[c] * (0.5 * LP_F(k, b)) + Rs1[c] * (0.5 * LP_DF(k, b));
        }
#pragma unroll
        for (int mm = 0; mm < 3; mm++) v += Rg0[a][mm] * LP_H(k, symi(a, mm)) + Rg1[a][mm] * LP_DH(k, symi(a, mm));
        out_r[slot(k, 1 + a) * ostride] = wt * v;
      }
#pragma unroll
      for (int s = 0; s < 6; s++) {
        const int j = s < 3 ? 0 : (s < 5 ? 1 : 2);
        const int m = s < 3 ? s : (s < 5 ? s - 2 : 2);
        double v = Rg0[j][m] * LP_F(k, j) + Rg1[j][m] * LP_DF(k, j);
        if (j != m) v += Rg0[m][j] * LP_F(k, m) + Rg1[m][j] * LP_DF(k, m);
        out_r[slot(k, 4 + s) * ostride] = wt * v;
      }
    }
  }

  if constexpr (TAN) {
    const double w0 = TR ? 0.25 : 1.0, w1 = TR ? 1.0 / 6.0 : 0.0, w2 = TR ? 0.125 : 0.0;
    // couplings of the normal strains: d2b[c][d] (symmetric) as (X0, X1, X2)
    const Jet<NJ> p_11 = jadd(jadd(jconst<NJ>(2.0 * A), jscale(e2, -6.0 * B)),
                              jadd(jscale(rho, 4.0 * C), jscale(e11, 8.0 * C)));
    const Jet<NJ> p_12 = jadd(jscale(e1, -6.0 * B), jscale(e12, 8.0 * C));
    const Jet<NJ> p_22 = jadd(jadd(jconst<NJ>(2.0 * A), jscale(e2, 6.0 * B)),
                              jadd(jscale(rho, 4.0 * C), jscale(e22, 8.0 * C)));
    double Xn[3][3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const Jet<NJ> x = jadd(jadd(jconst<NJ>(2.0 * cvol * Lv[i] * Lv[j]), jscale(p_11, L1[i] * L1[j])),
                               jadd(jscale(p_12, L1[i] * L2[j] + L2[i] * L1[j]), jscale(p_22, L2[i] * L2[j])));
        const double x1 = NJ > 1 ? x.c[NJ > 1 ? 1 : 0] : 0.0, x2 = NJ > 2 ? x.c[NJ > 2 ? 2 : 0] : 0.0;
        Xn[i][j][0] = w0 * x.c[0] + w1 * x1 + w2 * x2;
        Xn[i][j][1] = w1 * x.c[0] + w2 * x1;
        Xn[i][j][2] = w2 * x.c[0];
      }
    const double cs2 = 2.0 * cs;
    const double Xs0 = w0 * cs2, Xs1 = w1 * cs2, Xs2 = w2 * cs2;
    double gr[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) gr[a][b] = 2.0 * l2 * (L1[a] * L1[b] + L2[a] * L2[b]);
    // Hessian-of-measure weights
    double hn[3], hs[3], hg[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      hn[i] = colT(d1n[i]);
      hs[i] = colT(jscale(qs[i], cs2));
    }
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int mm = 0; mm < 3; mm++) hg[a][mm] = colT(d1g(a, mm));
    const double mass = TR ? damp / (2.0 * dt) + rho_m / (dt * dt) : 0.0;

    // contributions of the gradient measure c = (a, mm), entry (gi0, gi1), to a row
    auto add_grad = [&](double *acc, int a, int mm, double gi0, double gi1) {
#pragma unroll
      for (int b = 0; b < 3; b++) {
        const double x = gr[a][b];
        const double al = w0 * x * gi0 + w1 * x * gi1, be = w1 * x * gi0 + w2 * x * gi1;
        const int sb = symi(b, mm);
#pragma unroll
        for (int l = 0; l < 3; l++) {
          acc[slot(l, 1 + b)] += al * LP_H(l, sb) + (TR ? be * LP_DH(l, sb) : 0.0);
          acc[slot(l, 4 + sb)] += al * LP_F(l, b) + (TR ? be * LP_DF(l, b) : 0.0);
        }
      }
    };
#pragma unroll
    for (int k = 0; k < 3; k++) {
      // value row
      {
#pragma unroll
        for (int j = 0; j < 30; j++)
          out_d[(30 * slot(k, 0) + j) * ostride] = (TR && j == slot(k, 0)) ? wt * mass : 0.0;
      }
      // gradient rows (k, 1 + a)
#pragma unroll
      for (int a = 0; a < 3; a++) {
        double acc[30];
#pragma unroll
        for (int j = 0; j < 30; j++) acc[j] = 0.0;
        {  // normal strain c = a
          const double gi0 = LP_F(k, a), gi1 = LP_DF(k, a);
#pragma unroll
          for (int d = 0; d < 3; d++) {
            const double al = Xn[a][d][0] * gi0 + Xn[a][d][1] * gi1;
            const double be = Xn[a][d][1] * gi0 + Xn[a][d][2] * gi1;
#pragma unroll
            for (int l = 0; l < 3; l++) acc[slot(l, 1 + d)] += al * LP_F(l, d) + (TR ? be * LP_DF(l, d) : 0.0);
          }
        }
#pragma unroll
        for (int b = 0; b < 3; b++) {  // shear strains (a, b)
          if (b == a) continue;
          const double gi0 = 0.5 * LP_F(k, b), gi1 = 0.5 * LP_DF(k, b);
          const double al = Xs0 * gi0 + Xs1 * gi1, be = Xs1 * gi0 + Xs2 * gi1;
#pragma unroll
          for (int l = 0; l < 3; l++) {
            acc[slot(l, 1 + a)] += al * (0.5 * LP_F(l, b)) + (TR ? be * (0.5 * LP_DF(l, b)) : 0.0);
            acc[slot(l, 1 + b)] += al * (0.5 * LP_F(l, a)) + (TR ? be * (0.5 * LP_DF(l, a)) : 0.0);
          }
        }
#pragma unroll
        for (int mm = 0; mm < 3; mm++) add_grad(acc, a, mm, LP_H(k, symi(a, mm)), LP_DH(k, symi(a, mm)));
        // Hessians of the measures
        acc[slot(k, 1 + a)] += hn[a];
#pragma unroll
        for (int b = 0; b < 3; b++)
          if (b != a) acc[slot(k, 1 + b)] += 0.5 * hs[shear(a, b) - 3];
#pragma unroll
        for (int mm = 0; mm < 3; mm++) acc[slot(k, 4 + symi(a, mm))] += hg[a][mm];
        const int row = slot(k, 1 + a);
#pragma unroll
        for (int j = 0; j < 30; j++) out_d[(30 * row + j) * ostride] = wt * acc[j];
      }
      // Hessian rows (k, 4 + s)
#pragma unroll
      for (int s = 0; s < 6; s++) {
        const int j0 = s < 3 ? 0 : (s < 5 ? 1 : 2);
        const int m0 = s < 3 ? s : (s < 5 ? s - 2 : 2);
        double acc[30];
#pragma unroll
        for (int j = 0; j < 30; j++) acc[j] = 0.0;
        add_grad(acc, j0, m0, LP_F(k, j0), LP_DF(k, j0));
        acc[slot(k, 1 + j0)] += hg[j0][m0];
        if (j0 != m0) {
          add_grad(acc, m0, j0, LP_F(k, m0), LP_DF(k, m0));
          acc[slot(k, 1 + m0)] += hg[m0][j0];
        }
        const int row = slot(k, 4 + s);
#pragma unroll
        for (int j = 0; j < 30; j++) out_d[(30 * row + j) * ostride] = wt * acc[j];
      }
    }
  }
#undef LP_F
#undef LP_DF
#undef LP_H
#undef LP_DH
}

}  // namespace igap
