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
// Inputs per point (shared memory, column t, leading dimension ld; FP64, or
// floats for the FP32 law):
//   sm[slot]  m at the gradient and Hessian slots (m = u for the static law,
//             (u_n + u_{n-1})/2 for the transient one); at the value slots of
//             the transient law the inertia + damping residual term (read by
//             the residual only);
//   sd[slot]  delta = (u - u_{n-1})/2 (transient law only).
// Outputs: rr[30] and D[900] (row-major, row = test slot) scaled by wt,
// written to out_r[i * ostride] (FP64) and out_d[(30 i + j) * ostride] (in
// the arithmetic type T).
#pragma once
#include "df32.cuh"
#include "gram_common.cuh"
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

// input and output conversions of the arithmetic type (FP32: on the integer pipe)
template <typename T>
__device__ __forceinline__ T to_t(double x);
template <>
__device__ __forceinline__ double to_t<double>(double x) { return x; }
template <>
__device__ __forceinline__ float to_t<float>(double x) { return f64_to_pair(x).x; }
__device__ __forceinline__ double to_f64(double x) { return x; }
// the law's inputs as stored by the caller: FP64, or already in the FP32
// arithmetic type
template <typename T>
__device__ __forceinline__ T in_t(double x) { return to_t<T>(x); }
template <typename T>
__device__ __forceinline__ T in_t(float x) { return T(x); }
__device__ __forceinline__ double to_f64(float x) { return f32_to_f64(x); }

}  // namespace lawpt

template <int NJ, bool RES, bool TAN, typename T = double, typename IN = double>
__device__ __forceinline__ void gradelast_point(const IN *__restrict__ sm_in, const IN *__restrict__ sd_in,
                                                int ld, const double *par, double wt_in,
                                                double *__restrict__ out_r, T *__restrict__ out_d,
                                                int64_t ostride)
{
  // FP32: the point's inputs converted once into registers (on the integer
  // pipe); FP64: read from shared memory where they are used
  constexpr bool F32 = sizeof(T) == 4;
  T smv[F32 ? 30 : 1], sdv[F32 ? 30 : 1];
  if constexpr (F32) {
#pragma unroll
    for (int i = 0; i < 30; i++) {
      smv[i] = lawpt::in_t<T>(sm_in[i * ld]);
      sdv[i] = NJ > 1 ? lawpt::in_t<T>(sd_in[i * ld]) : T(0);
    }
  }
  const T wt = lawpt::to_t<T>(wt_in);
  using namespace lawpt;
  constexpr bool TR = NJ > 1;
#define LP_SM(i) (F32 ? smv[F32 ? (i) : 0] : T(sm_in[(i) * ld]))
#define LP_SD(i) (F32 ? sdv[F32 ? (i) : 0] : T(sd_in[(i) * ld]))
#define LP_F(k, a) (T((k) == (a) ? 1 : 0) + LP_SM(slot(k, 1 + (a))))
#define LP_DF(k, a) (TR ? LP_SD(slot(k, 1 + (a))) : T(0))
#define LP_H(k, s) (LP_SM(slot(k, 4 + (s))))
#define LP_DH(k, s) (TR ? LP_SD(slot(k, 4 + (s))) : T(0))
  // FP64: the correctly rounded square roots as constants (the reciprocals
  // below then fold at compile time; no FP64 square root or division per
  // point)
  T s2, s3, s6;
  if constexpr (sizeof(T) == 8) {
    s2 = T(1.4142135623730951);
    s3 = T(1.7320508075688772);
    s6 = T(2.449489742783178);
  } else {
    s2 = sqrt(T(2.0));
    s3 = sqrt(T(3.0));
    s6 = sqrt(T(6.0));
  }
  const T Lv[3] = {1 / s3, 1 / s3, 1 / s3};
  const T L1[3] = {1 / s2, -1 / s2, T(0.0)};
  const T L2[3] = {1 / s6, 1 / s6, -2 / s6};
  double Ad, Bd, Cd;
  landau(par, Ad, Bd, Cd);
  const T A = T(Ad), B = T(Bd), C = T(Cd);
  const T cvol = T(par[2]), cs = T(par[3]), l2 = T(par[4] * par[4]);
  // ---- measures (s-jets q0 + q1 s + q2 s^2) and the energy derivatives
  Jet<NJ, T> qn[3], qs[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    T q0 = T(0.0), q1 = T(0.0), q2 = T(0.0);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      q0 += LP_F(k, a) * LP_F(k, a);
      q2 += LP_DF(k, a) * LP_DF(k, a);
      q1 += LP_F(k, a) * LP_DF(k, a);
    }
    qn[a] = jconst<NJ, T>(T(0.5) * (q0 - T(1.0)));
    if constexpr (NJ > 1) qn[a].c[1] = q1;
    if constexpr (NJ > 2) qn[a].c[2] = T(0.5) * q2;
  }
#pragma unroll
  for (int c = 3; c < 6; c++) {
    const int a = c == 5 ? 1 : 0, b = c == 3 ? 1 : 2;
    T q0 = T(0.0), q1 = T(0.0), q2 = T(0.0);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      q0 += LP_F(k, a) * LP_F(k, b);
      q2 += LP_DF(k, a) * LP_DF(k, b);
      q1 += T(0.5) * LP_F(k, b) * LP_DF(k, a);
      q1 += T(0.5) * LP_F(k, a) * LP_DF(k, b);
    }
    qs[c - 3] = jconst<NJ, T>(T(0.5) * q0);
    if constexpr (NJ > 1) qs[c - 3].c[1] = q1;
    if constexpr (NJ > 2) qs[c - 3].c[2] = T(0.5) * q2;
  }
  // gradient measures only enter through G1[mm] = sum_a L1[a] q_(a,mm), G2 likewise
  Jet<NJ, T> G1[3], G2[3];
#pragma unroll
  for (int mm = 0; mm < 3; mm++) {
    G1[mm] = jzero<NJ, T>();
    G2[mm] = jzero<NJ, T>();
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const int s = symi(a, mm);
      T q0 = T(0.0), q1 = T(0.0), q2 = T(0.0);
#pragma unroll
      for (int k = 0; k < 3; k++) {
        q0 += LP_F(k, a) * LP_H(k, s);
        q2 += LP_DF(k, a) * LP_DH(k, s);
        q1 += LP_H(k, s) * LP_DF(k, a);
        q1 += LP_F(k, a) * LP_DH(k, s);
      }
      Jet<NJ, T> q = jconst<NJ, T>(q0);
      if constexpr (NJ > 1) q.c[1] = q1;
      if constexpr (NJ > 2) q.c[2] = q2;
      G1[mm] = jadd(G1[mm], jscale(q, L1[a]));
      G2[mm] = jadd(G2[mm], jscale(q, L2[a]));
    }
  }
  Jet<NJ, T> ev = jzero<NJ, T>(), e1 = jzero<NJ, T>(), e2 = jzero<NJ, T>();
#pragma unroll
  for (int i = 0; i < 3; i++) {
    ev = jadd(ev, jscale(qn[i], Lv[i]));
    e1 = jadd(e1, jscale(qn[i], L1[i]));
    e2 = jadd(e2, jscale(qn[i], L2[i]));
  }
  const Jet<NJ, T> e11 = jmul(e1, e1), e22 = jmul(e2, e2), e12 = jmul(e1, e2);
  const Jet<NJ, T> rho = jadd(e11, e22);
  const Jet<NJ, T> p_v = jscale(ev, T(2.0) * cvol);
  const Jet<NJ, T> p_1 = jadd(jadd(jscale(e1, T(2.0) * A), jscale(e12, -T(6.0) * B)), jscale(jmul(e1, rho), T(4.0) * C));
  const Jet<NJ, T> p_2 = jadd(jadd(jscale(e2, T(2.0) * A), jscale(jadd(e22, jscale(e11, -T(1.0))), T(3.0) * B)),
                           jscale(jmul(e2, rho), T(4.0) * C));
  // collapse weights: residual (sum_k t_k/(k+1), and the g1 part sum_k t_k/(k+2));
  // tangent (w0, w1, w2)
  // x / 3: FP64 multiplies by the rounded third (the FP64 division is a long
  // sequence on the FP64 pipe; the collapse sums stay within 1e-16 relative)
  auto div3 = [](T x) -> T {
    if constexpr (sizeof(T) == 8) return x * T(1.0 / 3.0);
    else return x / T(3.0);
  };
  auto colR0 = [&](const Jet<NJ, T> &t) -> T {
    if constexpr (NJ == 1) return t.c[0];
    else return t.c[0] + t.c[1] / T(2.0) + div3(t.c[2]) + t.c[3] / T(4.0);
  };
  auto colR1 = [&](const Jet<NJ, T> &t) -> T {
    if constexpr (NJ == 1) return T(0.0);
    else return t.c[0] / T(2.0) + div3(t.c[1]) + t.c[2] / T(4.0);
  };
  auto colT = [&](const Jet<NJ, T> &t) -> T {
    if constexpr (NJ == 1) return t.c[0];
    else return T(0.5) * (t.c[0] / T(2.0) + div3(t.c[1]) + t.c[2] / T(4.0));
  };
  // d1 of the normal strains
  Jet<NJ, T> d1n[3];
#pragma unroll
  for (int i = 0; i < 3; i++) d1n[i] = jadd(jadd(jscale(p_v, Lv[i]), jscale(p_1, L1[i])), jscale(p_2, L2[i]));
  // d1 of the gradient measures: 2 l2 (L1[a] G1 + L2[a] G2)
  auto d1g = [&](int a, int mm) -> Jet<NJ, T> {
    return jscale(jadd(jscale(G1[mm], L1[a]), jscale(G2[mm], L2[a])), T(2.0) * l2);
  };
  const T rho_m = T(par[5]), damp = T(par[6]), dt = T(par[7]);
  (void)rho_m; (void)damp; (void)dt;

  if constexpr (RES) {
    T Rn0[3], Rn1[3], Rs0[3], Rs1[3], Rg0[3][3], Rg1[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      Rn0[i] = colR0(d1n[i]); Rn1[i] = colR1(d1n[i]);
      const Jet<NJ, T> d = jscale(qs[i], T(2.0) * cs);
      Rs0[i] = colR0(d); Rs1[i] = colR1(d);
    }
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int mm = 0; mm < 3; mm++) {
        const Jet<NJ, T> d = d1g(a, mm);
        Rg0[a][mm] = colR0(d); Rg1[a][mm] = colR1(d);
      }
#pragma unroll
    for (int k = 0; k < 3; k++) {
      // value slot: inertia and damping of the transient law
      out_r[slot(k, 0) * ostride] = lawpt::to_f64(TR ? wt * LP_SM(slot(k, 0)) : T(0));
#pragma unroll
      for (int a = 0; a < 3; a++) {
        T v = Rn0[a] * LP_F(k, a) + Rn1[a] * LP_DF(k, a);
#pragma unroll
        for (int b = 0; b < 3; b++) {
          if (b == a) continue;
          const int c = shear(a, b) - 3;
          v += Rs0[c] * (T(0.5) * LP_F(k, b)) + Rs1[c] * (T(0.5) * LP_DF(k, b));
        }
#pragma unroll
        for (int mm = 0; mm < 3; mm++) v += Rg0[a][mm] * LP_H(k, symi(a, mm)) + Rg1[a][mm] * LP_DH(k, symi(a, mm));
        out_r[slot(k, 1 + a) * ostride] = lawpt::to_f64(wt * v);
      }
#pragma unroll
      for (int s = 0; s < 6; s++) {
        const int j = s < 3 ? 0 : (s < 5 ? 1 : 2);
        const int m = s < 3 ? s : (s < 5 ? s - 2 : 2);
        T v = Rg0[j][m] * LP_F(k, j) + Rg1[j][m] * LP_DF(k, j);
        if (j != m) v += Rg0[m][j] * LP_F(k, m) + Rg1[m][j] * LP_DF(k, m);
        out_r[slot(k, 4 + s) * ostride] = lawpt::to_f64(wt * v);
      }
    }
  }

  if constexpr (TAN) {
    const T w0 = TR ? T(0.25) : T(1.0), w1 = TR ? T(1.0) / T(6.0) : T(0.0), w2 = TR ? T(0.125) : T(0.0);
    // couplings of the normal strains: d2b[c][d] (symmetric) as (X0, X1, X2)
    const Jet<NJ, T> p_11 = jadd(jadd(jconst<NJ, T>(T(2.0) * A), jscale(e2, -T(6.0) * B)),
                              jadd(jscale(rho, T(4.0) * C), jscale(e11, T(8.0) * C)));
    const Jet<NJ, T> p_12 = jadd(jscale(e1, -T(6.0) * B), jscale(e12, T(8.0) * C));
    const Jet<NJ, T> p_22 = jadd(jadd(jconst<NJ, T>(T(2.0) * A), jscale(e2, T(6.0) * B)),
                              jadd(jscale(rho, T(4.0) * C), jscale(e22, T(8.0) * C)));
    T Xn[3][3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const Jet<NJ, T> x = jadd(jadd(jconst<NJ, T>(T(2.0) * cvol * Lv[i] * Lv[j]), jscale(p_11, L1[i] * L1[j])),
                               jadd(jscale(p_12, L1[i] * L2[j] + L2[i] * L1[j]), jscale(p_22, L2[i] * L2[j])));
        const T x1 = NJ > 1 ? x.c[NJ > 1 ? 1 : 0] : T(0.0), x2 = NJ > 2 ? x.c[NJ > 2 ? 2 : 0] : T(0.0);
        Xn[i][j][0] = w0 * x.c[0] + w1 * x1 + w2 * x2;
        Xn[i][j][1] = w1 * x.c[0] + w2 * x1;
        Xn[i][j][2] = w2 * x.c[0];
      }
    const T cs2 = T(2.0) * cs;
    const T Xs0 = w0 * cs2, Xs1 = w1 * cs2, Xs2 = w2 * cs2;
    T gr[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) gr[a][b] = T(2.0) * l2 * (L1[a] * L1[b] + L2[a] * L2[b]);
    // Hessian-of-measure weights
    T hn[3], hs[3], hg[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      hn[i] = colT(d1n[i]);
      hs[i] = colT(jscale(qs[i], cs2));
    }
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int mm = 0; mm < 3; mm++) hg[a][mm] = colT(d1g(a, mm));
    const T mass = TR ? damp / (T(2.0) * dt) + rho_m / (dt * dt) : T(0.0);

    // contributions of the gradient measure c = (a, mm), entry (gi0, gi1), to a row
    auto add_grad = [&](T *acc, int a, int mm, T gi0, T gi1) {
#pragma unroll
      for (int b = 0; b < 3; b++) {
        const T x = gr[a][b];
        const T al = w0 * x * gi0 + w1 * x * gi1, be = w1 * x * gi0 + w2 * x * gi1;
        const int sb = symi(b, mm);
#pragma unroll
        for (int l = 0; l < 3; l++) {
          acc[slot(l, 1 + b)] += al * LP_H(l, sb) + (TR ? be * LP_DH(l, sb) : T(0.0));
          acc[slot(l, 4 + sb)] += al * LP_F(l, b) + (TR ? be * LP_DF(l, b) : T(0.0));
        }
      }
    };
#pragma unroll
    for (int k = 0; k < 3; k++) {
      // value row
      {
#pragma unroll
        for (int j = 0; j < 30; j++)
          out_d[(30 * slot(k, 0) + j) * ostride] = (TR && j == slot(k, 0)) ? wt * mass : T(0);
      }
      // gradient rows (k, 1 + a)
#pragma unroll
      for (int a = 0; a < 3; a++) {
        T acc[30];
#pragma unroll
        for (int j = 0; j < 30; j++) acc[j] = T(0.0);
        {  // normal strain c = a
          const T gi0 = LP_F(k, a), gi1 = LP_DF(k, a);
#pragma unroll
          for (int d = 0; d < 3; d++) {
            const T al = Xn[a][d][0] * gi0 + Xn[a][d][1] * gi1;
            const T be = Xn[a][d][1] * gi0 + Xn[a][d][2] * gi1;
#pragma unroll
            for (int l = 0; l < 3; l++) acc[slot(l, 1 + d)] += al * LP_F(l, d) + (TR ? be * LP_DF(l, d) : T(0.0));
          }
        }
#pragma unroll
        for (int b = 0; b < 3; b++) {  // shear strains (a, b)
          if (b == a) continue;
          const T gi0 = T(0.5) * LP_F(k, b), gi1 = T(0.5) * LP_DF(k, b);
          const T al = Xs0 * gi0 + Xs1 * gi1, be = Xs1 * gi0 + Xs2 * gi1;
#pragma unroll
          for (int l = 0; l < 3; l++) {
            acc[slot(l, 1 + a)] += al * (T(0.5) * LP_F(l, b)) + (TR ? be * (T(0.5) * LP_DF(l, b)) : T(0.0));
            acc[slot(l, 1 + b)] += al * (T(0.5) * LP_F(l, a)) + (TR ? be * (T(0.5) * LP_DF(l, a)) : T(0.0));
          }
        }
#pragma unroll
        for (int mm = 0; mm < 3; mm++) add_grad(acc, a, mm, LP_H(k, symi(a, mm)), LP_DH(k, symi(a, mm)));
        // Hessians of the measures
        acc[slot(k, 1 + a)] += hn[a];
#pragma unroll
        for (int b = 0; b < 3; b++)
          if (b != a) acc[slot(k, 1 + b)] += T(0.5) * hs[shear(a, b) - 3];
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
        T acc[30];
#pragma unroll
        for (int j = 0; j < 30; j++) acc[j] = T(0.0);
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
#undef LP_SM
#undef LP_SD
}

}  // namespace igap
