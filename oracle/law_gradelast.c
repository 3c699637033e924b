/*
 * Finite-strain Toupin gradient elasticity: static law (phys/gradelast.c:7-1023,
 * parameters phys/physgradelast.c:21) and its three-level transient form
 * (phys/gradelasttime.c:7-9181, parameters phys/physgradelasttime.c:21) --
 * the project's own restatement from the stored-energy function, for the CPU
 * oracle.  TEST INFRASTRUCTURE ONLY.
 *
 * Energy.  With F = I + grad u, E = (F^T F - I)/2 and E_ab,m = dE_ab/dX_m:
 *   psi = c_v e_v^2 + c_s (E01^2 + E02^2 + E12^2)
 *       + A (e1^2 + e2^2) + B (e2^3 - 3 e1^2 e2) + C (e1^2 + e2^2)^2
 *       + l^2 sum_m [ (d_m e1)^2 + (d_m e2)^2 ]
 * e_v = tr E/sqrt3, e1 = (E00-E11)/sqrt2, e2 = (E00+E11-2E22)/sqrt6,
 * c_v = par[2], c_s = par[3], l = par[4]; A, B, C are the Landau coefficients
 * fixed by r = par[0], curv = par[1] (phys/gradelast.c:46-48).
 *
 * Static law: rr = dpsi/du, tt = d2psi/du2 by the chain rule through the 15
 * strain measures q = (E00,E11,E22,E01,E02,E12, E_aa,m), each quadratic in u:
 *   rr = sum_c psi_c grad q_c,  tt = sum_cd psi_cd grad q_c grad q_d^T
 *                                   + sum_c psi_c hess q_c.
 *
 * Transient law (u holds u, u_n, u_{n-1} at offsets 0, 30, 60).  The elastic
 * force is the average-vector-field discrete gradient between the midpoints
 * m = (u_n + u_{n-1})/2 and m + delta, delta = (u - u_{n-1})/2,
 *   f = int_0^1 grad psi(m + s delta) ds,
 * truncated at third order in delta:  f = sum_{k=0..3} g_k / (k+1), where g_k
 * is the s^k Taylor coefficient of g(s) = grad psi(m + s delta).  Its Jacobian
 * in u is  (1/2) sum_{k=0..2} T_k / (k+2),  T_k the s^k coefficient of the
 * static tangent along the same line.  Value entries add inertia and damping,
 *   rho (u - 2 u_n + u_{n-1}) / dt^2 + c (u - u_{n-1}) / (2 dt),
 * with rho = par[5], c = par[6], dt = par[7].  These identities were
 * established by probing the compiled reference law and are pinned by the
 * law-level tests.  All s-polynomials are carried as truncated Taylor jets.
 */
#include <math.h>
#include <string.h>

#define NQ 15
#define NJ 4 /* jet length: s^0..s^3 */

typedef struct { double c[NJ]; } jet;

static jet jconst(double a) { jet r; memset(&r, 0, sizeof r); r.c[0] = a; return r; }
static jet jadd(jet a, jet b) { for (int i = 0; i < NJ; i++) a.c[i] += b.c[i]; return a; }
static jet jscale(jet a, double s) { for (int i = 0; i < NJ; i++) a.c[i] *= s; return a; }
static jet jmul(jet a, jet b)
{
  jet r;
  for (int i = 0; i < NJ; i++) {
    double s = 0.0;
    for (int j = 0; j <= i; j++) s += a.c[j] * b.c[i - j];
    r.c[i] = s;
  }
  return r;
}

static int sym6(int j, int m)
{
  if (j > m) { int t = j; j = m; m = t; }
  static const int tab[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  return tab[j][m];
}

static const int PA[6] = {0, 1, 2, 0, 0, 1}, PB[6] = {0, 1, 2, 1, 2, 2};

void gradelast_coefficients(const double *par, double *A, double *B, double *C)
{
  double r = par[0], cv = par[1];
  double den = r * r - 2.0 * r * r * cv - r * (4.0 / 3.0 * r - 4.0 / 3.0 * r * cv);
  *B = -(4.0 / 3.0 * r - 4.0 / 3.0 * r * cv) / (r * r * den);
  *A = 2.0 * cv / den;
  *C = -1.0 / (r * r * den);
}

/* Split a 30-entry state into F (with or without identity) and H. */
static void unpack(const double *u, int with_identity, double F[3][3], double H[3][3][3])
{
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      F[i][j] = (with_identity && i == j ? 1.0 : 0.0) + u[10 * i + 1 + j];
      for (int m = 0; m < 3; m++) H[i][j][m] = u[10 * i + 4 + sym6(j, m)];
    }
}

/* grad q (15 x 30) at (F,H); linear in (F,H). */
static void grad_measures(double F[3][3], double H[3][3][3], double gq[NQ][30])
{
  memset(gq, 0, sizeof(double) * NQ * 30);
  for (int c = 0; c < 6; c++) {
    int a = PA[c], b = PB[c];
    for (int k = 0; k < 3; k++) {
      gq[c][10 * k + 1 + a] += 0.5 * F[k][b];
      gq[c][10 * k + 1 + b] += 0.5 * F[k][a];
    }
  }
  for (int a = 0; a < 3; a++)
    for (int m = 0; m < 3; m++) {
      int c = 6 + 3 * a + m;
      for (int k = 0; k < 3; k++) {
        gq[c][10 * k + 1 + a] += H[k][a][m];
        gq[c][10 * k + 4 + sym6(a, m)] += F[k][a];
      }
    }
}

/* q at (F,H) (F with identity) */
static void measures(double F[3][3], double H[3][3][3], double q[NQ])
{
  for (int c = 0; c < 6; c++) {
    int a = PA[c], b = PB[c];
    double s = 0.0;
    for (int k = 0; k < 3; k++) s += F[k][a] * F[k][b];
    q[c] = 0.5 * (s - (a == b ? 1.0 : 0.0));
  }
  for (int a = 0; a < 3; a++)
    for (int m = 0; m < 3; m++) {
      double s = 0.0;
      for (int k = 0; k < 3; k++) s += F[k][a] * H[k][a][m];
      q[6 + 3 * a + m] = s;
    }
}

/* purely quadratic part of q at an increment (dF without identity) */
static void measures_quad(double dF[3][3], double dH[3][3][3], double q2[NQ])
{
  for (int c = 0; c < 6; c++) {
    int a = PA[c], b = PB[c];
    double s = 0.0;
    for (int k = 0; k < 3; k++) s += dF[k][a] * dF[k][b];
    q2[c] = 0.5 * s;
  }
  for (int a = 0; a < 3; a++)
    for (int m = 0; m < 3; m++) {
      double s = 0.0;
      for (int k = 0; k < 3; k++) s += dF[k][a] * dH[k][a][m];
      q2[6 + 3 * a + m] = s;
    }
}

/* psi_c and psi_cd as jets of the measure jets. */
static void energy_derivs(const jet q[NQ], const double *par, jet d1[NQ], jet d2[NQ][NQ])
{
  const double s2 = sqrt(2.0), s3 = sqrt(3.0), s6 = sqrt(6.0);
  double A, B, C;
  gradelast_coefficients(par, &A, &B, &C);
  double cvol = par[2], cs = par[3], l2 = par[4] * par[4];
  const double Lv[3] = {1 / s3, 1 / s3, 1 / s3};
  const double L1[3] = {1 / s2, -1 / s2, 0.0};
  const double L2[3] = {1 / s6, 1 / s6, -2 / s6};
  jet ev = jconst(0), e1 = jconst(0), e2 = jconst(0);
  for (int i = 0; i < 3; i++) {
    ev = jadd(ev, jscale(q[i], Lv[i]));
    e1 = jadd(e1, jscale(q[i], L1[i]));
    e2 = jadd(e2, jscale(q[i], L2[i]));
  }
  jet e11 = jmul(e1, e1), e22 = jmul(e2, e2), e12 = jmul(e1, e2);
  jet rho = jadd(e11, e22);
  jet p_v = jscale(ev, 2.0 * cvol);
  jet p_1 = jadd(jadd(jscale(e1, 2.0 * A), jscale(e12, -6.0 * B)), jscale(jmul(e1, rho), 4.0 * C));
  jet p_2 = jadd(jadd(jscale(e2, 2.0 * A), jscale(jadd(e22, jscale(e11, -1.0)), 3.0 * B)),
                 jscale(jmul(e2, rho), 4.0 * C));
  jet p_11 = jadd(jadd(jconst(2.0 * A), jscale(e2, -6.0 * B)), jadd(jscale(rho, 4.0 * C), jscale(e11, 8.0 * C)));
  jet p_12 = jadd(jscale(e1, -6.0 * B), jscale(e12, 8.0 * C));
  jet p_22 = jadd(jadd(jconst(2.0 * A), jscale(e2, 6.0 * B)), jadd(jscale(rho, 4.0 * C), jscale(e22, 8.0 * C)));
  for (int i = 0; i < NQ; i++) {
    d1[i] = jconst(0);
    for (int j = 0; j < NQ; j++) d2[i][j] = jconst(0);
  }
  for (int i = 0; i < 3; i++) {
    d1[i] = jadd(jadd(jscale(p_v, Lv[i]), jscale(p_1, L1[i])), jscale(p_2, L2[i]));
    for (int j = 0; j < 3; j++)
      d2[i][j] = jadd(jadd(jconst(2.0 * cvol * Lv[i] * Lv[j]), jscale(p_11, L1[i] * L1[j])),
                      jadd(jscale(p_12, L1[i] * L2[j] + L2[i] * L1[j]), jscale(p_22, L2[i] * L2[j])));
  }
  for (int c = 3; c < 6; c++) { d1[c] = jscale(q[c], 2.0 * cs); d2[c][c] = jconst(2.0 * cs); }
  for (int m = 0; m < 3; m++) {
    jet g1 = jconst(0), g2 = jconst(0);
    for (int a = 0; a < 3; a++) {
      g1 = jadd(g1, jscale(q[6 + 3 * a + m], L1[a]));
      g2 = jadd(g2, jscale(q[6 + 3 * a + m], L2[a]));
    }
    for (int a = 0; a < 3; a++) {
      d1[6 + 3 * a + m] = jscale(jadd(jscale(g1, L1[a]), jscale(g2, L2[a])), 2.0 * l2);
      for (int b = 0; b < 3; b++)
        d2[6 + 3 * a + m][6 + 3 * b + m] = jconst(2.0 * l2 * (L1[a] * L1[b] + L2[a] * L2[b]));
    }
  }
}

/* Jets along the line m + s*delta: q(s) (degree 2 exact) and grad q(s)
 * (degree 1 exact).  delta == NULL gives the static point m. */
static void line_jets(const double *m, const double *delta, jet q[NQ], jet gq[NQ][30])
{
  double F[3][3], H[3][3][3], qm[NQ], g0[NQ][30];
  unpack(m, 1, F, H);
  measures(F, H, qm);
  grad_measures(F, H, g0);
  double g1[NQ][30], q1[NQ], q2[NQ];
  memset(g1, 0, sizeof g1);
  memset(q1, 0, sizeof q1);
  memset(q2, 0, sizeof q2);
  if (delta) {
    double dF[3][3], dH[3][3][3];
    unpack(delta, 0, dF, dH);
    grad_measures(dF, dH, g1);
    measures_quad(dF, dH, q2);
    for (int c = 0; c < NQ; c++) {
      double s = 0.0;
      for (int i = 0; i < 30; i++) s += g0[c][i] * delta[i];
      q1[c] = s;
    }
  }
  for (int c = 0; c < NQ; c++) {
    q[c] = jconst(qm[c]);
    q[c].c[1] = q1[c];
    q[c].c[2] = q2[c];
    for (int i = 0; i < 30; i++) {
      gq[c][i] = jconst(g0[c][i]);
      gq[c][i].c[1] = g1[c][i];
    }
  }
}

/* Jet of the static residual along the line. */
static void residual_jet(const jet q[NQ], jet gq[NQ][30], const double *par, jet r[30])
{
  jet d1[NQ], d2[NQ][NQ];
  energy_derivs(q, par, d1, d2);
  for (int i = 0; i < 30; i++) {
    jet s = jconst(0);
    for (int c = 0; c < NQ; c++) s = jadd(s, jmul(d1[c], gq[c][i]));
    r[i] = s;
  }
}

/* Jet of the static tangent along the line (row-major 30x30). */
static void tangent_jet(const jet q[NQ], jet gq[NQ][30], const double *par, jet *T)
{
  jet d1[NQ], d2[NQ][NQ];
  energy_derivs(q, par, d1, d2);
  static jet t[NQ][30];
  for (int c = 0; c < NQ; c++)
    for (int i = 0; i < 30; i++) {
      jet s = jconst(0);
      for (int d = 0; d < NQ; d++) s = jadd(s, jmul(d2[c][d], gq[d][i]));
      t[c][i] = s;
    }
  for (int i = 0; i < 30; i++)
    for (int j = 0; j < 30; j++) {
      jet s = jconst(0);
      for (int c = 0; c < NQ; c++) s = jadd(s, jmul(gq[c][i], t[c][j]));
      T[30 * i + j] = s;
    }
  /* constant Hessians of the measures, weighted by psi_c */
  for (int c = 0; c < 6; c++) {
    int a = PA[c], b = PB[c];
    for (int k = 0; k < 3; k++) {
      int ia = 10 * k + 1 + a, ib = 10 * k + 1 + b;
      T[30 * ia + ib] = jadd(T[30 * ia + ib], jscale(d1[c], 0.5));
      T[30 * ib + ia] = jadd(T[30 * ib + ia], jscale(d1[c], 0.5));
    }
  }
  for (int a = 0; a < 3; a++)
    for (int m = 0; m < 3; m++) {
      int c = 6 + 3 * a + m;
      for (int k = 0; k < 3; k++) {
        int iF = 10 * k + 1 + a, iH = 10 * k + 4 + sym6(a, m);
        T[30 * iF + iH] = jadd(T[30 * iF + iH], d1[c]);
        T[30 * iH + iF] = jadd(T[30 * iH + iF], d1[c]);
      }
    }
}

void gradelast_law_residual(double *rr, const double *u, const double *par)
{
  jet q[NQ], gq[NQ][30], r[30];
  line_jets(u, 0, q, gq);
  residual_jet(q, gq, par, r);
  for (int i = 0; i < 30; i++) rr[i] = r[i].c[0];
}

void gradelast_law_tangent(double *tt, const double *u, const double *par)
{
  static jet T[900];
  jet q[NQ], gq[NQ][30];
  line_jets(u, 0, q, gq);
  tangent_jet(q, gq, par, T);
  for (int i = 0; i < 900; i++) tt[i] = T[i].c[0];
}

static void transient_line(const double *u, double *m, double *delta)
{
  for (int i = 0; i < 30; i++) {
    m[i] = 0.5 * (u[30 + i] + u[60 + i]);
    delta[i] = 0.5 * (u[i] - u[60 + i]);
  }
}

void gradelasttime_law_residual(double *rr, const double *u, const double *par)
{
  double m[30], delta[30];
  transient_line(u, m, delta);
  jet q[NQ], gq[NQ][30], r[30];
  line_jets(m, delta, q, gq);
  residual_jet(q, gq, par, r);
  for (int i = 0; i < 30; i++) rr[i] = r[i].c[0] + r[i].c[1] / 2.0 + r[i].c[2] / 3.0 + r[i].c[3] / 4.0;
  const double rho = par[5], damp = par[6], dt = par[7];
  for (int d = 0; d < 3; d++) {
    int i = 10 * d;
    rr[i] += damp * (u[i] - u[60 + i]) / (2.0 * dt) + rho * (u[i] + u[60 + i] - 2.0 * u[30 + i]) / (dt * dt);
  }
}

void gradelasttime_law_tangent(double *tt, const double *u, const double *par)
{
  double m[30], delta[30];
  transient_line(u, m, delta);
  static jet T[900];
  jet q[NQ], gq[NQ][30];
  line_jets(m, delta, q, gq);
  tangent_jet(q, gq, par, T);
  for (int i = 0; i < 900; i++)
    tt[i] = 0.5 * (T[i].c[0] / 2.0 + T[i].c[1] / 3.0 + T[i].c[2] / 4.0);
  const double rho = par[5], damp = par[6], dt = par[7];
  for (int d = 0; d < 3; d++) {
    int i = 10 * d;
    tt[30 * i + i] += damp / (2.0 * dt) + rho / (dt * dt);
  }
}
