/*
 * CPU oracle: project-written C restatement of IGAP4's assembly path.
 * TEST INFRASTRUCTURE ONLY (see igap_oracle.h).  It keeps the reference's loop
 * structure (element loop, 4x4x4 points, naive 81x81 contraction) so that its
 * timing stands for the reference's CPU path, but every line is written here.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "igap_oracle.h"

#define MTOL 1.e-15 /* added to every knot-span denominator, src/meshcore_iga.c:10,303-307 */
#define NDDIM 10
#define NDOF 3

struct OracleCase {
  int p, nelem[3], nbasis[3], nknot[3];
  double *knots[3];
  double *w, *X;
  int law, torder, nquad;
  double par[9];
  int bc_type[36];
  double par_dirichlet[9];
  double neumann[36];
  int ndof;
  long nnz;
  long *rowptr;
  int *cols;
};

/* ------------------------------------------------------------ quadrature -- */
/* Newton iteration on the Legendre polynomial P_n (three-term recurrence),
 * then map [-1,1] -> [a,b]. Same rule as legendre_handle (src/quadrature.c:381)
 * computed by a different method; agreement is checked to round-off. */
void orc_gauss_legendre(int n, double a, double b, double *x, double *w)
{
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; i++) {
    double z = cos(pi * (i + 0.75) / (n + 0.5)), dp = 0.0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; k++) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1; p1 = p2;
      }
      if (n == 1) { p1 = z; p0 = 1.0; }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-17) break;
    }
    /* recompute derivative at the converged root */
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= n; k++) {
      double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1; p1 = p2;
    }
    dp = n * (z * p1 - p0) / (z * z - 1.0);
    double wi = 2.0 / ((1.0 - z * z) * dp * dp);
    /* roots come out descending in z, so -z ascends */
    x[i] = -z;
    w[i] = wi;
  }
  for (int i = 0; i < n; i++) {
    x[i] = 0.5 * (b - a) * x[i] + 0.5 * (b + a);
    w[i] = 0.5 * (b - a) * w[i];
  }
}

/* ------------------------------------------------------------------ mesh -- */
void orc_mesh_beam(const int nelem[3], const double L[3], int p, int perturb, double *knots,
                   double *w, double *X)
{
  /* open uniform knots on [0,1] (mesh/igabeam.c:36-45) */
  double *kv = knots;
  for (int d = 0; d < 3; d++) {
    int nk = nelem[d] + 1 + 2 * p;
    for (int k = 0; k < nk; k++)
      kv[k] = k <= p ? 0.0 : (k < nelem[d] + p ? (double)(k - p) / nelem[d] : 1.0);
    kv += nk;
  }
  /* Note: (k-p)*l with l=1/n as in the reference; keep that rounding */
  kv = knots;
  for (int d = 0; d < 3; d++) {
    int nk = nelem[d] + 1 + 2 * p;
    double l = 1.0 / nelem[d];
    for (int k = p + 1; k < nelem[d] + p; k++) kv[k] = (k - p) * l;
    kv += nk;
  }
  int nb[3] = {nelem[0] + p, nelem[1] + p, nelem[2] + p};
  long a = 0;
  for (int i = 0; i < nb[0]; i++)
    for (int j = 0; j < nb[1]; j++)
      for (int k = 0; k < nb[2]; k++, a++) {
        w[a] = 1.0;
        /* control points (mesh/igabeam.c:68-70) */
        double xi = ((double)i - 0.5) / ((double)(nb[0] - 2)) * L[0];
        double yj = ((double)j - 0.5) / ((double)(nb[1] - 2)) * L[1];
        double zk = ((double)k - 0.5) / ((double)(nb[2] - 2)) * L[2];
        if (perturb) { /* interior perturbation (mesh/igabeamtest.c:68-70) */
          double in = (double)(i > 2 && j > 2 && k > 2 && i < nb[0] - 2 && j < nb[1] - 2 && k < nb[2] - 2);
          xi += 0.2 * L[0] / nb[0] * in * sin(3 * i * k * j);
          yj += 0.2 * L[1] / nb[1] * in * sin(5 * i * k * j);
          zk += 0.2 * L[2] / nb[2] * in * sin(7 * i * k * j);
        }
        X[3 * a + 0] = xi; X[3 * a + 1] = yj; X[3 * a + 2] = zk;
      }
}

/* ----------------------------------------------------------------- basis -- */
/* 1-D values/derivatives of the p+1 functions active on span [kv[p],kv[p+1]]:
 * out[0..p] values, out[p+1..2p+1] first, out[2p+2..3p+2] second derivative.
 * Cox-de Boor triangle with MTOL on every denominator; for p=2 the operation
 * sequence is the one of src/meshcore_iga.c:300-307. */
static void bspline_1d(double *out, const double *kv, int p, double x)
{
  double lev[8][10];  /* lev[q][i] = N_{i,q} */
  double dlev[8][10]; /* first derivative of level q */
  for (int i = 0; i < 2 * p + 1; i++) lev[0][i] = 0.0;
  lev[0][p] = 1.0;
  for (int i = 0; i < 2 * p + 1; i++) dlev[0][i] = 0.0;
  for (int q = 1; q <= p; q++) {
    for (int i = 0; i < 2 * p + 1 - q; i++) {
      lev[q][i] = (x - kv[i]) / (kv[i + q] - kv[i] + MTOL) * lev[q - 1][i] +
                  (kv[i + q + 1] - x) / (kv[i + q + 1] - kv[i + 1] + MTOL) * lev[q - 1][i + 1];
      dlev[q][i] = (double)q / (kv[i + q] - kv[i] + MTOL) * lev[q - 1][i] -
                   (double)q / (kv[i + q + 1] - kv[i + 1] + MTOL) * lev[q - 1][i + 1];
    }
  }
  for (int i = 0; i <= p; i++) {
    out[i] = lev[p][i];
    out[p + 1 + i] = dlev[p][i];
    out[2 * p + 2 + i] = (double)p / (kv[i + p] - kv[i] + MTOL) * dlev[p - 1][i] -
                         (double)p / (kv[i + p + 1] - kv[i + 1] + MTOL) * dlev[p - 1][i + 1];
  }
}

void orc_eval_bspline(double *N, const double *const kv[3], int p, const double xq[3])
{
  double t[3][30];
  for (int d = 0; d < 3; d++) bspline_1d(t[d], kv[d], p, xq[d]);
  int q = p + 1;
  const double *nx = t[0], *dx = t[0] + q, *ddx = t[0] + 2 * q;
  const double *ny = t[1], *dy = t[1] + q, *ddy = t[1] + 2 * q;
  const double *nz = t[2], *dz = t[2] + q, *ddz = t[2] + 2 * q;
  for (int i = 0; i < q; i++)
    for (int j = 0; j < q; j++)
      for (int k = 0; k < q; k++) {
        double *o = N + NDDIM * (q * q * i + q * j + k);
        o[0] = nx[i] * ny[j] * nz[k];
        o[1] = dx[i] * ny[j] * nz[k];
        o[2] = nx[i] * dy[j] * nz[k];
        o[3] = nx[i] * ny[j] * dz[k];
        o[4] = ddx[i] * ny[j] * nz[k];
        o[5] = dx[i] * dy[j] * nz[k];
        o[6] = dx[i] * ny[j] * dz[k];
        o[7] = nx[i] * ddy[j] * nz[k];
        o[8] = nx[i] * dy[j] * dz[k];
        o[9] = nx[i] * ny[j] * ddz[k];
      }
}

/* Recursive basis evaluation with derivative coefficients a_{k,j}
 * (The NURBS Book eq. 2.9/2.10), with the right-end convention and the
 * 0/0 := 0 rules of src/meshcore_iga.c:344-380. */
static double evalN0(const double *kv, int nk, int i, int p, double xi)
{
  if (i == nk - p - 2 && fabs(xi - kv[nk - 1]) < 1.e-15 && fabs(kv[nk - 1] - kv[nk - 2]) < 1.e-15)
    return 1.0;
  if (p == 0) return (xi >= kv[i] && kv[i + 1] > xi) ? 1.0 : 0.0;
  double left = kv[i + p] - kv[i], right = kv[i + p + 1] - kv[i + 1];
  if (left == 0.0 && right == 0.0) return 0.0;
  if (left == 0.0) return (kv[i + p + 1] - xi) / right * evalN0(kv, nk, i + 1, p - 1, xi);
  if (right == 0.0) return (xi - kv[i]) / left * evalN0(kv, nk, i, p - 1, xi);
  return (xi - kv[i]) / left * evalN0(kv, nk, i, p - 1, xi) +
         (kv[i + p + 1] - xi) / right * evalN0(kv, nk, i + 1, p - 1, xi);
}

double orc_evalN(const double *kv, int nk, int k, int i, int p, double xi)
{
  if (k == 0) return evalN0(kv, nk, i, p, xi);
  if (k < 0 || k > p) return 0.0;
  double a[8][8];
  a[0][0] = 1.0;
  for (int r = 1; r <= k; r++) {
    double d0 = kv[i + p - r + 1] - kv[i];
    a[r][0] = d0 == 0.0 ? 0.0 : a[r - 1][0] / d0;
    for (int c = 1; c < r; c++) {
      double dc = kv[i + p + c - r + 1] - kv[i + c];
      a[r][c] = dc == 0.0 ? 0.0 : (a[r - 1][c] - a[r - 1][c - 1]) / dc;
    }
    double dr = kv[i + p + 1] - kv[i + r];
    a[r][r] = dr == 0.0 ? 0.0 : -a[r - 1][r - 1] / dr;
  }
  double s = 0.0;
  for (int j = 0; j <= k; j++) s += a[k][j] * evalN0(kv, nk, i + j, p - k, xi);
  double fac = 1.0;
  for (int j = p; j > p - k; j--) fac *= j; /* p!/(p-k)! */
  return s * fac;
}

/* ------------------------------------------------------------- geometry -- */
/* 3x3 inverse by cofactors (the role of matinv, src/mathutil.c:30-41). */
static void inv3(double *m)
{
  double c[9];
  c[0] = m[4] * m[8] - m[5] * m[7];
  c[1] = m[2] * m[7] - m[1] * m[8];
  c[2] = m[1] * m[5] - m[2] * m[4];
  c[3] = m[5] * m[6] - m[3] * m[8];
  c[4] = m[0] * m[8] - m[2] * m[6];
  c[5] = m[2] * m[3] - m[0] * m[5];
  c[6] = m[3] * m[7] - m[4] * m[6];
  c[7] = m[1] * m[6] - m[0] * m[7];
  c[8] = m[0] * m[4] - m[1] * m[3];
  double id = 1.0 / (m[0] * c[0] + m[1] * c[3] + m[2] * c[6]);
  for (int i = 0; i < 9; i++) m[i] = c[i] * id;
}

/* Physical basis R[nbpe][10] at one point, its Jacobian determinant and the
 * interpolated state u[(torder+1)*30]
 * (restates src/assmcore_iga.c:150-229). */
static void point_kernel(const OracleCase *c, int ex, int ey, int ez, const double xq[3],
                         const double *U_hist, double *R, double *detG_out, double *u)
{
  int p = c->p, q = p + 1, nbpe = q * q * q;
  const double *kv[3] = {c->knots[0] + ex, c->knots[1] + ey, c->knots[2] + ez};
  double N[64 * NDDIM];
  orc_eval_bspline(N, kv, p, xq);
  int nby = c->nbasis[1], nbz = c->nbasis[2];
  double wV[64], XV[3 * 64];
  long cp[64];
  for (int i = 0, b = 0; i < q; i++)
    for (int j = 0; j < q; j++)
      for (int k = 0; k < q; k++, b++) {
        cp[b] = (long)nby * nbz * (ex + i) + (long)nbz * (ey + j) + (ez + k);
        wV[b] = c->w[cp[b]];
        for (int d = 0; d < 3; d++) XV[3 * b + d] = c->X[3 * cp[b] + d];
      }
  /* rational basis by the quotient rule up to second order */
  double W[NDDIM] = {0};
  for (int b = 0; b < nbpe; b++)
    for (int k = 0; k < NDDIM; k++) W[k] += wV[b] * N[NDDIM * b + k];
  for (int b = 0; b < nbpe; b++) {
    double *r = R + NDDIM * b;
    const double *n = N + NDDIM * b;
    for (int k = 0; k < NDDIM; k++) r[k] = n[k] * wV[b] / W[0];
    for (int k = 1; k < NDDIM; k++) r[k] -= r[0] * W[k] / W[0];
    int a = 4;
    for (int i = 1; i < 4; i++)
      for (int j = i; j < 4; j++) r[a++] -= (r[j] * W[i] + r[i] * W[j]) / W[0];
  }
  /* geometry X (3 x 10) and its Jacobian G */
  double Xg[3 * NDDIM] = {0};
  for (int b = 0; b < nbpe; b++)
    for (int d = 0; d < 3; d++)
      for (int k = 0; k < NDDIM; k++) Xg[NDDIM * d + k] += XV[3 * b + d] * R[NDDIM * b + k];
  double G[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) G[3 * i + j] = Xg[NDDIM * i + 1 + j];
  *detG_out = G[0] * (G[4] * G[8] - G[5] * G[7]) - G[1] * (G[3] * G[8] - G[5] * G[6]) +
              G[2] * (G[3] * G[7] - G[4] * G[6]);
  inv3(G); /* G now holds dxi/dX */
  /* physical first and second derivatives */
  for (int b = 0; b < nbpe; b++) {
    double *r = R + NDDIM * b;
    double n[NDDIM];
    memcpy(n, r, sizeof(n));
    for (int i = 0; i < 3; i++) {
      r[1 + i] = 0.0;
      for (int j = 0; j < 3; j++) r[1 + i] += n[1 + j] * G[3 * j + i];
    }
    for (int k = 4; k < NDDIM; k++)
      for (int i = 0; i < 3; i++) n[k] -= r[1 + i] * Xg[NDDIM * i + k];
    /* symmetric parametric Hessian H (n[4..9]) -> G^T H G */
    double Hs[3][3] = {{n[4], n[5], n[6]}, {n[5], n[7], n[8]}, {n[6], n[8], n[9]}};
    int a = 4;
    for (int i = 0; i < 3; i++)
      for (int j = i; j < 3; j++) {
        double s = 0.0;
        for (int m = 0; m < 3; m++) {
          double t = 0.0;
          for (int l = 0; l < 3; l++) t += Hs[m][l] * G[3 * l + j];
          s += G[3 * m + i] * t;
        }
        r[a++] = s;
      }
  }
  /* interpolated state, every history level (src/assmcore_iga.c:209-224) */
  int nh = c->torder + 1;
  memset(u, 0, sizeof(double) * (size_t)nh * 30);
  for (int b = 0; b < nbpe; b++)
    for (int h = 0; h < nh; h++)
      for (int d = 0; d < NDOF; d++) {
        double Ub = U_hist[(long)h * c->ndof + NDOF * cp[b] + d];
        for (int k = 0; k < NDDIM; k++) u[30 * h + NDDIM * d + k] += R[NDDIM * b + k] * Ub;
      }
}

/* ---------------------------------------------------------------- pattern -- */
static long row_len(const OracleCase *c, int ix, int iy, int iz)
{
  int p = c->p, ii[3] = {ix, iy, iz};
  long n = NDOF;
  for (int d = 0; d < 3; d++) {
    int lo = ii[d] < p ? ii[d] : p;
    int hi = ii[d] > c->nbasis[d] - 1 - p ? c->nbasis[d] - 1 - ii[d] : p;
    n *= lo + 1 + hi;
  }
  return n;
}

static void build_pattern(OracleCase *c)
{
  int p = c->p, nbx = c->nbasis[0], nby = c->nbasis[1], nbz = c->nbasis[2];
  c->rowptr = (long *)malloc(sizeof(long) * ((size_t)c->ndof + 1));
  c->rowptr[0] = 0;
  long r = 0;
  for (int ix = 0; ix < nbx; ix++)
    for (int iy = 0; iy < nby; iy++)
      for (int iz = 0; iz < nbz; iz++)
        for (int d = 0; d < NDOF; d++, r++) c->rowptr[r + 1] = c->rowptr[r] + row_len(c, ix, iy, iz);
  c->nnz = c->rowptr[c->ndof];
  c->cols = (int *)malloc(sizeof(int) * (size_t)c->nnz);
  r = 0;
  for (int ix = 0; ix < nbx; ix++)
    for (int iy = 0; iy < nby; iy++)
      for (int iz = 0; iz < nbz; iz++)
        for (int d = 0; d < NDOF; d++, r++) {
          long s = c->rowptr[r];
          for (int jx = ix - p; jx <= ix + p; jx++) {
            if (jx < 0 || jx >= nbx) continue;
            for (int jy = iy - p; jy <= iy + p; jy++) {
              if (jy < 0 || jy >= nby) continue;
              for (int jz = iz - p; jz <= iz + p; jz++) {
                if (jz < 0 || jz >= nbz) continue;
                long cp = (long)nby * nbz * jx + (long)nbz * jy + jz;
                for (int e = 0; e < NDOF; e++) c->cols[s++] = (int)(NDOF * cp + e);
              }
            }
          }
        }
}

static double *csr_slot(const OracleCase *c, double *vals, int row, int col)
{
  long lo = c->rowptr[row], hi = c->rowptr[row + 1];
  while (lo < hi) {
    long mid = (lo + hi) / 2;
    if (c->cols[mid] < col) lo = mid + 1; else hi = mid;
  }
  return vals + lo; /* pattern is complete by construction */
}

/* ------------------------------------------------------------------- API -- */
OracleCase *orc_case_create(const int nelem[3], int p, const double *knots, const double *w,
                            const double *X, int law, const double *par, int nquad,
                            const int *bc_type, const double *par_dirichlet,
                            const double *neumann_tab)
{
  OracleCase *c = (OracleCase *)calloc(1, sizeof(OracleCase));
  c->p = p;
  long ncp = 1;
  const double *kv = knots;
  for (int d = 0; d < 3; d++) {
    c->nelem[d] = nelem[d];
    c->nbasis[d] = nelem[d] + p;
    c->nknot[d] = nelem[d] + 1 + 2 * p;
    c->knots[d] = (double *)malloc(sizeof(double) * (size_t)c->nknot[d]);
    memcpy(c->knots[d], kv, sizeof(double) * (size_t)c->nknot[d]);
    kv += c->nknot[d];
    ncp *= c->nbasis[d];
  }
  c->w = (double *)malloc(sizeof(double) * (size_t)ncp);
  c->X = (double *)malloc(sizeof(double) * 3 * (size_t)ncp);
  memcpy(c->w, w, sizeof(double) * (size_t)ncp);
  memcpy(c->X, X, sizeof(double) * 3 * (size_t)ncp);
  c->law = law;
  c->torder = law == ORC_LAW_GRADELASTTIME ? 2 : 0;
  orc_law_default_par(law, c->par);
  if (par) memcpy(c->par, par, sizeof(double) * 9);
  c->nquad = nquad > 0 ? nquad : 4;
  for (int i = 0; i < 36; i++) c->bc_type[i] = bc_type ? bc_type[i] : 1;
  for (int i = 0; i < 9; i++) c->par_dirichlet[i] = par_dirichlet ? par_dirichlet[i] : 0.0;
  for (int i = 0; i < 36; i++) c->neumann[i] = neumann_tab ? neumann_tab[i] : 0.0;
  c->ndof = (int)(NDOF * ncp);
  build_pattern(c);
  return c;
}

void orc_case_destroy(OracleCase *c)
{
  if (!c) return;
  for (int d = 0; d < 3; d++) free(c->knots[d]);
  free(c->w); free(c->X); free(c->rowptr); free(c->cols); free(c);
}
int orc_case_ndof(const OracleCase *c) { return c->ndof; }
int orc_case_torder(const OracleCase *c) { return c->torder; }
long orc_case_nnz(const OracleCase *c) { return c->nnz; }
void orc_case_pattern(const OracleCase *c, long *rowptr, int *cols)
{
  memcpy(rowptr, c->rowptr, sizeof(long) * ((size_t)c->ndof + 1));
  memcpy(cols, c->cols, sizeof(int) * (size_t)c->nnz);
}

static void elem_coords(const OracleCase *c, long e, int *ex, int *ey, int *ez)
{
  *ez = (int)(e % c->nelem[2]);
  *ey = (int)((e / c->nelem[2]) % c->nelem[1]);
  *ex = (int)(e / ((long)c->nelem[1] * c->nelem[2]));
}

/* volume residual of elements [e0,e1) (src/assmcore_iga.c:118-259) */
void orc_case_residual_elements(const OracleCase *c, const double *U_hist, double *RR, long e0,
                                long e1)
{
  int p = c->p, q = p + 1, nbpe = q * q * q, nq = c->nquad;
  double cq[16], wq[16];
  orc_gauss_legendre(nq, 0.0, 1.0, cq, wq);
  double R[64 * NDDIM], u[90], rr[30], val[3 * 64];
  int nby = c->nbasis[1], nbz = c->nbasis[2];
  for (long e = e0; e < e1; e++) {
    int ex, ey, ez;
    elem_coords(c, e, &ex, &ey, &ez);
    double x0[3] = {c->knots[0][ex + p], c->knots[1][ey + p], c->knots[2][ez + p]};
    double x1[3] = {c->knots[0][ex + p + 1], c->knots[1][ey + p + 1], c->knots[2][ez + p + 1]};
    memset(val, 0, sizeof(val));
    for (int qx = 0; qx < nq; qx++)
      for (int qy = 0; qy < nq; qy++)
        for (int qz = 0; qz < nq; qz++) {
          double xq[3] = {(-cq[qx] + 1.0) * x0[0] + cq[qx] * x1[0],
                          (-cq[qy] + 1.0) * x0[1] + cq[qy] * x1[1],
                          (-cq[qz] + 1.0) * x0[2] + cq[qz] * x1[2]};
          double detG;
          point_kernel(c, ex, ey, ez, xq, U_hist, R, &detG, u);
          orc_law_residual(c->law, rr, u, c->par);
          double wt = wq[qx] * wq[qy] * wq[qz] * (x1[0] - x0[0]) * (x1[1] - x0[1]) * (x1[2] - x0[2]) * detG;
          for (int b = 0; b < nbpe; b++)
            for (int d = 0; d < NDOF; d++) {
              double t = 0.0;
              for (int k = 0; k < NDDIM; k++) t += R[NDDIM * b + k] * rr[NDDIM * d + k];
              val[NDOF * b + d] += wt * t;
            }
        }
    for (int i = 0, b = 0; i < q; i++)
      for (int j = 0; j < q; j++)
        for (int k = 0; k < q; k++, b++) {
          long cp = (long)nby * nbz * (ex + i) + (long)nbz * (ey + j) + (ez + k);
          for (int d = 0; d < NDOF; d++) RR[NDOF * cp + d] += val[NDOF * b + d];
        }
  }
}

/* Face frame: (u,v) face-parallel directions, n the normal; strides in the
 * control-point numbering (src/assmcore_iga.c:276-313). */
static void face_frame(const OracleCase *c, int face, int dir[3], long stride[3])
{
  long sx = (long)c->nbasis[1] * c->nbasis[2], sy = c->nbasis[2], sz = 1;
  switch (face / 2) {
  case 0: dir[0] = 1; dir[1] = 2; dir[2] = 0; stride[0] = sy; stride[1] = sz; stride[2] = sx; break;
  case 1: dir[0] = 0; dir[1] = 2; dir[2] = 1; stride[0] = sx; stride[1] = sz; stride[2] = sy; break;
  default: dir[0] = 0; dir[1] = 1; dir[2] = 2; stride[0] = sx; stride[1] = sy; stride[2] = sz; break;
  }
}

/* Dirichlet data on one face layer (restates dirichlet_iga,
 * src/assmcore_iga.c:861-934): affine u_d = a.X interpolated in the face
 * spline space. out has nbasis[dir0]*nbasis[dir1] entries. */
static void dirichlet_face(const OracleCase *c, int face, int order, int d, double *out)
{
  int dir[3]; long st[3];
  face_frame(c, face, dir, st);
  int p = c->p;
  double pf[3];
  pf[0] = c->par_dirichlet[3 * d + dir[0]];
  pf[1] = c->par_dirichlet[3 * d + dir[1]];
  pf[2] = c->par_dirichlet[3 * d + dir[2]];
  const double *kn = c->knots[dir[2]];
  int nkn = c->nknot[dir[2]];
  double Z = (face % 2 == 0) ? kn[0] : kn[nkn - 1] - 1.e-15;
  double *d1[2];
  for (int b = 0; b < 2; b++) {
    int dd = dir[b], nb = c->nbasis[dd];
    const double *kv = c->knots[dd];
    d1[b] = (double *)malloc(sizeof(double) * (size_t)nb);
    double W0 = kv[p];
    double vec[8] = {0}, mat[64];
    vec[0] = pf[b] * W0;
    if (p > 1) vec[1] = pf[b];
    for (int i = 0; i < p; i++)
      for (int j = 0; j < p; j++) mat[p * i + j] = orc_evalN(kv, c->nknot[dd], i, j, p, W0);
    /* solve mat . x = vec (small dense, Gaussian elimination with pivoting) */
    double x[8];
    {
      double A[64], bb[8];
      memcpy(A, mat, sizeof(double) * (size_t)(p * p));
      memcpy(bb, vec, sizeof(double) * (size_t)p);
      for (int k = 0; k < p; k++) {
        int piv = k;
        for (int r = k + 1; r < p; r++) if (fabs(A[p * r + k]) > fabs(A[p * piv + k])) piv = r;
        for (int cc = 0; cc < p; cc++) { double t = A[p * k + cc]; A[p * k + cc] = A[p * piv + cc]; A[p * piv + cc] = t; }
        { double t = bb[k]; bb[k] = bb[piv]; bb[piv] = t; }
        for (int r = k + 1; r < p; r++) {
          double f = A[p * r + k] / A[p * k + k];
          for (int cc = k; cc < p; cc++) A[p * r + cc] -= f * A[p * k + cc];
          bb[r] -= f * bb[k];
        }
      }
      for (int k = p - 1; k >= 0; k--) {
        double s = bb[k];
        for (int cc = k + 1; cc < p; cc++) s -= A[p * k + cc] * x[cc];
        x[k] = s / A[p * k + k];
      }
    }
    for (int i = 0; i < p; i++) d1[b][i] = x[i];
    for (int i = p; i < nb; i++) d1[b][i] = d1[b][i - 1] + (kv[i + p] - kv[i]) / ((double)p) * pf[b];
  }
  int n0 = c->nbasis[dir[0]], n1 = c->nbasis[dir[1]];
  for (int i = 0; i < n0; i++)
    for (int j = 0; j < n1; j++) out[(long)n1 * i + j] = d1[0][i] + d1[1][j] + pf[2] * Z;
  (void)order; /* the high-order layer adds 0 (src/assmcore_iga.c:929-930) */
  free(d1[0]); free(d1[1]);
}

void orc_case_residual(const OracleCase *c, const double *U_hist, double *RR)
{
  memset(RR, 0, sizeof(double) * (size_t)c->ndof);
  long nel = (long)c->nelem[0] * c->nelem[1] * c->nelem[2];
  orc_case_residual_elements(c, U_hist, RR, 0, nel);
  int p = c->p, q = p + 1, nq = c->nquad;
  double cq[16], wq[16];
  orc_gauss_legendre(nq, 0.0, 1.0, cq, wq);
  /* Neumann faces, standard and high order (src/assmcore_iga.c:273-405) */
  for (int face = 0; face < 6; face++) {
    int dir[3]; long st[3];
    face_frame(c, face, dir, st);
    const double *kn = c->knots[dir[2]];
    int nkn = c->nknot[dir[2]];
    double zq = (face % 2 == 0) ? kn[0] : kn[nkn - 1];
    int lay0 = (face % 2 == 0) ? 0 : c->nelem[dir[2]] + p - 1;
    int lay1 = (face % 2 == 0) ? 1 : c->nelem[dir[2]] + p - 2;
    for (int order = 0; order < 2; order++)
      for (int d = 0; d < NDOF; d++) {
        if (c->bc_type[6 * face + 3 * order + d] != 1) continue;
        double t = c->neumann[6 * face + 3 * order + d];
        for (int ea = 0; ea < c->nelem[dir[0]]; ea++)
          for (int eb = 0; eb < c->nelem[dir[1]]; eb++) {
            const double *ka = c->knots[dir[0]], *kb = c->knots[dir[1]];
            double a0 = ka[ea + p], a1 = ka[ea + p + 1], b0 = kb[eb + p], b1 = kb[eb + p + 1];
            double v[2 * 64];
            memset(v, 0, sizeof(v));
            for (int qa = 0; qa < nq; qa++)
              for (int qb = 0; qb < nq; qb++) {
                double xa = (-cq[qa] + 1.0) * a0 + cq[qa] * a1;
                double xb = (-cq[qb] + 1.0) * b0 + cq[qb] * b1;
                double wt = wq[qa] * wq[qb] * (a1 - a0) * (b1 - b0);
                int ia = 0;
                for (int i = 0; i < q; i++)
                  for (int j = 0; j < q; j++) {
                    double Nab = orc_evalN(ka, c->nknot[dir[0]], 0, ea + i, p, xa) *
                                 orc_evalN(kb, c->nknot[dir[1]], 0, eb + j, p, xb);
                    if (order == 0) {
                      v[ia++] -= wt * Nab * t;
                    } else {
                      v[ia++] -= wt * (Nab * orc_evalN(kn, nkn, 1, lay0, p, zq)) * t;
                      v[ia++] -= wt * (Nab * orc_evalN(kn, nkn, 1, lay1, p, zq)) * t;
                    }
                  }
              }
            int ia = 0;
            for (int i = 0; i < q; i++)
              for (int j = 0; j < q; j++) {
                long base = st[0] * (ea + i) + st[1] * (eb + j);
                RR[NDOF * (base + st[2] * lay0) + d] += v[ia++];
                if (order == 1) RR[NDOF * (base + st[2] * lay1) + d] += v[ia++];
              }
          }
      }
  }
  /* Dirichlet rows: U - g, inserted after the additive phase
   * (src/assmcore_iga.c:411-494) */
  for (int face = 0; face < 6; face++) {
    int dir[3]; long st[3];
    face_frame(c, face, dir, st);
    int nz = c->nbasis[dir[2]];
    int layer[2] = {(face % 2 == 0) ? 0 : nz - 1, (face % 2 == 0) ? 1 : nz - 2};
    int n0 = c->nbasis[dir[0]], n1 = c->nbasis[dir[1]];
    double *g = (double *)malloc(sizeof(double) * (size_t)n0 * n1);
    for (int order = 0; order < 2; order++)
      for (int d = 0; d < NDOF; d++) {
        if (c->bc_type[6 * face + 3 * order + d] != 0) continue;
        dirichlet_face(c, face, order, d, g);
        for (int i = 0; i < n0; i++)
          for (int j = 0; j < n1; j++) {
            long row = NDOF * (st[0] * i + st[1] * j + st[2] * layer[order]) + d;
            RR[row] = U_hist[row] - g[(long)n1 * i + j];
          }
      }
    free(g);
  }
}

/* volume tangent of elements [e0,e1) (src/assmcore_iga.c:607-764) */
void orc_case_tangent_elements(const OracleCase *c, const double *U_hist, double *vals, long e0,
                               long e1)
{
  int p = c->p, q = p + 1, nbpe = q * q * q, nq = c->nquad, ne = NDOF * nbpe;
  double cq[16], wq[16];
  orc_gauss_legendre(nq, 0.0, 1.0, cq, wq);
  double R[64 * NDDIM], u[90], tt[900];
  double *val = (double *)malloc(sizeof(double) * (size_t)ne * ne);
  int idx[3 * 64];
  int nby = c->nbasis[1], nbz = c->nbasis[2];
  for (long e = e0; e < e1; e++) {
    int ex, ey, ez;
    elem_coords(c, e, &ex, &ey, &ez);
    double x0[3] = {c->knots[0][ex + p], c->knots[1][ey + p], c->knots[2][ez + p]};
    double x1[3] = {c->knots[0][ex + p + 1], c->knots[1][ey + p + 1], c->knots[2][ez + p + 1]};
    memset(val, 0, sizeof(double) * (size_t)ne * ne);
    for (int qx = 0; qx < nq; qx++)
      for (int qy = 0; qy < nq; qy++)
        for (int qz = 0; qz < nq; qz++) {
          double xq[3] = {(-cq[qx] + 1.0) * x0[0] + cq[qx] * x1[0],
                          (-cq[qy] + 1.0) * x0[1] + cq[qy] * x1[1],
                          (-cq[qz] + 1.0) * x0[2] + cq[qz] * x1[2]};
          double detG;
          point_kernel(c, ex, ey, ez, xq, U_hist, R, &detG, u);
          orc_law_tangent(c->law, tt, u, c->par);
          double wt = wq[qx] * wq[qy] * wq[qz] * (x1[0] - x0[0]) * (x1[1] - x0[1]) * (x1[2] - x0[2]) * detG;
          for (int b = 0; b < nbpe; b++)
            for (int d = 0; d < NDOF; d++) {
              int row = NDOF * b + d;
              for (int b2 = 0; b2 < nbpe; b2++)
                for (int d2 = 0; d2 < NDOF; d2++) {
                  double t = 0.0;
                  for (int k = 0; k < NDDIM; k++)
                    for (int l = 0; l < NDDIM; l++)
                      t += R[NDDIM * b + k] * tt[30 * (NDDIM * d + k) + (NDDIM * d2 + l)] * R[NDDIM * b2 + l];
                  val[(long)ne * row + NDOF * b2 + d2] += wt * t;
                }
            }
        }
    for (int i = 0, b = 0; i < q; i++)
      for (int j = 0; j < q; j++)
        for (int k = 0; k < q; k++, b++) {
          long cp = (long)nby * nbz * (ex + i) + (long)nbz * (ey + j) + (ez + k);
          for (int d = 0; d < NDOF; d++) idx[NDOF * b + d] = (int)(NDOF * cp + d);
        }
    for (int r = 0; r < ne; r++)
      for (int cc = 0; cc < ne; cc++) *csr_slot(c, vals, idx[r], idx[cc]) += val[(long)ne * r + cc];
  }
  free(val);
}

void orc_case_tangent(const OracleCase *c, const double *U_hist, double *vals)
{
  memset(vals, 0, sizeof(double) * (size_t)c->nnz);
  long nel = (long)c->nelem[0] * c->nelem[1] * c->nelem[2];
  orc_case_tangent_elements(c, U_hist, vals, 0, nel);
  /* Dirichlet rows and columns zeroed, unit diagonal
   * (MatZeroRowsColumns at src/assmcore_iga.c:780-846) */
  char *flag = (char *)calloc((size_t)c->ndof, 1);
  for (int face = 0; face < 6; face++) {
    int dir[3]; long st[3];
    face_frame(c, face, dir, st);
    int nz = c->nbasis[dir[2]];
    int layer[2] = {(face % 2 == 0) ? 0 : nz - 1, (face % 2 == 0) ? 1 : nz - 2};
    for (int order = 0; order < 2; order++)
      for (int d = 0; d < NDOF; d++) {
        if (c->bc_type[6 * face + 3 * order + d] != 0) continue;
        for (int i = 0; i < c->nbasis[dir[0]]; i++)
          for (int j = 0; j < c->nbasis[dir[1]]; j++)
            flag[NDOF * (st[0] * i + st[1] * j + st[2] * layer[order]) + d] = 1;
      }
  }
  for (int r = 0; r < c->ndof; r++)
    for (long s = c->rowptr[r]; s < c->rowptr[r + 1]; s++)
      if (flag[r] || flag[c->cols[s]]) vals[s] = (flag[r] && c->cols[s] == r) ? 1.0 : 0.0;
  free(flag);
}

/* ------------------------------------------------------- field sampling -- */
/* iga_plotfield's sampling loop (src/mgl/plotcore_iga.c:16-282, restated in
 * field_sampling.h) with this file's basis and inverse and the restated
 * field callbacks of laws.c. */
#include "field_sampling.h"

int orc_law_field(int law, double *f, const double *u, const double *par);
static void fs_orc_basis(double *N, double *kv[3], int p, double xq[3])
{
  const double *k[3] = {kv[0], kv[1], kv[2]};
  orc_eval_bspline(N, k, p, xq);
}
static void fs_field_gradelast(double *f, double *u, double *par) { orc_law_field(ORC_LAW_GRADELAST, f, u, par); }
static void fs_field_gradelasttime(double *f, double *u, double *par)
{
  orc_law_field(ORC_LAW_GRADELASTTIME, f, u, par);
}
static void fs_field_lingrad(double *f, double *u, double *par) { orc_law_field(ORC_LAW_LINGRAD, f, u, par); }

int orc_case_field(OracleCase *c, const double *U_hist, int nppe, double *field, double *xq, double *X)
{
  const int nf = c->law == ORC_LAW_GRADELASTTIME ? 6 : 33;
  fs_field_fn fn = c->law == ORC_LAW_GRADELAST       ? fs_field_gradelast
                   : c->law == ORC_LAW_GRADELASTTIME ? fs_field_gradelasttime
                                                     : fs_field_lingrad;
  fs_sample(c->p, c->nelem, c->knots, c->w, c->X, U_hist, c->ndof, c->torder + 1, c->par, nf, nppe, fs_orc_basis,
            inv3, fn, field, xq, X);
  return nf;
}
