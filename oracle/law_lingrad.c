/*
 * Linear isotropic strain-gradient law (lambda, mu, ell) -- CPU definition.
 *
 * The reference has no such law; this is the project's own plugin with the
 * reference's per-point callback ABI (residual_ptr / tangent_ptr,
 * include/physimpl.h:6-7): u[10*d+k] holds displacement component d with
 * k = 0 value, 1..3 d/dx,dy,dz, 4..9 d2/dxx,dxy,dxz,dyy,dyz,dzz (the layout the
 * assembly builds at src/assmcore_iga.c:209-229); rr[10*d+k] = dpsi/du[10*d+k];
 * tt[30*row+col] = d rr[row] / d u[col].
 *
 * Energy (small strain eps = sym grad u, kappa_ijm = d_m eps_ij):
 *   psi = lambda/2 (eps_kk)^2 + mu eps_ij eps_ij
 *       + ell^2 [ lambda/2 (kappa_kkm kappa_kkm) + mu kappa_ijm kappa_ijm ]
 * par = {lambda, mu, ell}.  The law is linear, so tt is constant and
 * rr = tt . u exactly.
 *
 * Test infrastructure (oracle): the device law in the product is written
 * independently and checked against this file.
 */
#include <math.h>
#include <string.h>

static const int SYM_J[6] = {0, 0, 0, 1, 1, 2};
static const int SYM_M[6] = {0, 1, 2, 1, 2, 2};

static int sym_index(int j, int m)
{
  if (j > m) { int t = j; j = m; m = t; }
  for (int s = 0; s < 6; s++)
    if (SYM_J[s] == j && SYM_M[s] == m) return s;
  return -1;
}

void lingrad_residual(double *rr, double *u, double *par)
{
  const double lam = par[0], mu = par[1], ell = par[2];
  double g[3][3];    /* g[i][j] = u_i,j */
  double h[3][3][3]; /* h[i][j][m] = u_i,jm */
  for (int i = 0; i < 3; i++) {
    for (int j = 0; j < 3; j++) g[i][j] = u[10 * i + 1 + j];
    for (int j = 0; j < 3; j++)
      for (int m = 0; m < 3; m++) h[i][j][m] = u[10 * i + 4 + sym_index(j, m)];
  }
  double eps[3][3], kap[3][3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      eps[i][j] = 0.5 * (g[i][j] + g[j][i]);
      for (int m = 0; m < 3; m++) kap[i][j][m] = 0.5 * (h[i][j][m] + h[j][i][m]);
    }
  double tr = eps[0][0] + eps[1][1] + eps[2][2];
  double trk[3];
  for (int m = 0; m < 3; m++) trk[m] = kap[0][0][m] + kap[1][1][m] + kap[2][2][m];
  double sig[3][3], tau[3][3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      sig[i][j] = 2.0 * mu * eps[i][j] + (i == j ? lam * tr : 0.0);
      for (int m = 0; m < 3; m++)
        tau[i][j][m] = ell * ell * (2.0 * mu * kap[i][j][m] + (i == j ? lam * trk[m] : 0.0));
    }
  for (int d = 0; d < 3; d++) {
    rr[10 * d] = 0.0;
    for (int j = 0; j < 3; j++) rr[10 * d + 1 + j] = sig[d][j];
    for (int s = 0; s < 6; s++) {
      int j = SYM_J[s], m = SYM_M[s];
      rr[10 * d + 4 + s] = (j == m) ? tau[d][j][j] : tau[d][j][m] + tau[d][m][j];
    }
  }
}

void lingrad_tangent(double *tt, double *u, double *par)
{
  (void)u;
  double e[30], col[30];
  for (int c = 0; c < 30; c++) {
    memset(e, 0, sizeof(e));
    e[c] = 1.0;
    lingrad_residual(col, e, par);
    for (int r = 0; r < 30; r++) tt[30 * r + c] = col[r];
  }
}

/* Densities for the integral of the law over the body, in the layout of the
 * reference's density callbacks (include/physimpl.h:9-10): h[0] the stored
 * energy psi above, h[1] = 1 (the integral is the volume).  Boundary: h[0] =
 * u0 * traction (the traction's work term), h[1] = 0. */
void lingrad_density(double h[], double u[], double *par)
{
  const double lam = par[0], mu = par[1], ell = par[2];
  double eps[3][3], kap[3][3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      eps[i][j] = 0.5 * (u[10 * i + 1 + j] + u[10 * j + 1 + i]);
      for (int m = 0; m < 3; m++)
        kap[i][j][m] = 0.5 * (u[10 * i + 4 + sym_index(j, m)] + u[10 * j + 4 + sym_index(i, m)]);
    }
  double tr = eps[0][0] + eps[1][1] + eps[2][2], ee = 0.0, kk = 0.0, tk = 0.0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      ee += eps[i][j] * eps[i][j];
      for (int m = 0; m < 3; m++) kk += kap[i][j][m] * kap[i][j][m];
    }
  for (int m = 0; m < 3; m++) {
    const double t = kap[0][0][m] + kap[1][1][m] + kap[2][2][m];
    tk += t * t;
  }
  h[0] = 0.5 * lam * tr * tr + mu * ee + ell * ell * (0.5 * lam * tk + mu * kk);
  h[1] = 1.0;
}

void lingrad_densityb(double h[], double u[], double traction, double *par, int order)
{
  (void)par;
  (void)order;
  h[0] = u[0] * traction;
  h[1] = 0.0;
}

/* Field callback of the linear law (field_ptr, include/physimpl.h:8), 33
 * values in the static gradient law's layout: f[0..29] = u, f[30] = tr eps,
 * f[31] = |dev eps|, f[32] = psi. */
void lingrad_field(double *f, double *u, double *par)
{
  for (int i = 0; i < 30; i++) f[i] = u[i];
  double eps[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) eps[i][j] = 0.5 * (u[10 * i + 1 + j] + u[10 * j + 1 + i]);
  const double tr = eps[0][0] + eps[1][1] + eps[2][2];
  double dd = 0.0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      const double v = eps[i][j] - (i == j ? tr / 3.0 : 0.0);
      dd += v * v;
    }
  double h[2];
  lingrad_density(h, u, par);
  f[30] = tr;
  f[31] = sqrt(dd);
  f[32] = h[0];
}
