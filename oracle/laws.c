/*
 * Law dispatch of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 * Default parameters are those of the reference's plugin constructors
 * (phys/physgradelast.c:21, phys/physgradelasttime.c:21) and the linear law's
 * lambda = mu = 1, ell = 0.1.
 */
#include <math.h>
#include <string.h>
#include "igap_oracle.h"

void lingrad_residual(double *rr, double *u, double *par);
void lingrad_tangent(double *tt, double *u, double *par);
void lingrad_field(double *f, double *u, double *par);
void gradelast_law_residual(double *rr, const double *u, const double *par);
void gradelast_law_tangent(double *tt, const double *u, const double *par);
void gradelasttime_law_residual(double *rr, const double *u, const double *par);
void gradelasttime_law_tangent(double *tt, const double *u, const double *par);

void orc_law_default_par(int law, double *par)
{
  static const double st[9] = {0.25, 0.50, 360., 180., 0.05, 1.0, 1.0, 1.e-3 * (1. / 2.), 0.0};
  static const double tr[9] = {0.25, 0.50, 500., 250., 0.025, 1.0, 1.0, 1.e-3 * (1. / 2.), 0.0};
  static const double li[9] = {1.0, 1.0, 0.1, 0, 0, 0, 0, 0, 0};
  memcpy(par, law == ORC_LAW_GRADELAST ? st : law == ORC_LAW_GRADELASTTIME ? tr : li,
         9 * sizeof(double));
}

void orc_law_residual(int law, double *rr, const double *u, const double *par)
{
  if (law == ORC_LAW_GRADELAST) gradelast_law_residual(rr, u, par);
  else if (law == ORC_LAW_GRADELASTTIME) gradelasttime_law_residual(rr, u, par);
  else lingrad_residual(rr, (double *)u, (double *)par);
}

void orc_law_tangent(int law, double *tt, const double *u, const double *par)
{
  if (law == ORC_LAW_GRADELAST) gradelast_law_tangent(tt, u, par);
  else if (law == ORC_LAW_GRADELASTTIME) gradelasttime_law_tangent(tt, u, par);
  else lingrad_tangent(tt, (double *)u, (double *)par);
}

/* Deviatoric strain coordinates of the Green-Lagrange strain of u (30
 * entries): E = (F^T F - I)/2 with F = I + grad u, e1 = (E00 - E11)/sqrt 2,
 * e2 = (E00 + E11 - 2 E22)/sqrt 6 (the comp[25], comp[26] of the field
 * callbacks, phys/gradelast.c:1107-1147). */
static void strain_e1e2(const double *u, double *e1, double *e2)
{
  double F[3][3], E[3];
  for (int k = 0; k < 3; k++)
    for (int a = 0; a < 3; a++) F[k][a] = (k == a ? 1.0 : 0.0) + u[10 * k + 1 + a];
  for (int a = 0; a < 3; a++) {
    double v = 0.0;
    for (int k = 0; k < 3; k++) v += F[k][a] * F[k][a];
    E[a] = 0.5 * (v - 1.0);
  }
  *e1 = (E[0] - E[1]) / sqrt(2.0);
  *e2 = (E[0] + E[1] - 2.0 * E[2]) / sqrt(6.0);
}

/* Sector code of (e1, e2) in the normalised Landau polynomial
 *   phi = (3/2 rho^2 + 2 r (1-c) e2 (e2^2 - 3 e1^2) - 3 r^2 c rho) / (r^4 (1/2 + c)),
 * rho = e1^2 + e2^2, r = par[0], c = par[1] (phys/gradelast.c:1151-1155):
 * inside the well phi < -1/2: 3 if e2 < 0, else 1 if e1 > 0, else 2 if e1 < 0. */
static double sector_code(double e1, double e2, const double *par)
{
  const double r = par[0], c = par[1], rho = e1 * e1 + e2 * e2;
  const double phi = (1.5 * rho * rho + 2.0 * r * (1.0 - c) * e2 * (e2 * e2 - 3.0 * e1 * e1) - 3.0 * r * r * c * rho) /
                     (r * r * r * r * (0.5 + c));
  if (phi < -0.5) {
    if (e2 < 0.0) return 3.0;
    if (e1 > 0.0) return 1.0;
    if (e1 < 0.0) return 2.0;
  }
  return 0.0;
}

/* Field callbacks (field_ptr, include/physimpl.h:8), restated: gradelast 33
 * values (u, e1, e2, sector code; phys/gradelast.c:1105-1156), gradelasttime
 * 6 (midpoint displacement of levels 1 and 2, e1, e2, sector code;
 * phys/gradelasttime.c:9242-9297), the linear law 33 (law_lingrad.c).
 * Returns the number of fields. */
int orc_law_field(int law, double *f, const double *u, const double *par)
{
  double e1, e2;
  if (law == ORC_LAW_GRADELAST) {
    for (int i = 0; i < 30; i++) f[i] = u[i];
    strain_e1e2(u, &e1, &e2);
    f[30] = e1;
    f[31] = e2;
    f[32] = sector_code(e1, e2, par);
    return 33;
  }
  if (law == ORC_LAW_GRADELASTTIME) {
    double mid[30];
    for (int i = 0; i < 30; i++) mid[i] = 0.5 * (u[30 + i] + u[60 + i]);
    for (int d = 0; d < 3; d++) f[d] = mid[10 * d];
    strain_e1e2(mid, &e1, &e2);
    f[3] = e1;
    f[4] = e2;
    f[5] = sector_code(e1, e2, par);
    return 6;
  }
  lingrad_field(f, (double *)u, (double *)par);
  return 33;
}
