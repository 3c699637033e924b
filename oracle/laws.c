/*
 * Law dispatch of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 * Default parameters are those of the reference's plugin constructors
 * (phys/physgradelast.c:21, phys/physgradelasttime.c:21) and the linear law's
 * lambda = mu = 1, ell = 0.1.
 */
#include <string.h>
#include "igap_oracle.h"

void lingrad_residual(double *rr, double *u, double *par);
void lingrad_tangent(double *tt, double *u, double *par);
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
