/*
 * Field sampling on the plot lattice (TEST INFRASTRUCTURE ONLY): the sampling
 * loop of iga_plotfield (src/mgl/plotcore_iga.c:16-282) restated without the
 * MathGL rendering.  The reference file itself does not compile: it declares
 * `BC *bc = app->bc[0]` for a BC handle (plotcore_iga.c:45) and dereferences
 * it as a struct (:47).  So the loop here is the project's; the tensor-product
 * basis, the 3x3 inverse and the law's field callback are passed in -- the
 * reference's compiled eval_Bspline / matinv / phys->field in
 * oracle/ref_driver.c, the project's restatements in oracle/igap_oracle.c.
 *
 * Lattice: nppe samples per element and direction plus the far face of the
 * last element, (nppe nelem[d] + 1) points per direction, stored x-major,
 * z fastest.  Sample s of element e in direction d sits at the knot
 * coordinate (k0 + 1e-15) + (k1 - k0) s / nppe - 2e-15 [s == nppe], k0 and k1
 * the element's knot span (plotcore_iga.c:166-168, same order of operations).
 * Affine periodic terms (par_periodic) are not added: the path rejects
 * periodic meshes.
 */
#ifndef IGAP_FIELD_SAMPLING_H
#define IGAP_FIELD_SAMPLING_H

#include <string.h>

typedef void (*fs_basis_fn)(double *N, double *kv[3], int p, double xq[3]);
typedef void (*fs_inverse_fn)(double *G); /* 3 x 3 row-major, in place */
typedef void (*fs_field_fn)(double *f, double *u, double *par);

/* U: [nlev][ldu] state, DOF 3 cp + d of control point cp (x-major, z fastest).
 * Outputs (any may be NULL): f [npoints][nfield], xq and X [npoints][3]. */
static void fs_sample(int p, const int nelem[3], double *const knots[3], const double *w, const double *X,
                      const double *U, long ldu, int nlev, double *par, int nfield, int nppe,
                      fs_basis_fn basis, fs_inverse_fn inverse, fs_field_fn field, double *out_f,
                      double *out_xq, double *out_X)
{
  enum { ND = 10, MAXB = 64 };
  const int q = p + 1, nb = q * q * q;
  const long n[3] = {(long)nppe * nelem[0] + 1, (long)nppe * nelem[1] + 1, (long)nppe * nelem[2] + 1};
  const long nby = nelem[1] + p, nbz = nelem[2] + p;
  double N[MAXB * ND], R[MAXB * ND], W[ND], Xg[3 * ND], G[9], u[3 * 30], f[64], wV[MAXB], XV[3 * MAXB];
  long cp[MAXB];
  for (long gx = 0; gx < n[0]; gx++)
    for (long gy = 0; gy < n[1]; gy++)
      for (long gz = 0; gz < n[2]; gz++) {
        const long g[3] = {gx, gy, gz};
        int e[3], s[3];
        double xq[3];
        double *kv[3];
        for (int d = 0; d < 3; d++) {
          e[d] = (int)(g[d] / nppe);
          if (e[d] == nelem[d]) e[d]--; /* the far face belongs to the last element */
          s[d] = (int)(g[d] - (long)nppe * e[d]);
          const double k0 = knots[d][e[d] + p], k1 = knots[d][e[d] + p + 1];
          xq[d] = k0 + 1.e-15 + (k1 - k0) * s[d] / nppe - 2 * 1.e-15 * (s[d] == nppe);
          kv[d] = knots[d] + e[d];
        }
        for (int i = 0, b = 0; i < q; i++)
          for (int j = 0; j < q; j++)
            for (int k = 0; k < q; k++, b++) {
              cp[b] = nby * nbz * (e[0] + i) + nbz * (e[1] + j) + (e[2] + k);
              wV[b] = w[cp[b]];
              for (int d = 0; d < 3; d++) XV[3 * b + d] = X[3 * cp[b] + d];
            }
        basis(N, kv, p, xq);
        /* rational basis by the quotient rule, second order */
        for (int k = 0; k < ND; k++) {
          W[k] = 0.0;
          for (int b = 0; b < nb; b++) W[k] += wV[b] * N[ND * b + k];
        }
        for (int b = 0; b < nb; b++) {
          double *r = R + ND * b;
          for (int k = 0; k < ND; k++) r[k] = N[ND * b + k] * wV[b] / W[0];
          for (int k = 1; k < ND; k++) r[k] -= r[0] * W[k] / W[0];
          int a = 4;
          for (int i = 1; i < 4; i++)
            for (int j = i; j < 4; j++) r[a++] -= (r[j] * W[i] + r[i] * W[j]) / W[0];
        }
        /* geometry, its Jacobian and the inverse */
        for (int i = 0; i < 3 * ND; i++) Xg[i] = 0.0;
        for (int b = 0; b < nb; b++)
          for (int d = 0; d < 3; d++)
            for (int k = 0; k < ND; k++) Xg[ND * d + k] += XV[3 * b + d] * R[ND * b + k];
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) G[3 * i + j] = Xg[ND * i + 1 + j];
        inverse(G);
        /* physical first and second derivatives */
        for (int b = 0; b < nb; b++) {
          double *r = R + ND * b, t[ND];
          memcpy(t, r, sizeof(t));
          for (int i = 0; i < 3; i++) {
            r[1 + i] = 0.0;
            for (int j = 0; j < 3; j++) r[1 + i] += t[1 + j] * G[3 * j + i];
          }
          for (int k = 4; k < ND; k++)
            for (int i = 0; i < 3; i++) t[k] -= r[1 + i] * Xg[ND * i + k];
          const double H[3][3] = {{t[4], t[5], t[6]}, {t[5], t[7], t[8]}, {t[6], t[8], t[9]}};
          int a = 4;
          for (int i = 0; i < 3; i++)
            for (int j = i; j < 3; j++) {
              double acc = 0.0;
              for (int m = 0; m < 3; m++) {
                double h = 0.0;
                for (int l = 0; l < 3; l++) h += H[m][l] * G[3 * l + j];
                acc += G[3 * m + i] * h;
              }
              r[a++] = acc;
            }
        }
        /* state of every level (plotcore_iga.c:228-248) */
        memset(u, 0, sizeof(u));
        for (int b = 0; b < nb; b++)
          for (int h = 0; h < nlev; h++)
            for (int d = 0; d < 3; d++) {
              const double ub = U[(long)h * ldu + 3 * cp[b] + d];
              for (int k = 0; k < ND; k++) u[30 * h + ND * d + k] += R[ND * b + k] * ub;
            }
        const long o = (gx * n[1] + gy) * n[2] + gz;
        if (out_f) {
          field(f, u, par);
          for (int i = 0; i < nfield; i++) out_f[o * nfield + i] = f[i];
        }
        for (int d = 0; d < 3; d++) {
          if (out_xq) out_xq[3 * o + d] = xq[d];
          if (out_X) out_X[3 * o + d] = Xg[ND * d];
        }
      }
}

#endif
