/*
 * CPU oracle: the project's own C restatement of IGAP4's element assembly path
 * (TEST INFRASTRUCTURE -- only tests/, the smoke check and the benchmark's CPU
 * baseline may load it; the product never does).
 *
 * Every function cites the reference routine it restates.  The restatement is
 * pinned against the reference's own code compiled from source
 * (oracle/_ref, see oracle/build_ref.sh) and against committed golden vectors
 * (tests/golden/).
 */
#ifndef IGAP_ORACLE_H
#define IGAP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_LAW_GRADELAST = 0, ORC_LAW_GRADELASTTIME = 1, ORC_LAW_LINGRAD = 2 };

typedef struct OracleCase OracleCase;

/* Gauss-Legendre rule of n points on [a,b], ascending nodes
 * (restates legendre_handle, src/quadrature.c:381-430, rescale :432). */
void orc_gauss_legendre(int n, double a, double b, double *x, double *w);

/* Control-point lattice of a box beam with per-direction element counts
 * (formulas of mesh/igabeam.c:34-72; perturb=1 adds mesh/igabeamtest.c:68-70).
 * knots: 3 concatenated vectors of nelem[d]+1+2p entries; w: ncp; X: 3*ncp. */
void orc_mesh_beam(const int nelem[3], const double L[3], int p, int perturb, double *knots,
                   double *w, double *X);

/* Tensor-product B-spline values and 1st/2nd derivatives at one point
 * (restates eval_Bspline, src/meshcore_iga.c:243-327, generalised to degree p).
 * kv[d] points at the knot vector offset by the element index; N has
 * (p+1)^3 * 10 entries, layout N[10*b+k]. */
void orc_eval_bspline(double *N, const double *const kv[3], int p, const double xq[3]);

/* One basis function (derivative order k) by recursion
 * (restates evalN, src/meshcore_iga.c:329-384). */
double orc_evalN(const double *kv, int nk, int k, int i, int p, double xi);

/* Case set-up: mesh arrays as produced by orc_mesh_beam (copied). */
OracleCase *orc_case_create(const int nelem[3], int p, const double *knots, const double *w,
                            const double *X, int law, const double *par, int nquad,
                            const int *bc_type, const double *par_dirichlet,
                            const double *neumann_tab);
void orc_case_destroy(OracleCase *c);
int orc_case_ndof(const OracleCase *c);
int orc_case_torder(const OracleCase *c);
long orc_case_nnz(const OracleCase *c);
/* CSR pattern of the tangent (restates setnz_iga src/assmcore_iga.c:1054-1087
 * plus the column set the element loop inserts). */
void orc_case_pattern(const OracleCase *c, long *rowptr, int *cols);
/* Residual Vec (restates Residual_iga, src/assmcore_iga.c:16-502).
 * U_hist: [(torder+1)][ndof]. */
void orc_case_residual(const OracleCase *c, const double *U_hist, double *RR);
/* Tangent CSR values in the pattern of orc_case_pattern
 * (restates Tangent_iga, src/assmcore_iga.c:507-858). */
void orc_case_tangent(const OracleCase *c, const double *U_hist, double *vals);
/* Volume element loop only (no boundary terms), for a subset of elements
 * [e0,e1) in x-major order; used for a bounded CPU timing sample. */
void orc_case_tangent_elements(const OracleCase *c, const double *U_hist, double *vals, long e0,
                               long e1);
void orc_case_residual_elements(const OracleCase *c, const double *U_hist, double *RR, long e0,
                                long e1);

/* The law's field on the plot lattice of iga_plotfield (restates
 * src/mgl/plotcore_iga.c:16-282 without MathGL; oracle/field_sampling.h):
 * field [npoints][nfield], xq / X [npoints][3]; returns nfield. */
int orc_case_field(OracleCase *c, const double *U_hist, int nppe, double *field, double *xq, double *X);
/* Field callback of a law (33 values, 6 for gradelasttime); returns the count. */
int orc_law_field(int law, double *f, const double *u, const double *par);

/* Laws (per point): residual rr[30], tangent tt[900] of u[(torder+1)*30]. */
void orc_law_residual(int law, double *rr, const double *u, const double *par);
void orc_law_tangent(int law, double *tt, const double *u, const double *par);
void orc_law_default_par(int law, double *par);

#ifdef __cplusplus
}
#endif
#endif
