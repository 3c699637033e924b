/*
 * CPU oracle driver around the reference's OWN compiled code (test
 * infrastructure; built into oracle/_ref/libigapref.so by oracle/build_ref.sh
 * from the sources under the reference tree, never copied into this repo).
 *
 * It sets up one IGAP4 problem through the reference's public API
 * (IGAPInitialize, IGAPMeshAdd, IGAPPhysAdd, IGAPBCAdd, IGAPAssmInit:
 * src/interface.c:23-203) and then calls the registered SNES callbacks
 * Residual_iga / Tangent_iga (src/assmcore_iga.c:16,507) on a given state,
 * exposing the assembled Vec and AIJ matrix as plain arrays for ctypes.
 *
 * Project-written pieces (no reference counterpart):
 *  - a mesh constructor with a per-direction element count; it fills the same
 *    global fields of struct __Mesh (include/meshimpl.h:24-28) with the knot
 *    and control-point formulas of mesh/igabeam.c:34-72 (and the perturbation
 *    of mesh/igabeamtest.c:68-70), generalised from 2^mref per direction;
 *  - a BC whose Neumann callback reads a constant 6x2x3 traction table from
 *    par_neumann (same signature as neumann_default_iga,
 *    src/assmcore_iga.c:1036-1052);
 *  - the linear isotropic strain-gradient law (oracle/law_lingrad.c), which the
 *    reference does not contain.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "petscsnes.h"
#include "igapimpl.h"
#include "interface.h"
#include "physgradelast.h"
#include "physgradelasttime.h"
#include "postcore.h"
#include "ioutil.h"
#include "meshigabeam.h"
#include "meshigabeamtest.h"
#include "gradelast.h"
#include "gradelasttime.h"
#include "quadrature.h"
#include "meshcore.h"

int oracle_stub_vec_size(Vec v);
double *oracle_stub_vec_array(Vec v);
long oracle_stub_mat_nnz(Mat A);
void oracle_stub_mat_csr(Mat A, long *rowptr, int *cols, double *vals);

/* project law (oracle/law_lingrad.c) */
void lingrad_residual(double *rr, double *u, double *par);
void lingrad_tangent(double *tt, double *u, double *par);

enum { LAW_GRADELAST = 0, LAW_GRADELASTTIME = 1, LAW_LINGRAD = 2 };
enum { MESH_BEAM = 0, MESH_BEAMTEST = 1, MESH_REF_IGABEAM = 2, MESH_REF_IGABEAMTEST = 3 };

typedef struct {
  IGAP igap;
  int torder;
  int ndof_total;
} RefCase;

/* ---- mesh: per-direction element counts, igabeam formulas ------------- */
static Mesh mesh_beam_dir(const int nelem[3], const double L[3], int porder, const int periodic[3],
                          int perturb)
{
  Mesh mesh = (Mesh)calloc(1, sizeof(struct __Mesh));
  int *bcp = (int *)malloc(3 * sizeof(int));
  int *neg = (int *)malloc(3 * sizeof(int));
  double **kv = (double **)malloc(3 * sizeof(double *));
  for (int d = 0; d < 3; d++) {
    bcp[d] = periodic[d];
    neg[d] = nelem[d];
    int nk = nelem[d] + 1 + 2 * porder;
    kv[d] = (double *)malloc((size_t)nk * sizeof(double));
    double h = 1.0 / nelem[d];
    for (int k = 0; k < nk; k++) {
      if (!periodic[d]) {
        if (k < porder + 1) kv[d][k] = 0.0;
        else if (k < nelem[d] + porder) kv[d][k] = (k - porder) * h;
        else kv[d][k] = 1.0;
      } else {
        kv[d][k] = (k - porder) * h;
      }
    }
  }
  int nb[3] = {nelem[0] + porder, nelem[1] + porder, nelem[2] + porder};
  size_t ncp = (size_t)nb[0] * nb[1] * nb[2];
  double *w = (double *)malloc(ncp * sizeof(double));
  double *X = (double *)malloc(3 * ncp * sizeof(double));
  size_t a = 0;
  for (int i = 0; i < nb[0]; i++)
    for (int j = 0; j < nb[1]; j++)
      for (int k = 0; k < nb[2]; k++) {
        w[a] = 1.0;
        X[3 * a + 0] = ((double)i - 0.5) / ((double)(nb[0] - 2)) * L[0];
        X[3 * a + 1] = ((double)j - 0.5) / ((double)(nb[1] - 2)) * L[1];
        X[3 * a + 2] = ((double)k - 0.5) / ((double)(nb[2] - 2)) * L[2];
        if (perturb) {
          double in = (double)(i > 2 && j > 2 && k > 2 && i < nb[0] - 2 && j < nb[1] - 2 && k < nb[2] - 2);
          X[3 * a + 0] += 0.2 * L[0] / nb[0] * in * sin(3 * i * k * j);
          X[3 * a + 1] += 0.2 * L[1] / nb[1] * in * sin(5 * i * k * j);
          X[3 * a + 2] += 0.2 * L[2] / nb[2] * in * sin(7 * i * k * j);
        }
        a++;
      }
  mesh->porder = porder;
  mesh->bc_periodic = bcp;
  mesh->nelem_global = neg;
  mesh->knotVector_global = kv;
  mesh->wVector_global = w;
  mesh->XVector_global = X;
  return mesh;
}

/* ---- project linear law plugin, same struct as PhysGradElast ---------- */
void lingrad_density(double h[], double u[], double *par);
void lingrad_densityb(double h[], double u[], double t, double *par, int o);
void lingrad_field(double *f, double *u, double *par);
static void lingrad_assert(double *par) { (void)par; }

static Phys phys_lingrad(const double *par)
{
  Phys phys = (Phys)malloc(sizeof(struct __Phys));
  phys->ndim = 3; phys->ndof = 3; phys->torder = 0; phys->sorder = 2;
  phys->ndensity = 2; phys->nfield = 33;
  phys->par_mat = (double *)calloc(9, sizeof(double));
  double def[3] = {1.0, 1.0, 0.1}; /* lambda, mu, ell */
  for (int i = 0; i < 3; i++) phys->par_mat[i] = par ? par[i] : def[i];
  phys->residual = lingrad_residual;
  phys->tangent = lingrad_tangent;
  phys->field = lingrad_field;
  phys->density = lingrad_density;
  phys->densityb = lingrad_densityb;
  phys->assert_par_mat = lingrad_assert;
  return phys;
}

/* ---- BC: constant traction table in par_neumann[(2*3)*face+3*order+dof] -- */
static void neumann_table(double *out, double par_neumann[], int face_id, int bc_order, int idof,
                          double xq[])
{
  (void)xq;
  *out = par_neumann[6 * face_id + 3 * bc_order + idof];
}

void *ref_case_create(const int nelem[3], const double L[3], int porder, const int periodic[3],
                      int mesh_kind, int law, const double *par_mat, const int *bc_type,
                      const double *par_dirichlet, const double *neumann_tab,
                      const double *par_periodic)
{
  RefCase *c = (RefCase *)calloc(1, sizeof(RefCase));
  IGAPInitialize(&c->igap);
  Mesh mesh;
  if (mesh_kind == MESH_REF_IGABEAM || mesh_kind == MESH_REF_IGABEAMTEST) {
    int mref = 0;
    while ((1 << mref) < nelem[0]) mref++;
    mesh = (mesh_kind == MESH_REF_IGABEAM ? MeshIGABeam : MeshIGABeamTest)(
        L[0], L[1], L[2], mref, porder, periodic[0], periodic[1], periodic[2]);
  } else {
    mesh = mesh_beam_dir(nelem, L, porder, periodic, mesh_kind == MESH_BEAMTEST);
  }
  IGAPMeshAdd(c->igap, mesh);
  Phys phys;
  if (law == LAW_GRADELAST) phys = PhysGradElast();
  else if (law == LAW_GRADELASTTIME) phys = PhysGradElastTime();
  else phys = phys_lingrad(par_mat);
  if (par_mat && law != LAW_LINGRAD)
    for (int i = 0; i < 9; i++) phys->par_mat[i] = par_mat[i];
  IGAPPhysAdd(c->igap, phys);

  BC bc = (BC)malloc(sizeof(struct __BC));
  bc->bc_type = (int *)malloc(36 * sizeof(int));
  bc->par_periodic = (double *)calloc(9, sizeof(double));
  bc->par_dirichlet = (double *)calloc(9, sizeof(double));
  bc->par_neumann = (double *)calloc(36, sizeof(double));
  for (int i = 0; i < 36; i++) bc->bc_type[i] = bc_type ? bc_type[i] : 1;
  for (int i = 0; i < 9; i++) {
    if (par_dirichlet) bc->par_dirichlet[i] = par_dirichlet[i];
    if (par_periodic) bc->par_periodic[i] = par_periodic[i];
  }
  for (int i = 0; i < 36; i++) bc->par_neumann[i] = neumann_tab ? neumann_tab[i] : 0.0;
  bc->neumann = neumann_table;
  IGAPBCAdd(c->igap, bc);

  IGAPAssmInit(c->igap);
  c->torder = c->igap->core->phys[0]->torder;
  c->ndof_total = c->igap->iocomm->nDof;
  return c;
}

/* iga_intdensity (src/postcore_iga.c:13-377) on the current U_hist; returns
 * the number of densities written to HH. */
int ref_case_density(void *h, double *HH)
{
  RefCase *c = (RefCase *)h;
  iga_intdensity(HH, c->igap->core);
  return c->igap->core->phys[0]->ndensity;
}

/* IGAPSolvSaveSolution / IGAPSolvLoadSolution of the reference (src/interface.c:271-300). */
void ref_case_save(void *h, const char *fname) { IGAPSolvSaveSolution(((RefCase *)h)->igap, fname); }
/* IGAPSolvLoadSolution minus its final copy into the SNES vector (no solver
 * here): read_solution (src/ioutil.c:127) on the same levels. */
void ref_case_load(void *h, const char *fname)
{
  RefCase *c = (RefCase *)h;
  double *U = c->igap->core->U_hist;
  const int n = c->igap->iocomm->nDof;
  if (c->torder == 0) {
    read_solution(fname, U, c->igap->iocomm, 0, 1);
  } else {
    read_solution(fname, U, c->igap->iocomm, 1, c->torder + 1);
    for (int i = 0; i < n; i++) U[i] = U[n + i];
  }
}

/* Field sampling: the reference's basis (eval_Bspline, src/meshcore_iga.c:
 * 243-327), 3 x 3 inverse (matinv, src/mathutil.c:17-41) and the law's field
 * callback (phys->field) driven by the restated plot loop of
 * oracle/field_sampling.h (the reference's own plotcore_iga.c does not
 * compile), on the ghosted local state of plotcore_iga.c:62-80. */
#include "field_sampling.h"
void matinv(double *mat, int n);
static void fs_ref_basis(double *N, double *kv[3], int p, double xq[3]) { eval_Bspline(N, kv, p, xq); }
static void fs_ref_inverse(double *G) { matinv(G, 3); }

int ref_case_field(void *h, int nppe, double *field, double *xq, double *X)
{
  RefCase *c = (RefCase *)h;
  Core core = c->igap->core;
  Mesh m = core->mesh[0];
  Phys ph = core->phys[0];
  Comm cm = core->comm[0];
  const int nself = cm->nselfIdx, nloc = cm->nselfIdx + cm->nrecvIdx, nlev = ph->torder + 1;
  double *U = (double *)calloc((size_t)nlev * nloc, sizeof(double));
  for (int l = 0; l < nlev; l++)
    for (int i = 0; i < nself; i++) U[(size_t)l * nloc + cm->selfIdx[i]] = core->U_hist[(size_t)l * nself + i];
  fs_sample(m->porder, m->nelem, m->knotVector, m->wVector, m->XVector, U, nloc, nlev, ph->par_mat, ph->nfield, nppe,
            fs_ref_basis, fs_ref_inverse, ph->field, field, xq, X);
  free(U);
  return ph->nfield;
}

int ref_case_ndof(void *h) { return ((RefCase *)h)->ndof_total; }
int ref_case_torder(void *h) { return ((RefCase *)h)->torder; }

/* U_hist layout: [(torder+1)][nDof], level 0 = current iterate. */
void ref_case_set_state(void *h, const double *U_hist)
{
  RefCase *c = (RefCase *)h;
  memcpy(c->igap->core->U_hist, U_hist, sizeof(double) * (size_t)(c->torder + 1) * c->ndof_total);
}
void ref_case_get_state(void *h, double *U_hist)
{
  RefCase *c = (RefCase *)h;
  memcpy(U_hist, c->igap->core->U_hist, sizeof(double) * (size_t)(c->torder + 1) * c->ndof_total);
}

void ref_case_residual(void *h, double *out)
{
  RefCase *c = (RefCase *)h;
  Vec U;
  VecDuplicate(c->igap->assm->RR, &U);
  memcpy(oracle_stub_vec_array(U), c->igap->core->U_hist, sizeof(double) * (size_t)c->ndof_total);
  c->igap->assm->Residual(NULL, U, c->igap->assm->RR, c->igap->core);
  memcpy(out, oracle_stub_vec_array(c->igap->assm->RR), sizeof(double) * (size_t)c->ndof_total);
  VecDestroy(&U);
}

long ref_case_tangent(void *h)
{
  RefCase *c = (RefCase *)h;
  Vec U;
  VecDuplicate(c->igap->assm->RR, &U);
  memcpy(oracle_stub_vec_array(U), c->igap->core->U_hist, sizeof(double) * (size_t)c->ndof_total);
  c->igap->assm->Tangent(NULL, U, c->igap->assm->TT, c->igap->assm->TT, c->igap->core);
  VecDestroy(&U);
  return oracle_stub_mat_nnz(c->igap->assm->TT);
}
void ref_case_tangent_csr(void *h, long *rowptr, int *cols, double *vals)
{
  oracle_stub_mat_csr(((RefCase *)h)->igap->assm->TT, rowptr, cols, vals);
}

/* globalIdx of the local (ghosted) numbering, built by IGAPAssmInit */
int ref_case_nlocal(void *h)
{
  Comm cm = ((RefCase *)h)->igap->core->comm[0];
  return cm->nselfIdx + cm->nrecvIdx;
}
void ref_case_global_idx(void *h, int *out)
{
  Comm cm = ((RefCase *)h)->igap->core->comm[0];
  memcpy(out, cm->globalIdx, sizeof(int) * (size_t)(cm->nselfIdx + cm->nrecvIdx));
}
/* Partitioned mesh as stored after mpipart_iga: knots per direction, w, X. */
void ref_case_mesh_info(void *h, int *nelem, int *nknot, int *nbasis)
{
  Mesh m = ((RefCase *)h)->igap->core->mesh[0];
  for (int d = 0; d < 3; d++) { nelem[d] = m->nelem[d]; nknot[d] = m->nknot[d]; nbasis[d] = m->nbasis[d]; }
}
void ref_case_mesh_arrays(void *h, double *knots /* concatenated */, double *w, double *X)
{
  Mesh m = ((RefCase *)h)->igap->core->mesh[0];
  int p = m->porder;
  size_t off = 0;
  for (int d = 0; d < 3; d++) {
    memcpy(knots + off, m->knotVector[d], sizeof(double) * (size_t)m->nknot[d]);
    off += (size_t)m->nknot[d];
  }
  size_t ncp = (size_t)(m->nelem[0] + p) * (m->nelem[1] + p) * (m->nelem[2] + p);
  memcpy(w, m->wVector, sizeof(double) * ncp);
  memcpy(X, m->XVector, sizeof(double) * 3 * ncp);
}

void ref_case_destroy(void *h)
{
  RefCase *c = (RefCase *)h;
  /* IGAPFinalize also destroys the SNES, which IGAPSolvInit never created
   * here; free the pieces owned by AssmInit directly instead. */
  VecDestroy(&c->igap->assm->RR);
  MatDestroy(&c->igap->assm->TT);
  free(c);
}

/* ---- law and quadrature entry points ---------------------------------- */
void ref_law_residual(int law, double *rr, double *u, double *par)
{
  if (law == LAW_GRADELAST) gradelast_residual(rr, u, par);
  else if (law == LAW_GRADELASTTIME) gradelasttime_residual(rr, u, par);
  else lingrad_residual(rr, u, par);
}
void ref_law_tangent(int law, double *tt, double *u, double *par)
{
  if (law == LAW_GRADELAST) gradelast_tangent(tt, u, par);
  else if (law == LAW_GRADELASTTIME) gradelasttime_tangent(tt, u, par);
  else lingrad_tangent(tt, u, par);
}
void ref_law_default_par(int law, double *par)
{
  Phys p = law == LAW_GRADELAST ? PhysGradElast() : law == LAW_GRADELASTTIME ? PhysGradElastTime() : phys_lingrad(NULL);
  memcpy(par, p->par_mat, 9 * sizeof(double));
}
void ref_gauss_legendre(int n, double a, double b, double *x, double *w) { legendre_handle(x, w, n, a, b); }
void ref_eval_bspline(double *N, double *kv0, double *kv1, double *kv2, double *xq)
{
  double *kv[3] = {kv0, kv1, kv2};
  eval_Bspline(N, kv, 2, xq);
}
double ref_evalN(double *kv, int nk, int k, int i, int p, double xi) { return evalN(kv, nk, k, i, p, xi); }
