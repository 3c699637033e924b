/*
 * Test driver for the IGAP4-facing glue (igap4_gb300/host/igapgpu_igap.c).
 * Builds a one-rank Core the way IGAPAssmInit leaves it (partitioned mesh,
 * identity comm, U_hist levels), registers a law plugin, and calls
 * Residual_gpu / Tangent_gpu through the PETSc-signature callbacks, with the
 * oracle's single-rank Vec/Mat stand-ins as the PETSc objects.
 * Test infrastructure only.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "igapgpu_igap.h"

int oracle_stub_vec_size(Vec v);
double *oracle_stub_vec_array(Vec v);
long oracle_stub_mat_nnz(Mat A);
void oracle_stub_mat_csr(Mat A, long *rowptr, int *cols, double *vals);

/* stand-in law plugins: only their addresses identify the law */
static void law_static(double *r, double *u, double *p) { (void)r; (void)u; (void)p; }
static void law_transient(double *r, double *u, double *p) { (void)r; (void)u; (void)p; }
static void law_linear(double *r, double *u, double *p) { (void)r; (void)u; (void)p; }
static double g_table[36];
static void neumann_table(double *out, double par[], int f, int o, int d, double xq[])
{
  (void)par; (void)xq;
  *out = g_table[6 * f + 3 * o + d];
}

/* A one-rank Core laid out as IGAPAssmInit leaves it, with its storage. */
typedef struct {
  struct __Mesh mesh;
  struct __Phys phys;
  struct __BC bc;
  struct __Comm comm;
  struct __Core core;
  Phys pa[1];
  Mesh ma[1];
  BC ba[1];
  Comm ca[1];
  int ne[3], nb[3], nk[3], boun[6], bct[36];
  double *kv[3], parm[9], zero9[9], parneu[1];
  int *gidx;
  double *uh;
  int ndof;
} TestCore;

static void core_build(TestCore *t, const int *nelem, const double *knots, const double *w,
                       const double *X, int law, const double *par, const int *bc_type,
                       const double *table, const double *U_hist)
{
  IGAPGPURegisterLaw(law_static, IGAPGPU_LAW_GRADELAST);
  IGAPGPURegisterLaw(law_transient, IGAPGPU_LAW_GRADELASTTIME);
  IGAPGPURegisterLaw(law_linear, IGAPGPU_LAW_LINGRAD);
  const int p = 2;
  memset(t, 0, sizeof *t);
  const double *kp = knots;
  for (int d = 0; d < 3; d++) {
    t->ne[d] = nelem[d]; t->nb[d] = nelem[d] + p; t->nk[d] = nelem[d] + 1 + 2 * p;
    t->kv[d] = (double *)kp;
    kp += t->nk[d];
  }
  for (int f = 0; f < 6; f++) t->boun[f] = f;
  t->mesh.porder = p; t->mesh.nelem = t->ne; t->mesh.nbasis = t->nb; t->mesh.nknot = t->nk;
  t->mesh.knotVector = t->kv; t->mesh.wVector = (double *)w; t->mesh.XVector = (double *)X;
  t->mesh.nboun = 6; t->mesh.boun = t->boun;
  const int ncp = t->nb[0] * t->nb[1] * t->nb[2];
  t->ndof = 3 * ncp;
  memcpy(t->parm, par, sizeof t->parm);
  t->phys.ndim = 3; t->phys.ndof = 3; t->phys.sorder = 2; t->phys.par_mat = t->parm;
  t->phys.torder = law == IGAPGPU_LAW_GRADELASTTIME ? 2 : 0;
  t->phys.residual = law == IGAPGPU_LAW_GRADELAST ? law_static
                     : law == IGAPGPU_LAW_GRADELASTTIME ? law_transient : law_linear;
  memcpy(t->bct, bc_type, sizeof t->bct);
  memcpy(g_table, table, sizeof g_table);
  t->bc.bc_type = t->bct; t->bc.par_periodic = t->zero9; t->bc.par_dirichlet = t->zero9;
  t->bc.par_neumann = t->parneu; t->bc.neumann = neumann_table;
  t->gidx = (int *)malloc(sizeof(int) * (size_t)t->ndof);
  for (int i = 0; i < t->ndof; i++) t->gidx[i] = i;
  t->comm.nselfIdx = t->ndof;
  t->comm.globalIdx = t->gidx; t->comm.selfIdx = t->gidx;
  const int nh = t->phys.torder + 1;
  t->uh = (double *)malloc(sizeof(double) * (size_t)nh * t->ndof);
  memcpy(t->uh, U_hist, sizeof(double) * (size_t)nh * t->ndof);
  t->pa[0] = &t->phys; t->ma[0] = &t->mesh; t->ba[0] = &t->bc; t->ca[0] = &t->comm;
  t->core.phys = t->pa; t->core.mesh = t->ma; t->core.bc = t->ba; t->core.comm = t->ca;
  t->core.U_hist = t->uh;
}

static void core_free(TestCore *t)
{
  free(t->gidx);
  free(t->uh);
}

/* returns 0 on success; RR (ndof), CSR of the stub AIJ after Tangent_gpu,
 * and Kx = the MATSHELL multiply of the device matrix applied to Kx_in */
int glue_run(const int *nelem, const double *knots, const double *w, const double *X, int law,
             const double *par, const int *bc_type, const double *table, const double *U_hist,
             double *RR, long *rowptr, int *cols, double *vals, long *nnz_out, double *Kx_in,
             double *Kx_out)
{
  TestCore t;
  core_build(&t, nelem, knots, w, X, law, par, bc_type, table, U_hist);
  Core core = &t.core;
  const int ndof = t.ndof, p = 2;
  const int *nb = t.nb;
  int rc = IGAPGPUAssmInit(core);
  if (rc) return rc;
  Vec U, F;
  VecCreateMPI(0, ndof, ndof, &U);
  VecDuplicate(U, &F);
  memcpy(oracle_stub_vec_array(U), U_hist, sizeof(double) * (size_t)ndof);
  rc = Residual_gpu(NULL, U, F, core);
  if (rc) return rc;
  memcpy(RR, oracle_stub_vec_array(F), sizeof(double) * (size_t)ndof);
  /* AIJ with the reference's preallocation (setnz_iga row lengths) */
  int *dnz = (int *)malloc(sizeof(int) * (size_t)ndof), *onz = (int *)calloc((size_t)ndof, sizeof(int));
  int a = 0;
  for (int ix = 0; ix < nb[0]; ix++)
    for (int iy = 0; iy < nb[1]; iy++)
      for (int iz = 0; iz < nb[2]; iz++)
        for (int d = 0; d < 3; d++) {
          int ii[3] = {ix, iy, iz}, len = 3;
          for (int q = 0; q < 3; q++)
            len *= (ii[q] < p ? ii[q] : p) + 1 + (ii[q] > nb[q] - 1 - p ? nb[q] - 1 - ii[q] : p);
          dnz[a++] = len;
        }
  Mat K;
  MatCreateAIJ(0, ndof, ndof, ndof, ndof, 0, dnz, 0, onz, &K);
  IGAPGPUSetHostMatrix(core, 1);
  rc = Tangent_gpu(NULL, U, K, K, core);
  if (rc) return rc;
  *nnz_out = oracle_stub_mat_nnz(K);
  oracle_stub_mat_csr(K, rowptr, cols, vals);
  /* MATSHELL multiply of the device matrix, through MatMult's dispatch */
  Mat S;
  rc = IGAPGPUCreateMatShell(core, &S);
  if (rc) return rc;
  Vec x, y;
  VecDuplicate(U, &x);
  VecDuplicate(U, &y);
  memcpy(oracle_stub_vec_array(x), Kx_in, sizeof(double) * (size_t)ndof);
  rc = MatMult(S, x, y);
  memcpy(Kx_out, oracle_stub_vec_array(y), sizeof(double) * (size_t)ndof);
  IGAPGPUFinalize(core);
  MatDestroy(&S); MatDestroy(&K);
  VecDestroy(&U); VecDestroy(&F); VecDestroy(&x); VecDestroy(&y);
  free(dnz); free(onz);
  core_free(&t);
  return rc;
}

/* The reference's solver set-up and Newton loop (IGAPSolvInit,
 * src/interface.c:207-250, and IGAPSolvSolve, :302-328) with the GPU
 * callbacks and the MATSHELL in place of Residual_iga / Tangent_iga and the
 * AIJ matrix; -pc_type jacobi is applied as the runtime option would.
 * U (in: initial iterate, out: solution); returns 0 or the first error. */
int glue_snes_run(const int *nelem, const double *knots, const double *w, const double *X, int law,
                  const double *par, const int *bc_type, const double *table, double *U_hist,
                  int restart, int *newton_its, int *ksp_its, int *reason, double *fnorm)
{
  TestCore t;
  core_build(&t, nelem, knots, w, X, law, par, bc_type, table, U_hist);
  Core core = &t.core;
  int rc = IGAPGPUAssmInit(core);
  if (rc) return rc;
  Vec RR, U;
  VecCreateMPI(0, t.ndof, t.ndof, &RR);
  VecDuplicate(RR, &U);
  Mat TT;
  if ((rc = IGAPGPUCreateMatShell(core, &TT))) return rc;
  SNES snes;
  KSP ksp;
  PC pc;
  SNESLineSearch ls;
  SNESCreate(MPI_COMM_WORLD, &snes);
  SNESSetFunction(snes, RR, Residual_gpu, core);
  SNESSetJacobian(snes, TT, TT, Tangent_gpu, core);
  SNESSetTolerances(snes, 1.e-10, 1.e-20, 1.e-20, 1, 1e9);
  SNESSetType(snes, SNESNEWTONLS);
  SNESGetLineSearch(snes, &ls);
  SNESLineSearchSetType(ls, SNESLINESEARCHBT);
  SNESLineSearchSetOrder(ls, SNES_LINESEARCH_ORDER_CUBIC);
  SNESGetKSP(snes, &ksp);
  KSPGetPC(ksp, &pc);
  KSPSetInitialGuessNonzero(ksp, PETSC_TRUE);
  KSPSetTolerances(ksp, 1e-8, PETSC_DEFAULT, 1e8, 100000);
  KSPSetType(ksp, KSPGMRES);
  KSPGMRESSetRestart(ksp, restart);
  KSPGMRESSetOrthogonalization(ksp, KSPGMRESModifiedGramSchmidtOrthogonalization);
  KSPSetPCSide(ksp, PC_RIGHT);
  PCSetType(pc, PCJACOBI);
  SNESSetFromOptions(snes);
  /* IGAPSolvGuess: U <- U_hist[0] */
  memcpy(oracle_stub_vec_array(U), t.uh, sizeof(double) * (size_t)t.ndof);
  SNESConvergedReason r = SNES_CONVERGED_ITERATING;
  double fn = 0.0, fold = 999.0;
  int its = 0, kits = 0;
  for (int sub = 0; sub < 200; sub++) {
    if ((rc = SNESSolve(snes, NULL, U))) break;
    PetscInt k;
    KSPGetIterationNumber(ksp, &k);
    kits += k;
    SNESGetConvergedReason(snes, &r);
    SNESGetFunctionNorm(snes, &fn);
    if (fabs(fold - fn) / fold < 1.e-6) r = SNES_DIVERGED_LINE_SEARCH;
    fold = fn;
    its++;
    if (r != SNES_DIVERGED_MAX_IT) break;
  }
  memcpy(U_hist, oracle_stub_vec_array(U), sizeof(double) * (size_t)t.ndof);
  *newton_its = its;
  *ksp_its = kits;
  *reason = (int)r;
  *fnorm = fn;
  IGAPGPUFinalize(core);
  SNESDestroy(&snes);
  MatDestroy(&TT);
  VecDestroy(&RR);
  VecDestroy(&U);
  core_free(&t);
  return rc;
}

/* Error paths: the callbacks on a Core without a device context, and the
 * MATSHELL operations on a matrix that is not a shell, return PETSc error
 * classes (positive). */
int glue_errors(int *codes)
{
  struct __Core none;
  memset(&none, 0, sizeof none);
  Vec U, F;
  VecCreateMPI(0, 3, 3, &U);
  VecDuplicate(U, &F);
  codes[0] = Residual_gpu(NULL, U, F, &none);
  codes[1] = Tangent_gpu(NULL, U, NULL, NULL, &none);
  Mat K;
  int dnz[3] = {1, 1, 1}, onz[3] = {0, 0, 0};
  MatCreateAIJ(0, 3, 3, 3, 3, 0, dnz, 0, onz, &K);
  codes[2] = MatMult_gpu(K, U, F);
  codes[3] = MatGetDiagonal_gpu(K, F);
  codes[4] = IGAPGPUPetscError(IGAPGPU_ERR_CUDA);
  codes[5] = IGAPGPUPetscError(IGAPGPU_ERR_NOMEM);
  MatDestroy(&K);
  VecDestroy(&U);
  VecDestroy(&F);
  return 0;
}
