/*
 * Test driver for the IGAP4-facing glue (igap4_gb300/host/igapgpu_igap.c).
 * Builds a one-rank Core the way IGAPAssmInit leaves it (partitioned mesh,
 * identity comm, U_hist levels), registers a law plugin, and calls
 * Residual_gpu / Tangent_gpu through the PETSc-signature callbacks, with the
 * oracle's single-rank Vec/Mat stand-ins as the PETSc objects.
 * Test infrastructure only.
 */
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

/* returns 0 on success; RR (ndof), CSR of the stub AIJ after Tangent_gpu */
int glue_run(const int *nelem, const double *knots, const double *w, const double *X, int law,
             const double *par, const int *bc_type, const double *table, const double *U_hist,
             double *RR, long *rowptr, int *cols, double *vals, long *nnz_out, double *Kx_in,
             double *Kx_out)
{
  IGAPGPURegisterLaw(law_static, IGAPGPU_LAW_GRADELAST);
  IGAPGPURegisterLaw(law_transient, IGAPGPU_LAW_GRADELASTTIME);
  IGAPGPURegisterLaw(law_linear, IGAPGPU_LAW_LINGRAD);
  const int p = 2;
  struct __Mesh mesh;
  memset(&mesh, 0, sizeof mesh);
  int ne[3], nb[3], nk[3];
  double *kv[3];
  const double *kp = knots;
  for (int d = 0; d < 3; d++) {
    ne[d] = nelem[d]; nb[d] = nelem[d] + p; nk[d] = nelem[d] + 1 + 2 * p;
    kv[d] = (double *)kp;
    kp += nk[d];
  }
  int boun[6] = {0, 1, 2, 3, 4, 5};
  mesh.porder = p; mesh.nelem = ne; mesh.nbasis = nb; mesh.nknot = nk; mesh.knotVector = kv;
  mesh.wVector = (double *)w; mesh.XVector = (double *)X; mesh.nboun = 6; mesh.boun = boun;
  const int ncp = nb[0] * nb[1] * nb[2], ndof = 3 * ncp;
  struct __Phys phys;
  memset(&phys, 0, sizeof phys);
  double parm[9];
  memcpy(parm, par, sizeof parm);
  phys.ndim = 3; phys.ndof = 3; phys.sorder = 2; phys.par_mat = parm;
  phys.torder = law == IGAPGPU_LAW_GRADELASTTIME ? 2 : 0;
  phys.residual = law == IGAPGPU_LAW_GRADELAST ? law_static
                  : law == IGAPGPU_LAW_GRADELASTTIME ? law_transient : law_linear;
  struct __BC bc;
  int bct[36];
  double zero9[9] = {0}, parneu[1] = {0};
  memcpy(bct, bc_type, sizeof bct);
  memcpy(g_table, table, sizeof g_table);
  bc.bc_type = bct; bc.par_periodic = zero9; bc.par_dirichlet = zero9; bc.par_neumann = parneu;
  bc.neumann = neumann_table;
  struct __Comm comm;
  memset(&comm, 0, sizeof comm);
  comm.nselfIdx = ndof;
  int *gidx = (int *)malloc(sizeof(int) * (size_t)ndof);
  for (int i = 0; i < ndof; i++) gidx[i] = i;
  comm.globalIdx = gidx; comm.selfIdx = gidx;
  const int nh = phys.torder + 1;
  double *uh = (double *)malloc(sizeof(double) * (size_t)nh * ndof);
  memcpy(uh, U_hist, sizeof(double) * (size_t)nh * ndof);
  Phys pa[1] = {&phys};
  Mesh ma[1] = {&mesh};
  BC ba[1] = {&bc};
  Comm ca[1] = {&comm};
  struct __Core core = {pa, ma, ba, ca, uh};
  int rc = IGAPGPUAssmInit(&core);
  if (rc) return rc;
  Vec U, F;
  VecCreateMPI(0, ndof, ndof, &U);
  VecDuplicate(U, &F);
  memcpy(oracle_stub_vec_array(U), U_hist, sizeof(double) * (size_t)ndof);
  rc = Residual_gpu(NULL, U, F, &core);
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
  IGAPGPUSetHostMatrix(&core, 1);
  rc = Tangent_gpu(NULL, U, K, K, &core);
  if (rc) return rc;
  *nnz_out = oracle_stub_mat_nnz(K);
  oracle_stub_mat_csr(K, rowptr, cols, vals);
  /* MATSHELL multiply of the device matrix */
  Vec x, y;
  VecDuplicate(U, &x);
  VecDuplicate(U, &y);
  memcpy(oracle_stub_vec_array(x), Kx_in, sizeof(double) * (size_t)ndof);
  rc = MatMult_gpu(&core, x, y);
  memcpy(Kx_out, oracle_stub_vec_array(y), sizeof(double) * (size_t)ndof);
  IGAPGPUFinalize(&core);
  free(dnz); free(onz); free(gidx); free(uh);
  return rc;
}
