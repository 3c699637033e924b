/*
 * IGAP4-facing host layer over libigapgpu.so (see igapgpu_igap.h).
 * Host code only moves data between IGAP4's structs / PETSc objects and the
 * device context; all residual, tangent and multiply arithmetic runs on the GPU.
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "igapgpu_igap.h"

#define MAXLAW 32
#define MAXCORE 32

static struct { residual_ptr fn; int id; } g_law[MAXLAW];
static int g_nlaw;
static struct { Core core; igapgpu_t ctx; int host_matrix; } g_core[MAXCORE];

int IGAPGPURegisterLaw(residual_ptr residual, int law_id)
{
  for (int i = 0; i < g_nlaw; i++)
    if (g_law[i].fn == residual) { g_law[i].id = law_id; return 0; }
  if (g_nlaw >= MAXLAW) return IGAPGPU_ERR_ARG;
  g_law[g_nlaw].fn = residual;
  g_law[g_nlaw].id = law_id;
  g_nlaw++;
  return 0;
}

/* Registered first; otherwise IGAP4's own symbol names
 * (phys/gradelast.c:7, phys/gradelasttime.c:7). */
static int law_of(Phys phys)
{
  for (int i = 0; i < g_nlaw; i++)
    if (g_law[i].fn == phys->residual) return g_law[i].id;
  Dl_info info;
  if (dladdr((void *)phys->residual, &info) && info.dli_sname) {
    if (!strcmp(info.dli_sname, "gradelast_residual")) return IGAPGPU_LAW_GRADELAST;
    if (!strcmp(info.dli_sname, "gradelasttime_residual")) return IGAPGPU_LAW_GRADELASTTIME;
    if (!strcmp(info.dli_sname, "lingrad_residual")) return IGAPGPU_LAW_LINGRAD;
  }
  return -1;
}

static int slot_of(Core core)
{
  for (int i = 0; i < MAXCORE; i++)
    if (g_core[i].core == core) return i;
  return -1;
}

igapgpu_t IGAPGPUContext(Core core)
{
  int s = slot_of(core);
  return s < 0 ? NULL : g_core[s].ctx;
}

/* Upload history levels 1..torder from core->U_hist: the reference's
 * callbacks read every level from there on each call (src/assmcore_iga.c:69-80). */
static int upload_history(Core core, igapgpu_t ctx)
{
  const int torder = core->phys[0]->torder, n = core->comm[0]->nselfIdx;
  for (int l = 1; l <= torder; l++) {
    int rc = igapgpu_set_history(ctx, l, core->U_hist + (size_t)l * n);
    if (rc) return rc;
  }
  return 0;
}

int IGAPGPUAssmInit(Core core)
{
  Mesh mesh = core->mesh[0];
  Phys phys = core->phys[0];
  BC bc = core->bc[0];
  if (mesh->nsendPart || mesh->nrecvPart || core->comm[0]->nrecvIdx) {
    fprintf(stderr, "IGAPGPUAssmInit: one rank, non-periodic meshes only\n");
    return IGAPGPU_ERR_ARG;
  }
  if (phys->ndim != 3 || phys->ndof != 3) return IGAPGPU_ERR_ARG;
  igapgpu_mesh_desc md;
  md.porder = mesh->porder;
  for (int d = 0; d < 3; d++) {
    md.nelem[d] = mesh->nelem[d];
    md.knots[d] = mesh->knotVector[d];
  }
  md.w = mesh->wVector;
  md.X = mesh->XVector;
  igapgpu_phys_desc pd;
  pd.law = law_of(phys);
  if (pd.law < 0) {
    fprintf(stderr, "IGAPGPUAssmInit: law plugin not known to the GPU path (no CPU fallback)\n");
    return IGAPGPU_ERR_LAW;
  }
  for (int i = 0; i < 9; i++) pd.par[i] = phys->par_mat[i];
  igapgpu_bc_desc bd;
  for (int i = 0; i < 36; i++) bd.bc_type[i] = bc->bc_type[i];
  for (int i = 0; i < 9; i++) {
    bd.par_periodic[i] = bc->par_periodic[i];
    bd.par_dirichlet[i] = bc->par_dirichlet[i];
  }
  /* the device integrates constant tractions: sample the callback at two
   * face points and require equal values */
  for (int f = 0; f < 6; f++)
    for (int o = 0; o < 2; o++)
      for (int d = 0; d < 3; d++) {
        double xa[3] = {0.25, 0.25, 0.25}, xb[3] = {0.75, 0.6, 0.4}, va = 0, vb = 0;
        bc->neumann(&va, bc->par_neumann, f, o, d, xa);
        bc->neumann(&vb, bc->par_neumann, f, o, d, xb);
        if (va != vb) {
          fprintf(stderr, "IGAPGPUAssmInit: position-dependent traction is not supported\n");
          return IGAPGPU_ERR_ARG;
        }
        bd.neumann[6 * f + 3 * o + d] = va;
      }
  int s = slot_of(core);
  if (s < 0) s = slot_of(NULL);
  if (s < 0) return IGAPGPU_ERR_NOMEM;
  igapgpu_t ctx = NULL;
  int rc = igapgpu_assm_init(&ctx, &md, &pd, &bd, 4);
  if (rc) return rc;
  g_core[s].core = core;
  g_core[s].ctx = ctx;
  g_core[s].host_matrix = 0;
  rc = igapgpu_set_history(ctx, 0, core->U_hist);
  if (rc) return rc;
  return upload_history(core, ctx);
}

/* When on, Tangent_gpu also writes the device CSR into the PETSc AIJ matrix P
 * (for host preconditioners such as ASM); off keeps it on the device
 * (MATSHELL). */
int IGAPGPUSetHostMatrix(Core core, int on)
{
  int s = slot_of(core);
  if (s < 0) return IGAPGPU_ERR_STATE;
  g_core[s].host_matrix = on;
  return 0;
}

int IGAPGPUFinalize(Core core)
{
  int s = slot_of(core);
  if (s < 0) return 0;
  int rc = igapgpu_finalize(g_core[s].ctx);
  g_core[s].core = NULL;
  g_core[s].ctx = NULL;
  return rc;
}

/* PETSc's error classes (petscerror.h); the stand-in header used by the
 * tests defines the same values. */
#ifndef PETSC_ERR_MEM
#define PETSC_ERR_MEM 55
#endif
#ifndef PETSC_ERR_ARG_WRONG
#define PETSC_ERR_ARG_WRONG 62
#endif
#ifndef PETSC_ERR_ARG_WRONGSTATE
#define PETSC_ERR_ARG_WRONGSTATE 73
#endif
#ifndef PETSC_ERR_LIB
#define PETSC_ERR_LIB 76
#endif

PetscErrorCode IGAPGPUPetscError(int rc)
{
  switch (rc) {
  case IGAPGPU_OK: return 0;
  case IGAPGPU_ERR_NOMEM: return PETSC_ERR_MEM;
  case IGAPGPU_ERR_ARG:
  case IGAPGPU_ERR_LAW: return PETSC_ERR_ARG_WRONG;
  case IGAPGPU_ERR_STATE: return PETSC_ERR_ARG_WRONGSTATE;
  default: return PETSC_ERR_LIB;
  }
}

/* report a library failure once, in PETSc's terms */
static PetscErrorCode fail(const char *where, int rc)
{
  if (!rc) return 0;
  const char *msg = igapgpu_last_error();
  fprintf(stderr, "%s: igapgpu error %d: %s\n", where, rc, msg ? msg : "");
  return IGAPGPUPetscError(rc);
}

PetscErrorCode Residual_gpu(SNES snes, Vec U, Vec F, void *core_)
{
  (void)snes;
  Core core = (Core)core_;
  igapgpu_t ctx = IGAPGPUContext(core);
  if (!ctx) return fail("Residual_gpu", IGAPGPU_ERR_STATE);
  const int n = core->comm[0]->nselfIdx;
  const PetscScalar *u;
  PetscScalar *f;
  VecGetArrayRead(U, &u);
  memcpy(core->U_hist, u, sizeof(double) * (size_t)n); /* side effect of Residual_iga */
  int rc = upload_history(core, ctx);
  VecGetArray(F, &f);
  if (!rc) rc = igapgpu_residual(ctx, u, f);
  VecRestoreArray(F, &f);
  VecRestoreArrayRead(U, &u);
  return fail("Residual_gpu", rc);
}

PetscErrorCode Tangent_gpu(SNES snes, Vec U, Mat A, Mat P, void *core_)
{
  (void)snes;
  Core core = (Core)core_;
  int s = slot_of(core);
  if (s < 0) return fail("Tangent_gpu", IGAPGPU_ERR_STATE);
  igapgpu_t ctx = g_core[s].ctx;
  const int n = core->comm[0]->nselfIdx;
  const PetscScalar *u;
  VecGetArrayRead(U, &u);
  memcpy(core->U_hist, u, sizeof(double) * (size_t)n); /* side effect of Tangent_iga */
  int rc = upload_history(core, ctx);
  if (!rc) rc = igapgpu_tangent(ctx, u, NULL);
  VecRestoreArrayRead(U, &u);
  if (rc) return fail("Tangent_gpu", rc);
  if (g_core[s].host_matrix) {
    int64_t ndof, nnz;
    igapgpu_sizes(ctx, &ndof, &nnz, NULL, NULL);
    int64_t *rowptr = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ndof + 1));
    int32_t *cols = (int32_t *)malloc(sizeof(int32_t) * (size_t)nnz);
    double *vals = (double *)malloc(sizeof(double) * (size_t)nnz);
    if (!rowptr || !cols || !vals) {
      free(rowptr); free(cols); free(vals);
      return fail("Tangent_gpu", IGAPGPU_ERR_NOMEM);
    }
    rc = igapgpu_pattern(ctx, rowptr, cols);
    if (!rc) rc = igapgpu_tangent(ctx, NULL, vals);
    if (!rc) {
      for (int64_t r = 0; r < ndof; r++) {
        PetscInt row = (PetscInt)r;
        PetscInt len = (PetscInt)(rowptr[r + 1] - rowptr[r]);
        MatSetValues(P, 1, &row, len, (const PetscInt *)(cols + rowptr[r]), vals + rowptr[r], INSERT_VALUES);
      }
      MatAssemblyBegin(P, MAT_FINAL_ASSEMBLY);
      MatAssemblyEnd(P, MAT_FINAL_ASSEMBLY);
    }
    free(rowptr);
    free(cols);
    free(vals);
  }
  if (A != P) {
    MatAssemblyBegin(A, MAT_FINAL_ASSEMBLY);
    MatAssemblyEnd(A, MAT_FINAL_ASSEMBLY);
  }
  return fail("Tangent_gpu", rc);
}

static igapgpu_t shell_context(Mat A)
{
  void *core = NULL;
  if (MatShellGetContext(A, &core)) return NULL;
  return IGAPGPUContext((Core)core);
}

PetscErrorCode MatMult_gpu(Mat A, Vec x, Vec y)
{
  igapgpu_t ctx = shell_context(A);
  if (!ctx) return fail("MatMult_gpu", IGAPGPU_ERR_STATE);
  const PetscScalar *xa;
  PetscScalar *ya;
  VecGetArrayRead(x, &xa);
  VecGetArray(y, &ya);
  int rc = igapgpu_matmult(ctx, xa, ya);
  VecRestoreArray(y, &ya);
  VecRestoreArrayRead(x, &xa);
  return fail("MatMult_gpu", rc);
}

PetscErrorCode MatGetDiagonal_gpu(Mat A, Vec d)
{
  igapgpu_t ctx = shell_context(A);
  if (!ctx) return fail("MatGetDiagonal_gpu", IGAPGPU_ERR_STATE);
  PetscScalar *da;
  VecGetArray(d, &da);
  int rc = igapgpu_get_diagonal(ctx, da);
  VecRestoreArray(d, &da);
  return fail("MatGetDiagonal_gpu", rc);
}

PetscErrorCode IGAPGPUCreateMatShell(Core core, Mat *A)
{
  igapgpu_t ctx = IGAPGPUContext(core);
  if (!ctx || !A) return fail("IGAPGPUCreateMatShell", IGAPGPU_ERR_STATE);
  const PetscInt n = (PetscInt)core->comm[0]->nselfIdx;
  PetscErrorCode ierr = MatCreateShell(PETSC_COMM_WORLD, n, n, n, n, (void *)core, A);
  if (ierr) return ierr;
  ierr = MatShellSetOperation(*A, MATOP_MULT, (void (*)(void))MatMult_gpu);
  if (ierr) return ierr;
  return MatShellSetOperation(*A, MATOP_GET_DIAGONAL, (void (*)(void))MatGetDiagonal_gpu);
}
