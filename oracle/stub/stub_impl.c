/*
 * Implementation of the single-rank MPI / PETSc stand-ins declared in
 * oracle/stub/mpi.h and oracle/stub/petscsnes.h.  Test infrastructure only:
 * it exists so that the reference's unmodified sources can be compiled and run
 * as the CPU oracle.  Nothing in the product links it.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "mpi.h"
#include "petscsnes.h"

/* ------------------------------------------------------------------ MPI -- */
static size_t type_size(MPI_Datatype t) { return t == MPI_INT ? sizeof(int) : sizeof(double); }

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm c) { (void)c; return MPI_SUCCESS; }

static void copy_if(void *dst, const void *src, size_t n)
{
  if (n && dst != src) memmove(dst, src, n);
}
int MPI_Scatter(const void *sb, int sc, MPI_Datatype st, void *rb, int rc, MPI_Datatype rt,
                int root, MPI_Comm c)
{
  (void)sc; (void)st; (void)root; (void)c;
  copy_if(rb, sb, (size_t)rc * type_size(rt));
  return MPI_SUCCESS;
}
int MPI_Scatterv(const void *sb, const int *scs, const int *ds, MPI_Datatype st, void *rb, int rc,
                 MPI_Datatype rt, int root, MPI_Comm c)
{
  (void)scs; (void)root; (void)c;
  copy_if(rb, (const char *)sb + (size_t)ds[0] * type_size(st), (size_t)rc * type_size(rt));
  return MPI_SUCCESS;
}
int MPI_Gather(const void *sb, int sc, MPI_Datatype st, void *rb, int rc, MPI_Datatype rt,
               int root, MPI_Comm c)
{
  (void)rc; (void)rt; (void)root; (void)c;
  copy_if(rb, sb, (size_t)sc * type_size(st));
  return MPI_SUCCESS;
}
int MPI_Gatherv(const void *sb, int sc, MPI_Datatype st, void *rb, const int *rcs, const int *ds,
                MPI_Datatype rt, int root, MPI_Comm c)
{
  (void)rcs; (void)root; (void)c;
  copy_if((char *)rb + (size_t)ds[0] * type_size(rt), sb, (size_t)sc * type_size(st));
  return MPI_SUCCESS;
}
int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c)
{
  (void)b; (void)n; (void)t; (void)root; (void)c;
  return MPI_SUCCESS;
}
int MPI_Allreduce(const void *sb, void *rb, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{
  (void)op; (void)c;
  copy_if(rb, sb, (size_t)n * type_size(t));
  return MPI_SUCCESS;
}

/* Self messages: a send record is kept until a receive with the same tag
 * waits on it.  Requests encode (kind, slot). */
#define MAXMSG 4096
static struct { const void *buf; size_t bytes; int tag; int live; } g_send[MAXMSG];
static struct { void *buf; size_t bytes; int tag; int live; } g_recv[MAXMSG];
static int g_nsend, g_nrecv;

int MPI_Isend(const void *buf, int n, MPI_Datatype t, int dest, int tag, MPI_Comm c,
              MPI_Request *req)
{
  (void)dest; (void)c;
  if (g_nsend >= MAXMSG) { fprintf(stderr, "stub MPI: too many sends\n"); abort(); }
  g_send[g_nsend].buf = buf; g_send[g_nsend].bytes = (size_t)n * type_size(t);
  g_send[g_nsend].tag = tag; g_send[g_nsend].live = 1;
  *req = 2 * g_nsend; g_nsend++;
  return MPI_SUCCESS;
}
int MPI_Irecv(void *buf, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Request *req)
{
  (void)src; (void)c;
  if (g_nrecv >= MAXMSG) { fprintf(stderr, "stub MPI: too many recvs\n"); abort(); }
  g_recv[g_nrecv].buf = buf; g_recv[g_nrecv].bytes = (size_t)n * type_size(t);
  g_recv[g_nrecv].tag = tag; g_recv[g_nrecv].live = 1;
  *req = 2 * g_nrecv + 1; g_nrecv++;
  return MPI_SUCCESS;
}
int MPI_Wait(MPI_Request *req, MPI_Status *st)
{
  (void)st;
  if (*req % 2 == 0) return MPI_SUCCESS; /* sends complete when matched */
  int r = *req / 2;
  if (!g_recv[r].live) return MPI_SUCCESS;
  for (int s = 0; s < g_nsend; s++) {
    if (g_send[s].live && g_send[s].tag == g_recv[r].tag) {
      if (g_send[s].bytes != g_recv[r].bytes) { fprintf(stderr, "stub MPI: size mismatch\n"); abort(); }
      memcpy(g_recv[r].buf, g_send[s].buf, g_recv[r].bytes);
      g_send[s].live = 0; g_recv[r].live = 0;
      break;
    }
  }
  if (g_recv[r].live) { fprintf(stderr, "stub MPI: unmatched self receive\n"); abort(); }
  /* reset the tables once every message has been consumed */
  int any = 0;
  for (int s = 0; s < g_nsend; s++) any |= g_send[s].live;
  for (int q = 0; q < g_nrecv; q++) any |= g_recv[q].live;
  if (!any) { g_nsend = 0; g_nrecv = 0; }
  return MPI_SUCCESS;
}

/* ---------------------------------------------------------------- PETSc -- */
struct _p_Vec { int n; double *a; };
typedef PetscErrorCode (*MultFn)(Mat, Vec, Vec);
typedef PetscErrorCode (*DiagFn)(Mat, Vec);
struct _p_Mat {
  int n;
  int shell;   /* MATSHELL: ctx + operations, no storage */
  void *ctx;
  MultFn mult;
  DiagFn diag;
  int *cap;    /* preallocated capacity per row */
  int *len;    /* entries used per row */
  int *start;  /* offset of each row in cols/vals */
  int *cols;
  double *vals;
  long nnz_cap;
};
struct _p_PC { int jacobi; };
struct _p_KSP {
  struct _p_PC pc;
  double rtol, abstol, dtol;
  int maxits, restart, its;
};
struct _p_SNESLineSearch { int order; };
struct _p_SNES {
  struct _p_KSP ksp;
  struct _p_SNESLineSearch ls;
  SNESFunctionFn f;
  void *fctx;
  Vec r;
  SNESJacobianFn J;
  void *jctx;
  Mat A, P;
  double abstol, rtol, stol;
  int maxit, its;
  double fnorm;
  SNESConvergedReason reason;
};

static const char *const g_reasons_storage[] = {
  "DIVERGED_LOCAL_MIN", "DIVERGED_INNER", "DIVERGED_LINE_SEARCH", "DIVERGED_MAX_IT",
  "DIVERGED_FNORM_NAN", "DIVERGED_LINEAR_SOLVE", "DIVERGED_FUNCTION_COUNT",
  "DIVERGED_FUNCTION_DOMAIN", "CONVERGED_ITERATING", "", "CONVERGED_FNORM_ABS",
  "CONVERGED_FNORM_RELATIVE", "CONVERGED_SNORM_RELATIVE", "CONVERGED_ITS"};
const char *const *SNESConvergedReasons = g_reasons_storage + 8;

PetscErrorCode KSPGMRESModifiedGramSchmidtOrthogonalization(KSP k, PetscInt i) { (void)k; (void)i; return 0; }
PetscErrorCode KSPGMRESClassicalGramSchmidtOrthogonalization(KSP k, PetscInt i) { (void)k; (void)i; return 0; }
PetscErrorCode PetscInitialize(int *ac, char ***av, const char *f, const char *h) { (void)ac; (void)av; (void)f; (void)h; return 0; }
PetscErrorCode PetscFinalize(void) { return 0; }

PetscErrorCode VecCreateMPI(MPI_Comm c, PetscInt n, PetscInt N, Vec *v)
{
  (void)c; (void)N;
  Vec x = (Vec)malloc(sizeof(*x));
  x->n = n; x->a = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
  *v = x;
  return 0;
}
PetscErrorCode VecDuplicate(Vec v, Vec *w) { return VecCreateMPI(0, v->n, v->n, w); }
PetscErrorCode VecDestroy(Vec *v) { if (*v) { free((*v)->a); free(*v); *v = 0; } return 0; }
PetscErrorCode VecSet(Vec v, PetscScalar a) { for (int i = 0; i < v->n; i++) v->a[i] = a; return 0; }
PetscErrorCode VecSetValues(Vec v, PetscInt n, const PetscInt *idx, const PetscScalar *val, InsertMode m)
{
  for (int i = 0; i < n; i++) {
    if (idx[i] < 0) continue;
    if (idx[i] >= v->n) { fprintf(stderr, "stub Vec: index out of range\n"); abort(); }
    if (m == ADD_VALUES) v->a[idx[i]] += val[i]; else v->a[idx[i]] = val[i];
  }
  return 0;
}
PetscErrorCode VecAssemblyBegin(Vec v) { (void)v; return 0; }
PetscErrorCode VecAssemblyEnd(Vec v) { (void)v; return 0; }
PetscErrorCode VecGetArray(Vec v, PetscScalar **a) { *a = v->a; return 0; }
PetscErrorCode VecRestoreArray(Vec v, PetscScalar **a) { (void)v; *a = 0; return 0; }
PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar **a) { *a = v->a; return 0; }
PetscErrorCode VecRestoreArrayRead(Vec v, const PetscScalar **a) { (void)v; *a = 0; return 0; }

PetscErrorCode MatCreateAIJ(MPI_Comm c, PetscInt m, PetscInt n, PetscInt M, PetscInt N,
                            PetscInt d_nz, const PetscInt d_nnz[], PetscInt o_nz,
                            const PetscInt o_nnz[], Mat *A)
{
  (void)c; (void)n; (void)M; (void)N;
  Mat a = (Mat)calloc(1, sizeof(*a));
  a->n = m;
  a->cap = (int *)malloc(sizeof(int) * (size_t)m);
  a->len = (int *)calloc((size_t)m, sizeof(int));
  a->start = (int *)malloc(sizeof(int) * (size_t)(m + 1));
  long tot = 0;
  for (int i = 0; i < m; i++) {
    int cap = (d_nnz ? d_nnz[i] : d_nz) + (o_nnz ? o_nnz[i] : o_nz);
    a->cap[i] = cap; a->start[i] = (int)tot; tot += cap;
  }
  a->start[m] = (int)tot;
  a->nnz_cap = tot;
  a->cols = (int *)malloc(sizeof(int) * (size_t)(tot > 0 ? tot : 1));
  a->vals = (double *)calloc((size_t)(tot > 0 ? tot : 1), sizeof(double));
  *A = a;
  return 0;
}
PetscErrorCode MatSetOption(Mat A, MatOption op, PetscBool f) { (void)A; (void)op; (void)f; return 0; }
PetscErrorCode MatZeroEntries(Mat A) { memset(A->vals, 0, sizeof(double) * (size_t)A->nnz_cap); return 0; }

static double *mat_slot(Mat A, int r, int c)
{
  int *cols = A->cols + A->start[r];
  int lo = 0, hi = A->len[r];
  while (lo < hi) {
    int mid = (lo + hi) / 2;
    if (cols[mid] < c) lo = mid + 1; else hi = mid;
  }
  if (lo < A->len[r] && cols[lo] == c) return A->vals + A->start[r] + lo;
  if (A->len[r] >= A->cap[r]) {
    fprintf(stderr, "stub Mat: row %d exceeds preallocation %d\n", r, A->cap[r]);
    abort();
  }
  double *vals = A->vals + A->start[r];
  memmove(cols + lo + 1, cols + lo, sizeof(int) * (size_t)(A->len[r] - lo));
  memmove(vals + lo + 1, vals + lo, sizeof(double) * (size_t)(A->len[r] - lo));
  cols[lo] = c; vals[lo] = 0.0; A->len[r]++;
  return vals + lo;
}
PetscErrorCode MatSetValues(Mat A, PetscInt m, const PetscInt im[], PetscInt n,
                            const PetscInt in[], const PetscScalar v[], InsertMode mode)
{
  for (int i = 0; i < m; i++) {
    if (im[i] < 0) continue;
    for (int j = 0; j < n; j++) {
      if (in[j] < 0) continue;
      double *s = mat_slot(A, im[i], in[j]);
      if (mode == ADD_VALUES) *s += v[(size_t)i * n + j]; else *s = v[(size_t)i * n + j];
    }
  }
  return 0;
}
PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType t) { (void)A; (void)t; return 0; }
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType t) { (void)A; (void)t; return 0; }
PetscErrorCode MatZeroRowsColumns(Mat A, PetscInt n, const PetscInt rows[], PetscScalar diag,
                                  Vec x, Vec b)
{
  (void)x; (void)b;
  char *flag = (char *)calloc((size_t)A->n, 1);
  for (int i = 0; i < n; i++) flag[rows[i]] = 1;
  for (int r = 0; r < A->n; r++) {
    for (int k = 0; k < A->len[r]; k++) {
      int c = A->cols[A->start[r] + k];
      if (flag[r] || flag[c]) A->vals[A->start[r] + k] = 0.0;
    }
  }
  for (int r = 0; r < A->n; r++)
    if (flag[r]) *mat_slot(A, r, r) = diag;
  free(flag);
  return 0;
}
PetscErrorCode MatGetSize(Mat A, PetscInt *m, PetscInt *n)
{
  if (m) *m = A->n;
  if (n) *n = A->n;
  return 0;
}
PetscErrorCode MatMult(Mat A, Vec x, Vec y)
{
  if (A->shell) {
    if (!A->mult) { fprintf(stderr, "stub Mat: MATSHELL without MATOP_MULT\n"); return PETSC_ERR_ARG_WRONGSTATE; }
    return A->mult(A, x, y);
  }
  for (int r = 0; r < A->n; r++) {
    double acc = 0.0;
    for (int k = 0; k < A->len[r]; k++) acc += A->vals[A->start[r] + k] * x->a[A->cols[A->start[r] + k]];
    y->a[r] = acc;
  }
  return 0;
}
PetscErrorCode MatGetDiagonal(Mat A, Vec d)
{
  if (A->shell) {
    if (!A->diag) { fprintf(stderr, "stub Mat: MATSHELL without MATOP_GET_DIAGONAL\n"); return PETSC_ERR_ARG_WRONGSTATE; }
    return A->diag(A, d);
  }
  for (int r = 0; r < A->n; r++) {
    d->a[r] = 0.0;
    for (int k = 0; k < A->len[r]; k++)
      if (A->cols[A->start[r] + k] == r) d->a[r] = A->vals[A->start[r] + k];
  }
  return 0;
}
PetscErrorCode MatCreateShell(MPI_Comm c, PetscInt m, PetscInt n, PetscInt M, PetscInt N, void *ctx, Mat *A)
{
  (void)c; (void)n; (void)M; (void)N;
  Mat a = (Mat)calloc(1, sizeof(*a));
  a->n = m;
  a->shell = 1;
  a->ctx = ctx;
  *A = a;
  return 0;
}
PetscErrorCode MatShellSetOperation(Mat A, MatOperation op, void (*fn)(void))
{
  if (!A->shell) return PETSC_ERR_ARG_WRONG;
  if (op == MATOP_MULT) A->mult = (MultFn)fn;
  else if (op == MATOP_GET_DIAGONAL) A->diag = (DiagFn)fn;
  else return PETSC_ERR_ARG_WRONG;
  return 0;
}
PetscErrorCode MatShellGetContext(Mat A, void *ctx)
{
  if (!A || !A->shell) return PETSC_ERR_ARG_WRONG;
  *(void **)ctx = A->ctx;
  return 0;
}
PetscErrorCode MatDestroy(Mat *A)
{
  if (*A) {
    free((*A)->cap); free((*A)->len); free((*A)->start); free((*A)->cols); free((*A)->vals);
    free(*A); *A = 0;
  }
  return 0;
}

/* Accessors used by the oracle driver (not PETSc API). */
int oracle_stub_vec_size(Vec v) { return v->n; }
double *oracle_stub_vec_array(Vec v) { return v->a; }
long oracle_stub_mat_nnz(Mat A)
{
  long s = 0;
  for (int r = 0; r < A->n; r++) s += A->len[r];
  return s;
}
/* Copy out as CSR (rowptr n+1, cols nnz, vals nnz), rows in order, columns ascending. */
void oracle_stub_mat_csr(Mat A, long *rowptr, int *cols, double *vals)
{
  long p = 0;
  rowptr[0] = 0;
  for (int r = 0; r < A->n; r++) {
    memcpy(cols + p, A->cols + A->start[r], sizeof(int) * (size_t)A->len[r]);
    memcpy(vals + p, A->vals + A->start[r], sizeof(double) * (size_t)A->len[r]);
    p += A->len[r];
    rowptr[r + 1] = p;
  }
}

/* SNES / KSP / PC: settings as IGAPSolvInit leaves them; SNESSolve is a
 * plain Newton / GMRES driver that calls the registered callbacks. */
PetscErrorCode SNESCreate(MPI_Comm c, SNES *s)
{
  (void)c;
  SNES n = (SNES)calloc(1, sizeof(*n));
  n->abstol = 1e-50; n->rtol = 1e-8; n->stol = 1e-8; n->maxit = 50;
  n->ksp.rtol = 1e-5; n->ksp.abstol = 1e-50; n->ksp.dtol = 1e5; n->ksp.maxits = 10000; n->ksp.restart = 30;
  n->ksp.pc.jacobi = 1;
  *s = n;
  return 0;
}
PetscErrorCode SNESSetFunction(SNES s, Vec r, SNESFunctionFn f, void *ctx) { s->r = r; s->f = f; s->fctx = ctx; return 0; }
PetscErrorCode SNESSetJacobian(SNES s, Mat A, Mat P, SNESJacobianFn f, void *ctx)
{
  s->A = A; s->P = P; s->J = f; s->jctx = ctx;
  return 0;
}
PetscErrorCode SNESSetTolerances(SNES s, PetscReal a, PetscReal r, PetscReal st, PetscInt mi, PetscInt mf)
{
  (void)mf;
  if (a != PETSC_DEFAULT) s->abstol = a;
  if (r != PETSC_DEFAULT) s->rtol = r;
  if (st != PETSC_DEFAULT) s->stol = st;
  if (mi != PETSC_DEFAULT) s->maxit = mi;
  return 0;
}
PetscErrorCode SNESSetType(SNES s, SNESType t) { (void)s; return strcmp(t, SNESNEWTONLS) ? PETSC_ERR_ARG_WRONG : 0; }
PetscErrorCode SNESGetLineSearch(SNES s, SNESLineSearch *ls) { *ls = &s->ls; return 0; }
PetscErrorCode SNESLineSearchSetType(SNESLineSearch ls, SNESLineSearchType t) { (void)ls; (void)t; return 0; }
PetscErrorCode SNESLineSearchSetOrder(SNESLineSearch ls, SNESLineSearchOrder o) { ls->order = (int)o; return 0; }
PetscErrorCode SNESGetKSP(SNES s, KSP *k) { *k = &s->ksp; return 0; }
PetscErrorCode SNESSetFromOptions(SNES s) { (void)s; return 0; }
PetscErrorCode SNESGetConvergedReason(SNES s, SNESConvergedReason *r) { *r = s->reason; return 0; }
PetscErrorCode SNESGetFunctionNorm(SNES s, PetscReal *f) { *f = s->fnorm; return 0; }
PetscErrorCode SNESGetIterationNumber(SNES s, PetscInt *i) { *i = s->its; return 0; }
PetscErrorCode SNESDestroy(SNES *s) { if (*s) free(*s); *s = 0; return 0; }
PetscErrorCode KSPGetPC(KSP k, PC *pc) { *pc = &k->pc; return 0; }
PetscErrorCode KSPSetInitialGuessNonzero(KSP k, PetscBool f) { (void)k; (void)f; return 0; }
PetscErrorCode KSPSetTolerances(KSP k, PetscReal r, PetscReal a, PetscReal d, PetscInt m)
{
  if (r != PETSC_DEFAULT) k->rtol = r;
  if (a != PETSC_DEFAULT) k->abstol = a;
  if (d != PETSC_DEFAULT) k->dtol = d;
  if (m != PETSC_DEFAULT) k->maxits = m;
  return 0;
}
PetscErrorCode KSPSetType(KSP k, KSPType t) { (void)k; return strcmp(t, KSPGMRES) ? PETSC_ERR_ARG_WRONG : 0; }
PetscErrorCode KSPGMRESSetRestart(KSP k, PetscInt r) { k->restart = r; return 0; }
PetscErrorCode KSPGMRESSetOrthogonalization(KSP k, PetscErrorCode (*fn)(KSP, PetscInt)) { (void)k; (void)fn; return 0; }
PetscErrorCode KSPSetPCSide(KSP k, PCSide s) { (void)k; return s == PC_RIGHT ? 0 : PETSC_ERR_ARG_WRONG; }
PetscErrorCode KSPGetIterationNumber(KSP k, PetscInt *i) { *i = k->its; return 0; }
PetscErrorCode KSPCGSetType(KSP k, KSPCGType t) { (void)k; (void)t; return 0; }
PetscErrorCode PCSetType(PC pc, PCType t)
{
  if (!strcmp(t, PCJACOBI)) pc->jacobi = 1;
  else if (!strcmp(t, PCNONE)) pc->jacobi = 0;
  else if (!strcmp(t, PCASM)) {
    fprintf(stderr, "stub PC: PCASM taken as Jacobi\n");
    pc->jacobi = 1;
  } else return PETSC_ERR_ARG_WRONG;
  return 0;
}
PetscErrorCode PCASMSetType(PC pc, PCASMType t) { (void)pc; (void)t; return 0; }
PetscErrorCode PCJacobiSetUseAbs(PC pc, PetscBool f) { (void)pc; (void)f; return 0; }

static double vnorm(int n, const double *a)
{
  double s = 0.0;
  for (int i = 0; i < n; i++) s += a[i] * a[i];
  return sqrt(s);
}

/* Right-preconditioned GMRES(m) with modified Gram-Schmidt on A x = b from
 * x = 0; z = M^-1 v with M = diag(P) (or the identity). */
static PetscErrorCode ksp_gmres(KSP k, Mat A, Mat P, Vec b, Vec x)
{
  const int n = b->n, m = k->restart > 0 ? (k->restart < 200 ? k->restart : 200) : 30;
  PetscErrorCode ierr = 0;
  double *dinv = (double *)malloc(sizeof(double) * (size_t)n);
  double *V = (double *)malloc(sizeof(double) * (size_t)n * (m + 1));
  double *Z = (double *)malloc(sizeof(double) * (size_t)n * m);
  double *H = (double *)calloc((size_t)(m + 1) * m, sizeof(double));
  double *cs = (double *)malloc(sizeof(double) * m), *sn = (double *)malloc(sizeof(double) * m);
  double *g = (double *)malloc(sizeof(double) * (m + 1)), *yv = (double *)malloc(sizeof(double) * m);
  Vec vin, vout;
  VecDuplicate(b, &vin);
  VecDuplicate(b, &vout);
  if (k->pc.jacobi) {
    Vec d;
    VecDuplicate(b, &d);
    ierr = MatGetDiagonal(P, d);
    for (int i = 0; i < n && !ierr; i++) dinv[i] = d->a[i] != 0.0 ? 1.0 / d->a[i] : 1.0;
    VecDestroy(&d);
  } else {
    for (int i = 0; i < n; i++) dinv[i] = 1.0;
  }
  memset(x->a, 0, sizeof(double) * (size_t)n);
  const double bnorm = vnorm(n, b->a);
  const double tol = fmax(k->rtol * bnorm, k->abstol);
  k->its = 0;
  double rnorm = bnorm;
  while (!ierr && rnorm > tol && k->its < k->maxits) {
    /* r = b - A x */
    memcpy(vin->a, x->a, sizeof(double) * (size_t)n);
    if ((ierr = MatMult(A, vin, vout))) break;
    for (int i = 0; i < n; i++) V[i] = b->a[i] - vout->a[i];
    double beta = vnorm(n, V);
    if (beta == 0.0) { rnorm = 0.0; break; }
    for (int i = 0; i < n; i++) V[i] /= beta;
    for (int i = 0; i <= m; i++) g[i] = 0.0;
    g[0] = beta;
    int j = 0;
    for (; j < m && k->its < k->maxits; j++) {
      double *zj = Z + (size_t)n * j, *w = V + (size_t)n * (j + 1);
      for (int i = 0; i < n; i++) zj[i] = dinv[i] * V[(size_t)n * j + i];
      memcpy(vin->a, zj, sizeof(double) * (size_t)n);
      if ((ierr = MatMult(A, vin, vout))) break;
      memcpy(w, vout->a, sizeof(double) * (size_t)n);
      for (int q = 0; q <= j; q++) {
        const double *vq = V + (size_t)n * q;
        double h = 0.0;
        for (int i = 0; i < n; i++) h += w[i] * vq[i];
        H[q * m + j] = h;
        for (int i = 0; i < n; i++) w[i] -= h * vq[i];
      }
      double hn = vnorm(n, w);
      H[(j + 1) * m + j] = hn;
      if (hn != 0.0)
        for (int i = 0; i < n; i++) w[i] /= hn;
      for (int q = 0; q < j; q++) {
        double a = H[q * m + j], c = H[(q + 1) * m + j];
        H[q * m + j] = cs[q] * a + sn[q] * c;
        H[(q + 1) * m + j] = -sn[q] * a + cs[q] * c;
      }
      double a = H[j * m + j], c = H[(j + 1) * m + j], r = hypot(a, c);
      cs[j] = r != 0.0 ? a / r : 1.0;
      sn[j] = r != 0.0 ? c / r : 0.0;
      H[j * m + j] = r;
      H[(j + 1) * m + j] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      k->its++;
      rnorm = fabs(g[j + 1]);
      if (rnorm <= tol || hn == 0.0) { j++; break; }
    }
    if (ierr) break;
    for (int q = j - 1; q >= 0; q--) {
      double s = g[q];
      for (int t = q + 1; t < j; t++) s -= H[q * m + t] * yv[t];
      yv[q] = s / H[q * m + q];
    }
    for (int q = 0; q < j; q++)
      for (int i = 0; i < n; i++) x->a[i] += yv[q] * Z[(size_t)n * q + i];
    if (rnorm > k->dtol * bnorm) break;
  }
  VecDestroy(&vin);
  VecDestroy(&vout);
  free(dinv); free(V); free(Z); free(H); free(cs); free(sn); free(g); free(yv);
  return ierr;
}

/* Newton with a backtracking line search on 1/2 |F|^2 (full step first,
 * then quadratic backtracking, step kept in [0.1, 0.5] of the previous). */
PetscErrorCode SNESSolve(SNES s, Vec b, Vec x)
{
  (void)b;
  if (!s->f || !s->J || !s->A) return PETSC_ERR_ARG_WRONGSTATE;
  PetscErrorCode ierr;
  const int n = x->n;
  Vec F = s->r, Y, Xb;
  int ownF = 0;
  if (!F) { VecDuplicate(x, &F); ownF = 1; }
  VecDuplicate(x, &Y);
  VecDuplicate(x, &Xb);
  s->its = 0;
  s->reason = SNES_CONVERGED_ITERATING;
  if ((ierr = s->f(s, x, F, s->fctx))) goto done;
  double fnorm = vnorm(n, F->a);
  const double fnorm0 = fnorm;
  for (;;) {
    if (!isfinite(fnorm)) { s->reason = SNES_DIVERGED_FNORM_NAN; break; }
    if (fnorm <= s->abstol) { s->reason = SNES_CONVERGED_FNORM_ABS; break; }
    if (s->its > 0 && fnorm <= s->rtol * fnorm0) { s->reason = SNES_CONVERGED_FNORM_RELATIVE; break; }
    if (s->its >= s->maxit) { s->reason = SNES_DIVERGED_MAX_IT; break; }
    if ((ierr = s->J(s, x, s->A, s->P ? s->P : s->A, s->jctx))) break;
    /* J Y = F, x <- x - lam Y */
    if ((ierr = ksp_gmres(&s->ksp, s->A, s->P ? s->P : s->A, F, Y))) break;
    memcpy(Xb->a, x->a, sizeof(double) * (size_t)n);
    const double f0 = 0.5 * fnorm * fnorm, slope = -fnorm * fnorm;
    double lam = 1.0, fn = fnorm;
    int ok = 0;
    for (int ls = 0; ls < 30; ls++) {
      for (int i = 0; i < n; i++) x->a[i] = Xb->a[i] - lam * Y->a[i];
      if ((ierr = s->f(s, x, F, s->fctx))) break;
      fn = vnorm(n, F->a);
      const double fl = 0.5 * fn * fn;
      if (isfinite(fl) && fl <= f0 + 1e-4 * lam * slope) { ok = 1; break; }
      double lnew = isfinite(fl) ? -slope * lam * lam / (2.0 * (fl - f0 - lam * slope)) : 0.5 * lam;
      lam = fmin(fmax(lnew, 0.1 * lam), 0.5 * lam);
    }
    if (ierr) break;
    s->its++;
    fnorm = fn;
    if (!ok) { s->reason = SNES_DIVERGED_LINE_SEARCH; break; }
    if (lam * vnorm(n, Y->a) <= s->stol * vnorm(n, x->a)) { s->reason = SNES_CONVERGED_SNORM_RELATIVE; break; }
  }
  s->fnorm = fnorm;
done:
  VecDestroy(&Y);
  VecDestroy(&Xb);
  if (ownF) VecDestroy(&F);
  return ierr;
}
