/*
 * Minimal single-rank PETSc stand-in used ONLY to compile the reference's own
 * C sources (src/assmcore_iga.c, src/interface.c, ...) into the CPU oracle.
 * Test infrastructure: never linked into the product library.
 *
 * Vec is a plain double array.  Mat is a row-compressed AIJ matrix whose
 * per-row capacity comes from the MatCreateAIJ preallocation
 * (src/interface.c:191, setnz_iga src/assmcore_iga.c:1054-1087); entries are
 * created on first MatSetValues (zeros included, as PETSc does), so after one
 * assembly the stored pattern equals the one PETSc would hold.
 * A Mat may also be a MATSHELL (MatCreateShell / MatShellSetOperation /
 * MatShellGetContext), whose MatMult and MatGetDiagonal call the registered
 * operations.  SNES/KSP/PC keep what IGAPSolvInit (src/interface.c:207-250)
 * sets, and SNESSolve runs a plain Newton method with a backtracking line
 * search over right-preconditioned GMRES(restart, modified Gram-Schmidt),
 * Jacobi from MatGetDiagonal of the preconditioning matrix (PCASM is taken
 * as Jacobi, with a warning), calling the registered residual and Jacobian
 * callbacks and MatMult of the operator: enough to drive the SNES callbacks
 * and a MATSHELL the way PETSc does, not a model of PETSc's arithmetic.
 */
#ifndef IGAP_ORACLE_STUB_PETSCSNES_H
#define IGAP_ORACLE_STUB_PETSCSNES_H

#include "mpi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef int PetscErrorCode;
typedef int PetscInt;
typedef double PetscScalar;
typedef double PetscReal;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;

#define PETSC_NULL 0
#define PETSC_COMM_WORLD MPI_COMM_WORLD
#define PETSC_COMM_SELF MPI_COMM_WORLD
/* error classes (petscerror.h values) */
#define PETSC_ERR_MEM 55
#define PETSC_ERR_ARG_WRONG 62
#define PETSC_ERR_ARG_WRONGSTATE 73
#define PETSC_ERR_LIB 76
#define PETSC_DEFAULT -2
#define PETSC_DECIDE -1

typedef struct _p_Vec *Vec;
typedef struct _p_Mat *Mat;
typedef struct _p_SNES *SNES;
typedef struct _p_KSP *KSP;
typedef struct _p_PC *PC;
typedef struct _p_SNESLineSearch *SNESLineSearch;

typedef enum { NOT_SET_VALUES, INSERT_VALUES, ADD_VALUES } InsertMode;
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef enum {
  MAT_KEEP_NONZERO_PATTERN,
  MAT_NO_OFF_PROC_ZERO_ROWS,
  MAT_SUBSET_OFF_PROC_ENTRIES,
  MAT_SYMMETRIC,
  MAT_SYMMETRY_ETERNAL
} MatOption;

typedef enum { MATOP_MULT = 3, MATOP_GET_DIAGONAL = 17 } MatOperation;

typedef const char *SNESType;
typedef const char *KSPType;
typedef const char *PCType;
typedef const char *SNESLineSearchType;
#define SNESNEWTONLS "newtonls"
#define SNESLINESEARCHBT "bt"
#define KSPGMRES "gmres"
#define KSPMINRES "minres"
#define KSPCG "cg"
#define PCASM "asm"
#define PCJACOBI "jacobi"
#define PCNONE "none"
typedef enum { SNES_LINESEARCH_ORDER_LINEAR = 1, SNES_LINESEARCH_ORDER_QUADRATIC = 2,
               SNES_LINESEARCH_ORDER_CUBIC = 3 } SNESLineSearchOrder;
typedef enum { PC_LEFT, PC_RIGHT, PC_SYMMETRIC } PCSide;
typedef enum { PC_ASM_BASIC = 3, PC_ASM_RESTRICT = 1, PC_ASM_INTERPOLATE = 2, PC_ASM_NONE = 0 } PCASMType;
typedef enum { KSP_CG_SYMMETRIC = 0 } KSPCGType;

typedef enum {
  SNES_CONVERGED_FNORM_ABS = 2,
  SNES_CONVERGED_FNORM_RELATIVE = 3,
  SNES_CONVERGED_SNORM_RELATIVE = 4,
  SNES_CONVERGED_ITS = 5,
  SNES_DIVERGED_FUNCTION_DOMAIN = -1,
  SNES_DIVERGED_FUNCTION_COUNT = -2,
  SNES_DIVERGED_LINEAR_SOLVE = -3,
  SNES_DIVERGED_FNORM_NAN = -4,
  SNES_DIVERGED_MAX_IT = -5,
  SNES_DIVERGED_LINE_SEARCH = -6,
  SNES_DIVERGED_INNER = -7,
  SNES_DIVERGED_LOCAL_MIN = -8,
  SNES_CONVERGED_ITERATING = 0
} SNESConvergedReason;
extern const char *const *SNESConvergedReasons;

typedef PetscErrorCode (*SNESFunctionFn)(SNES, Vec, Vec, void *);
typedef PetscErrorCode (*SNESJacobianFn)(SNES, Vec, Mat, Mat, void *);
PetscErrorCode KSPGMRESModifiedGramSchmidtOrthogonalization(KSP, PetscInt);
PetscErrorCode KSPGMRESClassicalGramSchmidtOrthogonalization(KSP, PetscInt);

PetscErrorCode PetscInitialize(int *argc, char ***argv, const char *file, const char *help);
PetscErrorCode PetscFinalize(void);

/* Vec */
PetscErrorCode VecCreateMPI(MPI_Comm comm, PetscInt n, PetscInt N, Vec *v);
PetscErrorCode VecDuplicate(Vec v, Vec *w);
PetscErrorCode VecDestroy(Vec *v);
PetscErrorCode VecSet(Vec v, PetscScalar a);
PetscErrorCode VecSetValues(Vec v, PetscInt n, const PetscInt *idx, const PetscScalar *val,
                            InsertMode mode);
PetscErrorCode VecAssemblyBegin(Vec v);
PetscErrorCode VecAssemblyEnd(Vec v);
PetscErrorCode VecGetArray(Vec v, PetscScalar **a);
PetscErrorCode VecRestoreArray(Vec v, PetscScalar **a);
PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar **a);
PetscErrorCode VecRestoreArrayRead(Vec v, const PetscScalar **a);

/* Mat (AIJ) */
PetscErrorCode MatCreateAIJ(MPI_Comm comm, PetscInt m, PetscInt n, PetscInt M, PetscInt N,
                            PetscInt d_nz, const PetscInt d_nnz[], PetscInt o_nz,
                            const PetscInt o_nnz[], Mat *A);
PetscErrorCode MatSetOption(Mat A, MatOption op, PetscBool flg);
PetscErrorCode MatZeroEntries(Mat A);
PetscErrorCode MatSetValues(Mat A, PetscInt m, const PetscInt idxm[], PetscInt n,
                            const PetscInt idxn[], const PetscScalar v[], InsertMode mode);
PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType t);
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType t);
PetscErrorCode MatZeroRowsColumns(Mat A, PetscInt n, const PetscInt rows[], PetscScalar diag,
                                  Vec x, Vec b);
PetscErrorCode MatDestroy(Mat *A);
PetscErrorCode MatGetSize(Mat A, PetscInt *m, PetscInt *n);
PetscErrorCode MatMult(Mat A, Vec x, Vec y);
PetscErrorCode MatGetDiagonal(Mat A, Vec d);

/* MATSHELL */
PetscErrorCode MatCreateShell(MPI_Comm comm, PetscInt m, PetscInt n, PetscInt M, PetscInt N,
                              void *ctx, Mat *A);
PetscErrorCode MatShellSetOperation(Mat A, MatOperation op, void (*fn)(void));
PetscErrorCode MatShellGetContext(Mat A, void *ctx);

/* SNES / KSP / PC */
PetscErrorCode SNESCreate(MPI_Comm comm, SNES *s);
PetscErrorCode SNESSetFunction(SNES s, Vec r, SNESFunctionFn f, void *ctx);
PetscErrorCode SNESSetJacobian(SNES s, Mat A, Mat P, SNESJacobianFn f, void *ctx);
PetscErrorCode SNESSetTolerances(SNES s, PetscReal abstol, PetscReal rtol, PetscReal stol,
                                 PetscInt maxit, PetscInt maxf);
PetscErrorCode SNESSetType(SNES s, SNESType t);
PetscErrorCode SNESGetLineSearch(SNES s, SNESLineSearch *ls);
PetscErrorCode SNESLineSearchSetType(SNESLineSearch ls, SNESLineSearchType t);
PetscErrorCode SNESLineSearchSetOrder(SNESLineSearch ls, SNESLineSearchOrder o);
PetscErrorCode SNESGetKSP(SNES s, KSP *k);
PetscErrorCode SNESSetFromOptions(SNES s);
PetscErrorCode SNESSolve(SNES s, Vec b, Vec x);
PetscErrorCode SNESGetConvergedReason(SNES s, SNESConvergedReason *r);
PetscErrorCode SNESGetFunctionNorm(SNES s, PetscReal *fnorm);
PetscErrorCode SNESGetIterationNumber(SNES s, PetscInt *its);
PetscErrorCode SNESDestroy(SNES *s);
PetscErrorCode KSPGetPC(KSP k, PC *pc);
PetscErrorCode KSPSetInitialGuessNonzero(KSP k, PetscBool flg);
PetscErrorCode KSPSetTolerances(KSP k, PetscReal rtol, PetscReal abstol, PetscReal dtol,
                                PetscInt maxits);
PetscErrorCode KSPSetType(KSP k, KSPType t);
PetscErrorCode KSPGMRESSetRestart(KSP k, PetscInt r);
PetscErrorCode KSPGMRESSetOrthogonalization(KSP k, PetscErrorCode (*fn)(KSP, PetscInt));
PetscErrorCode KSPSetPCSide(KSP k, PCSide side);
PetscErrorCode KSPGetIterationNumber(KSP k, PetscInt *its);
PetscErrorCode KSPCGSetType(KSP k, KSPCGType t);
PetscErrorCode PCSetType(PC pc, PCType t);
PetscErrorCode PCASMSetType(PC pc, PCASMType t);
PetscErrorCode PCJacobiSetUseAbs(PC pc, PetscBool flg);

#ifdef __cplusplus
}
#endif
#endif
