/*
 * IGAP4-facing host layer over libigapgpu.so (C99).
 *
 * Drop-in replacements for the SNES callbacks that IGAPAssmInit registers in
 * struct __Assm (include/assmimpl.h:7-15, src/interface.c:201-202), same
 * signatures, same side effect (U_hist[0] <- U, src/assmcore_iga.c:68,557):
 *
 *   PetscErrorCode Residual_gpu(SNES, Vec U, Vec F, void *core);   // Residual_iga
 *   PetscErrorCode Tangent_gpu(SNES, Vec U, Mat A, Mat P, void *core); // Tangent_iga
 *
 * plus the set-up IGAPGPUAssmInit(core), which reads the partitioned mesh,
 * the law and the boundary data from IGAP4's own structs (one rank), and the
 * MATSHELL that stands in for the AIJ tangent IGAPAssmInit creates
 * (src/interface.c:191) and SNES receives (src/interface.c:219): its
 * MATOP_MULT and MATOP_GET_DIAGONAL operations run on the device matrix.
 *
 * Errors: every PetscErrorCode returned here is 0 or a positive PETSc error
 * class (PETSC_ERR_MEM, PETSC_ERR_ARG_WRONG, PETSC_ERR_ARG_WRONGSTATE,
 * PETSC_ERR_LIB), so SNES/KSP propagate them like their own; the library's
 * message goes to stderr and stays readable through igapgpu_last_error().
 *
 * Compile inside IGAP4 (after petscsnes.h and IGAP4's headers) or stand-alone
 * with igap_types.h.  The glue never computes residual or tangent values on
 * the CPU: an unknown law or a missing GPU is an error.
 */
#ifndef IGAPGPU_IGAP_H
#define IGAPGPU_IGAP_H

#include "petscsnes.h"
#include "igap_types.h"
#include "igapgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Map a law plugin's per-point residual callback to a device law id
 * (IGAPGPU_LAW_*).  IGAP4's own gradelast / gradelasttime are also found by
 * symbol name when the process exports them. */
int IGAPGPURegisterLaw(residual_ptr residual, int law_id);

/* Create the device context of a Core (after IGAPAssmInit built comm and
 * the partitioned mesh).  Returns 0 or an IGAPGPU_ERR_* code. */
int IGAPGPUAssmInit(Core core);
/* When on, Tangent_gpu also copies the device CSR into the PETSc AIJ matrix P
 * (for host-side preconditioners); off (default) keeps it on the device. */
int IGAPGPUSetHostMatrix(Core core, int on);
/* Destroy the device context of a Core. */
int IGAPGPUFinalize(Core core);
/* The device context of a Core (NULL if none). */
igapgpu_t IGAPGPUContext(Core core);

/* PETSc error class of an IGAPGPU_ERR_* code (0 stays 0). */
PetscErrorCode IGAPGPUPetscError(int rc);

PetscErrorCode Residual_gpu(SNES snes, Vec U, Vec F, void *core);
PetscErrorCode Tangent_gpu(SNES snes, Vec U, Mat A, Mat P, void *core);
/* A MATSHELL of the Core's device matrix (local and global size = the DOF
 * count of the one rank, shell context = core) with MATOP_MULT =
 * MatMult_gpu and MATOP_GET_DIAGONAL = MatGetDiagonal_gpu; pass it to
 * SNESSetJacobian as A and P in place of the AIJ matrix. */
PetscErrorCode IGAPGPUCreateMatShell(Core core, Mat *A);
/* MATSHELL operations, PETSc's MATOP_MULT / MATOP_GET_DIAGONAL signatures;
 * the Core comes from MatShellGetContext. */
PetscErrorCode MatMult_gpu(Mat A, Vec x, Vec y);
PetscErrorCode MatGetDiagonal_gpu(Mat A, Vec d);

#ifdef __cplusplus
}
#endif
#endif
