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
 * MATSHELL operations MatMult / MatGetDiagonal of the device matrix.
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

PetscErrorCode Residual_gpu(SNES snes, Vec U, Vec F, void *core);
PetscErrorCode Tangent_gpu(SNES snes, Vec U, Mat A, Mat P, void *core);
/* MATSHELL operations (ctx = Core): MATOP_MULT, MATOP_GET_DIAGONAL. */
PetscErrorCode MatMult_gpu(void *core, Vec x, Vec y);
PetscErrorCode MatGetDiagonal_gpu(void *core, Vec d);

#ifdef __cplusplus
}
#endif
#endif
