/*
 * igapgpu.h -- C ABI of libigapgpu.so, the GB300 (sm_103a) implementation of
 * IGAP4's element assembly and Newton-Krylov inner loop on one GPU.
 *
 * Plain C types only.  Every array argument may be a host pointer or a CUDA
 * device pointer; the library inspects it (cudaPointerGetAttributes) and
 * stages host data through device buffers it owns.  With device pointers the
 * call is asynchronous on the context's stream; with any host pointer the call
 * returns after the host data are consumed / produced.
 *
 * Numbering follows the reference on one rank: control point
 *   cp = (ny+p)(nz+p) ix + (nz+p) iy + iz,  DOF = 3 cp + d
 * (src/interface.c:163-168, src/commcore_iga.c:28-37), state history
 * U_hist[(torder+1)][ndof] with level 0 the current iterate
 * (include/coreimpl.h:17, src/assmcore_iga.c:66-80).
 *
 * Errors: every entry point returns IGAPGPU_OK (0) or a negative code; the
 * text of the last error is available from igapgpu_last_error().  There is no
 * CPU fallback: without a usable GPU, igapgpu_assm_init fails.
 *
 * Threads: a context is used by one host thread at a time (as IGAP4 drives
 * its Core from one thread per rank); distinct contexts on distinct streams
 * may run concurrently, but the first call of each kernel kind sets its
 * shared-memory limit once, so make one call per kind before going parallel.
 */
#ifndef IGAPGPU_H
#define IGAPGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IGAPGPU_OK 0
#define IGAPGPU_ERR_ARG -1       /* invalid argument / unsupported configuration */
#define IGAPGPU_ERR_CUDA -2      /* CUDA runtime error */
#define IGAPGPU_ERR_NOMEM -3     /* device allocation failed */
#define IGAPGPU_ERR_LAW -4       /* unknown constitutive law: no CPU fallback */
#define IGAPGPU_ERR_NUMERIC -5   /* non-finite residual norm / breakdown */
#define IGAPGPU_ERR_STATE -6     /* call order violated (e.g. matmult before tangent) */
#define IGAPGPU_ERR_TIMEOUT -7   /* a bounded device wait expired */

/* Laws: the reference's two plugins and the project's linear law. */
#define IGAPGPU_LAW_GRADELAST 0     /* phys/gradelast.c, torder 0, par[9] */
#define IGAPGPU_LAW_GRADELASTTIME 1 /* phys/gradelasttime.c, torder 2, par[9] */
#define IGAPGPU_LAW_LINGRAD 2       /* linear isotropic strain gradient, par = {lambda, mu, ell} */

/* Precision of the element contractions (norms, Krylov dots and the multiply stay FP64).
 * In both tensor-core modes the residual's contractions run in double-FP32 arithmetic
 * (pairs of floats, compensated sums; the reference's laws keep their FP64 law between
 * them): relative error <= 1e-12 vs FP64 (measured ~1e-14); IGAPGPU_RES_DF=0 keeps FP64. */
#define IGAPGPU_PREC_FP64 0  /* FP64 everywhere */
#define IGAPGPU_PREC_SPLIT 1 /* tangent on the tensor cores: TF32x3 products (hi*hi + hi*lo + lo*hi),
                                FP32 accumulate; relative error <= 1e-5 (measured ~2e-6) */
#define IGAPGPU_PREC_OZAKI 2 /* FP64-quality tangent on the tensor cores (linear law): the sqrt(w)-weighted
                                Gram operands split error-free into four BF16 slices with a power-of-two
                                scale per row (Ozaki scheme), exact FP32 accumulation of the leading
                                product, FP64 recombination; relative error <= 1e-9 (measured ~1e-11);
                                other laws, or slices that do not fit in memory: the FP64 kernel;
                                single lattices only */

typedef struct igapgpu_ctx *igapgpu_t;

/* Mesh of one rank (the global mesh on one GPU), as struct __Mesh holds it
 * after partitioning (include/meshimpl.h:6-16). */
typedef struct {
  int porder;             /* B-spline degree, 2 */
  int nelem[3];           /* elements per direction */
  const double *knots[3]; /* knot vectors, nelem[d] + 1 + 2 porder entries */
  const double *w;        /* weights, prod(nelem+porder) entries, x-major, z fastest */
  const double *X;        /* control points, 3 per weight */
} igapgpu_mesh_desc;

/* Law selection and parameters (struct __Phys, include/physimpl.h:13-28). */
typedef struct {
  int law;
  double par[9];
} igapgpu_phys_desc;

/* Boundary data (struct __BC, include/bcimpl.h:8-15) with the Neumann
 * callback replaced by a constant traction table.  Index 6*face + 3*order + d;
 * faces 0/1 = x-min/x-max, 2/3 = y, 4/5 = z; bc_type 1 = Neumann, 0 = Dirichlet. */
typedef struct {
  int bc_type[36];
  double par_periodic[9]; /* affine periodic offset; must be 0 on a non-periodic mesh */
  double par_dirichlet[9];
  double neumann[36];
} igapgpu_bc_desc;

/* Newton-Krylov options (defaults of IGAPSolvInit, src/interface.c:207-250). */
typedef struct {
  double snes_abstol;  /* |F| below this: converged (1e-10) */
  double snes_rtol;    /* relative to |F_0| (1e-20) */
  double snes_stol;    /* |dU| / |U| step tolerance (1e-20) */
  int snes_max_it;     /* Newton iterations (the reference loops SNES max_it=1 up to 10000) */
  int linesearch;      /* 0 = full step, 1 = backtracking (cubic) */
  int ksp_restart;     /* GMRES restart length */
  double ksp_rtol;     /* relative residual tolerance of the linear solve */
  double ksp_abstol;
  double ksp_dtol;
  int ksp_max_it;
  int pc;              /* 0 = none, 1 = Jacobi, 2 = point-block Jacobi (3 x 3 blocks of each control point),
                          3 = cell-block Jacobi (blocks of 2 x 2 x 2 control points, up to 24 x 24; single lattice),
                          4 = restricted additive Schwarz: the cells of 3 extended by one control-point layer
                              (up to 192 DOFs), FP32 subdomain solves, each DOF from its own cell (the
                              reference's default PCASM / PC_ASM_RESTRICT, src/interface.c:240-241; single lattice) */
  int use_graphs;      /* 1: assembly and GMRES cycles replayed as CUDA graphs */
  int orth;            /* GMRES orthogonalisation: 0 = modified Gram-Schmidt (the reference's
                          KSPGMRESModifiedGramSchmidtOrthogonalization, src/interface.c:234);
                          1 = classical Gram-Schmidt applied twice (CGS2: two block passes per
                          Arnoldi step instead of one dot and one update per basis vector;
                          graph GMRES only, the host-driven GMRES always uses MGS) */
  double snes_f0_max;  /* > 0: an initial iterate whose |F| exceeds this is rejected before any Newton
                          step (reason IGAPGPU_REASON_REJECTED, U unchanged): a predicted guess is
                          tried against the residual of the plain guess without a second solve */
} igapgpu_solver_opts;

#define IGAPGPU_REASON_REJECTED (-9) /* igapgpu_solve: initial |F| above snes_f0_max */

typedef struct {
  int newton_its;
  int ksp_its_total;
  int ksp_its_last;
  int converged;     /* 1 converged, 0 not (reason < 0) */
  int reason;        /* PETSc-like SNESConvergedReason value */
  double fnorm0;
  double fnorm;
} igapgpu_solve_stats;

/* IGAPAssmInit (src/interface.c:131-203): upload the mesh, build the CSR
 * pattern (setnz_iga, src/assmcore_iga.c:1054-1087, plus the columns the
 * element loop inserts), the element colouring, the Dirichlet row list and the
 * Neumann load; allocate the state history, residual and matrix.
 * nquad: Gauss points per direction (4 as the reference, 3 allowed). */
int igapgpu_assm_init(igapgpu_t *ctx, const igapgpu_mesh_desc *mesh,
                      const igapgpu_phys_desc *phys, const igapgpu_bc_desc *bc, int nquad);
/* Frees every device buffer of the context (IGAPFinalize, src/interface.c:362). */
int igapgpu_finalize(igapgpu_t ctx);

int igapgpu_sizes(igapgpu_t ctx, int64_t *ndof, int64_t *nnz, int *torder, int64_t *nelem);
/* CSR pattern: rowptr[ndof+1] (int64), cols[nnz] (int32), rows in DOF order,
 * columns ascending -- the AIJ structure PETSc holds after the first
 * MatSetValues of Tangent_iga (MAT_KEEP_NONZERO_PATTERN, src/interface.c:196). */
int igapgpu_pattern(igapgpu_t ctx, int64_t *rowptr, int32_t *cols);

/* Dirichlet rows (unique) and their prescribed values g: the rows
 * Residual_iga sets to U - g (src/assmcore_iga.c:451-495) and Tangent_iga
 * clears with MatZeroRowsColumns (src/assmcore_iga.c:844).  rows / values may be NULL, host or device. */
int igapgpu_dirichlet(igapgpu_t ctx, int64_t *count, int64_t *rows, double *values);
/* U[r] = g_r on every Dirichlet row (U host or device), so that an initial
 * iterate meets the constraints the Newton correction does not move. */
int igapgpu_impose_dirichlet(igapgpu_t ctx, double *U);

/* iga_intdensity (src/postcore_iga.c:13-377): the law's densities integrated
 * over the body on the current U_hist, minus the traction term on the Neumann
 * faces.  HH receives *ndensity values (at most 16): the static gradient law
 * 13 (energy, 2 dpsi/dE_ab, sector fractions), the transient law 2 (energy
 * incl. kinetic, volume), the linear law 2 (energy, volume). */
int igapgpu_density(igapgpu_t ctx, double *HH, int *ndensity);

/* Field sampling of iga_plotfield (src/mgl/plotcore_iga.c:16-282) into a
 * headless buffer instead of a MathGL frame: the law's field callback
 * (include/physimpl.h:8) on the current U_hist at a lattice of nppe samples
 * per element and direction plus the far faces, (nppe nelem[d] + 1) points
 * per direction, x-major, z fastest.  field [npoints][nfield]: the static
 * gradient law 33 (u[0..29], e1, e2, sector code: phys/gradelast.c:1105), the
 * transient law 6 (midpoint displacement, e1, e2, sector code:
 * phys/gradelasttime.c:9242), the linear law 33 (u[0..29], tr eps, |dev eps|,
 * psi).  xq [npoints][3]: the knot coordinates the reference plots against;
 * X [npoints][3]: physical positions.  Outputs may be NULL, host or device;
 * with all three NULL only *nfield and *npoints are set.  1 <= nppe <= 64. */
int igapgpu_sample_field(igapgpu_t ctx, int nppe, double *field, double *xq, double *X, int *nfield,
                         int64_t *npoints);

/* Race check of the colour-partitioned scatter (a debug aid): counts[nnz]
 * receives, per CSR slot, how many element contributions landed in it when
 * every element adds 1 to each of its slots with a plain read-modify-write,
 * colour by colour.  Without lost updates that is the number of elements
 * whose support holds both control points of the slot.  Host or device. */
int igapgpu_debug_slot_counts(igapgpu_t ctx, double *counts);

/* IGAPSolvSaveSolution / IGAPSolvLoadSolution (src/interface.c:271-300): the
 * reference's solution file (write_solution / read_solution, src/ioutil.c:
 * 90-159), raw FP64 levels in DOF order; static laws level 0, the transient
 * law levels 1..torder (load also sets level 0 = level 1). */
int igapgpu_save_solution(igapgpu_t ctx, const char *fname);
int igapgpu_load_solution(igapgpu_t ctx, const char *fname);

/* State history U_hist[level] (level 0 current, 1 = u_n, 2 = u_{n-1}). */
int igapgpu_set_history(igapgpu_t ctx, int level, const double *U);
int igapgpu_get_history(igapgpu_t ctx, int level, double *U);
/* Time advance of the three-level scheme: u_{n-1} <- u_n, u_n <- U_hist[0].
 * The reference has no such routine; its callers shift the history. */
int igapgpu_shift_history(igapgpu_t ctx);

/* Residual_iga (src/assmcore_iga.c:16-502): RR = volume residual + Neumann
 * load, Dirichlet rows replaced by U - g.  Side effect as in the reference:
 * U_hist[0] <- U.  U may be NULL (use U_hist[0]). */
int igapgpu_residual(igapgpu_t ctx, const double *U, double *RR);
/* Tangent_iga (src/assmcore_iga.c:507-858): CSR values of dRR/dU in the
 * pattern order, Dirichlet rows and columns zeroed with unit diagonal
 * (MatZeroRowsColumns).  vals may be NULL: the context's own matrix (used by
 * igapgpu_matmult / the Newton solver) is assembled.  U may be NULL. */
int igapgpu_tangent(igapgpu_t ctx, const double *U, double *vals);
/* Residual and tangent in one fused element pass (same results as the two
 * calls above).  RR / vals may be NULL as above. */
int igapgpu_assemble(igapgpu_t ctx, const double *U, double *RR, double *vals);

/* MatMult of the context's matrix (MATSHELL MATOP_MULT): y = K x. */
int igapgpu_matmult(igapgpu_t ctx, const double *x, double *y);
/* VecNorm(NORM_2) of a device or host vector of the context's size, in FP64
 * (the Newton residual norm, SNESGetFunctionNorm at src/interface.c:322). */
int igapgpu_norm2(igapgpu_t ctx, const double *x, double *out);
/* igapgpu_norm2 without any device allocation.  No counterpart in the
 * reference.  For callers that cannot obtain device memory from cudaMalloc:
 * applications whose pool allocator already owns the GPU's memory (PyTorch's
 * caching allocator, a PETSc device pool), and code that must not allocate or
 * free because cudaMalloc / cudaFree can synchronise the whole device.
 * x: n doubles in device memory; out: host or device pointer to one double;
 * stream: cudaStream_t (NULL = default stream).  No context is needed.
 * Scratch: a fixed 64 KiB array of partial sums compiled into the library,
 * present on every GPU that loads it until the process exits; hence
 * n <= 33,554,432 (8192 partial sums of 4096 elements), larger n is rejected
 * with IGAPGPU_ERR_ARG.  The first call on each device looks up the array's
 * device address (cudaGetSymbolAddress, with that device current); make that
 * first call before any stream capture.  All calls share the one array, so
 * calls that overlap on the GPU race; serialise them on one stream. */
int igapgpu_norm2_noalloc(const double *x, int64_t n, double *out, void *stream);
/* MatGetDiagonal (MATOP_GET_DIAGONAL, used by Jacobi). */
int igapgpu_get_diagonal(igapgpu_t ctx, double *diag);

/* KSPSolve on the context's matrix: right-preconditioned GMRES(restart) with
 * modified Gram-Schmidt (src/interface.c:228-239), FP64, nonzero guess. */
int igapgpu_ksp_solve(igapgpu_t ctx, const double *b, double *x, const igapgpu_solver_opts *opts,
                      int *its, double *rnorm);
/* IGAPSolvSolve (src/interface.c:302-328) on the device: Newton with the
 * chosen line search, each step assembling the tangent and solving with
 * GMRES; U is the initial iterate on entry and the solution on exit. */
int igapgpu_solve(igapgpu_t ctx, double *U, const igapgpu_solver_opts *opts,
                  igapgpu_solve_stats *stats);
void igapgpu_default_solver_opts(igapgpu_solver_opts *opts);

/* Replace the constant traction table (index 6*face + 3*order + d) and
 * recompute the Neumann load on the device; bc_type is unchanged.  Used by
 * time-dependent loading (the reference's neumann callback may depend on
 * par_neumann, include/bcimpl.h:6). */
int igapgpu_set_neumann(igapgpu_t ctx, const double *table);

int igapgpu_set_precision(igapgpu_t ctx, int mode);
/* Run on the caller's CUDA stream (cudaStream_t passed as void*); NULL
 * restores the context's own (non-blocking) stream, so the legacy default
 * stream is selected with cudaStreamLegacy. */
int igapgpu_set_stream(igapgpu_t ctx, void *stream);
int igapgpu_synchronize(igapgpu_t ctx);
const char *igapgpu_last_error(void);

/* Kernel launches issued by this library since load (for accounting). */
int64_t igapgpu_launch_count(void);

/* Timing of the element-assembly kernels with CUDA events recorded on the
 * launching stream around each colour batch.  enable=1 resets and starts,
 * enable=0 stops; igapgpu_profile_read synchronises and returns the summed
 * kernel time (ms), the number of element-kernel launches and the number of
 * elements they processed since the last reset. */
int igapgpu_profile(igapgpu_t ctx, int enable);
int igapgpu_profile_read(igapgpu_t ctx, double *elem_ms, int64_t *launches, int64_t *elements);
/* The same for one kernel kind: 0 = the residual / FP64 element kernel
 * (residual and/or FP64 tangent), 1 = the tensor-core tangent kernel, 2 = the
 * nonlinear laws' all-points law kernel (-1: all kinds). */
int igapgpu_profile_read_kind(igapgpu_t ctx, int kind, double *elem_ms, int64_t *launches,
                              int64_t *elements);

/* Tensor-core self-test: D (128 x 32) = A (128 x 16) . B (32 x 16)^T of small
 * integers through tcgen05.mma kind::tf32 with the operand layout of the
 * split-precision tangent (variant 0) or with LBO/SBO swapped (variant 1).
 * out: 4096 floats on the host, row-major. */
int igapgpu_tc_selftest(int variant, float *out);

/* Measured FP64 FMA throughput of this GPU (TFLOP/s) from a register-only
 * kernel; used as the denominator of FP64-bound roofline fractions. */
int igapgpu_measure_fp64_peak(double *tflops);
/* The same for FP32 FMA (TFLOP/s, an FMA counted as 2): the denominator of the
 * double-FP32 residual kernel's roofline. */
int igapgpu_measure_fp32_peak(double *tflops);
/* Failure-detection self-test (no counterpart in the reference): a kernel
 * waits, with the bounded acquire-poll loop of the batched kernels, for a
 * zeroed counter to reach `target` (0: at once; 1: never, so the wait expires
 * after `limit` <= 2^24 polls).  *status receives the device error word: 0, or
 * 3 when the wait expired.  The kernel always returns; the context stays
 * usable. */
int igapgpu_wait_selftest(int target, unsigned int limit, int *status);


/* ---------------------------------------------------------------------
 * Batched instances (no counterpart in the reference): many independent
 * beams assembled by one persistent launch per kernel.  The returned context
 * is the block-diagonal union of the instances -- DOFs and CSR rows of
 * instance i follow those of instance i-1 -- and every igapgpu_* call above
 * applies to it (residual, tangent, solve, matmult, graphs, pattern, history,
 * Dirichlet).  All instances share one law; parameters, meshes and boundary
 * conditions are per instance.  igapgpu_set_neumann sets the same traction
 * table on every instance.  Elements of all instances form one colour-major
 * work queue; an element waits (bounded) until its instance's elements of the
 * earlier colours are finished, so CSR slots receive contributions in the
 * same order as the single-instance colour launches (bit-identical results). */
typedef struct {
  int grab_fp64;        /* elements per queue fetch, FP64 element kernel (>= 1) */
  int ctas_per_sm_fp64; /* resident CTAs per SM (capped by the kernel's occupancy) */
  int grab_tc;          /* elements per queue fetch, tensor-core tangent kernel */
  int order;            /* 0: instances in input order within a colour; 1: largest first */
} igapgpu_batch_schedule;

int igapgpu_batch_init(igapgpu_t *ctx, int ninst, const igapgpu_mesh_desc *meshes,
                       const igapgpu_phys_desc *phys, const igapgpu_bc_desc *bcs, int nquad);
/* dof_off / elem_off: [ninst+1] prefix offsets (may be NULL). */
int igapgpu_batch_info(igapgpu_t ctx, int *ninst, int64_t *dof_off, int64_t *elem_off);
/* FP64 2-norm of each instance's segment of x (host or device), norms[ninst] host. */
int igapgpu_batch_norms(igapgpu_t ctx, const double *x, double *norms);
int igapgpu_batch_set_schedule(igapgpu_t ctx, const igapgpu_batch_schedule *s);
int igapgpu_batch_get_schedule(igapgpu_t ctx, igapgpu_batch_schedule *s);
/* Times candidate schedules of both kernels on the current state (each
 * candidate runs `reps` times on a prefix of `frac` of the work queue), keeps
 * the fastest and returns it; ms_fp64 / ms_tc: best time of each kernel on the
 * prefix (may be NULL).  Leaves the context's residual and matrix invalid. */
int igapgpu_batch_autotune(igapgpu_t ctx, int reps, double frac, igapgpu_batch_schedule *best,
                           double *ms_fp64, double *ms_tc);

/* ---- learned Newton predictor (no counterpart in the reference) --------
 * 3-D convolutional network on the control-point lattice (nx, ny, nz):
 * channels 9 -> 32 -> 32 -> 32 -> 3, 3x3x3 kernels, zero padding, ReLU after
 * the first three layers.  storage 1 = bfloat16 weights and activations,
 * 0 = float (gradient checks); FP32 accumulation; FP32 master weights and Adam.
 * Parameter layout: weights layer by layer [Co][27][Ci] (tap t = 9(dx+1) +
 * 3(dy+1) + dz+1), then biases.  Tensors are device FP32, [B][nx][ny][nz][C]. */
typedef struct igapgpu_net igapgpu_net;
int igapgpu_net_create(igapgpu_net **net, int nx, int ny, int nz, int batch_max, int storage);
int igapgpu_net_destroy(igapgpu_net *net);
int64_t igapgpu_net_num_params(igapgpu_net *net);
int igapgpu_net_set_stream(igapgpu_net *net, void *stream);
int igapgpu_net_set_params(igapgpu_net *net, const float *params);
int igapgpu_net_get_params(igapgpu_net *net, float *params);
int igapgpu_net_get_grads(igapgpu_net *net, float *grads);
int igapgpu_net_forward(igapgpu_net *net, const float *in, float *out, int batch);
/* forward + mean-square loss against target + backward (gradients zeroed
 * first); lr > 0 then applies one Adam step.  loss: host float. */
int igapgpu_net_train_step(igapgpu_net *net, const float *in, const float *target, int batch, float lr,
                           float *loss);

#ifdef __cplusplus
}
#endif
#endif
