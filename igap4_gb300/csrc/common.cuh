// Internal definitions shared by the translation units of libigapgpu.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <atomic>
#include <string>
#include <utility>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "igapgpu.h"

namespace igap {

// NVTX range over an entry point (visible in Nsight timelines; no cost
// without a tool attached).
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

constexpr int P = 2;                    // B-spline degree handled on the device
constexpr int P1 = P + 1;               // basis functions per direction per element
constexpr int NB = P1 * P1 * P1;        // 27 basis functions per element
constexpr int NDD = 10;                 // value, 3 first, 6 second derivatives
constexpr int NE = 3 * NB;              // 81 element DOFs
constexpr int TAB = 3 * P1 + 2;         // 1-D table entry: N, dN, ddN of 3 functions, xi, h
constexpr int MAXQ = 6;                 // max Gauss points per direction
// sizes that follow the B-spline degree (the kernels above P are the quadratic
// ones; the cubic path of cubic.cu instantiates these for degree 3)
template <int PD>
struct Deg {
  static constexpr int P1 = PD + 1, NB = P1 * P1 * P1, NE = 3 * NB, TAB = 3 * P1 + 2;
};
// basis-table entry length of a degree
__host__ __device__ constexpr int tab_len(int pd) { return 3 * (pd + 1) + 2; }

// Reference-ABI constants (include/physimpl.h, src/assmcore_iga.c)
constexpr int NFACE = 6;

void set_error(const char *fmt, ...);
extern std::atomic<int64_t> g_launches;
inline void count_launch(int n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

#define IGAP_CUDA(call)                                                              \
  do {                                                                               \
    cudaError_t _e = (call);                                                         \
    if (_e != cudaSuccess) {                                                         \
      ::igap::set_error("CUDA error %s at %s:%d: %s", cudaGetErrorName(_e), __FILE__, \
                        __LINE__, cudaGetErrorString(_e));                           \
      return IGAPGPU_ERR_CUDA;                                                       \
    }                                                                                \
  } while (0)

#define IGAP_CHECK_LAUNCH() IGAP_CUDA(cudaGetLastError())

// Device-resident problem description used by the element kernels.
struct DevMesh {
  int nelem[3];
  int nbasis[3];           // nelem + P
  int nquad;
  int npts;                // nquad^3
  const double *tab[3];    // [nelem_d][nquad][TAB] 1-D basis tables (with the knot-span MTOL)
  const double *wq;        // [nquad] Gauss weights on [0,1]
  const double *w;         // [ncp]
  const double *X;         // [3*ncp]
  const int64_t *rowptr;   // [ndof+1] (global CSR positions; a batch instance's rows)
  int64_t ndof;            // stride between history levels of the state
  int64_t dof_off;         // first DOF of this mesh in the state / residual vectors
  const double *geo;       // geometry cache [nelem][npts][272] or null
  const float *geof;       // FP32 copy of the geometry cache (split tangent) or null
  const float *gop;        // Gram operands of the linear law in MMA layout (split tangent) or null
};

struct DevLaw {
  int law;
  int nhist;               // torder + 1
  double par[9];
  const double *Dconst;    // 900 constant tangent of a linear law (or null)
  // sparse form of Dconst: rows (CSR) for the residual, and per (d,k,e)
  // segments (entries l with D[(d,k),(e,l)] != 0) for the split tangent
  const int *dptr;         // [31]
  const int *dcol;         // [nnz]
  const double *dval;      // [nnz]
  const int *sptr;         // [91]
  const int *sl;           // [nnz]
  const float *sval;       // [nnz]
  int dnnz;
  // weighted law outputs per point, [nelem][30][npts] and [nelem][900][npts]
  // (point-minor), when computed for all points before the colour launches
  // (else null)
  const double *preR;
  const double *preD;
  // the tangent's outputs in FP32 (split mode: the law in FP32 arithmetic,
  // stored in the preD buffer), else null
  const float *preDf;
};

struct GraphWork;
struct Batch;

// One work item of a batched launch: element (ex, ey, ez) of instance inst,
// whose colour (ex mod 3, ey mod 3, ez mod 3) is col.
struct BatchItem {
  int inst;
  int col;
  int ex;
  int eyz;  // ey << 16 | ez
};

// Arguments of the persistent batched kernels.
struct BatchArgs {
  const DevMesh *meshes;   // [ninst]
  const DevLaw *laws;      // [ninst]
  const BatchItem *items;  // colour-major work queue
  int64_t nitems;
  int *head;               // queue head (reset before each launch)
  int *done;               // [ninst] finished items per instance
  const int *need;         // [ninst*27] items of the instance in colours before each colour
  int grab;                // items taken per fetch
  int *err;                // device error word
};

struct Context {
  // problem
  int law, torder, nquad, prec;
  int porder = P;                  // B-spline degree: 2, or 3 (cubic.cu)
  double par[9];
  int nelem[3], nbasis[3];
  int64_t ndof, nnz, nelem_total, ncp;
  igapgpu_bc_desc bc;
  std::vector<double> h_knots[3];  // host copies of the knot vectors (boundary data)
  double nfac[6][2];               // Neumann normal-derivative factors of the two boundary layers
  // device buffers
  double *d_tab[3] = {nullptr, nullptr, nullptr};
  double *d_tabn[3] = {nullptr, nullptr, nullptr}; // plain Cox-de Boor (face integrals)
  double *d_knots[3] = {nullptr, nullptr, nullptr};
  double *d_wq = nullptr, *d_xq = nullptr;
  double *d_w = nullptr, *d_X = nullptr;
  double *d_Uhist = nullptr;   // [(torder+1)][ndof]
  double *d_RR = nullptr;      // [ndof]
  double *d_vals = nullptr;    // [nnz] the context's matrix
  int64_t *d_rowptr = nullptr; // [ndof+1]
  int32_t *d_cols = nullptr;   // [nnz]
  double *d_Dconst = nullptr;  // [900]
  double *d_Fneu = nullptr;    // [ndof] Neumann load (state independent)
  int *d_err = nullptr;        // device error word (bounded waits that expired)
  int *d_bct = nullptr;        // bc_type table on the device [36]
  double *d_neu = nullptr;     // traction table on the device [36]
  double *d_geo = nullptr;     // geometry cache (physical basis + weight per point)
  float *d_geof = nullptr;     // FP32 copy for the split-precision tangent
  float *d_gop = nullptr;      // linear law: sqrt(w)-weighted Gram operands in MMA layout (split tangent)
  int gop_state = -1;          // -1 not decided, 0 off, 1 on
  void *d_oz = nullptr;        // linear law: BF16 slices of the Gram operands (FP64-quality tensor-core tangent)
  void *d_ozexp = nullptr;     // their per-row power-of-two exponents (int8, 88 per element)
  int oz_state = -1;           // -1 not decided, 0 off, 1 on
  float2 *d_rpc = nullptr;     // linear law: derivative and weight pairs per point (double-FP32 residual)
  float2 *d_rel = nullptr;     // its per-element residual pairs [element][81]
  float2 *d_upair = nullptr;   // the state as pairs [ndof]
  int rpc_state = -1;          // -1 not decided, 0 off, 1 linear law, 2 the reference's laws
  double *d_lin = nullptr;     // the reference's laws: law inputs of every point [point][64] (double-FP32 residual)
  bool law_df = false;         // the last law launch took its residual inputs from d_lin
  double *d_preR = nullptr;    // law outputs of every point (nonlinear laws, when it fits)
  double *d_preD = nullptr;
  int pre_state = -1;          // -1 not decided, 0 off, 1 on
  double *d_dens = nullptr;    // per-element density sums + result (igapgpu_density, lazy)
  int *d_dsparse = nullptr;    // sparse constant tangent: dptr | dcol | sptr | sl
  double *d_dval = nullptr;
  float *d_sval = nullptr;
  int dnnz = 0;
  int64_t n_dir = 0;           // Dirichlet rows (unique, last writer wins)
  int64_t *d_dir_rows = nullptr;
  double *d_dir_g = nullptr;
  double *d_stage_a = nullptr, *d_stage_b = nullptr; // host-pointer staging [ndof]
  double *d_stage_v = nullptr;                       // host-pointer staging [nnz] (lazy)
  bool matrix_valid = false;
  // Krylov workspace (lazy)
  int ksp_restart = 0;
  double *d_V = nullptr;       // [(restart+1)][ndof]
  double *d_Z = nullptr;       // [restart][ndof] (right-preconditioned directions)
  double *d_work = nullptr;    // [4][ndof]
  double *d_diag = nullptr;    // [ndof]
  double *d_bdiag = nullptr;   // [3 ndof] inverted 3 x 3 point blocks (point-block Jacobi)
  double *d_cinv = nullptr;    // [cells][24 x 24] inverted cell blocks (cell-block Jacobi, lazy)
  float *d_asmz = nullptr;     // [cells][24 x 192] subdomain inverse rows (restricted additive Schwarz, lazy)
  double *d_red = nullptr;     // device scalars (norms, Hessenberg column) [red_cap]
  double *h_red = nullptr;     // pinned host mirror of d_red [red_cap]
  double *d_partial = nullptr; // per-block partial sums of the reductions
  int red_cap = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  // CUDA graphs (graph.cu)
  GraphWork *gmres_graph = nullptr;
  cudaGraphExec_t asm_graph[12] = {};  // key: residual + 2 tangent + 4 precision mode
  int64_t asm_graph_nodes[12] = {};
  bool capturing = false;
  // batched instances (batch.cu): this context is then their block-diagonal union
  Batch *batch = nullptr;
  bool sub = false;  // an instance of a batch (no matrix or state of its own)
  int geo_mode = -1;  // geometry cache: -1 by free memory, 0 none, 1 FP64, 2 FP64 + FP32
  std::vector<int64_t> h_rowptr;  // host CSR offsets (kept for instances of a batch)
  // element-kernel timing (igapgpu_profile)
  bool prof = false;
  // per kernel kind: 0 = residual / FP64 element kernel, 1 = tensor-core
  // tangent kernel, 2 = the nonlinear laws' all-points law kernel
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_ev[3];
  int64_t prof_launches[3] = {0, 0, 0}, prof_elements[3] = {0, 0, 0};

  DevMesh devmesh() const {
    DevMesh m;
    for (int d = 0; d < 3; d++) {
      m.nelem[d] = nelem[d];
      m.nbasis[d] = nbasis[d];
      m.tab[d] = d_tab[d];
    }
    m.nquad = nquad;
    m.npts = nquad * nquad * nquad;
    m.wq = d_wq;
    m.w = d_w;
    m.X = d_X;
    m.rowptr = d_rowptr;
    m.ndof = ndof;
    m.dof_off = 0;
    m.geo = d_geo;
    m.geof = d_geof;
    m.gop = d_gop;
    return m;
  }
  DevLaw devlaw() const {
    DevLaw l;
    l.law = law;
    l.nhist = torder + 1;
    for (int i = 0; i < 9; i++) l.par[i] = par[i];
    l.Dconst = d_Dconst;
    l.dnnz = dnnz;
    l.dptr = d_dsparse;
    l.dcol = d_dsparse ? d_dsparse + 31 : nullptr;
    l.sptr = d_dsparse ? d_dsparse + 31 + dnnz : nullptr;
    l.sl = d_dsparse ? d_dsparse + 31 + dnnz + 91 : nullptr;
    l.dval = d_dval;
    l.sval = d_sval;
    l.preR = nullptr;
    l.preD = nullptr;
    l.preDf = nullptr;
    return l;
  }
};

// Pointer classification: true if ptr is device (or managed) memory.
bool is_device_ptr(const void *p);

// context.cu
int check_instance_args(const igapgpu_mesh_desc *mesh, const igapgpu_phys_desc *phys,
                        const igapgpu_bc_desc *bc, int nquad);
Context *new_context(const igapgpu_mesh_desc *mesh, const igapgpu_phys_desc *phys,
                     const igapgpu_bc_desc *bc, int nquad);
int context_init(Context *c, const igapgpu_mesh_desc *mesh);
int context_free(Context *c);

// assemble.cu
int launch_assembly(Context *c, bool do_res, bool do_tan, double *RR, double *vals);
// law outputs at every point of a nonlinear law in one launch; sets preR/preD
// of `L` when the buffers exist (else leaves them null)
int launch_law_points(Context *c, bool do_res, bool do_tan, DevLaw &L);
int launch_basis_tables(Context *c);
int launch_lingrad_dconst(Context *c);
int launch_neumann(Context *c, const double nfac[NFACE][2]);
int launch_dirichlet_matrix(Context *c, double *vals);
int launch_dirichlet_residual(Context *c, double *RR);
int launch_impose_dirichlet(Context *c, double *U);
int launch_pattern_cols(Context *c);
int launch_pattern_cols_at(Context *c, const int64_t *rowptr, int32_t *cols, int64_t coff);
int launch_dirichlet_matrix_batch(Context *c, const int *d_inst, const int *d_nbs, const int64_t *d_off,
                                  double *vals);
int launch_geometry_cache(Context *c);
int launch_geometry_cache_f32(Context *c);
// tc_tangent.cu
int launch_tc_tangent(Context *c, double *vals, const DevLaw &L);
// tc_gram.cu (linear isotropic law with the FP32 geometry cache)
int launch_tc_gram(Context *c, double *vals);
// cached: every instance has its Gram operands (d_gop); persistent CTAs per SM of nsm
int launch_tc_gram_batch(Context *c, const BatchArgs &a, int nsm, double *vals, bool cached);
// cubic.cu (degree 3: basis tables, pattern, Neumann load, Dirichlet columns,
// FP64 element kernel)
int launch_basis_tables_p3(Context *c);
int launch_pattern_cols_p3(Context *c);
int launch_neumann_p3(Context *c, const double nfac[NFACE][2]);
int launch_dirichlet_matrix_p3(Context *c, double *vals);
int launch_assembly_p3(Context *c, bool do_res, bool do_tan, double *RR, double *vals);
// tc_ozaki.cu (linear law, BF16 slices, FP64-quality)
int ensure_ozaki_operands(Context *c);
int launch_tc_ozaki(Context *c, double *vals);
// res_df.cu (linear law residual in double-FP32 arithmetic)
int ensure_res_pairs(Context *c);
int launch_res_df(Context *c, double *RR);
// the reference's laws: law inputs by pair interpolation, projection on pairs
int launch_law_in_df(Context *c);
int launch_res_law_df(Context *c, const double *preR, double *RR);
int launch_res_df_batch(Context *c, const DevMesh *meshes, const DevLaw *laws, const int64_t *eoff,
                        const int *einst, const int64_t *doff, int ninst, int64_t nel, float2 *rel, double *RR);
// builds d_gop once (linear law, FP64 geometry cache present, memory allows)
int ensure_gram_operands(Context *c);
// krylov.cu
int spmv(Context *c, const double *vals, const double *x, double *y);
bool spmv_df(const Context *c);
int ksp_gmres(Context *c, const double *b, double *x, const igapgpu_solver_opts *o, int *its,
              double *rnorm);
int dev_norm2(Context *c, const double *x, double *out);
struct CellGeom;
CellGeom cell_geom(const Context *c);
int ensure_cblock(Context *c, int64_t ncell);
// restricted additive Schwarz (pc = 4): set-up of the subdomain rows into Z
// (cells x 24 x 192 floats) from the context matrix
int asm_setup(Context *c, float *Z);
// batch.cu
int launch_batch_assembly(Context *c, bool do_res, bool do_tan, double *RR, double *vals);
void batch_release(Context *c);
int batch_set_neumann(Context *c, const double *table);
int batch_prepare_split(Context *c);
// element kernels over a batch work queue (assemble.cu, tc_tangent.cu)
int launch_element_batch(Context *c, const BatchArgs &a, int law, bool do_res, bool do_tan, int grid,
                         const double *Uhist, double *RR, double *vals);
int launch_tc_batch(Context *c, const BatchArgs &a, int law, int grid, const double *Uhist, double *vals);
int element_batch_occupancy(int law, bool do_res, bool do_tan, int *blocks_per_sm);
// graph.cu
int ksp_gmres_graph(Context *c, const double *b, double *x, const igapgpu_solver_opts *o, int *its,
                    double *rnorm);
int assembly_graph(Context *c, bool do_res, bool do_tan);
void graph_release(Context *c);

}  // namespace igap

// The opaque handle of the C ABI is the context itself.
struct igapgpu_ctx : public igap::Context {};
