// CUDA-graph execution of the Newton-Krylov step.
//
// * GMRES(m) with modified Gram-Schmidt and right Jacobi preconditioning,
//   device-resident: the Hessenberg column, the Givens rotations and the
//   convergence test run in single-thread kernels, so one restart cycle
//   (residual, m Arnoldi steps, least-squares update of x) is one graph with
//   no host synchronisation inside.  Once the residual estimate reaches the
//   tolerance a device flag predicates the remaining steps of the cycle off.
//   The host reads one small state record per cycle.
// * The assembly (colour launches, Dirichlet rows and columns) is captured
//   once per (residual, tangent, precision) and replayed.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>
#include <vector>

#include "common.cuh"
#include "spmv.cuh"
#include "asm_pc.cuh"

namespace igap {

struct GmState {
  int done;      // converged (or broke down) in this cycle
  int its;       // Arnoldi steps completed in this cycle
  double beta;   // |r| at the start of the cycle
  double rnorm;  // residual estimate
  double rnorm0; // |r| of the first cycle (negative before it)
  double tol;
  double rtol, abstol;
};

namespace {
constexpr int RB = 304, RT = 512;

__global__ void gm_reset(GmState *st) { st->done = 0; st->its = 0; }

template <bool DF>
__global__ void __launch_bounds__(256) gm_spmv(const int64_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
                                               const double *__restrict__ vals, const double *__restrict__ x,
                                               double *__restrict__ y, int64_t n, const GmState *st, int nb0,
                                               int nb1, int nb2)
{
  if (st && st->done) return;
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / SPMV_G;
  const int sub = threadIdx.x % SPMV_G;
  const double s = spmv_row<DF>(rowptr, cols, vals, x, row, row < n, sub, nb0, nb1, nb2);
  if (sub == 0 && row < n) y[row] = s;
}

__global__ void __launch_bounds__(RT) gm_dot_partial(const double *__restrict__ a, const double *__restrict__ b,
                                                     int64_t n, double *partial, const GmState *st)
{
  if (st && st->done) return;
  __shared__ double sh[RT / 32];
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s = fma(a[i], b[i], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < RT / 32 ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
  }
}

__global__ void gm_dot_final(const double *partial, int np, double *out, int sqrt_flag, const GmState *st)
{
  if (st && st->done) return;
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += partial[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (int)(blockDim.x / 32) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[0] = sqrt_flag ? sqrt(s) : s;
  }
}

__global__ void gm_sub_from(double *r, const double *b, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    r[i] = b[i] - r[i];
}
__global__ void gm_axpy_neg(double *y, const double *x, const double *coef, int64_t n, const GmState *st)
{
  if (st->done) return;
  const double a = coef[0];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = fma(-a, x[i], y[i]);
}
__global__ void gm_scale_div(double *y, const double *x, const double *den, int64_t n, const GmState *st)
{
  if (st->done) return;
  const double inv = 1.0 / den[0];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = x[i] * inv;
}
__global__ void gm_precond(double *z, const double *v, const double *diag, int pc, int64_t n, CellGeom cg,
                           const GmState *st)
{
  if (st->done) return;
  if (pc == 2) {  // point-block Jacobi: diag holds the inverted 3 x 3 blocks
    bdiag_apply(z, v, diag, n / 3);
    return;
  }
  if (pc == 3) {  // cell-block Jacobi: diag holds the inverted cell blocks
    cblock_apply(z, v, diag, cg, cell_count(cg));
    return;
  }
  if (pc == 4) {  // restricted additive Schwarz: diag holds the subdomain rows (FP32)
    asm_apply(z, v, reinterpret_cast<const float *>(diag), cg, cell_count(cg));
    return;
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double d = pc ? diag[i] : 1.0;
    z[i] = v[i] / (d != 0.0 ? d : 1.0);
  }
}
// start of a cycle: beta = |r| is in *beta_in
__global__ void gm_cycle_init(GmState *st, const double *beta_in, double *g, int m)
{
  const double beta = beta_in[0];
  if (st->rnorm0 < 0.0) {
    st->rnorm0 = beta;
    st->tol = fmax(st->rtol * beta, st->abstol);
  }
  st->beta = beta;
  st->rnorm = beta;
  st->its = 0;
  st->done = (beta <= st->tol || !isfinite(beta)) ? 1 : 0;
  for (int i = 0; i <= m; i++) g[i] = 0.0;
  g[0] = beta;
}
// Classical Gram-Schmidt pass over basis vectors 0..cnt-1 (blockIdx.y):
// per row block the partial dot products with w, then per vector a fixed-order
// sum (deterministic), then w -= V h.
constexpr int MD_BLOCKS = 64;
__global__ void __launch_bounds__(256) gm_mdot_partial(const double *__restrict__ V, const double *__restrict__ w,
                                                       int64_t n, double *partial, const GmState *st)
{
  if (st->done) return;
  __shared__ double sh[8];
  const double *v = V + (size_t)blockIdx.y * n;
  double s = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    s = fma(v[r], w[r], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < 8 ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = s;
  }
}
// one warp per vector: h[i] = sum of its MD_BLOCKS partials
__global__ void gm_mdot_final(const double *partial, int cnt, double *h, const GmState *st)
{
  if (st->done) return;
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (i >= cnt) return;
  double s = 0.0;
  for (int k = lane; k < MD_BLOCKS; k += 32) s += partial[i * MD_BLOCKS + k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) h[i] = s;
}
__global__ void __launch_bounds__(256) gm_vupdate(double *__restrict__ w, const double *__restrict__ V,
                                                  const double *__restrict__ h, int cnt, int64_t n,
                                                  const GmState *st)
{
  if (st->done) return;
  __shared__ double hs[1024];
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) hs[i] = h[i];
  __syncthreads();
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double s = w[r];
    for (int i = 0; i < cnt; i++) s = fma(-hs[i], V[(size_t)i * n + r], s);
    w[r] = s;
  }
}
// Givens update of Hessenberg column j (column-major, leading dim m+1); with
// corr (the second Gram-Schmidt pass) h[0..j] += corr[0..j] first.
__global__ void gm_givens(double *H, double *cs, double *sn, double *g, int j, int m, GmState *st,
                          const double *corr = nullptr)
{
  if (st->done) return;
  double *h = H + (size_t)j * (m + 1);
  if (corr)
    for (int i = 0; i <= j; i++) h[i] += corr[i];
  for (int i = 0; i < j; i++) {
    const double t = cs[i] * h[i] + sn[i] * h[i + 1];
    h[i + 1] = -sn[i] * h[i] + cs[i] * h[i + 1];
    h[i] = t;
  }
  double den = hypot(h[j], h[j + 1]);
  const bool breakdown = !(den > 0.0) || !isfinite(den);
  if (breakdown) den = 1e-300;
  cs[j] = h[j] / den;
  sn[j] = h[j + 1] / den;
  h[j] = den;
  h[j + 1] = 0.0;
  g[j + 1] = -sn[j] * g[j];
  g[j] = cs[j] * g[j];
  st->rnorm = fabs(g[j + 1]);
  st->its = j + 1;
  if (st->rnorm <= st->tol || breakdown || !isfinite(st->rnorm)) st->done = 1;
}
// y = H(1:its,1:its)^{-1} g(1:its)
__global__ void gm_backsolve(const double *H, const double *g, double *y, int m, const GmState *st)
{
  const int k = st->its;
  for (int i = k - 1; i >= 0; i--) {
    double s = g[i];
    for (int l = i + 1; l < k; l++) s -= H[(size_t)l * (m + 1) + i] * y[l];
    y[i] = s / H[(size_t)i * (m + 1) + i];
  }
}
// x += sum_{i < its} y_i Z_i
__global__ void gm_update_x(double *x, const double *Z, const double *y, int64_t n, const GmState *st)
{
  const int k = st->its;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
    double s = x[idx];
    for (int i = 0; i < k; i++) s = fma(y[i], Z[(size_t)i * n + idx], s);
    x[idx] = s;
  }
}
__global__ void get_diag_kernel_g(const int64_t *rowptr, const int32_t *cols, const double *vals,
                                  double *diag, int64_t n)
{
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  int64_t lo = rowptr[r], hi = rowptr[r + 1];
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (cols[mid] < r) lo = mid + 1; else hi = mid;
  }
  diag[r] = (lo < rowptr[r + 1] && cols[lo] == r) ? vals[lo] : 0.0;
}
}  // namespace

// Graph workspace held by the context.
struct GraphWork {
  int m = 0, pc = -1, orth = -1;
  bool df = false;  // double-FP32 multiply
  cudaGraphExec_t exec = nullptr;
  int64_t nodes = 0;
  double *b = nullptr, *x = nullptr, *r = nullptr, *w = nullptr, *V = nullptr, *Z = nullptr;
  double *H = nullptr, *cs = nullptr, *sn = nullptr, *g = nullptr, *y = nullptr, *scal = nullptr;
  double *partial = nullptr, *diag = nullptr;
  GmState *st = nullptr;
  GmState *h_st = nullptr;
};

static void free_graph(GraphWork *gw)
{
  if (!gw) return;
  if (gw->exec) cudaGraphExecDestroy(gw->exec);
  void *bufs[] = {gw->b, gw->x, gw->r, gw->w, gw->V, gw->Z, gw->H, gw->cs, gw->sn, gw->g, gw->y,
                  gw->scal, gw->partial, gw->diag, gw->st};
  for (void *p : bufs)
    if (p) cudaFree(p);
  if (gw->h_st) cudaFreeHost(gw->h_st);
  delete gw;
}

void graph_release(Context *c)
{
  free_graph(c->gmres_graph);
  c->gmres_graph = nullptr;
  for (int i = 0; i < 12; i++) {
    if (c->asm_graph[i]) cudaGraphExecDestroy(c->asm_graph[i]);
    c->asm_graph[i] = nullptr;
  }
}


// Capture cannot begin on the legacy default stream; there the graph is
// recorded on the context's own stream (recording runs nothing) and later
// launched on the caller's stream.
static cudaStream_t capture_stream(const Context *c)
{
  return (c->stream == nullptr || c->stream == cudaStreamLegacy) ? c->own_stream : c->stream;
}

static int build_gmres_graph(Context *c, int m, int pc, int orth)
{
  free_graph(c->gmres_graph);
  c->gmres_graph = nullptr;
  GraphWork *gw = new GraphWork();
  const int64_t n = c->ndof;
  auto alloc = [&](double **p, size_t cnt) { return cudaMalloc((void **)p, sizeof(double) * cnt); };
  if (alloc(&gw->b, n) || alloc(&gw->x, n) || alloc(&gw->r, n) || alloc(&gw->w, n) ||
      alloc(&gw->V, (size_t)(m + 1) * n) || alloc(&gw->Z, (size_t)m * n) ||
      alloc(&gw->H, (size_t)(m + 1) * m) || alloc(&gw->cs, m) || alloc(&gw->sn, m) ||
      alloc(&gw->g, m + 1) || alloc(&gw->y, m) || alloc(&gw->scal, m + 2) ||
      alloc(&gw->partial, (size_t)(RB > MD_BLOCKS * (m + 1) ? RB : MD_BLOCKS * (m + 1))) ||
      alloc(&gw->diag, pc == 3   ? (size_t)cell_count(cell_geom(c)) * CBS * CBS
                       : pc == 4 ? (size_t)cell_count(cell_geom(c)) * AS_NC * AS_N / 2
                                 : (size_t)3 * n) ||
      cudaMalloc(&gw->st, sizeof(GmState)) != cudaSuccess ||
      cudaMallocHost(&gw->h_st, sizeof(GmState)) != cudaSuccess) {
    cudaGetLastError();
    free_graph(gw);
    set_error("GMRES graph workspace (restart %d) does not fit", m);
    return IGAPGPU_ERR_NOMEM;
  }
  gw->m = m;
  gw->pc = pc;
  gw->orth = orth;
  gw->df = spmv_df(c);
  auto gspmv = gw->df ? gm_spmv<true> : gm_spmv<false>;
  const unsigned vb = (unsigned)((n + 255) / 256 < 152 * 8 ? (n + 255) / 256 : 152 * 8);
  const unsigned sb = (unsigned)((n * SPMV_G + 255) / 256);
  cudaStream_t s = capture_stream(c);
  int64_t nodes = 0;
  IGAP_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  gm_reset<<<1, 1, 0, s>>>(gw->st);
  const int nb0 = (c->batch || c->porder != P) ? 0 : c->nbasis[0];
  gspmv<<<sb, 256, 0, s>>>(c->d_rowptr, c->d_cols, c->d_vals, gw->x, gw->r, n, nullptr, nb0, c->nbasis[1],
                           c->nbasis[2]);
  gm_sub_from<<<vb, 256, 0, s>>>(gw->r, gw->b, n);
  gm_dot_partial<<<RB, RT, 0, s>>>(gw->r, gw->r, n, gw->partial, nullptr);
  gm_dot_final<<<1, 1024, 0, s>>>(gw->partial, RB, gw->scal, 1, nullptr);
  gm_cycle_init<<<1, 1, 0, s>>>(gw->st, gw->scal, gw->g, m);
  gm_scale_div<<<vb, 256, 0, s>>>(gw->V, gw->r, gw->scal, n, gw->st);
  nodes += 7;
  for (int j = 0; j < m; j++) {
    double *vj = gw->V + (size_t)j * n, *zj = gw->Z + (size_t)j * n, *vn = gw->V + (size_t)(j + 1) * n;
    double *hcol = gw->H + (size_t)j * (m + 1);
    gm_precond<<<vb, 256, 0, s>>>(zj, vj, gw->diag, pc, n, cell_geom(c), gw->st);
    gspmv<<<sb, 256, 0, s>>>(c->d_rowptr, c->d_cols, c->d_vals, zj, gw->w, n, gw->st, nb0, c->nbasis[1],
                             c->nbasis[2]);
    nodes += 2;
    if (orth == 1) {  // CGS2: two block passes h = V^T w, w -= V h
      const dim3 gp(MD_BLOCKS, (unsigned)(j + 1));
      const unsigned fb = (unsigned)((j + 1 + 7) / 8);
      gm_mdot_partial<<<gp, 256, 0, s>>>(gw->V, gw->w, n, gw->partial, gw->st);
      gm_mdot_final<<<fb, 256, 0, s>>>(gw->partial, j + 1, hcol, gw->st);
      gm_vupdate<<<vb, 256, 0, s>>>(gw->w, gw->V, hcol, j + 1, n, gw->st);
      gm_mdot_partial<<<gp, 256, 0, s>>>(gw->V, gw->w, n, gw->partial, gw->st);
      gm_mdot_final<<<fb, 256, 0, s>>>(gw->partial, j + 1, gw->y, gw->st);
      gm_vupdate<<<vb, 256, 0, s>>>(gw->w, gw->V, gw->y, j + 1, n, gw->st);
      nodes += 6;
    } else {
      for (int i = 0; i <= j; i++) {
        gm_dot_partial<<<RB, RT, 0, s>>>(gw->w, gw->V + (size_t)i * n, n, gw->partial, gw->st);
        gm_dot_final<<<1, 1024, 0, s>>>(gw->partial, RB, hcol + i, 0, gw->st);
        gm_axpy_neg<<<vb, 256, 0, s>>>(gw->w, gw->V + (size_t)i * n, hcol + i, n, gw->st);
        nodes += 3;
      }
    }
    gm_dot_partial<<<RB, RT, 0, s>>>(gw->w, gw->w, n, gw->partial, gw->st);
    gm_dot_final<<<1, 1024, 0, s>>>(gw->partial, RB, hcol + j + 1, 1, gw->st);
    gm_scale_div<<<vb, 256, 0, s>>>(vn, gw->w, hcol + j + 1, n, gw->st);
    gm_givens<<<1, 1, 0, s>>>(gw->H, gw->cs, gw->sn, gw->g, j, m, gw->st, orth == 1 ? gw->y : nullptr);
    nodes += 4;
  }
  gm_backsolve<<<1, 1, 0, s>>>(gw->H, gw->g, gw->y, m, gw->st);
  gm_update_x<<<vb, 256, 0, s>>>(gw->x, gw->Z, gw->y, n, gw->st);
  nodes += 2;
  cudaGraph_t graph;
  cudaError_t e = cudaStreamEndCapture(s, &graph);
  if (e != cudaSuccess) {
    free_graph(gw);
    set_error("GMRES graph capture failed: %s", cudaGetErrorString(e));
    return IGAPGPU_ERR_CUDA;
  }
  e = cudaGraphInstantiate(&gw->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    free_graph(gw);
    set_error("GMRES graph instantiation failed: %s", cudaGetErrorString(e));
    return IGAPGPU_ERR_CUDA;
  }
  gw->nodes = nodes;
  c->gmres_graph = gw;
  return IGAPGPU_OK;
}

// GMRES on the context matrix through the cycle graph; b, x device vectors.
int ksp_gmres_graph(Context *c, const double *b, double *x, const igapgpu_solver_opts *o, int *its_out,
                    double *rnorm_out)
{
  const int m = o->ksp_restart > 0 ? o->ksp_restart : 30;
  const int pc = (o->pc >= 1 && o->pc <= 4) ? o->pc : 0;
  const int orth = o->orth == 1 ? 1 : 0;
  if (m > 1000) {
    set_error("graph GMRES: restart %d above 1000", m);
    return IGAPGPU_ERR_ARG;
  }
  if ((pc == 3 || pc == 4) && c->porder != P) {
    set_error("block preconditioners (pc = 3, 4) use the quadratic stencil; degree 3 takes pc 0, 1 or 2");
    return IGAPGPU_ERR_ARG;
  }
  if ((pc == 3 || pc == 4) && c->batch) {
    set_error("block preconditioners (pc = 3, 4) need a single lattice; a batch takes pc 0, 1 or 2");
    return IGAPGPU_ERR_ARG;
  }
  if (!c->gmres_graph || c->gmres_graph->m != m || c->gmres_graph->pc != pc || c->gmres_graph->orth != orth ||
      c->gmres_graph->df != spmv_df(c)) {
    int r = build_gmres_graph(c, m, pc, orth);
    if (r) return r;
  }
  GraphWork *gw = c->gmres_graph;
  const int64_t n = c->ndof;
  cudaStream_t s = c->stream;
  IGAP_CUDA(cudaMemcpyAsync(gw->b, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  IGAP_CUDA(cudaMemcpyAsync(gw->x, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  if (pc == 1) {
    get_diag_kernel_g<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(c->d_rowptr, c->d_cols, c->d_vals, gw->diag, n);
    count_launch();
    IGAP_CHECK_LAUNCH();
  } else if (pc == 2) {
    bdiag_invert_kernel<<<(unsigned)((n / 3 + 255) / 256), 256, 0, s>>>(c->d_rowptr, c->d_cols, c->d_vals, gw->diag,
                                                                      n / 3);
    count_launch();
    IGAP_CHECK_LAUNCH();
  } else if (pc == 3) {
    const CellGeom cg = cell_geom(c);
    const int64_t ncell = cell_count(cg);
    cblock_invert_kernel<<<(unsigned)((ncell + CB_WARPS - 1) / CB_WARPS), 32 * CB_WARPS, 0, s>>>(c->d_rowptr, c->d_vals,
                                                                                              gw->diag, cg, ncell);
    count_launch();
    IGAP_CHECK_LAUNCH();
  } else if (pc == 4) {
    int r = asm_setup(c, reinterpret_cast<float *>(gw->diag));
    if (r) return r;
  }
  GmState h0;
  memset(&h0, 0, sizeof h0);
  h0.rnorm0 = -1.0;
  h0.rtol = o->ksp_rtol;
  h0.abstol = o->ksp_abstol;
  IGAP_CUDA(cudaMemcpyAsync(gw->st, &h0, sizeof h0, cudaMemcpyHostToDevice, s));
  int its = 0;
  double rnorm = 0.0;
  for (;;) {
    IGAP_CUDA(cudaGraphLaunch(gw->exec, s));
    count_launch((int)gw->nodes);
    IGAP_CUDA(cudaMemcpyAsync(gw->h_st, gw->st, sizeof(GmState), cudaMemcpyDeviceToHost, s));
    IGAP_CUDA(cudaStreamSynchronize(s));
    const GmState st = *gw->h_st;
    its += st.its;
    rnorm = st.rnorm;
    if (!isfinite(rnorm)) {
      set_error("GMRES: non-finite residual");
      return IGAPGPU_ERR_NUMERIC;
    }
    if (st.rnorm0 > 0 && st.beta > o->ksp_dtol * st.rnorm0) {
      set_error("GMRES diverged (dtol)");
      return IGAPGPU_ERR_NUMERIC;
    }
    if (rnorm <= st.tol || its >= o->ksp_max_it) break;
    if (st.its == 0 && st.done) break;  // already converged at the cycle start
  }
  IGAP_CUDA(cudaMemcpyAsync(x, gw->x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  if (its_out) *its_out = its;
  if (rnorm_out) *rnorm_out = rnorm;
  return IGAPGPU_OK;
}

// Residual and/or tangent assembly into the context buffers (d_RR, d_vals),
// captured once per (res, tan, precision) and replayed.
int assembly_graph(Context *c, bool do_res, bool do_tan)
{
  const int key = (do_res ? 1 : 0) + (do_tan ? 2 : 0) + 4 * c->prec;
  if (!c->asm_graph[key]) {
    // first use: run it directly (one-time set-up such as kernel attributes
    // and constant tables happens outside the capture), then capture it
    int r0 = launch_assembly(c, do_res, do_tan, c->d_RR, c->d_vals);
    if (r0) return r0;
    if (do_tan) c->matrix_valid = true;
    const bool prof = c->prof;
    c->prof = false;
    c->capturing = true;
    cudaStream_t user = c->stream;
    c->stream = capture_stream(c);
    IGAP_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const int64_t l0 = g_launches.load();
    int r = launch_assembly(c, do_res, do_tan, c->d_RR, c->d_vals);
    cudaGraph_t graph;
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    c->stream = user;
    c->capturing = false;
    c->prof = prof;
    if (r) return r;
    if (e != cudaSuccess) {
      set_error("assembly graph capture failed: %s", cudaGetErrorString(e));
      return IGAPGPU_ERR_CUDA;
    }
    c->asm_graph_nodes[key] = g_launches.load() - l0;
    g_launches.fetch_sub(c->asm_graph_nodes[key]);  // counted at replay
    e = cudaGraphInstantiate(&c->asm_graph[key], graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      c->asm_graph[key] = nullptr;
      set_error("assembly graph instantiation failed: %s", cudaGetErrorString(e));
      return IGAPGPU_ERR_CUDA;
    }
    return IGAPGPU_OK;
  }
  // the error word is cleared inside the graph; it is read after the replay
  // when a kernel of the graph has bounded waits
  const bool waits = c->batch || (c->prec != IGAPGPU_PREC_FP64 && do_tan);
  if (waits) IGAP_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
  IGAP_CUDA(cudaGraphLaunch(c->asm_graph[key], c->stream));
  count_launch((int)c->asm_graph_nodes[key]);
  if (do_tan) c->matrix_valid = true;
  if (waits) {
    int herr = 0;
    IGAP_CUDA(cudaMemcpyAsync(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    IGAP_CUDA(cudaStreamSynchronize(c->stream));
    if (herr) {
      set_error("tensor-core tangent: a bounded mbarrier wait expired (code %d)", herr);
      return IGAPGPU_ERR_TIMEOUT;
    }
  }
  return IGAPGPU_OK;
}

}  // namespace igap
