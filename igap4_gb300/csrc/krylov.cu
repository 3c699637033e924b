// Newton-Krylov inner loop on the device: CSR SpMV (the MATSHELL multiply),
// Jacobi diagonal, FP64 reductions, right-preconditioned GMRES(m) with
// modified Gram-Schmidt (src/interface.c:228-241 options) and the Newton
// driver of IGAPSolvSolve (src/interface.c:302-328).
//
// All vectors stay in HBM; the only host traffic per GMRES iteration is the
// new Hessenberg column (j+2 doubles) needed for the Givens update.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>
#include <vector>

#include "common.cuh"
#include "spmv.cuh"
#include "asm_pc.cuh"

namespace igap {

constexpr int RED_BLOCKS = 304;  // 2 x 152 SMs
constexpr int RED_THREADS = 512;

// y = A x, SPMV_G lanes per row (spmv_row; structured columns when nb0 > 0;
// DF: double-FP32 products on the FP32 pipe).
template <bool DF>
__global__ void __launch_bounds__(256) spmv_csr_kernel(const int64_t *__restrict__ rowptr,
                                                       const int32_t *__restrict__ cols,
                                                       const double *__restrict__ vals,
                                                       const double *__restrict__ x,
                                                       double *__restrict__ y, int64_t n, int nb0, int nb1,
                                                       int nb2)
{
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / SPMV_G;
  const int sub = threadIdx.x % SPMV_G;
  const double s = spmv_row<DF>(rowptr, cols, vals, x, row, row < n, sub, nb0, nb1, nb2);
  if (sub == 0 && row < n) y[row] = s;
}

__global__ void get_diag_kernel(const int64_t *rowptr, const int32_t *cols, const double *vals,
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

// Deterministic two-pass dot product: partial sums per block, then one block.
__global__ void __launch_bounds__(RED_THREADS) dot_partial_kernel(const double *__restrict__ a,
                                                                  const double *__restrict__ b,
                                                                  int64_t n, double *partial)
{
  __shared__ double sh[RED_THREADS / 32];
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s = fma(a[i], b[i], s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < RED_THREADS / 32 ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
  }
}
// out[0] = sum(partial) ; if sqrt_flag: out[0] = sqrt(out[0])
__global__ void dot_final_kernel(const double *partial, int np, double *out, int sqrt_flag)
{
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += partial[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (int)(blockDim.x / 32) ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[0] = sqrt_flag ? sqrt(s) : s;
  }
}

// y += alpha * x with alpha = sign * (*palpha) (device scalar) or host scalar
__global__ void axpy_dev_kernel(double *y, const double *x, const double *palpha, double sign,
                                int64_t n)
{
  const double a = sign * palpha[0];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = fma(a, x[i], y[i]);
}
__global__ void axpby_kernel(double *y, const double *x, double a, double b, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}
// y = x / (*pden)  (device scalar)
__global__ void scale_div_kernel(double *y, const double *x, const double *pden, int64_t n)
{
  const double inv = 1.0 / pden[0];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = x[i] * inv;
}
// z = v / diag (Jacobi; zero diagonal -> 1, as PCJACOBI)
__global__ void cblock_kernel(double *z, const double *v, const double *inv, CellGeom g, int64_t ncell)
{
  cblock_apply(z, v, inv, g, ncell);
}

__global__ void bdiag_kernel(double *z, const double *v, const double *inv, int64_t ncp)
{
  bdiag_apply(z, v, inv, ncp);
}

__global__ void jacobi_kernel(double *z, const double *v, const double *diag, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double d = diag[i];
    z[i] = v[i] / (d != 0.0 ? d : 1.0);
  }
}
// r = b - r
__global__ void sub_from_kernel(double *r, const double *b, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    r[i] = b[i] - r[i];
}

static unsigned vec_blocks(int64_t n)
{
  int64_t b = (n + 255) / 256;
  return (unsigned)(b < 152 * 8 ? b : 152 * 8);
}

// IGAPGPU_SPMV_DF=1: the multiply of the split and FP64-quality modes in
// double-FP32 arithmetic on the FP32 pipe.  Off by default: measured at
// 128x32x32 it takes 0.55 ms against 0.375 ms for the FP64 multiply (the
// integer-pipe splits of the value and of x cost more issue slots per
// nonzero than the FP64 FMA they replace).
bool spmv_df(const Context *c)
{
  const char *e = getenv("IGAPGPU_SPMV_DF");
  return e && e[0] == '1' && c->prec != IGAPGPU_PREC_FP64;
}

int spmv(Context *c, const double *vals, const double *x, double *y)
{
  const int64_t n = c->ndof;
  // a batch's rows belong to different lattices; the structured columns are
  // those of the quadratic stencil
  const int nb0 = (c->batch || c->porder != P) ? 0 : c->nbasis[0];
  auto kern = spmv_df(c) ? spmv_csr_kernel<true> : spmv_csr_kernel<false>;
  kern<<<(unsigned)((n * SPMV_G + 255) / 256), 256, 0, c->stream>>>(c->d_rowptr, c->d_cols, vals, x, y, n, nb0,
                                                                    c->nbasis[1], c->nbasis[2]);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

// out (device scalar) = a . b  or |a| (sqrt_flag)
static int dev_dot(Context *c, const double *a, const double *b, double *out, int sqrt_flag)
{
  dot_partial_kernel<<<RED_BLOCKS, RED_THREADS, 0, c->stream>>>(a, b, c->ndof, c->d_partial);
  dot_final_kernel<<<1, 1024, 0, c->stream>>>(c->d_partial, RED_BLOCKS, out, sqrt_flag);
  count_launch(2);
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

static int ensure_krylov(Context *c, int restart)
{
  if (c->d_work == nullptr) {
    if (cudaMalloc(&c->d_work, sizeof(double) * 4 * c->ndof) != cudaSuccess ||
        cudaMalloc(&c->d_diag, sizeof(double) * c->ndof) != cudaSuccess ||
        cudaMalloc(&c->d_bdiag, sizeof(double) * 3 * c->ndof) != cudaSuccess) {
      cudaGetLastError();
      set_error("Krylov workspace allocation failed");
      return IGAPGPU_ERR_NOMEM;
    }
  }
  if (restart + 8 > c->red_cap) {
    cudaFree(c->d_red);
    cudaFreeHost(c->h_red);
    c->d_red = nullptr;
    c->h_red = nullptr;
    c->red_cap = 0;
    if (cudaMalloc(&c->d_red, sizeof(double) * (restart + 8)) != cudaSuccess ||
        cudaMallocHost(&c->h_red, sizeof(double) * (restart + 8)) != cudaSuccess) {
      cudaGetLastError();
      set_error("reduction scratch allocation failed");
      return IGAPGPU_ERR_NOMEM;
    }
    c->red_cap = restart + 8;
  }
  if (restart > c->ksp_restart) {
    if (c->d_V) cudaFree(c->d_V);
    if (c->d_Z) cudaFree(c->d_Z);
    c->d_V = c->d_Z = nullptr;
    if (cudaMalloc(&c->d_V, sizeof(double) * (size_t)(restart + 1) * c->ndof) != cudaSuccess ||
        cudaMalloc(&c->d_Z, sizeof(double) * (size_t)restart * c->ndof) != cudaSuccess) {
      cudaGetLastError();
      c->ksp_restart = 0;
      set_error("GMRES basis of restart %d does not fit", restart);
      return IGAPGPU_ERR_NOMEM;
    }
    c->ksp_restart = restart;
  }
  return IGAPGPU_OK;
}

int dev_norm2(Context *c, const double *x, double *out)
{
  int r = ensure_krylov(c, 1);
  if (r) return r;
  r = dev_dot(c, x, x, c->d_red, 1);
  if (r) return r;
  IGAP_CUDA(cudaMemcpyAsync(c->h_red, c->d_red, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  *out = c->h_red[0];
  return IGAPGPU_OK;
}

// Lattice cells of the cell-block Jacobi preconditioner (2 x 2 x 2 control points).
CellGeom cell_geom(const Context *c)
{
  CellGeom g;
  for (int d = 0; d < 3; d++) {
    g.nb[d] = c->nbasis[d];
    g.nc[d] = (c->nbasis[d] + 1) / 2;
  }
  return g;
}

int ensure_cblock(Context *c, int64_t ncell)
{
  if (c->batch) {
    set_error("cell-block Jacobi (pc = 3) needs a single lattice; a batch takes pc 0, 1 or 2");
    return IGAPGPU_ERR_ARG;
  }
  if (!c->d_cinv && cudaMalloc(&c->d_cinv, sizeof(double) * (size_t)ncell * CBS * CBS) != cudaSuccess) {
    cudaGetLastError();
    c->d_cinv = nullptr;
    set_error("cell-block Jacobi: allocation of %lld blocks failed", (long long)ncell);
    return IGAPGPU_ERR_NOMEM;
  }
  return IGAPGPU_OK;
}

static __global__ void asm_kernel(double *z, const double *v, const float *Zi, CellGeom g, int64_t ncell)
{
  asm_apply(z, v, Zi, g, ncell);
}

int asm_setup(Context *c, float *Z)
{
  if (c->batch) {
    set_error("additive Schwarz (pc = 4) needs a single lattice; a batch takes pc 0, 1 or 2");
    return IGAPGPU_ERR_ARG;
  }
  static bool attr = false;
  if (!attr) {
    IGAP_CUDA(cudaFuncSetAttribute(asm_setup_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)asm_smem_bytes()));
    attr = true;
  }
  const CellGeom cg = cell_geom(c);
  asm_setup_kernel<<<(unsigned)cell_count(cg), AS_THREADS, asm_smem_bytes(), c->stream>>>(c->d_rowptr, c->d_vals, Z,
                                                                                          cg);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

// Right-preconditioned GMRES(m) with MGS, x in/out (device), b device.
int ksp_gmres(Context *c, const double *b, double *x, const igapgpu_solver_opts *o, int *its_out,
              double *rnorm_out)
{
  const int m = o->ksp_restart > 0 ? o->ksp_restart : 30;
  int r = ensure_krylov(c, m);
  if (r) return r;
  const int64_t n = c->ndof;
  double *V = c->d_V, *Z = c->d_Z, *w = c->d_work, *rvec = c->d_work + n;
  const unsigned vb = vec_blocks(n);
  const CellGeom cg = cell_geom(c);
  const int64_t ncell = cell_count(cg);
  if ((o->pc == 3 || o->pc == 4) && c->porder != P) {
    set_error("block preconditioners (pc = 3, 4) use the quadratic stencil; degree 3 takes pc 0, 1 or 2");
    return IGAPGPU_ERR_ARG;
  }
  if (o->pc == 1) {
    get_diag_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(c->d_rowptr, c->d_cols, c->d_vals, c->d_diag, n);
    count_launch();
  } else if (o->pc == 2) {  // point-block Jacobi: inverted 3 x 3 blocks, 9 per control point
    bdiag_invert_kernel<<<(unsigned)((n / 3 + 255) / 256), 256, 0, c->stream>>>(c->d_rowptr, c->d_cols, c->d_vals,
                                                                               c->d_bdiag, n / 3);
    count_launch();
    IGAP_CHECK_LAUNCH();
  } else if (o->pc == 3) {  // cell-block Jacobi: inverted blocks of the 2 x 2 x 2 control-point cells
    if ((r = ensure_cblock(c, ncell))) return r;
    cblock_invert_kernel<<<(unsigned)((ncell + CB_WARPS - 1) / CB_WARPS), 32 * CB_WARPS, 0, c->stream>>>(
        c->d_rowptr, c->d_vals, c->d_cinv, cg, ncell);
    count_launch();
    IGAP_CHECK_LAUNCH();
  } else if (o->pc == 4) {  // restricted additive Schwarz
    if (!c->d_asmz && cudaMalloc(&c->d_asmz, sizeof(float) * (size_t)ncell * AS_NC * AS_N) != cudaSuccess) {
      cudaGetLastError();
      c->d_asmz = nullptr;
      set_error("additive Schwarz: allocation of %lld subdomains failed", (long long)ncell);
      return IGAPGPU_ERR_NOMEM;
    }
    if ((r = asm_setup(c, c->d_asmz))) return r;
  }
  std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
  double rnorm0 = -1.0, rnorm = 0.0;
  int its = 0;
  for (;;) {
    // r = b - A x
    if ((r = spmv(c, c->d_vals, x, rvec))) return r;
    sub_from_kernel<<<vb, 256, 0, c->stream>>>(rvec, b, n);
    count_launch();
    double beta;
    if ((r = dev_dot(c, rvec, rvec, c->d_red, 1))) return r;
    IGAP_CUDA(cudaMemcpyAsync(c->h_red, c->d_red, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    IGAP_CUDA(cudaStreamSynchronize(c->stream));
    beta = c->h_red[0];
    if (!isfinite(beta)) {
      set_error("GMRES: non-finite residual norm");
      return IGAPGPU_ERR_NUMERIC;
    }
    if (rnorm0 < 0) rnorm0 = beta;
    rnorm = beta;
    const double tol = fmax(o->ksp_rtol * rnorm0, o->ksp_abstol);
    if (beta <= tol || its >= o->ksp_max_it) break;
    if (beta > o->ksp_dtol * rnorm0) {
      set_error("GMRES diverged (dtol)");
      return IGAPGPU_ERR_NUMERIC;
    }
    scale_div_kernel<<<vb, 256, 0, c->stream>>>(V, rvec, c->d_red, n);
    count_launch();
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    for (; j < m && its < o->ksp_max_it; j++, its++) {
      double *vj = V + (size_t)j * n, *zj = Z + (size_t)j * n, *vn = V + (size_t)(j + 1) * n;
      if (o->pc == 1) {
        jacobi_kernel<<<vb, 256, 0, c->stream>>>(zj, vj, c->d_diag, n);
        count_launch();
      } else if (o->pc == 2) {
        bdiag_kernel<<<vb, 256, 0, c->stream>>>(zj, vj, c->d_bdiag, n / 3);
        count_launch();
      } else if (o->pc == 3) {
        cblock_kernel<<<vb, 256, 0, c->stream>>>(zj, vj, c->d_cinv, cg, ncell);
        count_launch();
      } else if (o->pc == 4) {
        asm_kernel<<<vb, 256, 0, c->stream>>>(zj, vj, c->d_asmz, cg, ncell);
        count_launch();
      } else {
        IGAP_CUDA(cudaMemcpyAsync(zj, vj, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
      }
      if ((r = spmv(c, c->d_vals, zj, w))) return r;
      for (int i = 0; i <= j; i++) {  // modified Gram-Schmidt
        if ((r = dev_dot(c, w, V + (size_t)i * n, c->d_red + 1 + i, 0))) return r;
        axpy_dev_kernel<<<vb, 256, 0, c->stream>>>(w, V + (size_t)i * n, c->d_red + 1 + i, -1.0, n);
        count_launch();
      }
      if ((r = dev_dot(c, w, w, c->d_red + 2 + j, 1))) return r;
      scale_div_kernel<<<vb, 256, 0, c->stream>>>(vn, w, c->d_red + 2 + j, n);
      count_launch();
      IGAP_CUDA(cudaMemcpyAsync(c->h_red, c->d_red + 1, sizeof(double) * (j + 2), cudaMemcpyDeviceToHost, c->stream));
      IGAP_CUDA(cudaStreamSynchronize(c->stream));
      double *h = &H[(size_t)j * (m + 1)];
      for (int i = 0; i <= j + 1; i++) h[i] = c->h_red[i];
      for (int i = 0; i < j; i++) {  // previous rotations
        double t = cs[i] * h[i] + sn[i] * h[i + 1];
        h[i + 1] = -sn[i] * h[i] + cs[i] * h[i + 1];
        h[i] = t;
      }
      double den = hypot(h[j], h[j + 1]);
      if (den == 0.0) den = 1e-300;
      cs[j] = h[j] / den;
      sn[j] = h[j + 1] / den;
      h[j] = den;
      h[j + 1] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      rnorm = fabs(g[j + 1]);
      if (!isfinite(rnorm)) {
        set_error("GMRES: breakdown");
        return IGAPGPU_ERR_NUMERIC;
      }
      if (rnorm <= tol) { j++; its++; break; }
    }
    // y = H^{-1} g (upper triangular j x j), x += Z y
    for (int i = j - 1; i >= 0; i--) {
      double s = g[i];
      for (int k = i + 1; k < j; k++) s -= H[(size_t)k * (m + 1) + i] * y[k];
      y[i] = s / H[(size_t)i * (m + 1) + i];
    }
    for (int i = 0; i < j; i++) {
      axpby_kernel<<<vb, 256, 0, c->stream>>>(x, Z + (size_t)i * n, y[i], 1.0, n);
      count_launch();
    }
    IGAP_CHECK_LAUNCH();
    if (rnorm <= tol || its >= o->ksp_max_it) {
      // true residual of the final iterate
      if ((r = spmv(c, c->d_vals, x, rvec))) return r;
      sub_from_kernel<<<vb, 256, 0, c->stream>>>(rvec, b, n);
      count_launch();
      if ((r = dev_dot(c, rvec, rvec, c->d_red, 1))) return r;
      IGAP_CUDA(cudaMemcpyAsync(c->h_red, c->d_red, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      IGAP_CUDA(cudaStreamSynchronize(c->stream));
      rnorm = c->h_red[0];
      break;
    }
  }
  if (its_out) *its_out = its;
  if (rnorm_out) *rnorm_out = rnorm;
  return IGAPGPU_OK;
}

}  // namespace igap

using namespace igap;

extern "C" {

void igapgpu_default_solver_opts(igapgpu_solver_opts *o)
{
  o->snes_abstol = 1e-10;
  o->snes_rtol = 1e-20;
  o->snes_stol = 1e-20;
  o->snes_max_it = 50;
  o->linesearch = 1;
  o->ksp_restart = 100;
  o->ksp_rtol = 1e-10;
  o->ksp_abstol = 1e-50;
  o->ksp_dtol = 1e8;
  o->ksp_max_it = 10000;
  o->pc = 1;
  o->use_graphs = 1;
  o->orth = 0;
  o->snes_f0_max = 0.0;
}

int igapgpu_norm2(igapgpu_t c, const double *x, double *out)
{
  if (!c || !x || !out) return IGAPGPU_ERR_ARG;
  const double *xd = x;
  if (!is_device_ptr(x)) {
    IGAP_CUDA(cudaMemcpyAsync(c->d_stage_a, x, sizeof(double) * c->ndof, cudaMemcpyHostToDevice, c->stream));
    xd = c->d_stage_a;
  }
  double v = 0.0;
  int r = dev_norm2(c, xd, &v);
  if (r) return r;
  if (is_device_ptr(out)) {
    IGAP_CUDA(cudaMemcpyAsync(out, c->d_red, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  } else {
    *out = v;
  }
  return IGAPGPU_OK;
}

int igapgpu_get_diagonal(igapgpu_t c, double *diag)
{
  if (!c || !diag) return IGAPGPU_ERR_ARG;
  if (!c->matrix_valid) {
    set_error("get_diagonal before the tangent was assembled");
    return IGAPGPU_ERR_STATE;
  }
  const bool dev = is_device_ptr(diag);
  double *d = dev ? diag : c->d_stage_b;
  get_diag_kernel<<<(unsigned)((c->ndof + 255) / 256), 256, 0, c->stream>>>(c->d_rowptr, c->d_cols, c->d_vals, d, c->ndof);
  count_launch();
  IGAP_CHECK_LAUNCH();
  if (!dev) {
    IGAP_CUDA(cudaMemcpyAsync(diag, d, sizeof(double) * c->ndof, cudaMemcpyDeviceToHost, c->stream));
    IGAP_CUDA(cudaStreamSynchronize(c->stream));
  }
  return IGAPGPU_OK;
}

int igapgpu_ksp_solve(igapgpu_t c, const double *b, double *x, const igapgpu_solver_opts *opts,
                      int *its, double *rnorm)
{
  NvtxRange range("igapgpu_ksp_solve");
  if (!c || !b || !x) return IGAPGPU_ERR_ARG;
  if (!c->matrix_valid) {
    set_error("ksp_solve before the tangent was assembled");
    return IGAPGPU_ERR_STATE;
  }
  igapgpu_solver_opts o;
  if (opts) o = *opts; else igapgpu_default_solver_opts(&o);
  const bool bh = !is_device_ptr(b), xh = !is_device_ptr(x);
  double *bd = (double *)b, *xd = x;
  if (bh) {
    IGAP_CUDA(cudaMemcpyAsync(c->d_stage_a, b, sizeof(double) * c->ndof, cudaMemcpyHostToDevice, c->stream));
    bd = c->d_stage_a;
  }
  if (xh) {
    IGAP_CUDA(cudaMemcpyAsync(c->d_stage_b, x, sizeof(double) * c->ndof, cudaMemcpyHostToDevice, c->stream));
    xd = c->d_stage_b;
  }
  int r = ksp_gmres(c, bd, xd, &o, its, rnorm);
  if (r) return r;
  if (xh) {
    IGAP_CUDA(cudaMemcpyAsync(x, xd, sizeof(double) * c->ndof, cudaMemcpyDeviceToHost, c->stream));
    IGAP_CUDA(cudaStreamSynchronize(c->stream));
  }
  return IGAPGPU_OK;
}

// Newton with backtracking on 1/2|F|^2 (SNESNEWTONLS + BT, src/interface.c:217-224).
int igapgpu_solve(igapgpu_t c, double *U, const igapgpu_solver_opts *opts, igapgpu_solve_stats *st)
{
  NvtxRange range("igapgpu_solve");
  if (!c || !U) return IGAPGPU_ERR_ARG;
  igapgpu_solver_opts o;
  if (opts) o = *opts; else igapgpu_default_solver_opts(&o);
  igapgpu_solve_stats S;
  memset(&S, 0, sizeof S);
  const int64_t n = c->ndof;
  const bool uh = !is_device_ptr(U);
  int r = ensure_krylov(c, o.ksp_restart > 0 ? o.ksp_restart : 30);
  if (r) return r;
  double *Ud = c->d_Uhist;  // the iterate lives in U_hist[0]
  if (uh) IGAP_CUDA(cudaMemcpyAsync(Ud, U, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  else if (U != Ud) IGAP_CUDA(cudaMemcpyAsync(Ud, U, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
  double *F = c->d_RR, *dx = c->d_work + 2 * n, *Ubak = c->d_stage_a, *negF = c->d_stage_b;
  const unsigned vb = vec_blocks(n);
  auto residual = [&]() { return o.use_graphs ? assembly_graph(c, true, false) : launch_assembly(c, true, false, F, nullptr); };
  if ((r = residual())) return r;
  double fnorm;
  if ((r = dev_norm2(c, F, &fnorm))) return r;
  S.fnorm0 = fnorm;
  S.reason = 0;
  if (o.snes_f0_max > 0.0 && !(fnorm <= o.snes_f0_max)) {  // rejected initial iterate: U unchanged
    S.reason = IGAPGPU_REASON_REJECTED;
    S.fnorm = fnorm;
    if (uh) IGAP_CUDA(cudaMemcpyAsync(U, Ud, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    IGAP_CUDA(cudaStreamSynchronize(c->stream));
    if (st) *st = S;
    return IGAPGPU_OK;
  }
  for (int it = 0; it < o.snes_max_it; it++) {
    if (!isfinite(fnorm)) { S.reason = -4; break; }
    if (fnorm <= o.snes_abstol) { S.reason = 2; break; }
    if (fnorm <= o.snes_rtol * S.fnorm0) { S.reason = 3; break; }
    // J dx = -F
    if ((r = o.use_graphs ? assembly_graph(c, false, true) : launch_assembly(c, false, true, nullptr, c->d_vals)))
      return r;
    c->matrix_valid = true;
    IGAP_CUDA(cudaMemsetAsync(dx, 0, sizeof(double) * n, c->stream));
    axpby_kernel<<<vb, 256, 0, c->stream>>>(negF, F, -1.0, 0.0, n);
    count_launch();
    int kits = 0;
    double kr = 0.0;
    r = o.use_graphs ? ksp_gmres_graph(c, negF, dx, &o, &kits, &kr) : ksp_gmres(c, negF, dx, &o, &kits, &kr);
    if (r == IGAPGPU_ERR_NUMERIC) { S.reason = -3; break; }
    if (r) return r;
    S.ksp_its_last = kits;
    S.ksp_its_total += kits;
    // line search
    IGAP_CUDA(cudaMemcpyAsync(Ubak, Ud, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
    const double f0 = 0.5 * fnorm * fnorm, slope = -fnorm * fnorm;  // d/dl 1/2|F(U+l dx)|^2 at 0
    double lam = 1.0, lam_prev = 0.0, f_prev = 0.0, fn = 0.0;
    bool ok = false;
    for (int ls = 0; ls < 40; ls++) {
      IGAP_CUDA(cudaMemcpyAsync(Ud, Ubak, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
      axpby_kernel<<<vb, 256, 0, c->stream>>>(Ud, dx, lam, 1.0, n);
      count_launch();
      if ((r = residual())) return r;
      if ((r = dev_norm2(c, F, &fn))) return r;
      const double fl = 0.5 * fn * fn;
      if (o.linesearch == 0 || (isfinite(fl) && fl <= f0 + 1e-4 * lam * slope)) { ok = true; break; }
      double lnew;
      if (ls == 0 || !isfinite(fl)) {
        lnew = isfinite(fl) ? -slope / (2.0 * (fl - f0 - slope)) : 0.5 * lam;
      } else {  // cubic through f0, slope, (lam, fl), (lam_prev, f_prev)
        double t1 = fl - f0 - lam * slope, t2 = f_prev - f0 - lam_prev * slope;
        double a = (t1 / (lam * lam) - t2 / (lam_prev * lam_prev)) / (lam - lam_prev);
        double bb = (-lam_prev * t1 / (lam * lam) + lam * t2 / (lam_prev * lam_prev)) / (lam - lam_prev);
        if (a == 0.0) lnew = -slope / (2.0 * bb);
        else {
          double disc = bb * bb - 3.0 * a * slope;
          lnew = disc < 0 ? 0.5 * lam : (-bb + sqrt(disc)) / (3.0 * a);
        }
      }
      lam_prev = lam;
      f_prev = fl;
      lam = fmin(fmax(lnew, 0.1 * lam), 0.5 * lam);
    }
    S.newton_its = it + 1;
    if (!ok) { S.reason = -6; fnorm = fn; break; }
    fnorm = fn;
    // step tolerance |lam dx| <= stol |U|
    double dxn, un;
    if ((r = dev_norm2(c, dx, &dxn))) return r;
    if ((r = dev_norm2(c, Ud, &un))) return r;
    if (lam * dxn <= o.snes_stol * un) { S.reason = 4; break; }
  }
  if (S.reason == 0) S.reason = (fnorm <= o.snes_abstol) ? 2 : -5;
  S.fnorm = fnorm;
  S.converged = S.reason > 0;
  if (uh) {
    IGAP_CUDA(cudaMemcpyAsync(U, Ud, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  } else if (U != Ud) {
    IGAP_CUDA(cudaMemcpyAsync(U, Ud, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
  }
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  if (st) *st = S;
  return IGAPGPU_OK;
}

}  // extern "C"
