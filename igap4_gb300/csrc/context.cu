// C ABI of libigapgpu.so: context lifecycle, set-up (IGAPAssmInit role) and
// the Residual / Tangent / MatMult entry points.  Host code here only prepares
// state-independent data (quadrature rule, CSR row offsets, Dirichlet rows and
// boundary values, Neumann normal-derivative factors); every per-iterate
// computation runs in the kernels of assemble.cu and krylov.cu.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>
#include <map>
#include <utility>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace igap {

std::atomic<int64_t> g_launches{0};
static char g_err[512] = "";
static std::mutex g_err_mu;

void set_error(const char *fmt, ...)
{
  std::lock_guard<std::mutex> lk(g_err_mu);
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}

bool is_device_ptr(const void *p)
{
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Gauss-Legendre rule on [0,1] (the rule of legendre_handle,
// src/quadrature.c:381-430, computed by Newton iteration on P_n).
static void gauss_legendre01(int n, double *x, double *w)
{
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; i++) {
    double z = cos(pi * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; k++) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      double dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-17) break;
    }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= n; k++) {
      double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    double dp = n * (z * p1 - p0) / (z * z - 1.0);
    x[i] = 0.5 * (-z) + 0.5;
    w[i] = 0.5 * (2.0 / ((1.0 - z * z) * dp * dp));
  }
}

// B-spline basis function i (derivative order k) at xi, with the end-point
// and 0/0 conventions of evalN (src/meshcore_iga.c:329-384).
static double basis0(const double *kv, int nk, int i, int p, double xi)
{
  if (i == nk - p - 2 && fabs(xi - kv[nk - 1]) < 1.e-15 && fabs(kv[nk - 1] - kv[nk - 2]) < 1.e-15)
    return 1.0;
  if (p == 0) return (xi >= kv[i] && kv[i + 1] > xi) ? 1.0 : 0.0;
  double left = kv[i + p] - kv[i], right = kv[i + p + 1] - kv[i + 1];
  if (left == 0.0 && right == 0.0) return 0.0;
  if (left == 0.0) return (kv[i + p + 1] - xi) / right * basis0(kv, nk, i + 1, p - 1, xi);
  if (right == 0.0) return (xi - kv[i]) / left * basis0(kv, nk, i, p - 1, xi);
  return (xi - kv[i]) / left * basis0(kv, nk, i, p - 1, xi) +
         (kv[i + p + 1] - xi) / right * basis0(kv, nk, i + 1, p - 1, xi);
}
static double basis_deriv(const double *kv, int nk, int k, int i, int p, double xi)
{
  if (k == 0) return basis0(kv, nk, i, p, xi);
  double a[8][8];
  a[0][0] = 1.0;
  for (int r = 1; r <= k; r++) {
    double d0 = kv[i + p - r + 1] - kv[i];
    a[r][0] = d0 == 0.0 ? 0.0 : a[r - 1][0] / d0;
    for (int cc = 1; cc < r; cc++) {
      double dc = kv[i + p + cc - r + 1] - kv[i + cc];
      a[r][cc] = dc == 0.0 ? 0.0 : (a[r - 1][cc] - a[r - 1][cc - 1]) / dc;
    }
    double dr = kv[i + p + 1] - kv[i + r];
    a[r][r] = dr == 0.0 ? 0.0 : -a[r - 1][r - 1] / dr;
  }
  double s = 0.0;
  for (int j = 0; j <= k; j++) s += a[k][j] * basis0(kv, nk, i + j, p - k, xi);
  double fac = 1.0;
  for (int j = p; j > p - k; j--) fac *= j;
  return s * fac;
}

// Face frame: (a, b) face-parallel directions, n the normal
// (src/assmcore_iga.c:276-313, :418-437).
static void face_dirs(int face, int &da, int &db, int &dn)
{
  if (face / 2 == 0) { da = 1; db = 2; dn = 0; }
  else if (face / 2 == 1) { da = 0; db = 2; dn = 1; }
  else { da = 0; db = 1; dn = 2; }
}

// Affine Dirichlet data on one face (role of dirichlet_iga,
// src/assmcore_iga.c:861-934): values on the face's control points.
static void dirichlet_face(const Context *c, const std::vector<double> kn[3], int face, int d,
                           std::vector<double> &out)
{
  int da, db, dn;
  face_dirs(face, da, db, dn);
  const int p = c->porder;
  const int dirs[2] = {da, db};
  double pf[3] = {c->bc.par_dirichlet[3 * d + da], c->bc.par_dirichlet[3 * d + db],
                  c->bc.par_dirichlet[3 * d + dn]};
  const std::vector<double> &kz = kn[dn];
  const double Z = (face % 2 == 0) ? kz[0] : kz[kz.size() - 1] - 1.e-15;
  std::vector<double> d1[2];
  for (int bb = 0; bb < 2; bb++) {
    const int dd = dirs[bb], nb = c->nbasis[dd];
    const std::vector<double> &kv = kn[dd];
    d1[bb].assign(nb, 0.0);
    const double W0 = kv[p];
    // value and slope of the affine function at the first knot, matched by
    // the first p control values: solve  sum_j N_j^(i)(W0) x_j = v_i
    double A[4][4], v[4];
    for (int i = 0; i < p; i++) {
      v[i] = (i == 0) ? pf[bb] * W0 : (i == 1 ? pf[bb] : 0.0);
      for (int j = 0; j < p; j++) A[i][j] = basis_deriv(kv.data(), (int)kv.size(), i, j, p, W0);
    }
    if (p == 2) {  // the 2 x 2 solve by Cramer's rule
      double det = A[0][0] * A[1][1] - A[0][1] * A[1][0];
      d1[bb][0] = (v[0] * A[1][1] - A[0][1] * v[1]) / det;
      d1[bb][1] = (A[0][0] * v[1] - A[1][0] * v[0]) / det;
    } else {  // p x p: Gaussian elimination with partial pivoting
      for (int k = 0; k < p; k++) {
        int pr = k;
        for (int i = k + 1; i < p; i++)
          if (fabs(A[i][k]) > fabs(A[pr][k])) pr = i;
        for (int j = 0; j < p; j++) std::swap(A[k][j], A[pr][j]);
        std::swap(v[k], v[pr]);
        for (int i = k + 1; i < p; i++) {
          const double f = A[i][k] / A[k][k];
          for (int j = k; j < p; j++) A[i][j] -= f * A[k][j];
          v[i] -= f * v[k];
        }
      }
      for (int k = p - 1; k >= 0; k--) {
        double s = v[k];
        for (int j = k + 1; j < p; j++) s -= A[k][j] * d1[bb][j];
        d1[bb][k] = s / A[k][k];
      }
    }
    for (int i = p; i < nb; i++) d1[bb][i] = d1[bb][i - 1] + (kv[i + p] - kv[i]) / ((double)p) * pf[bb];
  }
  const int n0 = c->nbasis[da], n1 = c->nbasis[db];
  out.assign((size_t)n0 * n1, 0.0);
  for (int i = 0; i < n0; i++)
    for (int j = 0; j < n1; j++) out[(size_t)n1 * i + j] = d1[0][i] + d1[1][j] + pf[2] * Z;
}

static int free_ctx(Context *c)
{
  if (!c) return IGAPGPU_OK;
  graph_release(c);
  batch_release(c);
  void *bufs[] = {c->d_wq, c->d_xq, c->d_w, c->d_X, c->d_Uhist, c->d_RR, c->d_vals,
                  c->d_rowptr, c->d_cols, c->d_Dconst, c->d_Fneu, c->d_dir_rows, c->d_dir_g,
                  c->d_stage_a, c->d_stage_b, c->d_stage_v, c->d_V, c->d_Z, c->d_work,
                  c->d_diag, c->d_bdiag, c->d_cinv, c->d_asmz, c->d_red, c->d_partial, c->d_err, c->d_geo, c->d_geof, c->d_gop, c->d_oz, c->d_ozexp, c->d_rpc, c->d_rel, c->d_upair, c->d_lin, c->d_preR, c->d_preD, c->d_dens, c->d_dsparse, c->d_dval, c->d_sval, c->d_bct, c->d_neu};
  for (void *b : bufs)
    if (b) cudaFree(b);
  for (int d = 0; d < 3; d++) {
    if (c->d_tab[d]) cudaFree(c->d_tab[d]);
    if (c->d_tabn[d]) cudaFree(c->d_tabn[d]);
    if (c->d_knots[d]) cudaFree(c->d_knots[d]);
  }
  if (c->h_red) cudaFreeHost(c->h_red);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete static_cast<igapgpu_ctx *>(c);
  return IGAPGPU_OK;
}

template <typename T>
static int dev_alloc(T **p, size_t n)
{
  cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (n ? n : 1));
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaMalloc of %zu bytes failed: %s", sizeof(T) * n, cudaGetErrorString(e));
    return IGAPGPU_ERR_NOMEM;
  }
  return IGAPGPU_OK;
}

#define IGAP_TRY(x)            \
  do {                         \
    int _r = (x);              \
    if (_r) {                  \
      free_ctx(c);             \
      return _r;               \
    }                          \
  } while (0)

static int init_impl(Context *c, const igapgpu_mesh_desc *mesh)
{
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("no CUDA device: the GPU assembly has no CPU fallback");
    return IGAPGPU_ERR_CUDA;
  }
  if (!c->sub) {  // an instance of a batch runs on the batch's stream
    IGAP_CUDA(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
    c->stream = c->own_stream;
  }
  // mesh
  std::vector<double> kn[3];
  const int pd = c->porder;
  for (int d = 0; d < 3; d++) {
    const int nk = c->nelem[d] + 1 + 2 * pd;
    kn[d].assign(mesh->knots[d], mesh->knots[d] + nk);
    int r = dev_alloc(&c->d_knots[d], nk);
    if (r) return r;
    IGAP_CUDA(cudaMemcpy(c->d_knots[d], kn[d].data(), sizeof(double) * nk, cudaMemcpyHostToDevice));
    if ((r = dev_alloc(&c->d_tab[d], (size_t)c->nelem[d] * c->nquad * tab_len(pd)))) return r;
    if ((r = dev_alloc(&c->d_tabn[d], (size_t)c->nelem[d] * c->nquad * tab_len(pd)))) return r;
  }
  int r;
  if ((r = dev_alloc(&c->d_w, c->ncp))) return r;
  if ((r = dev_alloc(&c->d_X, 3 * c->ncp))) return r;
  IGAP_CUDA(cudaMemcpy(c->d_w, mesh->w, sizeof(double) * c->ncp, cudaMemcpyHostToDevice));
  IGAP_CUDA(cudaMemcpy(c->d_X, mesh->X, sizeof(double) * 3 * c->ncp, cudaMemcpyHostToDevice));
  // quadrature
  double xq[MAXQ], wq[MAXQ];
  gauss_legendre01(c->nquad, xq, wq);
  if ((r = dev_alloc(&c->d_xq, c->nquad))) return r;
  if ((r = dev_alloc(&c->d_wq, c->nquad))) return r;
  IGAP_CUDA(cudaMemcpy(c->d_xq, xq, sizeof(double) * c->nquad, cudaMemcpyHostToDevice));
  IGAP_CUDA(cudaMemcpy(c->d_wq, wq, sizeof(double) * c->nquad, cudaMemcpyHostToDevice));
  if ((r = pd == 3 ? launch_basis_tables_p3(c) : launch_basis_tables(c))) return r;
  // geometry cache: built once when it fits (leaving headroom for the matrix
  // and the Krylov workspace); IGAPGPU_GEOMETRY_CACHE=0 disables it; the
  // cubic path evaluates its geometry in the element kernel
  {
    const char *env = getenv("IGAPGPU_GEOMETRY_CACHE");
    const bool want = !(env && env[0] == '0') && pd == P;
    const size_t npts = (size_t)c->nquad * c->nquad * c->nquad;
    const size_t bytes = sizeof(double) * (size_t)c->nelem_total * npts * (NB * NDD + 2);
    size_t freeb = 0, totb = 0;
    IGAP_CUDA(cudaMemGetInfo(&freeb, &totb));
    const size_t need_other = (size_t)(3 * c->ncp) * 8 * 400;  // matrix, pattern, workspace (rough)
    bool use64, use32;
    if (c->geo_mode >= 0) {  // decided by the caller (the instances of a batch)
      use64 = want && c->geo_mode >= 1;
      use32 = use64 && c->geo_mode >= 2;
    } else {
      use64 = want && bytes + need_other + ((size_t)4 << 30) < freeb;
      use32 = use64 && bytes / 2 + need_other + ((size_t)4 << 30) < freeb - bytes;
    }
    if (use64) {
      if (cudaMalloc(&c->d_geo, bytes) != cudaSuccess) {
        cudaGetLastError();
        c->d_geo = nullptr;
      } else if ((r = launch_geometry_cache(c))) {
        return r;
      } else if (use32) {
        // FP32 copy used by the split-precision tangent
        if (cudaMalloc(&c->d_geof, bytes / 2) != cudaSuccess) {
          cudaGetLastError();
          c->d_geof = nullptr;
        } else if ((r = launch_geometry_cache_f32(c))) {
          return r;
        }
      }
    }
  }
  // CSR row offsets (setnz_iga, src/assmcore_iga.c:1074-1086, one rank)
  std::vector<int64_t> rowptr(c->ndof + 1);
  rowptr[0] = 0;
  {
    int64_t row = 0;
    auto cnt = [&](int i, int nb) { return (i < pd ? i : pd) + 1 + (i > nb - 1 - pd ? nb - 1 - i : pd); };
    for (int ix = 0; ix < c->nbasis[0]; ix++)
      for (int iy = 0; iy < c->nbasis[1]; iy++)
        for (int iz = 0; iz < c->nbasis[2]; iz++) {
          const int64_t len = 3LL * cnt(ix, c->nbasis[0]) * cnt(iy, c->nbasis[1]) * cnt(iz, c->nbasis[2]);
          for (int d = 0; d < 3; d++, row++) rowptr[row + 1] = rowptr[row] + len;
        }
  }
  c->nnz = rowptr[c->ndof];
  if (c->nnz > INT64_C(2147483647) * 8) {
    set_error("matrix too large");
    return IGAPGPU_ERR_ARG;
  }
  if (c->sub) {  // the batch owns matrix, pattern and state
    c->h_rowptr.swap(rowptr);
    if ((r = dev_alloc(&c->d_Fneu, c->ndof))) return r;
    if ((r = dev_alloc(&c->d_err, 1))) return r;
    IGAP_CUDA(cudaMemset(c->d_err, 0, sizeof(int)));
  } else {
  if ((r = dev_alloc(&c->d_rowptr, c->ndof + 1))) return r;
  if ((r = dev_alloc(&c->d_cols, c->nnz))) return r;
  if ((r = dev_alloc(&c->d_vals, c->nnz))) return r;
  IGAP_CUDA(cudaMemcpy(c->d_rowptr, rowptr.data(), sizeof(int64_t) * (c->ndof + 1), cudaMemcpyHostToDevice));
  if ((r = pd == 3 ? launch_pattern_cols_p3(c) : launch_pattern_cols(c))) return r;
  // state, residual, staging
  if ((r = dev_alloc(&c->d_Uhist, (size_t)(c->torder + 1) * c->ndof))) return r;
  IGAP_CUDA(cudaMemset(c->d_Uhist, 0, sizeof(double) * (c->torder + 1) * c->ndof));
  if ((r = dev_alloc(&c->d_RR, c->ndof))) return r;
  if ((r = dev_alloc(&c->d_stage_a, c->ndof))) return r;
  if ((r = dev_alloc(&c->d_stage_b, c->ndof))) return r;
  if ((r = dev_alloc(&c->d_Fneu, c->ndof))) return r;
  if ((r = dev_alloc(&c->d_err, 1))) return r;
  IGAP_CUDA(cudaMemset(c->d_err, 0, sizeof(int)));
  if ((r = dev_alloc(&c->d_red, 64))) return r;
  if ((r = dev_alloc(&c->d_partial, 1024))) return r;
  IGAP_CUDA(cudaMallocHost(&c->h_red, 64 * sizeof(double)));
  c->red_cap = 64;
  }
  // law constants
  if (c->law == IGAPGPU_LAW_LINGRAD) {
    if ((r = dev_alloc(&c->d_Dconst, 900))) return r;
    if ((r = launch_lingrad_dconst(c))) return r;
    // sparse form of the constant tangent (exact zeros skipped)
    double D[900];
    IGAP_CUDA(cudaMemcpy(D, c->d_Dconst, sizeof D, cudaMemcpyDeviceToHost));
    std::vector<int> dptr(31, 0), dcol, sptr(91, 0), sl;
    std::vector<double> dval;
    std::vector<float> sval;
    for (int i = 0; i < 30; i++) {
      for (int j = 0; j < 30; j++)
        if (D[30 * i + j] != 0.0) { dcol.push_back(j); dval.push_back(D[30 * i + j]); }
      dptr[i + 1] = (int)dcol.size();
    }
    for (int i = 0; i < 30; i++)
      for (int e = 0; e < 3; e++) {
        for (int l = 0; l < 10; l++)
          if (D[30 * i + 10 * e + l] != 0.0) { sl.push_back(l); sval.push_back((float)D[30 * i + 10 * e + l]); }
        sptr[3 * i + e + 1] = (int)sl.size();
      }
    c->dnnz = (int)dcol.size();
    std::vector<int> packed;
    packed.insert(packed.end(), dptr.begin(), dptr.end());
    packed.insert(packed.end(), dcol.begin(), dcol.end());
    packed.insert(packed.end(), sptr.begin(), sptr.end());
    packed.insert(packed.end(), sl.begin(), sl.end());
    if ((r = dev_alloc(&c->d_dsparse, packed.size()))) return r;
    if ((r = dev_alloc(&c->d_dval, dval.size()))) return r;
    if ((r = dev_alloc(&c->d_sval, sval.size()))) return r;
    IGAP_CUDA(cudaMemcpy(c->d_dsparse, packed.data(), sizeof(int) * packed.size(), cudaMemcpyHostToDevice));
    IGAP_CUDA(cudaMemcpy(c->d_dval, dval.data(), sizeof(double) * dval.size(), cudaMemcpyHostToDevice));
    IGAP_CUDA(cudaMemcpy(c->d_sval, sval.data(), sizeof(float) * sval.size(), cudaMemcpyHostToDevice));
  }
  // Neumann load (state independent): normal-derivative factors of the two
  // boundary layers, evalN(k=1) at the face coordinate (src/assmcore_iga.c:384-387)
  double (&nfac)[NFACE][2] = c->nfac;
  for (int d = 0; d < 3; d++) c->h_knots[d] = kn[d];
  for (int face = 0; face < NFACE; face++) {
    int da, db, dn;
    face_dirs(face, da, db, dn);
    const std::vector<double> &kz = kn[dn];
    const int nk = (int)kz.size();
    const double zq = (face % 2 == 0) ? kz[0] : kz[nk - 1];
    const int lay0 = (face % 2 == 0) ? 0 : c->nelem[dn] + pd - 1;
    const int lay1 = (face % 2 == 0) ? 1 : c->nelem[dn] + pd - 2;
    nfac[face][0] = basis_deriv(kz.data(), nk, 1, lay0, pd, zq);
    nfac[face][1] = basis_deriv(kz.data(), nk, 1, lay1, pd, zq);
  }
  if ((r = pd == 3 ? launch_neumann_p3(c, nfac) : launch_neumann(c, nfac))) return r;
  // Dirichlet rows and values, in the reference's insertion order; a row
  // listed twice keeps the last value (INSERT_VALUES, src/assmcore_iga.c:467,489)
  {
    std::map<int64_t, double> last;
    std::vector<int64_t> order;
    const int64_t sx = (int64_t)c->nbasis[1] * c->nbasis[2], sy = c->nbasis[2], sz = 1;
    for (int face = 0; face < NFACE; face++) {
      int da, db, dn;
      face_dirs(face, da, db, dn);
      const int64_t st[3] = {sx, sy, sz};
      const int nz = c->nbasis[dn];
      const int layer[2] = {(face % 2 == 0) ? 0 : nz - 1, (face % 2 == 0) ? 1 : nz - 2};
      for (int o = 0; o < 2; o++)
        for (int d = 0; d < 3; d++) {
          if (c->bc.bc_type[6 * face + 3 * o + d] != 0) continue;
          std::vector<double> g;
          dirichlet_face(c, kn, face, d, g);
          const int n1 = c->nbasis[db];
          for (int i = 0; i < c->nbasis[da]; i++)
            for (int j = 0; j < n1; j++) {
              const int64_t row = 3 * (st[da] * i + st[db] * j + st[dn] * layer[o]) + d;
              if (!last.count(row)) order.push_back(row);
              last[row] = g[(size_t)n1 * i + j];
            }
        }
    }
    c->n_dir = (int64_t)order.size();
    if (c->n_dir) {
      std::vector<double> gv(c->n_dir);
      for (int64_t i = 0; i < c->n_dir; i++) gv[i] = last[order[i]];
      if ((r = dev_alloc(&c->d_dir_rows, c->n_dir))) return r;
      if ((r = dev_alloc(&c->d_dir_g, c->n_dir))) return r;
      IGAP_CUDA(cudaMemcpy(c->d_dir_rows, order.data(), sizeof(int64_t) * c->n_dir, cudaMemcpyHostToDevice));
      IGAP_CUDA(cudaMemcpy(c->d_dir_g, gv.data(), sizeof(double) * c->n_dir, cudaMemcpyHostToDevice));
    }
  }
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  return IGAPGPU_OK;
}

// Copy a user array into device memory if needed; returns the device pointer.
static int stage_in(Context *c, const double *src, size_t n, double *scratch, const double **dev)
{
  if (!src) {
    *dev = nullptr;
    return IGAPGPU_OK;
  }
  if (is_device_ptr(src)) {
    *dev = src;
    return IGAPGPU_OK;
  }
  IGAP_CUDA(cudaMemcpyAsync(scratch, src, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  *dev = scratch;
  return IGAPGPU_OK;
}

static int set_current(Context *c, const double *U)
{
  if (!U) return IGAPGPU_OK;
  if (is_device_ptr(U)) {
    if (U != c->d_Uhist)
      IGAP_CUDA(cudaMemcpyAsync(c->d_Uhist, U, sizeof(double) * c->ndof, cudaMemcpyDeviceToDevice, c->stream));
  } else {
    IGAP_CUDA(cudaMemcpyAsync(c->d_Uhist, U, sizeof(double) * c->ndof, cudaMemcpyHostToDevice, c->stream));
  }
  return IGAPGPU_OK;
}


}  // namespace igap

namespace igap {

int check_instance_args(const igapgpu_mesh_desc *mesh, const igapgpu_phys_desc *phys,
                        const igapgpu_bc_desc *bc, int nquad)
{
  if (!mesh || !phys || !bc) {
    set_error("null argument");
    return IGAPGPU_ERR_ARG;
  }
  if (mesh->porder != 2 && mesh->porder != 3) {
    set_error("porder %d unsupported: the device bases are quadratic (as eval_Bspline) and cubic",
              mesh->porder);
    return IGAPGPU_ERR_ARG;
  }
  for (int d = 0; d < 3; d++)
    if (mesh->nelem[d] < mesh->porder || !mesh->knots[d]) {
      set_error("direction %d has %d elements; at least porder are required", d, mesh->nelem[d]);
      return IGAPGPU_ERR_ARG;
    }
  if (!mesh->w || !mesh->X) {
    set_error("mesh weights / control points missing");
    return IGAPGPU_ERR_ARG;
  }
  if (nquad < 1 || nquad > MAXQ) {
    set_error("nquad %d out of range 1..%d", nquad, MAXQ);
    return IGAPGPU_ERR_ARG;
  }
  if (phys->law != IGAPGPU_LAW_GRADELAST && phys->law != IGAPGPU_LAW_GRADELASTTIME &&
      phys->law != IGAPGPU_LAW_LINGRAD) {
    set_error("unknown law id %d (no CPU fallback)", phys->law);
    return IGAPGPU_ERR_LAW;
  }
  for (int i = 0; i < 9; i++)
    if (bc->par_periodic[i] != 0.0) {
      set_error("par_periodic must be zero on a non-periodic mesh");
      return IGAPGPU_ERR_ARG;
    }
  for (int i = 0; i < 36; i++)
    if (bc->bc_type[i] != 0 && bc->bc_type[i] != 1) {
      set_error("bc_type[%d] = %d; expected 0 (Dirichlet) or 1 (Neumann)", i, bc->bc_type[i]);
      return IGAPGPU_ERR_ARG;
    }
  return IGAPGPU_OK;
}

Context *new_context(const igapgpu_mesh_desc *mesh, const igapgpu_phys_desc *phys,
                     const igapgpu_bc_desc *bc, int nquad)
{
  igapgpu_ctx *c = new igapgpu_ctx();
  c->law = phys->law;
  c->torder = phys->law == IGAPGPU_LAW_GRADELASTTIME ? 2 : 0;
  memcpy(c->par, phys->par, sizeof c->par);
  c->nquad = nquad;
  c->prec = IGAPGPU_PREC_FP64;
  c->bc = *bc;
  c->porder = mesh->porder;
  c->ncp = 1;
  c->nelem_total = 1;
  for (int d = 0; d < 3; d++) {
    c->nelem[d] = mesh->nelem[d];
    c->nbasis[d] = mesh->nelem[d] + mesh->porder;
    c->ncp *= c->nbasis[d];
    c->nelem_total *= c->nelem[d];
  }
  c->ndof = 3 * c->ncp;
  return c;
}

int context_init(Context *c, const igapgpu_mesh_desc *mesh) { return init_impl(c, mesh); }
int context_free(Context *c) { return free_ctx(c); }

}  // namespace igap

using namespace igap;

extern "C" {

const char *igapgpu_last_error(void) { return g_err; }
int64_t igapgpu_launch_count(void) { return g_launches.load(); }

int igapgpu_assm_init(igapgpu_t *out, const igapgpu_mesh_desc *mesh, const igapgpu_phys_desc *phys,
                      const igapgpu_bc_desc *bc, int nquad)
{
  if (!out) {
    set_error("null argument");
    return IGAPGPU_ERR_ARG;
  }
  *out = nullptr;
  int r = check_instance_args(mesh, phys, bc, nquad);
  if (r) return r;
  Context *c = new_context(mesh, phys, bc, nquad);
  IGAP_TRY(init_impl(c, mesh));
  *out = static_cast<igapgpu_ctx *>(c);
  return IGAPGPU_OK;
}

int igapgpu_finalize(igapgpu_t c)
{
  if (c && c->stream) cudaStreamSynchronize(c->stream);
  return free_ctx(c);
}

int igapgpu_sizes(igapgpu_t c, int64_t *ndof, int64_t *nnz, int *torder, int64_t *nelem)
{
  if (!c) return IGAPGPU_ERR_ARG;
  if (ndof) *ndof = c->ndof;
  if (nnz) *nnz = c->nnz;
  if (torder) *torder = c->torder;
  if (nelem) *nelem = c->nelem_total;
  return IGAPGPU_OK;
}

int igapgpu_pattern(igapgpu_t c, int64_t *rowptr, int32_t *cols)
{
  if (!c) return IGAPGPU_ERR_ARG;
  if (rowptr) {
    cudaMemcpyKind k = is_device_ptr(rowptr) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    IGAP_CUDA(cudaMemcpyAsync(rowptr, c->d_rowptr, sizeof(int64_t) * (c->ndof + 1), k, c->stream));
  }
  if (cols) {
    cudaMemcpyKind k = is_device_ptr(cols) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    IGAP_CUDA(cudaMemcpyAsync(cols, c->d_cols, sizeof(int32_t) * c->nnz, k, c->stream));
  }
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  return IGAPGPU_OK;
}

int igapgpu_dirichlet(igapgpu_t c, int64_t *count, int64_t *rows, double *values)
{
  if (!c) return IGAPGPU_ERR_ARG;
  if (count) *count = c->n_dir;
  if (c->n_dir == 0) return IGAPGPU_OK;
  if (rows) {
    cudaMemcpyKind k = is_device_ptr(rows) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    IGAP_CUDA(cudaMemcpyAsync(rows, c->d_dir_rows, sizeof(int64_t) * c->n_dir, k, c->stream));
  }
  if (values) {
    cudaMemcpyKind k = is_device_ptr(values) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    IGAP_CUDA(cudaMemcpyAsync(values, c->d_dir_g, sizeof(double) * c->n_dir, k, c->stream));
  }
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  return IGAPGPU_OK;
}

int igapgpu_impose_dirichlet(igapgpu_t c, double *U)
{
  if (!c || !U) return IGAPGPU_ERR_ARG;
  if (c->n_dir == 0) return IGAPGPU_OK;
  if (is_device_ptr(U)) return launch_impose_dirichlet(c, U);
  // host vector: round trip through the residual scratch
  IGAP_CUDA(cudaMemcpyAsync(c->d_RR, U, sizeof(double) * c->ndof, cudaMemcpyHostToDevice, c->stream));
  int r = launch_impose_dirichlet(c, c->d_RR);
  if (r) return r;
  IGAP_CUDA(cudaMemcpyAsync(U, c->d_RR, sizeof(double) * c->ndof, cudaMemcpyDeviceToHost, c->stream));
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  return IGAPGPU_OK;
}

// Solution files of IGAPSolvSaveSolution / IGAPSolvLoadSolution
// (src/interface.c:271-300, write_solution / read_solution, src/ioutil.c:90-159):
// raw FP64 history levels in the universal DOF order, which on one rank with a
// non-periodic mesh is the DOF numbering 3 cp + d.  Static laws store level 0,
// the transient law levels 1..torder (loading also sets level 0 = level 1).
static void solution_levels(const Context *c, int *l0, int *l1)
{
  *l0 = c->torder == 0 ? 0 : 1;
  *l1 = c->torder == 0 ? 1 : c->torder + 1;
}

int igapgpu_save_solution(igapgpu_t c, const char *fname)
{
  if (!c || !fname) return IGAPGPU_ERR_ARG;
  int l0, l1;
  solution_levels(c, &l0, &l1);
  const size_t n = (size_t)(l1 - l0) * c->ndof;
  std::vector<double> h(n);
  IGAP_CUDA(cudaMemcpyAsync(h.data(), c->d_Uhist + (size_t)l0 * c->ndof, sizeof(double) * n,
                            cudaMemcpyDeviceToHost, c->stream));
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  FILE *f = fopen(fname, "wb");
  if (!f) {
    set_error("cannot open %s for writing", fname);
    return IGAPGPU_ERR_ARG;
  }
  const size_t w = fwrite(h.data(), sizeof(double), n, f);
  fclose(f);
  if (w != n) {
    set_error("short write to %s", fname);
    return IGAPGPU_ERR_ARG;
  }
  return IGAPGPU_OK;
}

int igapgpu_load_solution(igapgpu_t c, const char *fname)
{
  if (!c || !fname) return IGAPGPU_ERR_ARG;
  int l0, l1;
  solution_levels(c, &l0, &l1);
  const size_t n = (size_t)(l1 - l0) * c->ndof;
  std::vector<double> h(n);
  FILE *f = fopen(fname, "rb");
  if (!f) {
    set_error("cannot open %s", fname);
    return IGAPGPU_ERR_ARG;
  }
  const size_t r = fread(h.data(), sizeof(double), n, f);
  fclose(f);
  if (r != n) {
    set_error("%s holds %zu of the %zu values of this problem's solution file", fname, r, n);
    return IGAPGPU_ERR_ARG;
  }
  IGAP_CUDA(cudaMemcpyAsync(c->d_Uhist + (size_t)l0 * c->ndof, h.data(), sizeof(double) * n,
                            cudaMemcpyHostToDevice, c->stream));
  if (l0 == 1)
    IGAP_CUDA(cudaMemcpyAsync(c->d_Uhist, c->d_Uhist + c->ndof, sizeof(double) * c->ndof,
                              cudaMemcpyDeviceToDevice, c->stream));
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  return IGAPGPU_OK;
}

int igapgpu_set_history(igapgpu_t c, int level, const double *U)
{
  if (!c || !U || level < 0 || level > c->torder) {
    set_error("bad history level %d", level);
    return IGAPGPU_ERR_ARG;
  }
  const bool dev = is_device_ptr(U);
  IGAP_CUDA(cudaMemcpyAsync(c->d_Uhist + (size_t)level * c->ndof, U, sizeof(double) * c->ndof,
                            dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream));
  if (!dev) IGAP_CUDA(cudaStreamSynchronize(c->stream));
  return IGAPGPU_OK;
}

int igapgpu_get_history(igapgpu_t c, int level, double *U)
{
  if (!c || !U || level < 0 || level > c->torder) {
    set_error("bad history level %d", level);
    return IGAPGPU_ERR_ARG;
  }
  const bool dev = is_device_ptr(U);
  IGAP_CUDA(cudaMemcpyAsync(U, c->d_Uhist + (size_t)level * c->ndof, sizeof(double) * c->ndof,
                            dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream));
  if (!dev) IGAP_CUDA(cudaStreamSynchronize(c->stream));
  return IGAPGPU_OK;
}

int igapgpu_shift_history(igapgpu_t c)
{
  if (!c) return IGAPGPU_ERR_ARG;
  for (int l = c->torder; l >= 1; l--)
    IGAP_CUDA(cudaMemcpyAsync(c->d_Uhist + (size_t)l * c->ndof, c->d_Uhist + (size_t)(l - 1) * c->ndof,
                              sizeof(double) * c->ndof, cudaMemcpyDeviceToDevice, c->stream));
  return IGAPGPU_OK;
}

static int assemble_common(igapgpu_t c, const double *U, double *RR, double *vals, bool do_res,
                           bool do_tan)
{
  if (!c) return IGAPGPU_ERR_ARG;
  int r = set_current(c, U);
  if (r) return r;
  const bool rr_host = do_res && RR && !is_device_ptr(RR);
  const bool v_host = do_tan && vals && !is_device_ptr(vals);
  double *rr_dev = do_res ? ((RR && !rr_host) ? RR : c->d_RR) : nullptr;
  double *v_dev = do_tan ? ((vals && !v_host) ? vals : c->d_vals) : nullptr;
  r = launch_assembly(c, do_res, do_tan, rr_dev, v_dev);
  if (r) return r;
  if (do_tan && v_dev == c->d_vals) c->matrix_valid = true;
  if (rr_host) IGAP_CUDA(cudaMemcpyAsync(RR, rr_dev, sizeof(double) * c->ndof, cudaMemcpyDeviceToHost, c->stream));
  if (v_host) IGAP_CUDA(cudaMemcpyAsync(vals, v_dev, sizeof(double) * c->nnz, cudaMemcpyDeviceToHost, c->stream));
  if (rr_host || v_host || (U && !is_device_ptr(U))) IGAP_CUDA(cudaStreamSynchronize(c->stream));
  return IGAPGPU_OK;
}

int igapgpu_residual(igapgpu_t c, const double *U, double *RR)
{
  NvtxRange range("igapgpu_residual");
  return assemble_common(c, U, RR, nullptr, true, false);
}
int igapgpu_tangent(igapgpu_t c, const double *U, double *vals)
{
  NvtxRange range("igapgpu_tangent");
  return assemble_common(c, U, nullptr, vals, false, true);
}
int igapgpu_assemble(igapgpu_t c, const double *U, double *RR, double *vals)
{
  NvtxRange range("igapgpu_assemble");
  return assemble_common(c, U, RR, vals, true, true);
}

int igapgpu_matmult(igapgpu_t c, const double *x, double *y)
{
  NvtxRange range("igapgpu_matmult");
  if (!c || !x || !y) return IGAPGPU_ERR_ARG;
  if (!c->matrix_valid) {
    set_error("matmult before the tangent was assembled into the context matrix");
    return IGAPGPU_ERR_STATE;
  }
  const double *xd;
  int r = stage_in(c, x, c->ndof, c->d_stage_a, &xd);
  if (r) return r;
  const bool yh = !is_device_ptr(y);
  double *yd = yh ? c->d_stage_b : y;
  r = spmv(c, c->d_vals, xd, yd);
  if (r) return r;
  if (yh) {
    IGAP_CUDA(cudaMemcpyAsync(y, yd, sizeof(double) * c->ndof, cudaMemcpyDeviceToHost, c->stream));
    IGAP_CUDA(cudaStreamSynchronize(c->stream));
  }
  return IGAPGPU_OK;
}

int igapgpu_set_neumann(igapgpu_t c, const double *table)
{
  if (!c || !table) return IGAPGPU_ERR_ARG;
  if (c->batch) return batch_set_neumann(c, table);
  for (int i = 0; i < 36; i++) c->bc.neumann[i] = table[i];
  return c->porder == 3 ? launch_neumann_p3(c, c->nfac) : launch_neumann(c, c->nfac);
}

int igapgpu_set_precision(igapgpu_t c, int mode)
{
  if (!c) return IGAPGPU_ERR_ARG;
  if (mode != IGAPGPU_PREC_FP64 && mode != IGAPGPU_PREC_SPLIT && mode != IGAPGPU_PREC_OZAKI) {
    set_error("unknown precision mode %d", mode);
    return IGAPGPU_ERR_ARG;
  }
  if (mode != IGAPGPU_PREC_FP64 && c->porder != P) {
    set_error("degree %d assembles in FP64 only (the tensor-core tangents are quadratic)", c->porder);
    return IGAPGPU_ERR_ARG;
  }
  if (mode == IGAPGPU_PREC_OZAKI && c->batch) {
    set_error("IGAPGPU_PREC_OZAKI is for single lattices; a batch takes FP64 or split precision");
    return IGAPGPU_ERR_ARG;
  }
  c->prec = mode;
  int rc = IGAPGPU_OK;
  if (mode == IGAPGPU_PREC_SPLIT) rc = c->batch ? batch_prepare_split(c) : ensure_gram_operands(c);
  if (mode == IGAPGPU_PREC_OZAKI) rc = ensure_ozaki_operands(c);
  if (rc) return rc;
  // the residual of both tensor-core modes in double-FP32 arithmetic
  return mode == IGAPGPU_PREC_FP64 ? IGAPGPU_OK : ensure_res_pairs(c);
}

int igapgpu_set_stream(igapgpu_t c, void *s)
{
  if (!c) return IGAPGPU_ERR_ARG;
  c->stream = s ? (cudaStream_t)s : c->own_stream;
  return IGAPGPU_OK;
}

int igapgpu_profile(igapgpu_t c, int enable)
{
  if (!c) return IGAPGPU_ERR_ARG;
  if (enable) {
    IGAP_CUDA(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < 3; k++) {
      for (auto &p : c->prof_ev[k]) {
        cudaEventDestroy(p.first);
        cudaEventDestroy(p.second);
      }
      c->prof_ev[k].clear();
      c->prof_launches[k] = c->prof_elements[k] = 0;
    }
  }
  c->prof = enable != 0;
  return IGAPGPU_OK;
}

int igapgpu_profile_read_kind(igapgpu_t c, int kind, double *elem_ms, int64_t *launches,
                              int64_t *elements)
{
  if (!c || kind < -1 || kind > 2) return IGAPGPU_ERR_ARG;
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  double ms = 0.0;
  int64_t nl = 0, ne = 0;
  for (int k = 0; k < 3; k++) {
    if (kind >= 0 && k != kind) continue;
    for (auto &p : c->prof_ev[k]) {
      float t = 0.f;
      IGAP_CUDA(cudaEventElapsedTime(&t, p.first, p.second));
      ms += t;
    }
    nl += c->prof_launches[k];
    ne += c->prof_elements[k];
  }
  if (elem_ms) *elem_ms = ms;
  if (launches) *launches = nl;
  if (elements) *elements = ne;
  return IGAPGPU_OK;
}

int igapgpu_profile_read(igapgpu_t c, double *elem_ms, int64_t *launches, int64_t *elements)
{
  return igapgpu_profile_read_kind(c, -1, elem_ms, launches, elements);
}

int igapgpu_synchronize(igapgpu_t c)
{
  if (!c) return IGAPGPU_ERR_ARG;
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  return IGAPGPU_OK;
}

}  // extern "C"
