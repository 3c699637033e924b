// Integral of the law's densities over the body (iga_intdensity,
// src/postcore_iga.c:13-377): HH[i] = sum over elements and Gauss points of
// w_q |span| detG h_i(u_q), minus the traction term over the Neumann faces.
//
// Densities per law (the layout of the reference's density callbacks,
// include/physimpl.h:9-10):
//   gradelast (13): h0 the stored energy psi of the Green-Lagrange strain E
//     and its gradient; h1..h6 = 2 dpsi/dE_ab for ab = 00, 01, 02, 11, 12, 22;
//     h7..h9 indicators of the three deviatoric sectors of (e1, e2); h10..h12
//     the same sectors restricted to psi < -1/2.
//   gradelasttime (2): h0 = psi at the midpoint (u_n + u_{n-1})/2 plus the
//     kinetic energy rho/2 |(u_n - u_{n-1})/dt|^2; h1 = 1 (volume).
//   linear strain-gradient law (2): h0 = psi, h1 = 1.
// The boundary densities are the traction's work u . t on h0 (level 0, or the
// mean of levels 1 and 2 for the transient law), i.e. minus the Neumann load
// vector dotted with that state: the face integrals are the residual's.
//
// One CTA per element (a warp per point, lane 0 evaluates the density),
// per-element partial sums, then a fixed-order reduction: deterministic.
//
// Also here: the field sampling of iga_plotfield (src/mgl/plotcore_iga.c:
// 16-282) without its MathGL rendering.  The law's field callback
// (include/physimpl.h:8) is evaluated on a lattice of nppe samples per element
// and direction plus the far faces; the lattice, the sample coordinates (a
// 1e-15 shift into the span, plotcore_iga.c:166-168) and the basis with the
// knot-span MTOL are the plot loop's, the values go to a headless buffer.
// Fields per law:
//   gradelast (33, phys/gradelast.c:1105-1156): u[0..29] (value, gradient,
//     Hessian of the three components), e1, e2 (deviatoric strain
//     coordinates), and the sector code of the normalised Landau polynomial
//     (0 outside its well, 1, 2, 3 for e1 > 0, e1 < 0, e2 < 0 inside).
//   gradelasttime (6, phys/gradelasttime.c:9242-9297): the displacement
//     of the midpoint of levels 1 and 2, its e1, e2 and sector code.
//   linear strain-gradient law (33): u[0..29], tr eps, |dev eps|, psi.
#include <cuda_runtime.h>
#include <math.h>

#include "common.cuh"
#include "element.cuh"

namespace igap {

namespace {
constexpr int MAXD = 16;
constexpr int MAXF = 33;  // fields per sample point (gradelast and the linear law)

// psi, dpsi/dE and the sector quantities of the finite-strain gradient law at
// a state u (30 entries: value, gradient, Hessian of the three components).
struct GeDensity {
  double psi, S[6], e1, e2;
};

__device__ GeDensity gradelast_energy(const double *u, const double *par)
{
  double F[3][3], dF[3][3][3];
  for (int k = 0; k < 3; k++)
    for (int a = 0; a < 3; a++) {
      F[k][a] = (k == a ? 1.0 : 0.0) + u[10 * k + 1 + a];
      for (int m = 0; m < 3; m++) dF[k][a][m] = u[10 * k + 4 + sym6(a, m)];  // d_m F_ka
    }
  // E_ab and d_m E_ab, ab in (00, 01, 02, 11, 12, 22)
  const int PA[6] = {0, 0, 0, 1, 1, 2}, PB[6] = {0, 1, 2, 1, 2, 2};
  double E[6], dE[6][3];
  for (int s = 0; s < 6; s++) {
    const int a = PA[s], b = PB[s];
    double v = 0.0;
    for (int k = 0; k < 3; k++) v += F[k][a] * F[k][b];
    E[s] = 0.5 * (v - (a == b ? 1.0 : 0.0));
    for (int m = 0; m < 3; m++) {
      double g = 0.0;
      for (int k = 0; k < 3; k++) g += dF[k][a][m] * F[k][b] + F[k][a] * dF[k][b][m];
      dE[s][m] = 0.5 * g;
    }
  }
  const double r2 = sqrt(2.0), r3 = sqrt(3.0), r6 = sqrt(6.0);
  const double ev = (E[0] + E[3] + E[5]) / r3, e1 = (E[0] - E[3]) / r2, e2 = (E[0] + E[3] - 2.0 * E[5]) / r6;
  double g2 = 0.0;
  for (int m = 0; m < 3; m++) {
    const double d1 = (dE[0][m] - dE[3][m]) / r2, d2 = (dE[0][m] + dE[3][m] - 2.0 * dE[5][m]) / r6;
    g2 += d1 * d1 + d2 * d2;
  }
  double A, B, C;
  landau(par, A, B, C);
  const double cv = par[2], cs = par[3], l2 = par[4] * par[4];
  const double rho = e1 * e1 + e2 * e2;
  GeDensity o;
  o.psi = cv * ev * ev + cs * (E[1] * E[1] + E[2] * E[2] + E[4] * E[4]) + A * rho + B * e2 * (e2 * e2 - 3.0 * e1 * e1) +
          C * rho * rho + l2 * g2;
  const double Pv = 2.0 * cv * ev, P1 = 2.0 * e1 * (A - 3.0 * B * e2 + 2.0 * C * rho),
               P2 = 2.0 * A * e2 + 3.0 * B * (e2 * e2 - e1 * e1) + 4.0 * C * e2 * rho;
  o.S[0] = 2.0 * (Pv / r3 + P1 / r2 + P2 / r6);
  o.S[1] = 4.0 * cs * E[1];
  o.S[2] = 4.0 * cs * E[2];
  o.S[3] = 2.0 * (Pv / r3 - P1 / r2 + P2 / r6);
  o.S[4] = 4.0 * cs * E[4];
  o.S[5] = 2.0 * (Pv / r3 - 2.0 * P2 / r6);
  o.e1 = e1;
  o.e2 = e2;
  return o;
}

template <int LAWK>
__device__ void point_density(const double *u, const double *par, double *h)
{
  if constexpr (LAWK == 1) {
    const GeDensity g = gradelast_energy(u, par);
    h[0] = g.psi;
    for (int s = 0; s < 6; s++) h[1 + s] = g.S[s];
    const double e1 = g.e1, e2 = g.e2;
    h[7] = (e1 > 0 && e2 > -0.5 * e1) ? 1.0 : 0.0;
    h[8] = (e1 < 0 && e2 > 0.5 * e1) ? 1.0 : 0.0;
    h[9] = (e2 < 0.5 * e1 && e2 < -0.5 * e1) ? 1.0 : 0.0;
    const bool low = g.psi < -0.5;
    h[10] = (low && e1 > 0 && e2 > 0) ? 1.0 : 0.0;
    h[11] = (low && e1 < 0 && e2 > 0) ? 1.0 : 0.0;
    h[12] = (low && e2 < 0) ? 1.0 : 0.0;
  } else if constexpr (LAWK == 2) {
    double mid[30];
    for (int i = 0; i < 30; i++) mid[i] = 0.5 * (u[30 + i] + u[60 + i]);
    const GeDensity g = gradelast_energy(mid, par);
    const double rho_m = par[5], dt = par[7];
    double kin = 0.0;
    for (int d = 0; d < 3; d++) {
      const double v = u[30 + 10 * d] - u[60 + 10 * d];
      kin += v * v;
    }
    h[0] = g.psi + rho_m * kin / (2.0 * dt * dt);
    h[1] = 1.0;
  } else {
    const double lam = par[0], mu = par[1], ell = par[2];
    double eps[3][3], kap[3][3][3];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        eps[i][j] = 0.5 * (u[10 * i + 1 + j] + u[10 * j + 1 + i]);
        for (int m = 0; m < 3; m++) kap[i][j][m] = 0.5 * (u[10 * i + 4 + sym6(j, m)] + u[10 * j + 4 + sym6(i, m)]);
      }
    double tr = eps[0][0] + eps[1][1] + eps[2][2], ee = 0.0, kk = 0.0, tk = 0.0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        ee += eps[i][j] * eps[i][j];
        for (int m = 0; m < 3; m++) kk += kap[i][j][m] * kap[i][j][m];
      }
    for (int m = 0; m < 3; m++) {
      const double t = kap[0][0][m] + kap[1][1][m] + kap[2][2][m];
      tk += t * t;
    }
    h[0] = 0.5 * lam * tr * tr + mu * ee + ell * ell * (0.5 * lam * tk + mu * kk);
    h[1] = 1.0;
  }
}

struct DensSmem {
  ElemData E;
  PointScratch Pt[PW];
  double R[PW][NB * NDD];
  double acc[PW][MAXD];
};

template <int LAWK>
__global__ void __launch_bounds__(PW * 32) density_kernel(DevMesh m, DevLaw L, const double *__restrict__ Uhist,
                                                          double *__restrict__ partial, int nd)
{
  __shared__ DensSmem S;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t e = blockIdx.x;
  const int ez = (int)(e % m.nelem[2]), ey = (int)((e / m.nelem[2]) % m.nelem[1]),
            ex = (int)(e / ((int64_t)m.nelem[1] * m.nelem[2]));
  load_element(S.E, m, L.nhist, Uhist, ex, ey, ez, tid, PW * 32);
  __syncthreads();
  double my[MAXD];
  for (int i = 0; i < MAXD; i++) my[i] = 0.0;
  double *R = S.R[warp];
  PointScratch &P = S.Pt[warp];
  const int nchunk = (m.npts + PW - 1) / PW;
  for (int ch = 0; ch < nchunk; ch++) {
    const int q = ch * PW + warp;
    if (q < m.npts) {  // uniform across the warp
      double wt;
      if (m.geo) {
        const double *g = m.geo + (e * m.npts + q) * GEO_STRIDE;
        for (int i = lane; i < NB * NDD; i += 32) R[i] = __ldg(g + i);
        wt = __ldg(g + NB * NDD);
        __syncwarp();
      } else {
        wt = point_geometry(S.E, P, m, ex, ey, ez, q, lane, R);
      }
      if (lane < 30) {  // state of every history level, src/postcore_iga.c:230-245
        const int d = lane / NDD, k = lane % NDD;
        for (int h = 0; h < L.nhist; h++) {
          double s = 0.0;
          for (int b = 0; b < NB; b++) s += R[NDD * b + k] * S.E.U[h * NE + 3 * b + d];
          P.u[30 * h + lane] = s;
        }
      }
      __syncwarp();
      if (lane == 0) {
        double hh[MAXD];
        point_density<LAWK>(P.u, L.par, hh);
        for (int i = 0; i < nd; i++) my[i] += wt * hh[i];
      }
      __syncwarp();
    }
  }
  if (lane == 0)
    for (int i = 0; i < nd; i++) S.acc[warp][i] = my[i];
  __syncthreads();
  if (tid < nd) {
    double s = 0.0;
    for (int w = 0; w < PW; w++) s += S.acc[w][tid];
    partial[e * nd + tid] = s;
  }
}

// out[i] = sum_e partial[e][i] (block i), out[nd] = sum_k Fneu[k] ub[k]
// (block nd) with ub the level-0 state or the mean of levels 1 and 2.
__global__ void __launch_bounds__(1024) density_reduce_kernel(const double *__restrict__ partial, int64_t nelem,
                                                              int nd, const double *__restrict__ Fneu,
                                                              const double *__restrict__ Uhist, int64_t ndof,
                                                              int transient, double *__restrict__ out)
{
  __shared__ double red[32];
  const int i = blockIdx.x, tid = threadIdx.x;
  double s = 0.0;
  if (i < nd) {
    for (int64_t e = tid; e < nelem; e += 1024) s += partial[e * nd + i];
  } else {
    for (int64_t k = tid; k < ndof; k += 1024) {
      const double ub = transient ? 0.5 * (Uhist[ndof + k] + Uhist[2 * ndof + k]) : Uhist[k];
      s = fma(Fneu[k], ub, s);
    }
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((tid & 31) == 0) red[tid >> 5] = s;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int w = 0; w < 32; w++) t += red[w];
    out[i] = t;
  }
}

// ------------------------------------------------------------ field sampling
// Sector code of the deviatoric strain coordinates (e1, e2): with r = par[0],
// c = par[1], rho = e1^2 + e2^2 and the normalised Landau polynomial
//   phi = (3/2 rho^2 + 2 r (1 - c) e2 (e2^2 - 3 e1^2) - 3 r^2 c rho) / (r^4 (1/2 + c)),
// inside the well (phi < -1/2) the code is 3 for e2 < 0, else 1 for e1 > 0,
// else 2 for e1 < 0; 0 everywhere else.
__device__ double sector_code(double e1, double e2, const double *par)
{
  const double r = par[0], cv = par[1];
  const double rho = e1 * e1 + e2 * e2;
  const double phi = (1.5 * rho * rho + 2.0 * r * (1.0 - cv) * e2 * (e2 * e2 - 3.0 * e1 * e1) - 3.0 * r * r * cv * rho) /
                     (r * r * r * r * (0.5 + cv));
  if (phi < -0.5) {
    if (e2 < 0.0) return 3.0;
    if (e1 > 0.0) return 1.0;
    if (e1 < 0.0) return 2.0;
  }
  return 0.0;
}

template <int LAWK>
__device__ void point_field(const double *u, const double *par, double *f)
{
  if constexpr (LAWK == 1) {
    for (int i = 0; i < 30; i++) f[i] = u[i];
    const GeDensity g = gradelast_energy(u, par);
    f[30] = g.e1;
    f[31] = g.e2;
    f[32] = sector_code(g.e1, g.e2, par);
  } else if constexpr (LAWK == 2) {
    double mid[30];
    for (int i = 0; i < 30; i++) mid[i] = 0.5 * (u[30 + i] + u[60 + i]);
    for (int d = 0; d < 3; d++) f[d] = mid[NDD * d];
    const GeDensity g = gradelast_energy(mid, par);
    f[3] = g.e1;
    f[4] = g.e2;
    f[5] = sector_code(g.e1, g.e2, par);
  } else {
    for (int i = 0; i < 30; i++) f[i] = u[i];
    double eps[3][3];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) eps[i][j] = 0.5 * (u[NDD * i + 1 + j] + u[NDD * j + 1 + i]);
    const double tr = eps[0][0] + eps[1][1] + eps[2][2];
    double dd = 0.0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        const double v = eps[i][j] - (i == j ? tr / 3.0 : 0.0);
        dd += v * v;
      }
    double h[MAXD];
    point_density<0>(u, par, h);
    f[30] = tr;
    f[31] = sqrt(dd);
    f[32] = h[0];
  }
}

// 1-D tables at the sample coordinates: tab[(e * (nppe+1) + s) * TAB], sample
// s of element e at (k0 + 1e-15) + (k1 - k0) s / nppe - 2e-15 [s == nppe]
// (plotcore_iga.c:166-168, same order of operations), basis with the
// knot-span shift 1e-15 of eval_Bspline.
__global__ void sample_table_kernel(const double *__restrict__ knots, int nelem, int nppe, double *__restrict__ tab)
{
  const int ns = nppe + 1;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nelem * ns) return;
  const int e = t / ns, s = t % ns;
  const double *kv = knots + e;
  const double x0 = kv[P], x1 = kv[P + 1];
  const double x = __dsub_rn(__dadd_rn(__dadd_rn(x0, 1.e-15), __ddiv_rn(__dmul_rn(x1 - x0, (double)s), (double)nppe)),
                             s == nppe ? 2.e-15 : 0.0);
  basis_1d(kv, x, 1.e-15, tab + (size_t)t * TAB);
}

struct FieldSmem {
  ElemData E;
  PointScratch Pt[PW];
  double R[PW][NB * NDD];
};

// One CTA per element, a warp per sample point: the plot loop's geometry
// (point_geometry on the sample tables), the state of every level, the field.
// Lattice point (nppe ex + sx, nppe ey + sy, nppe ez + sz); the last element
// of a direction also takes the far face (s = nppe).
template <int LAWK>
__global__ void __launch_bounds__(PW * 32)
    field_kernel(DevMesh ms, DevLaw L, const double *__restrict__ Uhist, int nppe, int nf, double *__restrict__ out_f,
                 double *__restrict__ out_xq, double *__restrict__ out_X)
{
  __shared__ FieldSmem S;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t e = blockIdx.x;
  const int ez = (int)(e % ms.nelem[2]), ey = (int)((e / ms.nelem[2]) % ms.nelem[1]),
            ex = (int)(e / ((int64_t)ms.nelem[1] * ms.nelem[2]));
  load_element(S.E, ms, L.nhist, Uhist, ex, ey, ez, tid, PW * 32);
  __syncthreads();
  const int ns = nppe + 1;
  const int cx = nppe + (ex == ms.nelem[0] - 1 ? 1 : 0), cy = nppe + (ey == ms.nelem[1] - 1 ? 1 : 0),
            cz = nppe + (ez == ms.nelem[2] - 1 ? 1 : 0);
  const int64_t NY = (int64_t)nppe * ms.nelem[1] + 1, NZ = (int64_t)nppe * ms.nelem[2] + 1;
  double *R = S.R[warp];
  PointScratch &Pt = S.Pt[warp];
  for (int k = warp; k < cx * cy * cz; k += PW) {  // uniform across the warp
    const int sx = k / (cy * cz), sy = (k / cz) % cy, sz = k % cz;
    point_geometry(S.E, Pt, ms, ex, ey, ez, (sx * ns + sy) * ns + sz, lane, R);
    if (lane < 30) {  // plotcore_iga.c:228-248, every history level
      const int d = lane / NDD, kk = lane % NDD;
      for (int h = 0; h < L.nhist; h++) {
        double s = 0.0;
        for (int b = 0; b < NB; b++) s += R[NDD * b + kk] * S.E.U[h * NE + 3 * b + d];
        Pt.u[30 * h + lane] = s;
      }
    }
    __syncwarp();
    const int64_t g = (((int64_t)nppe * ex + sx) * NY + ((int64_t)nppe * ey + sy)) * NZ + ((int64_t)nppe * ez + sz);
    if (lane == 0 && out_f) {
      double f[MAXF];
      point_field<LAWK>(Pt.u, L.par, f);
      for (int i = 0; i < nf; i++) out_f[g * nf + i] = f[i];
    }
    if (lane < 3) {
      const int sd = lane == 0 ? sx : (lane == 1 ? sy : sz), ed = lane == 0 ? ex : (lane == 1 ? ey : ez);
      if (out_xq) out_xq[3 * g + lane] = ms.tab[lane][((size_t)ed * ns + sd) * TAB + 3 * P1];
      if (out_X) out_X[3 * g + lane] = Pt.Xg[NDD * lane];
    }
    __syncwarp();
  }
}

template <int LAWK>
static int run_field(Context *c, const DevMesh &ms, int nppe, int nf, double *f, double *xq, double *X)
{
  field_kernel<LAWK><<<(unsigned)c->nelem_total, PW * 32, 0, c->stream>>>(ms, c->devlaw(), c->d_Uhist, nppe, nf, f,
                                                                          xq, X);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

template <int LAWK>
static int run_density(Context *c, int nd)
{
  const DevMesh m = c->devmesh();
  const DevLaw L = c->devlaw();
  density_kernel<LAWK><<<(unsigned)c->nelem_total, PW * 32, 0, c->stream>>>(m, L, c->d_Uhist, c->d_dens, nd);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

}  // namespace

}  // namespace igap

using namespace igap;

extern "C" int igapgpu_density(igapgpu_t c, double *HH, int *ndensity)
{
  NvtxRange range("igapgpu_density");
  if (!c || !HH) {
    set_error("density: null argument");
    return IGAPGPU_ERR_ARG;
  }
  if (c->porder != P) {
    set_error("density: quadratic meshes only");
    return IGAPGPU_ERR_ARG;
  }
  if (c->batch) {
    set_error("density: not available on a batch context");
    return IGAPGPU_ERR_ARG;
  }
  const int nd = c->law == IGAPGPU_LAW_GRADELAST ? 13 : 2;
  if (!c->d_dens) {
    cudaError_t e = cudaMalloc(&c->d_dens, sizeof(double) * ((size_t)c->nelem_total * nd + MAXD + 1));
    if (e != cudaSuccess) {
      cudaGetLastError();
      c->d_dens = nullptr;
      set_error("density: cudaMalloc failed: %s", cudaGetErrorString(e));
      return IGAPGPU_ERR_NOMEM;
    }
  }
  int r = c->law == IGAPGPU_LAW_GRADELAST ? run_density<1>(c, nd)
          : c->law == IGAPGPU_LAW_GRADELASTTIME ? run_density<2>(c, nd)
                                                : run_density<0>(c, nd);
  if (r) return r;
  double *out = c->d_dens + (size_t)c->nelem_total * nd;
  density_reduce_kernel<<<nd + 1, 1024, 0, c->stream>>>(c->d_dens, c->nelem_total, nd, c->d_Fneu, c->d_Uhist,
                                                         c->ndof, c->law == IGAPGPU_LAW_GRADELASTTIME, out);
  count_launch();
  IGAP_CHECK_LAUNCH();
  double h[MAXD + 1];
  IGAP_CUDA(cudaMemcpyAsync(h, out, sizeof(double) * (nd + 1), cudaMemcpyDeviceToHost, c->stream));
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  // boundary: HH0 -= int u.t = -(-Fneu . ub), the residual's Neumann vector being -int N t
  h[0] += h[nd];
  for (int i = 0; i < nd; i++) HH[i] = h[i];
  if (ndensity) *ndensity = nd;
  return IGAPGPU_OK;
}

extern "C" int igapgpu_sample_field(igapgpu_t c, int nppe, double *field, double *xq, double *X, int *nfield,
                                    int64_t *npoints)
{
  NvtxRange range("igapgpu_sample_field");
  if (!c) {
    set_error("sample_field: null context");
    return IGAPGPU_ERR_ARG;
  }
  if (c->porder != P) {
    set_error("sample_field: quadratic meshes only");
    return IGAPGPU_ERR_ARG;
  }
  if (c->batch) {
    set_error("sample_field: not available on a batch context");
    return IGAPGPU_ERR_ARG;
  }
  if (nppe < 1 || nppe > 64) {
    set_error("sample_field: nppe = %d outside 1..64", nppe);
    return IGAPGPU_ERR_ARG;
  }
  const int nf = c->law == IGAPGPU_LAW_GRADELASTTIME ? 6 : MAXF;
  int64_t n[3];
  for (int d = 0; d < 3; d++) n[d] = (int64_t)nppe * c->nelem[d] + 1;
  const int64_t np = n[0] * n[1] * n[2];
  if (nfield) *nfield = nf;
  if (npoints) *npoints = np;
  if (!field && !xq && !X) return IGAPGPU_OK;  // size query
  const int ns = nppe + 1;
  // one device block: three sample tables, unit weights, staging of host outputs
  size_t off[7];
  size_t tot = 0;
  for (int d = 0; d < 3; d++) {
    off[d] = tot;
    tot += (size_t)c->nelem[d] * ns * TAB;
  }
  off[3] = tot;
  tot += (size_t)ns;
  double *outs[3] = {field, xq, X};
  const size_t len[3] = {(size_t)np * nf, (size_t)np * 3, (size_t)np * 3};
  bool host[3];
  for (int i = 0; i < 3; i++) {
    host[i] = outs[i] && !is_device_ptr(outs[i]);
    off[4 + i] = tot;
    if (host[i]) tot += len[i];
  }
  double *buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, sizeof(double) * tot);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("sample_field: cudaMalloc of %zu bytes failed: %s", sizeof(double) * tot, cudaGetErrorString(e));
    return IGAPGPU_ERR_NOMEM;
  }
  int rc = IGAPGPU_OK;
  do {
    std::vector<double> ones((size_t)ns, 1.0);
    e = cudaMemcpyAsync(buf + off[3], ones.data(), sizeof(double) * ns, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) break;
    DevMesh ms = c->devmesh();
    for (int d = 0; d < 3; d++) {
      const int cnt = c->nelem[d] * ns;
      sample_table_kernel<<<(cnt + 127) / 128, 128, 0, c->stream>>>(c->d_knots[d], c->nelem[d], nppe, buf + off[d]);
      count_launch();
      ms.tab[d] = buf + off[d];
    }
    ms.nquad = ns;
    ms.npts = ns * ns * ns;
    ms.wq = buf + off[3];
    ms.geo = nullptr;
    ms.geof = nullptr;
    double *dst[3];
    for (int i = 0; i < 3; i++) dst[i] = host[i] ? buf + off[4 + i] : outs[i];
    rc = c->law == IGAPGPU_LAW_GRADELAST       ? run_field<1>(c, ms, nppe, nf, dst[0], dst[1], dst[2])
         : c->law == IGAPGPU_LAW_GRADELASTTIME ? run_field<2>(c, ms, nppe, nf, dst[0], dst[1], dst[2])
                                               : run_field<0>(c, ms, nppe, nf, dst[0], dst[1], dst[2]);
    if (rc) break;
    for (int i = 0; i < 3 && e == cudaSuccess; i++)
      if (host[i])
        e = cudaMemcpyAsync(outs[i], dst[i], sizeof(double) * len[i], cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) break;
    e = cudaStreamSynchronize(c->stream);
  } while (0);
  if (e != cudaSuccess && rc == IGAPGPU_OK) {
    set_error("sample_field: CUDA error %s", cudaGetErrorString(e));
    rc = IGAPGPU_ERR_CUDA;
  }
  cudaStreamSynchronize(c->stream);
  cudaFree(buf);
  return rc;
}
