// Cubic C1 B-spline / NURBS elements (degree 3: 64 basis functions, 192
// DOFs per element) in FP64: the element loop of Residual_iga / Tangent_iga
// (src/assmcore_iga.c:16-502, 507-858) for a degree the reference's own
// eval_Bspline does not take (it exits for p != 2, src/meshcore_iga.c:293);
// the same operations generalised to any degree: Cox-de Boor tables with the
// knot-span MTOL shift, the tensor-product basis, the quotient rule, the
// geometry and its inverse, physical first and second derivatives, the
// interpolated state, the law at every point (the same device laws), the
// residual projection and the tangent contraction, scattered into the CSR
// pattern of the degree-3 stencil (7 x 7 x 7 control points per row).
// Elements are launched colour by colour with 4 colours per direction
// (elements ex, ex + 4 share no control point), so the scatter needs no
// atomics.  The pattern, the Neumann load and the Dirichlet columns follow
// the degree too.  Everything here is templated on the degree PD.
#include <cuda_runtime.h>
#include <stdlib.h>

#include "common.cuh"
#include "element.cuh"
#include "laws.cuh"

namespace igap {

#define MTOL3 1.e-15  // knot-span denominator shift of src/meshcore_iga.c:10

namespace {

// One 1-D table entry of degree PD at x (local knots kv[0..2PD+1], every
// knot-span denominator shifted by mt): N[0..PD], N', N'', x, span length.
template <int PD>
__device__ inline void basis_1d_t(const double *kv, double x, double mt, double *o)
{
  constexpr int P1d = PD + 1;
  double lev[PD + 1][2 * PD + 1], dlev[PD + 1][2 * PD + 1];
  for (int i = 0; i < 2 * PD + 1; i++) { lev[0][i] = 0.0; dlev[0][i] = 0.0; }
  lev[0][PD] = 1.0;
  for (int q = 1; q <= PD; q++)
    for (int i = 0; i < 2 * PD + 1 - q; i++) {
      const double dl = kv[i + q] - kv[i] + mt, dr = kv[i + q + 1] - kv[i + 1] + mt;
      const double a = (dl != 0.0) ? (x - kv[i]) / dl * lev[q - 1][i] : 0.0;
      const double b = (dr != 0.0) ? (kv[i + q + 1] - x) / dr * lev[q - 1][i + 1] : 0.0;
      lev[q][i] = a + b;
      const double da = (dl != 0.0) ? (double)q / dl * lev[q - 1][i] : 0.0;
      const double db = (dr != 0.0) ? (double)q / dr * lev[q - 1][i + 1] : 0.0;
      dlev[q][i] = da - db;
    }
  for (int i = 0; i <= PD; i++) {
    o[i] = lev[PD][i];
    o[P1d + i] = dlev[PD][i];
    const double dl = kv[i + PD] - kv[i] + mt, dr = kv[i + PD + 1] - kv[i + 1] + mt;
    const double a = (dl != 0.0) ? (double)PD / dl * dlev[PD - 1][i] : 0.0;
    const double b = (dr != 0.0) ? (double)PD / dr * dlev[PD - 1][i + 1] : 0.0;
    o[2 * P1d + i] = a - b;
  }
  o[3 * P1d] = x;
  o[3 * P1d + 1] = kv[PD + 1] - kv[PD];
}

template <int PD>
__device__ __forceinline__ int64_t stencil_pos_t(int ix, int iy, int iz, int jx, int jy, int jz, const int nb[3])
{
  const int lox = max(ix - PD, 0), loy = max(iy - PD, 0), loz = max(iz - PD, 0);
  const int cy = min(iy + PD, nb[1] - 1) - loy + 1;
  const int cz = min(iz + PD, nb[2] - 1) - loz + 1;
  return ((int64_t)(jx - lox) * cy + (jy - loy)) * cz + (jz - loz);
}
}  // namespace

template <int PD>
__global__ void basis_table_p_kernel(const double *knots, int nelem, const double *xq01, int nq, double *tab,
                                     int with_mtol)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nelem * nq) return;
  const int e = t / nq, iq = t % nq;
  const double *kv = knots + e;
  const double x0 = kv[PD], x1 = kv[PD + 1], c = xq01[iq];
  basis_1d_t<PD>(kv, (-c + 1.0) * x0 + c * x1, with_mtol ? MTOL3 : 0.0, tab + (size_t)t * Deg<PD>::TAB);
}

template <int PD>
__global__ void pattern_cols_p_kernel(const int64_t *rowptr, int32_t *cols, int64_t ndof, int nb0, int nb1, int nb2)
{
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= ndof) return;
  const int nb[3] = {nb0, nb1, nb2};
  int ix, iy, iz;
  cp_coords(r / 3, nb, ix, iy, iz);
  int64_t s = rowptr[r];
  for (int jx = max(ix - PD, 0); jx <= min(ix + PD, nb0 - 1); jx++)
    for (int jy = max(iy - PD, 0); jy <= min(iy + PD, nb1 - 1); jy++)
      for (int jz = max(iz - PD, 0); jz <= min(iz + PD, nb2 - 1); jz++) {
        const int64_t cp = ((int64_t)jx * nb1 + jy) * nb2 + jz;
        for (int e = 0; e < 3; e++) cols[s++] = (int32_t)(3 * cp + e);
      }
}

// Face integrals of the traction table (src/assmcore_iga.c:264-405), one
// thread per face control point, as neumann_kernel for the quadratic basis.
template <int PD>
__global__ void neumann_p_kernel(int face, const int *bc_type, const double *neumann, const double *tabn0,
                                 const double *tabn1, const double *wq, int nq, int ne_a, int ne_b, int nb_a, int nb_b,
                                 int64_t st_a, int64_t st_b, int64_t st_n, int lay0, int lay1, double nfac0,
                                 double nfac1, double *F)
{
  constexpr int TABp = Deg<PD>::TAB, P1d = PD + 1;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nb_a * nb_b) return;
  const int ia = t / nb_b, ib = t % nb_b;
  for (int order = 0; order < 2; order++)
    for (int d = 0; d < 3; d++) {
      const int key = 6 * face + 3 * order + d;
      if (bc_type[key] != 1) continue;
      const double tr = neumann[key];
      double v0 = 0.0, v1 = 0.0;
      for (int ea = max(0, ia - PD); ea <= min(ne_a - 1, ia); ea++)
        for (int eb = max(0, ib - PD); eb <= min(ne_b - 1, ib); eb++) {
          double s0 = 0.0, s1 = 0.0;
          for (int qa = 0; qa < nq; qa++)
            for (int qb = 0; qb < nq; qb++) {
              const double *ta = tabn0 + ((size_t)ea * nq + qa) * TABp;
              const double *tb = tabn1 + ((size_t)eb * nq + qb) * TABp;
              const double Nab = ta[ia - ea] * tb[ib - eb];
              const double wt = wq[qa] * wq[qb] * ta[3 * P1d + 1] * tb[3 * P1d + 1];
              if (order == 0) {
                s0 -= wt * Nab * tr;
              } else {
                s0 -= wt * (Nab * nfac0) * tr;
                s1 -= wt * (Nab * nfac1) * tr;
              }
            }
          v0 += s0;
          v1 += s1;
        }
      const int64_t base = st_a * ia + st_b * ib;
      F[3 * (base + st_n * lay0) + d] += v0;
      if (order == 1) F[3 * (base + st_n * lay1) + d] += v1;
    }
}

// MatZeroRowsColumns(diag = 1) for the degree-PD stencil.
template <int PD>
__global__ void dirichlet_matrix_p_kernel(const int64_t *rows, int64_t n, const int64_t *rowptr, const int32_t *cols,
                                          int nb0, int nb1, int nb2, double *vals)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int nb[3] = {nb0, nb1, nb2};
  const int64_t r = rows[t];
  int ix, iy, iz;
  cp_coords(r / 3, nb, ix, iy, iz);
  const int dr = (int)(r % 3);
  for (int64_t s = rowptr[r]; s < rowptr[r + 1]; s++) {
    const int32_t c = cols[s];
    vals[s] = (c == r) ? 1.0 : 0.0;
    if (c == r) continue;
    int jx, jy, jz;
    cp_coords(c / 3, nb, jx, jy, jz);
    vals[rowptr[c] + 3 * stencil_pos_t<PD>(jx, jy, jz, ix, iy, iz, nb) + dr] = 0.0;
  }
}

// --------------------------------------------------------- element kernel
template <int PD>
struct CubicCfg {
  static constexpr int NBp = Deg<PD>::NB, NEp = Deg<PD>::NE, TABp = Deg<PD>::TAB;
  static constexpr int NT = 512;
  static constexpr int NPAIRp = NBp * (NBp + 1) / 2;
  static constexpr int PPT = (NPAIRp + NT - 1) / NT;  // pairs per thread
};

template <int PD>
struct CubicSmem {
  static constexpr int NBp = Deg<PD>::NB, NEp = Deg<PD>::NE;
  double XV[3 * NBp];
  double wV[NBp];
  double U[3 * NEp];            // [nhist][NBp][3]
  double R[PW][NBp * NDD];      // physical basis of the chunk's points
  double W[PW][NDD];
  double Xg[PW][3 * NDD];
  double u[PW][90];
  double wt[PW];
  double rr[PW][30];
  double Dw[PW][900];
  double M[27 * NEp];           // B1 of one point: [(d, k = 1..9)][(c, e)]
};

// Geometry of point q of element (ex,ey,ez) by one warp (the lanes stride
// over the basis functions): physical R[NBp*10] and the quadrature weight
// w_q |span| detG (src/assmcore_iga.c:150-208).
template <int PD>
__device__ double cubic_geometry(CubicSmem<PD> &S, int w, const DevMesh &m, int ex, int ey, int ez, int q, int lane)
{
  constexpr int P1d = PD + 1, NBp = Deg<PD>::NB, TABp = Deg<PD>::TAB;
  const int nq = m.nquad;
  const int qx = q / (nq * nq), qy = (q / nq) % nq, qz = q % nq;
  const double *tx = m.tab[0] + ((size_t)ex * nq + qx) * TABp;
  const double *ty = m.tab[1] + ((size_t)ey * nq + qy) * TABp;
  const double *tz = m.tab[2] + ((size_t)ez * nq + qz) * TABp;
  double *R = S.R[w];
  for (int b = lane; b < NBp; b += 32) {
    const int i = b / (P1d * P1d), j = (b / P1d) % P1d, l = b % P1d;
    const double nx = tx[i], dx = tx[P1d + i], ddx = tx[2 * P1d + i];
    const double ny = ty[j], dy = ty[P1d + j], ddy = ty[2 * P1d + j];
    const double nz = tz[l], dz = tz[P1d + l], ddz = tz[2 * P1d + l];
    double *o = R + NDD * b;
    o[0] = nx * ny * nz;
    o[1] = dx * ny * nz;
    o[2] = nx * dy * nz;
    o[3] = nx * ny * dz;
    o[4] = ddx * ny * nz;
    o[5] = dx * dy * nz;
    o[6] = dx * ny * dz;
    o[7] = nx * ddy * nz;
    o[8] = nx * dy * dz;
    o[9] = nx * ny * ddz;
  }
  __syncwarp();
  if (lane < NDD) {
    double s = 0.0;
    for (int b = 0; b < NBp; b++) s += S.wV[b] * R[NDD * b + lane];
    S.W[w][lane] = s;
  }
  __syncwarp();
  const double *Wv = S.W[w];
  for (int b = lane; b < NBp; b += 32) {  // quotient rule
    double *r = R + NDD * b;
    const double wb = S.wV[b];
    for (int k = 0; k < NDD; k++) r[k] = r[k] * wb / Wv[0];
    for (int k = 1; k < NDD; k++) r[k] -= r[0] * Wv[k] / Wv[0];
    int a = 4;
    for (int i = 1; i < 4; i++)
      for (int j = i; j < 4; j++) { r[a] -= (r[j] * Wv[i] + r[i] * Wv[j]) / Wv[0]; a++; }
  }
  __syncwarp();
  if (lane < 30) {  // geometry X and its derivatives
    const int d = lane / NDD, k = lane % NDD;
    double s = 0.0;
    for (int b = 0; b < NBp; b++) s += S.XV[3 * b + d] * R[NDD * b + k];
    S.Xg[w][lane] = s;
  }
  __syncwarp();
  const double *Xg = S.Xg[w];
  double G[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) G[3 * i + j] = Xg[NDD * i + 1 + j];
  const double detG = G[0] * (G[4] * G[8] - G[5] * G[7]) - G[1] * (G[3] * G[8] - G[5] * G[6]) +
                      G[2] * (G[3] * G[7] - G[4] * G[6]);
  double Gi[9];
  {
    const double c0 = G[4] * G[8] - G[5] * G[7], c1 = G[2] * G[7] - G[1] * G[8], c2 = G[1] * G[5] - G[2] * G[4];
    const double c3 = G[5] * G[6] - G[3] * G[8], c4 = G[0] * G[8] - G[2] * G[6], c5 = G[2] * G[3] - G[0] * G[5];
    const double c6 = G[3] * G[7] - G[4] * G[6], c7 = G[1] * G[6] - G[0] * G[7], c8 = G[0] * G[4] - G[1] * G[3];
    const double id = 1.0 / (G[0] * c0 + G[1] * c3 + G[2] * c6);
    Gi[0] = c0 * id; Gi[1] = c1 * id; Gi[2] = c2 * id;
    Gi[3] = c3 * id; Gi[4] = c4 * id; Gi[5] = c5 * id;
    Gi[6] = c6 * id; Gi[7] = c7 * id; Gi[8] = c8 * id;
  }
  for (int b = lane; b < NBp; b += 32) {  // physical first and second derivatives
    double *r = R + NDD * b;
    double n[NDD];
    for (int k = 0; k < NDD; k++) n[k] = r[k];
    for (int i = 0; i < 3; i++) {
      double s = 0.0;
      for (int j = 0; j < 3; j++) s += n[1 + j] * Gi[3 * j + i];
      r[1 + i] = s;
    }
    for (int k = 4; k < NDD; k++)
      for (int i = 0; i < 3; i++) n[k] -= r[1 + i] * Xg[NDD * i + k];
    const double Hs[3][3] = {{n[4], n[5], n[6]}, {n[5], n[7], n[8]}, {n[6], n[8], n[9]}};
    int a = 4;
    for (int i = 0; i < 3; i++)
      for (int j = i; j < 3; j++) {
        double s = 0.0;
        for (int mm = 0; mm < 3; mm++) {
          double t = 0.0;
          for (int l = 0; l < 3; l++) t += Hs[mm][l] * Gi[3 * l + j];
          s += Gi[3 * mm + i] * t;
        }
        r[a++] = s;
      }
  }
  __syncwarp();
  return m.wq[qx] * m.wq[qy] * m.wq[qz] * tx[3 * P1d + 1] * ty[3 * P1d + 1] * tz[3 * P1d + 1] * detG;
}

// One CTA per element of one colour (elements ex = cx + 4 i, ...).
template <int PD, int LAWK, bool RES, bool TAN>
__global__ void __launch_bounds__(512, 1)
    cubic_element_kernel(DevMesh m, DevLaw L, int cx, int cy, int cz, int ncy, int ncz,
                         const double *__restrict__ Uhist, double *__restrict__ RR, double *__restrict__ vals)
{
  using Cfg = CubicCfg<PD>;
  constexpr int P1d = PD + 1, NBp = Cfg::NBp, NEp = Cfg::NEp, NT = Cfg::NT, NPAIRp = Cfg::NPAIRp, PPT = Cfg::PPT;
  extern __shared__ __align__(16) unsigned char cubic_smem_raw[];
  CubicSmem<PD> &S = *reinterpret_cast<CubicSmem<PD> *>(cubic_smem_raw);
  LawSmem<LAWK> &LS = *reinterpret_cast<LawSmem<LAWK> *>(cubic_smem_raw + sizeof(CubicSmem<PD>));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int bi = blockIdx.x;
  const int ez = cz + P1d * (bi % ncz), ey = cy + P1d * ((bi / ncz) % ncy), ex = cx + P1d * (bi / (ncz * ncy));
  const int nb1 = m.nbasis[1], nb2 = m.nbasis[2];
  const int nh = L.nhist;
  for (int t = tid; t < NBp; t += NT) {
    const int i = t / (P1d * P1d), j = (t / P1d) % P1d, l = t % P1d;
    const int64_t cp = ((int64_t)(ex + i) * nb1 + (ey + j)) * nb2 + (ez + l);
    S.wV[t] = m.w[cp];
    for (int d = 0; d < 3; d++) S.XV[3 * t + d] = m.X[3 * cp + d];
    for (int h = 0; h < nh; h++)
      for (int d = 0; d < 3; d++) S.U[h * NEp + 3 * t + d] = Uhist[(int64_t)h * m.ndof + 3 * cp + d];
  }
  __syncthreads();
  double acc[PPT][9];
#pragma unroll
  for (int p = 0; p < PPT; p++)
#pragma unroll
    for (int i = 0; i < 9; i++) acc[p][i] = 0.0;
  double racc = 0.0;
  // this thread's basis pairs (b <= c, row-major over the upper triangle)
  int pb[PPT], pcc[PPT];
#pragma unroll
  for (int p = 0; p < PPT; p++) {
    int b = 0, rem = tid + p * NT;
    if (rem >= NPAIRp) rem = 0;
    while (rem >= NBp - b) { rem -= NBp - b; b++; }
    pb[p] = b;
    pcc[p] = b + rem;
  }
  const int nchunk = (m.npts + PW - 1) / PW;
  const double *Dconst = L.Dconst;
  for (int ch = 0; ch < nchunk; ch++) {
    if (warp < PW) {
      const int w = warp, q = ch * PW + w;
      if (q >= m.npts) {  // padding point: no contribution
        for (int i = lane; i < NBp * NDD; i += 32) S.R[w][i] = 0.0;
        for (int i = lane; i < 30; i += 32) S.rr[w][i] = 0.0;
        if (TAN)
          for (int i = lane; i < 900; i += 32) S.Dw[w][i] = 0.0;
        __syncwarp();
      } else {
        const double wt = cubic_geometry<PD>(S, w, m, ex, ey, ez, q, lane);
        // interpolated state of every level (src/assmcore_iga.c:209-229)
        if (lane < 30) {
          const int d = lane / NDD, k = lane % NDD;
          for (int h = 0; h < nh; h++) {
            double s = 0.0;
            for (int b = 0; b < NBp; b++) s += S.R[w][NDD * b + k] * S.U[h * NEp + 3 * b + d];
            S.u[w][30 * h + lane] = s;
          }
        }
        __syncwarp();
        if constexpr (LAWK == 0) {  // constant tangent of the linear law
          if (RES && lane < 30) {
            double s = 0.0;
            for (int j = 0; j < 30; j++) s += Dconst[30 * lane + j] * S.u[w][j];
            S.rr[w][lane] = wt * s;
          }
          if (TAN)
            for (int i = lane; i < 900; i += 32) S.Dw[w][i] = wt * Dconst[i];
          __syncwarp();
        } else if constexpr (LAWK == 1) {
          gradelast_warp<1, RES, TAN, double>(S.u[w], L.par, false, wt, S.rr[w], S.Dw[w], LS.s[w], lane);
        } else {
          gradelast_warp<4, RES, TAN, double>(S.u[w], L.par, true, wt, S.rr[w], S.Dw[w], LS.s[w], lane);
        }
      }
    }
    __syncthreads();
    if (RES && tid < NEp) {  // projection: val[3b+d] += sum_k R[b,k] rr[10d+k]
      const int b = tid / 3, d = tid % 3;
      for (int w = 0; w < PW; w++) {
        double s = 0.0;
        for (int k = 0; k < NDD; k++) s += S.R[w][NDD * b + k] * S.rr[w][NDD * d + k];
        racc += s;
      }
    }
    if constexpr (TAN) {
      for (int w = 0; w < PW; w++) {
        const double *R = S.R[w], *Dw = S.Dw[w];
        // B1: M[(d,k-1),(c,e)] = sum_{l=1..9} Dw[(d,k),(e,l)] R[c,l]
        for (int t = tid; t < 27 * NEp; t += NT) {
          const int row = t / NEp, col = t % NEp;
          const int d = row / 9, k = row % 9 + 1, c = col / 3, e = col % 3;
          const double *drow = Dw + 30 * (10 * d + k) + 10 * e;
          const double *rc = R + NDD * c;
          double s = 0.0;
#pragma unroll
          for (int l = 1; l < NDD; l++) s = fma(drow[l], rc[l], s);
          S.M[t] = s;
        }
        __syncthreads();
        // B2: K[(b,d),(c,e)] += sum_k R[b,k] M[(d,k),(c,e)] + the value (mass) term
#pragma unroll
        for (int p = 0; p < PPT; p++) {
          const int pid = tid + p * NT;
          if (pid < NPAIRp) {
            const int b = pb[p], c = pcc[p];
            const double *rb = R + NDD * b;
            const double r0 = rb[0] * R[NDD * c];
#pragma unroll
            for (int d = 0; d < 3; d++)
#pragma unroll
              for (int e = 0; e < 3; e++) {
                const double *mc = S.M + (9 * d) * NEp + 3 * c + e;
                double s = acc[p][3 * d + e];
#pragma unroll
                for (int k = 0; k < 9; k++) s = fma(rb[k + 1], mc[NEp * k], s);
                if (d == e) s = fma(Dw[30 * (10 * d) + 10 * d], r0, s);
                acc[p][3 * d + e] = s;
              }
          }
        }
        __syncthreads();
      }
    }
    __syncthreads();  // the next chunk's points overwrite R, rr, Dw
  }
  // scatter (no two elements of a colour share a control point)
  const int nbv[3] = {m.nbasis[0], nb1, nb2};
  if (RES && tid < NEp) {
    const int b = tid / 3, d = tid % 3;
    const int i = b / (P1d * P1d), j = (b / P1d) % P1d, l = b % P1d;
    const int64_t cp = ((int64_t)(ex + i) * nb1 + (ey + j)) * nb2 + (ez + l);
    RR[3 * cp + d] += racc;
  }
  if constexpr (TAN) {
#pragma unroll
    for (int p = 0; p < PPT; p++) {
      const int pid = tid + p * NT;
      if (pid >= NPAIRp) continue;
      const int b = pb[p], c = pcc[p];
      const int bx = ex + b / (P1d * P1d), by = ey + (b / P1d) % P1d, bz = ez + b % P1d;
      const int cxp = ex + c / (P1d * P1d), cyp = ey + (c / P1d) % P1d, czp = ez + c % P1d;
      const int64_t cpb = ((int64_t)bx * nb1 + by) * nb2 + bz, cpc = ((int64_t)cxp * nb1 + cyp) * nb2 + czp;
      const int64_t pbc = stencil_pos_t<PD>(bx, by, bz, cxp, cyp, czp, nbv);
      const int64_t pcb = stencil_pos_t<PD>(cxp, cyp, czp, bx, by, bz, nbv);
      for (int d = 0; d < 3; d++)
        for (int e = 0; e < 3; e++) {
          vals[m.rowptr[3 * cpb + d] + 3 * pbc + e] += acc[p][3 * d + e];
          if (c != b) vals[m.rowptr[3 * cpc + e] + 3 * pcb + d] += acc[p][3 * d + e];
        }
    }
  }
}

// ---------------------------------------------------------------- launches
int launch_basis_tables_p3(Context *c)
{
  for (int d = 0; d < 3; d++) {
    const int n = c->nelem[d] * c->nquad;
    basis_table_p_kernel<3><<<(n + 127) / 128, 128, 0, c->stream>>>(c->d_knots[d], c->nelem[d], c->d_xq, c->nquad,
                                                                     c->d_tab[d], 1);
    basis_table_p_kernel<3><<<(n + 127) / 128, 128, 0, c->stream>>>(c->d_knots[d], c->nelem[d], c->d_xq, c->nquad,
                                                                     c->d_tabn[d], 0);
    count_launch(2);
    IGAP_CHECK_LAUNCH();
  }
  return IGAPGPU_OK;
}

int launch_pattern_cols_p3(Context *c)
{
  const int64_t n = c->ndof;
  pattern_cols_p_kernel<3><<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(c->d_rowptr, c->d_cols, n,
                                                                               c->nbasis[0], c->nbasis[1],
                                                                               c->nbasis[2]);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

int launch_neumann_p3(Context *c, const double nfac[NFACE][2])
{
  if (!c->d_bct) {
    IGAP_CUDA(cudaMalloc(&c->d_bct, 36 * sizeof(int)));
    IGAP_CUDA(cudaMalloc(&c->d_neu, 36 * sizeof(double)));
  }
  IGAP_CUDA(cudaMemcpyAsync(c->d_bct, c->bc.bc_type, 36 * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  IGAP_CUDA(cudaMemcpyAsync(c->d_neu, c->bc.neumann, 36 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  IGAP_CUDA(cudaMemsetAsync(c->d_Fneu, 0, sizeof(double) * c->ndof, c->stream));
  const int64_t sx = (int64_t)c->nbasis[1] * c->nbasis[2], sy = c->nbasis[2], sz = 1;
  for (int face = 0; face < NFACE; face++) {
    int da, db, dn;
    int64_t sa, sb, sn;
    if (face / 2 == 0) { da = 1; db = 2; dn = 0; sa = sy; sb = sz; sn = sx; }
    else if (face / 2 == 1) { da = 0; db = 2; dn = 1; sa = sx; sb = sz; sn = sy; }
    else { da = 0; db = 1; dn = 2; sa = sx; sb = sy; sn = sz; }
    const int lay0 = (face % 2 == 0) ? 0 : c->nbasis[dn] - 1;
    const int lay1 = (face % 2 == 0) ? 1 : c->nbasis[dn] - 2;
    const int n = c->nbasis[da] * c->nbasis[db];
    neumann_p_kernel<3><<<(n + 127) / 128, 128, 0, c->stream>>>(
        face, c->d_bct, c->d_neu, c->d_tabn[da], c->d_tabn[db], c->d_wq, c->nquad, c->nelem[da], c->nelem[db],
        c->nbasis[da], c->nbasis[db], sa, sb, sn, lay0, lay1, nfac[face][0], nfac[face][1], c->d_Fneu);
    count_launch();
    IGAP_CHECK_LAUNCH();
  }
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  return IGAPGPU_OK;
}

int launch_dirichlet_matrix_p3(Context *c, double *vals)
{
  if (c->n_dir == 0) return IGAPGPU_OK;
  dirichlet_matrix_p_kernel<3><<<(unsigned)((c->n_dir + 127) / 128), 128, 0, c->stream>>>(
      c->d_dir_rows, c->n_dir, c->d_rowptr, c->d_cols, c->nbasis[0], c->nbasis[1], c->nbasis[2], vals);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

template <int LAWK, bool RES, bool TAN>
static int run_cubic_colours(Context *c, double *RR, double *vals)
{
  constexpr int PD = 3, P1d = PD + 1;
  const DevMesh m = c->devmesh();
  const DevLaw L = c->devlaw();
  const size_t smem = sizeof(CubicSmem<PD>) + sizeof(LawSmem<LAWK>);
  auto kern = cubic_element_kernel<PD, LAWK, RES, TAN>;
  static bool attr_set = false;
  if (!attr_set) {
    IGAP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  for (int cx = 0; cx < P1d; cx++)
    for (int cy = 0; cy < P1d; cy++)
      for (int cz = 0; cz < P1d; cz++) {
        const int ncx = (c->nelem[0] - cx + PD) / P1d, ncy = (c->nelem[1] - cy + PD) / P1d,
                  ncz = (c->nelem[2] - cz + PD) / P1d;
        const int nblk = ncx * ncy * ncz;
        if (nblk <= 0) continue;
        kern<<<nblk, CubicCfg<PD>::NT, smem, c->stream>>>(m, L, cx, cy, cz, ncy, ncz, c->d_Uhist, RR, vals);
        count_launch();
        IGAP_CHECK_LAUNCH();
      }
  return IGAPGPU_OK;
}

// The assembly of launch_assembly for degree 3 (FP64): Neumann load, colour
// launches, Dirichlet rows and columns.
int launch_assembly_p3(Context *c, bool do_res, bool do_tan, double *RR, double *vals)
{
  if (do_res)
    IGAP_CUDA(cudaMemcpyAsync(RR, c->d_Fneu, sizeof(double) * c->ndof, cudaMemcpyDeviceToDevice, c->stream));
  if (do_tan) IGAP_CUDA(cudaMemsetAsync(vals, 0, sizeof(double) * c->nnz, c->stream));
  int rc = IGAPGPU_OK;
#define IGAP_P3(LK)                                                   \
  rc = (do_res && do_tan) ? run_cubic_colours<LK, true, true>(c, RR, vals)   \
       : do_res           ? run_cubic_colours<LK, true, false>(c, RR, vals)  \
                          : run_cubic_colours<LK, false, true>(c, RR, vals);
  if (do_res || do_tan) {
    if (c->law == IGAPGPU_LAW_LINGRAD) { IGAP_P3(0) }
    else if (c->law == IGAPGPU_LAW_GRADELAST) { IGAP_P3(1) }
    else if (c->law == IGAPGPU_LAW_GRADELASTTIME) { IGAP_P3(2) }
    else {
      set_error("unknown law %d", c->law);
      return IGAPGPU_ERR_LAW;
    }
  }
#undef IGAP_P3
  if (rc) return rc;
  if (do_res && (rc = launch_dirichlet_residual(c, RR))) return rc;
  if (do_tan && (rc = launch_dirichlet_matrix_p3(c, vals))) return rc;
  return IGAPGPU_OK;
}

}  // namespace igap
