// Element assembly on the device: residual Vec and CSR tangent of IGAP4's
// volume integral (src/assmcore_iga.c:118-259 and :607-764), plus the set-up
// kernels (1-D basis tables, CSR columns, Neumann load, Dirichlet rows).
//
// Element kernel (FP64): one CTA per element, 384 threads.
//   Phase A  -- warp w of 8 evaluates quadrature point q = 8*chunk + w:
//               basis (lane = basis function), rational quotient rule,
//               geometry, physical derivatives, interpolated state, law.
//   Phase B1 -- M[(d,k),(c,e)] = sum_l Dw[(d,k),(e,l)] R[c,l]   (27 x 81)
//   Phase B2 -- thread (b<=c) accumulates K[(b,.),(c,.)] += R[b,k] M[.,(c,.)]
//   Scatter  -- colour-partitioned: elements of one colour
//               (ex mod 3, ey mod 3, ez mod 3) share no control point, so the
//               CSR slots and residual rows they add into are disjoint.
// Slots are computed arithmetically from the clipped structured stencil.
#include <cuda_runtime.h>
#include <stdlib.h>
#include "common.cuh"
#include "laws.cuh"
#include "element.cuh"
#include "law_thread.cuh"

namespace igap {

constexpr uint32_t BATCH_WAIT_LIMIT = 1u << 24;  // polls of a colour counter (~2 s)

#define MTOL 1.e-15  // knot-span denominator shift of src/meshcore_iga.c:10,303-307

constexpr int THREADS = 384;
constexpr int NPAIR = NB * (NB + 1) / 2;  // 378 (b <= c) pairs

__constant__ unsigned char c_pair_b[NPAIR];
__constant__ unsigned char c_pair_c[NPAIR];

// ---------------------------------------------------------------- tables
// tab[(e*nq + iq)*TAB + ...]: N[0..2], dN[3..5], ddN[6..8], xi[9], h[10]
__global__ void basis_table_kernel(const double *knots, int nelem, const double *xq01, int nq,
                                   double *tab, int with_mtol)
{
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nelem * nq) return;
  int e = t / nq, iq = t % nq;
  const double *kv = knots + e;  // local knots kv[0..2P+1]
  double x0 = kv[P], x1 = kv[P + 1];
  double c = xq01[iq];
  double x = (-c + 1.0) * x0 + c * x1;
  basis_1d(kv, x, with_mtol ? MTOL : 0.0, tab + (size_t)t * TAB);
}

// ------------------------------------------------------------ pattern
__global__ void pattern_cols_kernel(const int64_t *rowptr, int32_t *cols, int64_t ndof, int nb0,
                                    int nb1, int nb2, int64_t coff)
{
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= ndof) return;
  const int nb[3] = {nb0, nb1, nb2};
  int ix, iy, iz;
  cp_coords(r / 3, nb, ix, iy, iz);
  int64_t s = rowptr[r];
  for (int jx = max(ix - P, 0); jx <= min(ix + P, nb0 - 1); jx++)
    for (int jy = max(iy - P, 0); jy <= min(iy + P, nb1 - 1); jy++)
      for (int jz = max(iz - P, 0); jz <= min(iz + P, nb2 - 1); jz++) {
        int64_t cp = ((int64_t)jx * nb1 + jy) * nb2 + jz;
        for (int e = 0; e < 3; e++) cols[s++] = (int32_t)(coff + 3 * cp + e);
      }
}

// ---------------------------------------------------- constant linear law
__global__ void lingrad_dconst_kernel(const double *par, double *D)
{
  int j = threadIdx.x;
  if (j >= 30) return;
  double u[30], rr[30];
  for (int i = 0; i < 30; i++) u[i] = (i == j) ? 1.0 : 0.0;
  lingrad_residual_dev(u, par, rr);
  for (int i = 0; i < 30; i++) D[30 * i + j] = rr[i];
}

// ------------------------------------------------------ element kernel
struct ElemSmem {
  ElemData E;
  PointScratch Pt[PW];
  double R[PW][NB * NDD];    // physical basis of the chunk's points
  double rr[PW][30];         // weighted residual integrand
  double Dw[PW][900];        // weighted tangent integrand
  double M[27 * 81];
};

// Residual-only elements: no tangent integrand or stage buffers, 256 threads,
// so that two CTAs share an SM.
struct ResSmem {
  ElemData E;
  PointScratch Pt[PW];
  double R[PW][NB * NDD];
  double rr[PW][30];
};

template <bool TAN>
struct ElemCfg {  // tangent (and residual): 384 threads, one CTA per SM
  static constexpr int NT = THREADS;
  static constexpr int MINB = 1;
  using Smem = ElemSmem;
};
template <>
struct ElemCfg<false> {
  static constexpr int NT = 256;
  static constexpr int MINB = 2;
  using Smem = ResSmem;
};

template <bool TAN>
__device__ __forceinline__ double *dw_ptr(typename ElemCfg<TAN>::Smem &S, int w)
{
  if constexpr (TAN) return S.Dw[w];
  else return nullptr;
}

// One element: load, quadrature (phase A, B1, B2) and the scatter into RR /
// vals.  COH: the read-modify-write of RR / vals bypasses L1 (a batched
// launch orders colours inside one kernel, through L2).
template <int LAWK, bool RES, bool TAN, bool COH>
__device__ __forceinline__ void element_body(typename ElemCfg<TAN>::Smem &S, LawSmem<LAWK> &LS, const DevMesh &m,
                                             const DevLaw &L, int ex, int ey, int ez,
                                             const double *__restrict__ Uhist, double *__restrict__ RR,
                                             double *__restrict__ vals)
{
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nb1 = m.nbasis[1], nb2 = m.nbasis[2];
  const int nh = L.nhist;
  // element data: weights, control points, state of every history level
  constexpr int NT = ElemCfg<TAN>::NT;
  load_element(S.E, m, nh, Uhist, ex, ey, ez, tid, NT);
  __syncthreads();

  double acc[9];
#pragma unroll
  for (int i = 0; i < 9; i++) acc[i] = 0.0;
  double racc = 0.0;
  const int pb = tid < NPAIR ? c_pair_b[tid] : 0;
  const int pc = tid < NPAIR ? c_pair_c[tid] : 0;

  const int nchunk = (m.npts + PW - 1) / PW;
  // Linear isotropic strain-gradient law: its tangent block of a basis pair
  // (b,c) is, with per-point Gram sums G1[i][j] = sum_q w dN_b/dx_i dN_c/dx_j
  // and G2[d][e] = sum_q w sum_m d2N_b/dx_d dx_m d2N_c/dx_e dx_m,
  //   K[(b,d),(c,e)] = lam G1[d][e] + mu (delta_de tr G1 + G1[e][d])
  //                  + ell^2 (lam G2[d][e] + mu (delta_de tr G2 + G2[e][d])),
  // the same sum as R^T D R of the assembly loop with this law's constant D
  // (36 instead of 81 + 27 x 81 x 9 / 378 FMAs per pair and point).
  constexpr bool ISO = (LAWK == 0) && TAN;
  double g1[9], g2[9];
#pragma unroll
  for (int i = 0; i < 9; i++) g1[i] = g2[i] = 0.0;
  for (int ch = 0; ch < nchunk; ch++) {
    if (warp < PW)
      point_setup<LAWK, RES, TAN, double>(S.E, S.Pt[warp], LS, m, L, ex, ey, ez, warp, ch * PW + warp,
                                          lane, S.R[warp], S.rr[warp], dw_ptr<TAN>(S, warp), !ISO);
    __syncthreads();
    if (RES && tid < NE) {
      const int bb = tid / 3, d = tid % 3;
      constexpr int K0 = LAWK == 0 ? 1 : 0;  // the linear law's value slot of rr is zero
      for (int w = 0; w < PW; w++) {
        double s = 0.0;
        for (int k = K0; k < NDD; k++) s += S.R[w][NDD * bb + k] * S.rr[w][NDD * d + k];
        racc += s;
      }
    }
    if constexpr (ISO) {
      // weighted derivatives of every basis function, once per point (the
      // tangent-integrand buffer is free in this form)
      for (int t = tid; t < PW * NB * 9; t += NT) {
        const int w = t / (NB * 9), r = t % (NB * 9);
        S.Dw[w][r] = S.Pt[w].wt * S.R[w][NDD * (r / 9) + 1 + r % 9];
      }
      __syncthreads();
      if (tid < NPAIR) {
        for (int w = 0; w < PW; w++) {
          const double *sb = S.Dw[w] + 9 * pb, *rc = S.R[w] + NDD * pc;  // sb: weighted slots 1..9 of b
          double gb[3], gc[3], hb[3][3], hc[3][3];
#pragma unroll
          for (int i = 0; i < 3; i++) {
            gb[i] = sb[i];
            gc[i] = rc[1 + i];
          }
          // Hessian components (xx, xy, xz, yy, yz, zz) -> symmetric 3 x 3
          hb[0][0] = sb[3]; hb[0][1] = hb[1][0] = sb[4]; hb[0][2] = hb[2][0] = sb[5];
          hb[1][1] = sb[6]; hb[1][2] = hb[2][1] = sb[7]; hb[2][2] = sb[8];
          hc[0][0] = rc[4]; hc[0][1] = hc[1][0] = rc[5]; hc[0][2] = hc[2][0] = rc[6];
          hc[1][1] = rc[7]; hc[1][2] = hc[2][1] = rc[8]; hc[2][2] = rc[9];
#pragma unroll
          for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
              g1[3 * i + j] = fma(gb[i], gc[j], g1[3 * i + j]);
              double t = g2[3 * i + j];
#pragma unroll
              for (int mm = 0; mm < 3; mm++) t = fma(hb[i][mm], hc[j][mm], t);
              g2[3 * i + j] = t;
            }
        }
      }
      __syncthreads();
    } else if constexpr (TAN) {
      for (int w = 0; w < PW; w++) {
        const double *R = S.R[w];
        const double *Dw = S.Dw[w];
        {
          // B1: M[(d,k-1),(c,e)] = sum_{l=1..9} Dw[(d,k),(e,l)] R[c,l]
          for (int t = tid; t < 27 * 81; t += NT) {
            const int row = t / 81, col = t % 81;
            const int d = row / 9, k = row % 9 + 1, c = col / 3, e = col % 3;
            const double *drow = Dw + 30 * (10 * d + k) + 10 * e;
            const double *rc = R + NDD * c;
            double s = 0.0;
#pragma unroll
            for (int l = 1; l < NDD; l++) s = fma(drow[l], rc[l], s);
            S.M[t] = s;
          }
        }
        __syncthreads();
        // B2: K[(b,d),(c,e)] += sum_k R[b,k] M[(d,k),(c,e)] + value (mass) term
        if (tid < NPAIR) {
          const double *rb = R + NDD * pb;
          double rbk[9];
#pragma unroll
          for (int k = 0; k < 9; k++) rbk[k] = rb[k + 1];
          const double r0 = rb[0] * R[NDD * pc];
#pragma unroll
          for (int d = 0; d < 3; d++)
#pragma unroll
            for (int e = 0; e < 3; e++) {
              const double *mc = S.M + (9 * d) * 81 + 3 * pc + e;
              double s = acc[3 * d + e];
#pragma unroll
              for (int k = 0; k < 9; k++) s = fma(rbk[k], mc[81 * k], s);
              if (d == e) s = fma(Dw[30 * (10 * d) + 10 * d], r0, s);
              acc[3 * d + e] = s;
            }
        }
        __syncthreads();
      }
    } else {
      __syncthreads();
    }
  }
  if (ISO && tid < NPAIR) {
    const double lam = L.par[0], mu = L.par[1], l2 = L.par[2] * L.par[2];
    const double t1 = g1[0] + g1[4] + g1[8], t2 = g2[0] + g2[4] + g2[8];
#pragma unroll
    for (int d = 0; d < 3; d++)
#pragma unroll
      for (int e = 0; e < 3; e++) {
        double k1 = lam * g1[3 * d + e] + mu * g1[3 * e + d];
        double k2 = lam * g2[3 * d + e] + mu * g2[3 * e + d];
        if (d == e) {
          k1 += mu * t1;
          k2 += mu * t2;
        }
        acc[3 * d + e] = k1 + l2 * k2;
      }
  }
  // scatter (conflict-free within a colour)
  const int nbv[3] = {m.nbasis[0], nb1, nb2};
  if (RES && tid < NE) {
    const int bb = tid / 3, d = tid % 3;
    const int i = bb / 9, j = (bb / 3) % 3, l = bb % 3;
    const int64_t cp = ((int64_t)(ex + i) * nb1 + (ey + j)) * nb2 + (ez + l);
    double *dst = RR + m.dof_off + 3 * cp + d;
    *dst = (COH ? __ldcg(dst) : *dst) + racc;
  }
  if (TAN && tid < NPAIR) {
    const int bi = pb / 9, bj = (pb / 3) % 3, bl = pb % 3;
    const int ci = pc / 9, cj = (pc / 3) % 3, cl = pc % 3;
    const int rx = ex + bi, ry = ey + bj, rz = ez + bl;
    const int sx = ex + ci, sy = ey + cj, sz = ez + cl;
    const int64_t cpb = ((int64_t)rx * nb1 + ry) * nb2 + rz;
    const int64_t cpc = ((int64_t)sx * nb1 + sy) * nb2 + sz;
    const int64_t pos_bc = stencil_pos(rx, ry, rz, sx, sy, sz, nbv);
    const int64_t pos_cb = stencil_pos(sx, sy, sz, rx, ry, rz, nbv);
    for (int d = 0; d < 3; d++)
      for (int e = 0; e < 3; e++) {
        double *p1 = vals + __ldg(m.rowptr + 3 * cpb + d) + 3 * pos_bc + e;
        *p1 = (COH ? __ldcg(p1) : *p1) + acc[3 * d + e];
        if (pb != pc) {
          double *p2 = vals + __ldg(m.rowptr + 3 * cpc + e) + 3 * pos_cb + d;
          *p2 = (COH ? __ldcg(p2) : *p2) + acc[3 * d + e];
        }
      }
  }
}

template <int LAWK, bool RES, bool TAN>
__global__ void __launch_bounds__(ElemCfg<TAN>::NT, ElemCfg<TAN>::MINB)
    element_kernel(DevMesh m, DevLaw L, int cx, int cy, int cz, int ncy, int ncz,
                   const double *__restrict__ Uhist, double *__restrict__ RR,
                   double *__restrict__ vals)
{
  using Smem = typename ElemCfg<TAN>::Smem;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem &S = *reinterpret_cast<Smem *>(smem_raw);
  LawSmem<LAWK> &LS = *reinterpret_cast<LawSmem<LAWK> *>(smem_raw + sizeof(Smem));
  // element of this colour
  const int b = blockIdx.x;
  const int iz = b % ncz, iy = (b / ncz) % ncy, ix = b / (ncz * ncy);
  element_body<LAWK, RES, TAN, false>(S, LS, m, L, cx + 3 * ix, cy + 3 * iy, cz + 3 * iz, Uhist, RR, vals);
}

// ------------------------------------------------- batched (persistent)
// Publishes the CTA's finished element: the barrier before the call orders
// every thread's stores before this thread's release at GPU scope.
__device__ __forceinline__ void release_add(int *p, int v)
{
  asm volatile("fence.acq_rel.gpu;\n\tred.relaxed.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Waits (bounded) until *p >= target; acquire at GPU scope.
__device__ __forceinline__ bool wait_count_ge(const int *p, int target, uint32_t limit = BATCH_WAIT_LIMIT)
{
  for (uint32_t i = 0; i < limit; i++) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    if (v >= target) return true;
    __nanosleep(128);
  }
  return false;
}

// Self-test of the expiry path of the bounded waits: thread 0 of every CTA
// waits for a counter that nothing increments, with a short poll limit, and
// the CTA reports the outcome in the error-word convention of the batched
// kernels (3 = a wait expired).  No fault and no hang: the kernel returns.
__global__ void wait_selftest_kernel(const int *counter, int target, uint32_t limit, int *err)
{
  __shared__ int expired;
  if (threadIdx.x == 0) expired = wait_count_ge(counter, target, limit) ? 0 : 1;
  __syncthreads();
  if (threadIdx.x == 0 && expired) atomicExch(err, 3);
}

// Persistent CTAs take elements of every instance from one colour-major
// queue (a CTA reserves its next fetch while it works on the current one;
// items are reserved only by running CTAs, in queue order).  An element of colour k of instance i starts only after all its
// instance's elements of colours < k are finished (a per-instance count
// reaching the number of those elements); they sit earlier in the queue and
// were taken by running CTAs, so every wait ends.  Each CSR slot and residual
// row therefore receives its element contributions in colour order, exactly
// as with one launch per colour.
template <int LAWK, bool RES, bool TAN>
__global__ void __launch_bounds__(ElemCfg<TAN>::NT, ElemCfg<TAN>::MINB)
    element_batch_kernel(BatchArgs a, const double *__restrict__ Uhist, double *__restrict__ RR,
                         double *__restrict__ vals)
{
  using Smem = typename ElemCfg<TAN>::Smem;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem &S = *reinterpret_cast<Smem *>(smem_raw);
  LawSmem<LAWK> &LS = *reinterpret_cast<LawSmem<LAWK> *>(smem_raw + sizeof(Smem));
  __shared__ int64_t s_base;
  __shared__ int s_abort;
  const int tid = threadIdx.x;
  int cur = -1;
  DevMesh m;  // current instance, in registers
  DevLaw L;
  // the queue position of the following fetch is taken one fetch ahead, so
  // the atomic's round trip overlaps the current elements
  int64_t next = 0;
  if (tid == 0) {
    s_abort = 0;
    next = atomicAdd(a.head, a.grab);
  }
  for (;;) {
    __syncthreads();
    if (tid == 0) s_base = next;
    __syncthreads();
    const int64_t base = s_base;
    if (base >= a.nitems || s_abort) break;
    if (tid == 0) next = atomicAdd(a.head, a.grab);
    const int64_t end = base + a.grab < a.nitems ? base + a.grab : a.nitems;
    for (int64_t it = base; it < end; it++) {
      const BatchItem w = a.items[it];
      if (w.inst != cur) {
        m = a.meshes[w.inst];
        L = a.laws[w.inst];
        cur = w.inst;
      }
      if (tid == 0 && w.col > 0) {
        if (!wait_count_ge(a.done + w.inst, a.need[27 * w.inst + w.col])) {
          s_abort = 1;
          atomicExch(a.err, 3);
        }
      }
      __syncthreads();
      if (s_abort) break;
      element_body<LAWK, RES, TAN, true>(S, LS, m, L, w.ex, w.eyz >> 16, w.eyz & 0xffff, Uhist, RR, vals);
      __syncthreads();
      if (tid == 0) release_add(a.done + w.inst, 1);
    }
  }
}

// ------------------------------------------------------ geometry cache
// State-independent per-point geometry: physical basis R (value, gradient,
// Hessian of the 27 rational basis functions) and the quadrature weight.
__global__ void __launch_bounds__(256) geometry_cache_kernel(DevMesh m, double *geo)
{
  __shared__ ElemData E;
  __shared__ PointScratch Pt[8];
  __shared__ double R[8][NB * NDD];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t e = blockIdx.x;
  const int ez = (int)(e % m.nelem[2]), ey = (int)((e / m.nelem[2]) % m.nelem[1]),
            ex = (int)(e / ((int64_t)m.nelem[1] * m.nelem[2]));
  load_element(E, m, 0, nullptr, ex, ey, ez, tid, 256);
  __syncthreads();
  for (int q = warp; q < m.npts; q += 8) {
    const double wt = point_geometry(E, Pt[warp], m, ex, ey, ez, q, lane, R[warp]);
    double *g = geo + (e * m.npts + q) * GEO_STRIDE;
    for (int i = lane; i < NB * NDD; i += 32) g[i] = R[warp][i];
    if (lane == 0) {
      g[NB * NDD] = wt;
      g[NB * NDD + 1] = 0.0;
    }
    __syncwarp();
  }
}

__global__ void geometry_f32_kernel(const double *geo, float *geof, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    geof[i] = (float)geo[i];
}

int launch_geometry_cache_f32(Context *c)
{
  const int64_t n = c->nelem_total * (int64_t)c->nquad * c->nquad * c->nquad * GEO_STRIDE;
  geometry_f32_kernel<<<152 * 16, 256, 0, c->stream>>>(c->d_geo, c->d_geof, n);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

int launch_geometry_cache(Context *c)
{
  DevMesh m = c->devmesh();
  m.geo = nullptr;
  geometry_cache_kernel<<<(unsigned)c->nelem_total, 256, 0, c->stream>>>(m, c->d_geo);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

// ----------------------------------------------------------- Neumann
// One thread per face control point of one face; both orders and all dofs.
__global__ void neumann_kernel(int face, const int *bc_type, const double *neumann,
                               const double *tabn0, const double *tabn1, const double *wq, int nq,
                               int ne_a, int ne_b, int nb_a, int nb_b, int64_t st_a, int64_t st_b,
                               int64_t st_n, int lay0, int lay1, double nfac0, double nfac1,
                               double *F)
{
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nb_a * nb_b) return;
  const int ia = t / nb_b, ib = t % nb_b;
  for (int order = 0; order < 2; order++)
    for (int d = 0; d < 3; d++) {
      const int key = 6 * face + 3 * order + d;
      if (bc_type[key] != 1) continue;
      const double tr = neumann[key];
      double v0 = 0.0, v1 = 0.0;
      for (int ea = max(0, ia - P); ea <= min(ne_a - 1, ia); ea++)
        for (int eb = max(0, ib - P); eb <= min(ne_b - 1, ib); eb++) {
          double s0 = 0.0, s1 = 0.0;
          for (int qa = 0; qa < nq; qa++)
            for (int qb = 0; qb < nq; qb++) {
              const double *ta = tabn0 + ((size_t)ea * nq + qa) * TAB;
              const double *tb = tabn1 + ((size_t)eb * nq + qb) * TAB;
              const double Nab = ta[ia - ea] * tb[ib - eb];
              const double wt = wq[qa] * wq[qb] * ta[3 * P1 + 1] * tb[3 * P1 + 1];
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

// ---------------------------------------------------------- Dirichlet
__global__ void dirichlet_residual_kernel(const int64_t *rows, const double *g, int64_t n,
                                          const double *U, double *RR)
{
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int64_t r = rows[t];
  RR[r] = U[r] - g[t];
}

// MatZeroRowsColumns(diag = 1): row r and column r of every Dirichlet DOF.
__global__ void dirichlet_matrix_kernel(const int64_t *rows, int64_t n, const int64_t *rowptr,
                                        const int32_t *cols, int nb0, int nb1, int nb2,
                                        double *vals)
{
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
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
    const int64_t pos = stencil_pos(jx, jy, jz, ix, iy, iz, nb);
    vals[rowptr[c] + 3 * pos + dr] = 0.0;
  }
}

// MatZeroRowsColumns on the block-diagonal matrix of a batch: rows carry
// their instance (inst), whose lattice is nbs[3*inst..] and first DOF dof_off[inst].
__global__ void dirichlet_matrix_batch_kernel(const int64_t *rows, const int *inst, int64_t n,
                                              const int64_t *rowptr, const int32_t *cols, const int *nbs,
                                              const int64_t *dof_off, double *vals)
{
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = inst[t];
  const int nb[3] = {nbs[3 * i], nbs[3 * i + 1], nbs[3 * i + 2]};
  const int64_t off = dof_off[i];
  const int64_t r = rows[t], rl = r - off;
  int ix, iy, iz;
  cp_coords(rl / 3, nb, ix, iy, iz);
  const int dr = (int)(rl % 3);
  for (int64_t s = rowptr[r]; s < rowptr[r + 1]; s++) {
    const int32_t c = cols[s];
    vals[s] = (c == r) ? 1.0 : 0.0;
    if (c == r) continue;
    int jx, jy, jz;
    cp_coords((c - off) / 3, nb, jx, jy, jz);
    const int64_t pos = stencil_pos(jx, jy, jz, ix, iy, iz, nb);
    vals[rowptr[c] + 3 * pos + dr] = 0.0;
  }
}

int launch_dirichlet_matrix_batch(Context *c, const int *d_inst, const int *d_nbs, const int64_t *d_off,
                                  double *vals)
{
  if (c->n_dir == 0) return IGAPGPU_OK;
  dirichlet_matrix_batch_kernel<<<(unsigned)((c->n_dir + 127) / 128), 128, 0, c->stream>>>(
      c->d_dir_rows, d_inst, c->n_dir, c->d_rowptr, c->d_cols, d_nbs, d_off, vals);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

int launch_pattern_cols_at(Context *c, const int64_t *rowptr, int32_t *cols, int64_t coff)
{
  const int64_t n = c->ndof;
  pattern_cols_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(
      rowptr, cols, n, c->nbasis[0], c->nbasis[1], c->nbasis[2], coff);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

// ------------------------------------------------------------ launches
// ------------------------------------------------- law at every point
// One CTA per (element, chunk of 8 points), one warp per point: geometry,
// state and the law as in the element kernel's phase A; the weighted law
// outputs (rr, D) go to global memory.  The law of a point does not depend on
// the colouring, so all points run in one launch, where the colour launches
// would evaluate one colour's elements at a time.
struct LawPtSmem {
  ElemData E;
  PointScratch Pt[PW];
  double R[PW][NB * NDD];
  double rr[PW][30];
  double D[PW][900];
};

template <int LAWK, bool RES, bool TAN>
__global__ void __launch_bounds__(PW * 32, 1)
    law_points_kernel(DevMesh m, DevLaw L, const double *__restrict__ Uhist, double *__restrict__ preR,
                      double *__restrict__ preD)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  LawPtSmem &S = *reinterpret_cast<LawPtSmem *>(smem_raw);
  LawSmem<LAWK> &LS = *reinterpret_cast<LawSmem<LAWK> *>(smem_raw + sizeof(LawPtSmem));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nchunk = (m.npts + PW - 1) / PW;
  const int64_t e = blockIdx.x / nchunk;
  const int ch = (int)(blockIdx.x % nchunk);
  const int ez = (int)(e % m.nelem[2]), ey = (int)((e / m.nelem[2]) % m.nelem[1]),
            ex = (int)(e / ((int64_t)m.nelem[1] * m.nelem[2]));
  load_element(S.E, m, L.nhist, Uhist, ex, ey, ez, tid, PW * 32);
  __syncthreads();
  point_setup<LAWK, RES, TAN, double>(S.E, S.Pt[warp], LS, m, L, ex, ey, ez, warp, ch * PW + warp, lane,
                                      S.R[warp], S.rr[warp], S.D[warp]);
  __syncthreads();
  const int q0 = ch * PW;
  const int nv = m.npts - q0 < PW ? m.npts - q0 : PW;
  // point-minor layout: [element][entry][point]
  if (RES)
    for (int i = tid; i < nv * 30; i += PW * 32)
      preR[(e * 30 + i % 30) * m.npts + q0 + i / 30] = S.rr[i / 30][i % 30];
  if (TAN)
    for (int i = tid; i < nv * 900; i += PW * 32)
      preD[(e * 900 + i % 900) * m.npts + q0 + i / 900] = S.D[i / 900][i % 900];
}

// ------------------------------------- law at every point, a thread per point
// Needs the geometry cache.  Phase 1 (a warp per point, 32 points per warp):
// the point's physical basis comes from the cache, the lanes of the 30 slots
// interpolate every history level (src/assmcore_iga.c:209-229, same order as
// point_setup) and store the law's inputs column-wise in shared memory.
// Phase 2: each thread evaluates its point's law (gradelast_point) and writes
// the weighted outputs in the point-minor layout [element][entry][point], so
// that a warp's stores are contiguous.
constexpr int LT_NT = 128;
// T: the law's arithmetic.  The FP32 law keeps its inputs as floats (the
// same values its phase 2 used to convert them to), and a launch that copies
// its inputs (PRE) needs no basis or state: the smaller shared-memory
// footprints let more CTAs share an SM.
template <typename T, bool PRE = false>
struct LawThreadSmem {
  static constexpr bool F32 = sizeof(T) == 4;
  T sm[30 * LT_NT];
  T sd[30 * LT_NT];
  double wt[LT_NT];
  double R[LT_NT / 32][PRE ? 1 : GEO_STRIDE];
  double U[LT_NT / 32][F32 || PRE ? 1 : 3 * NE];
  float Uf[LT_NT / 32][F32 && !PRE ? 3 * NE : 1];  // the element's state in FP32 (float law)
};

// T: the law's arithmetic (double; float for the tangent of the split mode,
// whose contraction runs in TF32x3 on the tensor cores).  PRE: phase 1 copies
// the law's inputs from lin (pair interpolation, law_in_df_kernel) instead of
// interpolating them.
template <int LAWK, bool RES, bool TAN, typename T = double, bool PRE = false>
__global__ void __launch_bounds__(LT_NT)
    law_thread_kernel(DevMesh m, DevLaw L, const double *__restrict__ Uhist, double *__restrict__ preR,
                      double *__restrict__ preD, int64_t npt_total, const double *__restrict__ lin)
{
  constexpr bool TR = LAWK == 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  LawThreadSmem<T, PRE> &S = *reinterpret_cast<LawThreadSmem<T, PRE> *>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t p0 = (int64_t)blockIdx.x * LT_NT;
  const int nh = L.nhist;
  const int nb1 = m.nbasis[1], nb2 = m.nbasis[2];
  const double rho_m = L.par[5], damp = L.par[6], dt = L.par[7];
  int64_t cur_e = -1;
  for (int j = 0; j < 32; j++) {
    const int t = warp * 32 + j;
    const int64_t p = p0 + t;
    if (p >= npt_total) break;  // uniform over the warp
    if constexpr (PRE) {
      const double *src = lin + p * 64;
      if (lane < 30) {
        S.sm[lane * LT_NT + t] = lawpt::to_t<T>(__ldg(src + lane));
        if (TR) S.sd[lane * LT_NT + t] = lawpt::to_t<T>(__ldg(src + 30 + lane));
      }
      if (lane == 30) S.wt[t] = __ldg(src + 60);
    } else {
      const int64_t e = p / m.npts;
      if (e != cur_e) {
        __syncwarp();
        const int ez = (int)(e % m.nelem[2]), ey = (int)((e / m.nelem[2]) % m.nelem[1]),
                  ex = (int)(e / ((int64_t)m.nelem[1] * m.nelem[2]));
        for (int i = lane; i < nh * NE; i += 32) {
          const int h = i / NE, r = i % NE, b = r / 3, d = r % 3;
          const int64_t cp = ((int64_t)(ex + b / 9) * nb1 + (ey + (b / 3) % 3)) * nb2 + (ez + b % 3);
          const double u = __ldg(Uhist + (int64_t)h * m.ndof + m.dof_off + 3 * cp + d);
          if constexpr (sizeof(T) == 4) S.Uf[warp][i] = f64_to_pair(u).x;
          else S.U[warp][i] = u;
        }
        cur_e = e;
      }
      const double *g = m.geo + p * GEO_STRIDE;
      for (int i = lane; i < GEO_STRIDE; i += 32) S.R[warp][i] = __ldg(g + i);
      __syncwarp();
      if (lane < 30) {
        const int d = lane / NDD, k = lane % NDD;
        double s[3] = {0.0, 0.0, 0.0};
        if constexpr (sizeof(T) == 4) {  // FP32 interpolation (the basis split on the integer pipe)
          float sf[3] = {0.f, 0.f, 0.f};
#pragma unroll
          for (int b = 0; b < NB; b++) {
            const float r = f64_to_pair(S.R[warp][NDD * b + k]).x;
#pragma unroll
            for (int h = 0; h < 3; h++)
              if (h < nh) sf[h] = fmaf(r, S.Uf[warp][h * NE + 3 * b + d], sf[h]);
          }
#pragma unroll
          for (int h = 0; h < 3; h++) s[h] = f32_to_f64(sf[h]);
        } else {
          for (int h = 0; h < nh; h++) {
            double acc = 0.0;
#pragma unroll
            for (int b = 0; b < NB; b++) acc += S.R[warp][NDD * b + k] * S.U[warp][h * NE + 3 * b + d];
            s[h] = acc;
          }
        }
        if (!TR) {
          S.sm[lane * LT_NT + t] = lawpt::to_t<T>(s[0]);
        } else if (k == 0) {
          // the value slots' inertia and damping term enters the residual only
          // (the tangent's value rows are the constant mass): no FP64 divisions
          // in a tangent-only launch
          S.sm[lane * LT_NT + t] = RES ? lawpt::to_t<T>(damp * (s[0] - s[2]) / (2.0 * dt) +
                                                        rho_m * (s[0] + s[2] - 2.0 * s[1]) / (dt * dt))
                                       : T(0);
        } else {
          S.sm[lane * LT_NT + t] = lawpt::to_t<T>(0.5 * (s[1] + s[2]));
          S.sd[lane * LT_NT + t] = lawpt::to_t<T>(0.5 * (s[0] - s[2]));
        }
      }
      if (lane == 0) S.wt[t] = S.R[warp][NB * NDD];
      __syncwarp();
    }
  }
  __syncthreads();
  const int64_t p = p0 + tid;
  if (p < npt_total) {
    const int64_t e = p / m.npts;
    const int q = (int)(p % m.npts);
    // the float law writes its tangent outputs as floats into the same buffer
    T *outd = reinterpret_cast<T *>(preD) + e * 900 * m.npts + q;
    gradelast_point<TR ? 4 : 1, RES, TAN, T>(S.sm + tid, S.sd + tid, LT_NT, L.par, S.wt[tid],
                                             preR + e * 30 * m.npts + q, outd, m.npts);
  }
}

template <int LAWK, bool RES, bool TAN, typename T = double, bool PRE = false>
static int run_law_points(Context *c, const DevLaw &L)
{
  const DevMesh m = c->devmesh();
  if (m.geo) {
    const size_t smem = sizeof(LawThreadSmem<T, PRE>);
    auto kern = law_thread_kernel<LAWK, RES, TAN, T, PRE>;
    static bool attr_set = false;
    if (!attr_set) {
      IGAP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      attr_set = true;
    }
    const int64_t npt = c->nelem_total * m.npts;
    const int64_t nblk = (npt + LT_NT - 1) / LT_NT;
    kern<<<(unsigned)nblk, LT_NT, smem, c->stream>>>(m, L, c->d_Uhist, c->d_preR, c->d_preD, npt, c->d_lin);
    count_launch();
    IGAP_CHECK_LAUNCH();
    return IGAPGPU_OK;
  }
  const size_t smem = sizeof(LawPtSmem) + sizeof(LawSmem<LAWK>);
  auto kern = law_points_kernel<LAWK, RES, TAN>;
  static bool attr_set = false;
  if (!attr_set) {
    IGAP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  const int nchunk = (m.npts + PW - 1) / PW;
  const int64_t nblk = c->nelem_total * nchunk;
  kern<<<(unsigned)nblk, PW * 32, smem, c->stream>>>(m, L, c->d_Uhist, c->d_preR, c->d_preD);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

int launch_law_points(Context *c, bool do_res, bool do_tan, DevLaw &L)
{
  c->law_df = false;
  if (c->law == IGAPGPU_LAW_LINGRAD || (!do_res && !do_tan)) return IGAPGPU_OK;
  if (c->pre_state < 0) {
    // decided once, outside any capture: the buffers are allocated when they
    // take at most a quarter of the free memory; IGAPGPU_LAW_PRECOMPUTE=0 turns
    // the precomputation off
    c->pre_state = 0;
    const char *env = getenv("IGAPGPU_LAW_PRECOMPUTE");
    const size_t npt = (size_t)c->nelem_total * c->nquad * c->nquad * c->nquad;
    size_t freeb = 0, totb = 0;
    if (!c->capturing && !(env && env[0] == '0') && cudaMemGetInfo(&freeb, &totb) == cudaSuccess &&
        npt * 930 * sizeof(double) < freeb / 4) {
      if (cudaMalloc(&c->d_preR, npt * 30 * sizeof(double)) == cudaSuccess &&
          cudaMalloc(&c->d_preD, npt * 900 * sizeof(double)) == cudaSuccess) {
        c->pre_state = 1;
      } else {
        cudaGetLastError();
        if (c->d_preR) cudaFree(c->d_preR);
        c->d_preR = nullptr;
      }
    }
  }
  if (c->pre_state != 1) return IGAPGPU_OK;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (c->prof) {
    IGAP_CUDA(cudaEventCreate(&e0));
    IGAP_CUDA(cudaEventCreate(&e1));
    IGAP_CUDA(cudaEventRecord(e0, c->stream));
  }
  // split precision: the tangent's law outputs in FP32 arithmetic (they feed
  // the TF32x3 contraction); the residual's law stays FP64.  IGAPGPU_LAW_F32=0
  // keeps FP64 for both.
  const char *lf = getenv("IGAPGPU_LAW_F32");
  const bool tan32 = do_tan && c->prec == IGAPGPU_PREC_SPLIT && c->d_geo && !(lf && lf[0] == '0');
  // the tensor-core modes' residual (residual alone, or beside the FP32-law
  // tangent): the law's inputs from pair interpolation, the projection on
  // pairs afterwards (launch_assembly)
  c->law_df = do_res && c->prec != IGAPGPU_PREC_FP64 && c->rpc_state == 2 && (tan32 || !do_tan);
  int rc = IGAPGPU_OK;
  if (c->law_df) rc = launch_law_in_df(c);
  if (rc) return rc;
  if (c->law == IGAPGPU_LAW_GRADELAST) {
    if (c->law_df) {
      rc = run_law_points<1, true, false, double, true>(c, L);
      if (!rc && do_tan) rc = run_law_points<1, false, true, float>(c, L);
    } else if (tan32) {
      if (do_res) rc = run_law_points<1, true, false>(c, L);
      if (!rc) rc = run_law_points<1, false, true, float>(c, L);
    } else {
      rc = (do_res && do_tan) ? run_law_points<1, true, true>(c, L)
           : do_res           ? run_law_points<1, true, false>(c, L)
                              : run_law_points<1, false, true>(c, L);
    }
  } else {
    if (c->law_df) {
      rc = run_law_points<2, true, false, double, true>(c, L);
      if (!rc && do_tan) rc = run_law_points<2, false, true, float>(c, L);
    } else if (tan32) {
      if (do_res) rc = run_law_points<2, true, false>(c, L);
      if (!rc) rc = run_law_points<2, false, true, float>(c, L);
    } else {
      rc = (do_res && do_tan) ? run_law_points<2, true, true>(c, L)
           : do_res           ? run_law_points<2, true, false>(c, L)
                              : run_law_points<2, false, true>(c, L);
    }
  }
  if (rc) return rc;
  if (c->prof) {
    IGAP_CUDA(cudaEventRecord(e1, c->stream));
    c->prof_ev[2].emplace_back(e0, e1);
    c->prof_launches[2]++;
    c->prof_elements[2] += c->nelem_total;
  }
  L.preR = c->d_preR;
  L.preD = tan32 ? nullptr : c->d_preD;
  L.preDf = tan32 ? reinterpret_cast<const float *>(c->d_preD) : nullptr;
  return IGAPGPU_OK;
}

template <int LAWK, bool RES, bool TAN>
static int run_colours(Context *c, const DevLaw &L, double *RR, double *vals)
{
  const DevMesh m = c->devmesh();
  const size_t smem = sizeof(typename ElemCfg<TAN>::Smem) + sizeof(LawSmem<LAWK>);
  auto kern = element_kernel<LAWK, RES, TAN>;
  static bool attr_set = false;
  if (!attr_set) {
    IGAP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (c->prof) {
    IGAP_CUDA(cudaEventCreate(&e0));
    IGAP_CUDA(cudaEventCreate(&e1));
    IGAP_CUDA(cudaEventRecord(e0, c->stream));
  }
  for (int cx = 0; cx < 3; cx++)
    for (int cy = 0; cy < 3; cy++)
      for (int cz = 0; cz < 3; cz++) {
        const int ncx = (c->nelem[0] - cx + 2) / 3, ncy = (c->nelem[1] - cy + 2) / 3,
                  ncz = (c->nelem[2] - cz + 2) / 3;
        const int nblk = ncx * ncy * ncz;
        if (nblk <= 0) continue;
        kern<<<nblk, ElemCfg<TAN>::NT, smem, c->stream>>>(m, L, cx, cy, cz, ncy, ncz, c->d_Uhist, RR, vals);
        count_launch();
        IGAP_CHECK_LAUNCH();
        if (c->prof) {
          c->prof_launches[0]++;
          c->prof_elements[0] += nblk;
        }
      }
  if (c->prof) {
    IGAP_CUDA(cudaEventRecord(e1, c->stream));
    c->prof_ev[0].emplace_back(e0, e1);
  }
  return IGAPGPU_OK;
}

static bool pairs_ready = false;
static int init_pairs()
{
  if (pairs_ready) return IGAPGPU_OK;
  unsigned char hb[NPAIR], hc[NPAIR];
  int n = 0;
  for (int b = 0; b < NB; b++)
    for (int cc = b; cc < NB; cc++) { hb[n] = (unsigned char)b; hc[n] = (unsigned char)cc; n++; }
  IGAP_CUDA(cudaMemcpyToSymbol(c_pair_b, hb, sizeof(hb)));
  IGAP_CUDA(cudaMemcpyToSymbol(c_pair_c, hc, sizeof(hc)));
  pairs_ready = true;
  return IGAPGPU_OK;
}

template <int LAWK, bool RES, bool TAN>
static int run_batch(Context *c, const BatchArgs &a, int grid, const double *Uhist, double *RR, double *vals)
{
  const size_t smem = sizeof(typename ElemCfg<TAN>::Smem) + sizeof(LawSmem<LAWK>);
  auto kern = element_batch_kernel<LAWK, RES, TAN>;
  static bool attr_set = false;
  if (!attr_set) {
    IGAP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  kern<<<grid, ElemCfg<TAN>::NT, smem, c->stream>>>(a, Uhist, RR, vals);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

template <int LAWK, bool RES, bool TAN>
static int batch_occ(int *nb)
{
  const size_t smem = sizeof(typename ElemCfg<TAN>::Smem) + sizeof(LawSmem<LAWK>);
  auto kern = element_batch_kernel<LAWK, RES, TAN>;
  IGAP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  IGAP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(nb, kern, ElemCfg<TAN>::NT, smem));
  return IGAPGPU_OK;
}

#define IGAP_BATCH_DISPATCH(FN, ...)                                                       \
  switch (law) {                                                                         \
  case IGAPGPU_LAW_LINGRAD:                                                              \
    if (do_res && do_tan) return FN<0, true, true>(__VA_ARGS__);                         \
    if (do_res) return FN<0, true, false>(__VA_ARGS__);                                  \
    return FN<0, false, true>(__VA_ARGS__);                                              \
  case IGAPGPU_LAW_GRADELAST:                                                            \
    if (do_res && do_tan) return FN<1, true, true>(__VA_ARGS__);                         \
    if (do_res) return FN<1, true, false>(__VA_ARGS__);                                  \
    return FN<1, false, true>(__VA_ARGS__);                                              \
  case IGAPGPU_LAW_GRADELASTTIME:                                                        \
    if (do_res && do_tan) return FN<2, true, true>(__VA_ARGS__);                         \
    if (do_res) return FN<2, true, false>(__VA_ARGS__);                                  \
    return FN<2, false, true>(__VA_ARGS__);                                              \
  default:                                                                               \
    set_error("unknown law %d", law);                                                    \
    return IGAPGPU_ERR_LAW;                                                              \
  }

int launch_element_batch(Context *c, const BatchArgs &a, int law, bool do_res, bool do_tan, int grid,
                         const double *Uhist, double *RR, double *vals)
{
  int rc = init_pairs();
  if (rc) return rc;
  IGAP_BATCH_DISPATCH(run_batch, c, a, grid, Uhist, RR, vals)
}

int element_batch_occupancy(int law, bool do_res, bool do_tan, int *blocks_per_sm)
{
  IGAP_BATCH_DISPATCH(batch_occ, blocks_per_sm)
}
#undef IGAP_BATCH_DISPATCH

int launch_assembly(Context *c, bool do_res, bool do_tan, double *RR, double *vals)
{
  int rc = init_pairs();
  if (rc) return rc;
  if (c->batch) return launch_batch_assembly(c, do_res, do_tan, RR, vals);
  if (c->porder == 3) return launch_assembly_p3(c, do_res, do_tan, RR, vals);
  if (do_res) {
    IGAP_CUDA(cudaMemcpyAsync(RR, c->d_Fneu, sizeof(double) * c->ndof, cudaMemcpyDeviceToDevice,
                              c->stream));
  }
  if (do_tan) IGAP_CUDA(cudaMemsetAsync(vals, 0, sizeof(double) * c->nnz, c->stream));
#define IGAP_DISPATCH(LK)                                                   \
  if (do_res && do_tan) rc = run_colours<LK, true, true>(c, L, RR, vals);   \
  else if (do_res) rc = run_colours<LK, true, false>(c, L, RR, vals);       \
  else rc = run_colours<LK, false, true>(c, L, RR, vals);
  // split precision: the tangent goes to the tensor cores (TF32x3);
  // FP64-quality tensor-core precision: the linear law's tangent from BF16
  // slices when they were built, else the FP64 kernel; the residual of both
  // modes below
  const bool oz_tan = do_tan && c->prec == IGAPGPU_PREC_OZAKI && c->d_oz;
  const bool fp64_tan = do_tan && c->prec != IGAPGPU_PREC_SPLIT && !oz_tan;
  // nonlinear laws: every point's law outputs in one launch, so that the
  // colour launches do not evaluate the law colour after colour
  DevLaw L = c->devlaw();
  rc = launch_law_points(c, do_res, do_tan, L);
  if (rc) return rc;
  // the residual of the tensor-core modes: double-FP32 kernels when their
  // buffers were built (the linear law's pair cache; the reference's laws'
  // law-input buffer, with the law outputs of every point)
  const bool law_df = do_res && c->law_df && c->pre_state == 1;
  const bool df_res = do_res && c->prec != IGAPGPU_PREC_FP64 && (c->d_rpc || law_df);
  if (df_res) {
    rc = law_df ? launch_res_law_df(c, c->d_preR, RR) : launch_res_df(c, RR);
    if (rc) return rc;
  }
  const bool k_res = do_res && !df_res, k_tan = fp64_tan;
  if (k_res || k_tan) {
    const bool do_res_k = k_res, do_tan_k = k_tan;
    {
      const bool do_res = do_res_k, do_tan = do_tan_k;
      if (c->law == IGAPGPU_LAW_LINGRAD) { IGAP_DISPATCH(0) }
      else if (c->law == IGAPGPU_LAW_GRADELAST) { IGAP_DISPATCH(1) }
      else if (c->law == IGAPGPU_LAW_GRADELASTTIME) { IGAP_DISPATCH(2) }
      else {
        set_error("unknown law %d", c->law);
        return IGAPGPU_ERR_LAW;
      }
    }
  }
#undef IGAP_DISPATCH
  if (rc) return rc;
  if (do_tan && !fp64_tan) {
    IGAP_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
    rc = oz_tan ? launch_tc_ozaki(c, vals) : launch_tc_tangent(c, vals, L);
    if (rc) return rc;
    if (!c->capturing) {  // a graph replay checks the error word itself
      int herr = 0;
      IGAP_CUDA(cudaMemcpyAsync(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      IGAP_CUDA(cudaStreamSynchronize(c->stream));
      if (herr) {
        set_error("tensor-core tangent: a bounded mbarrier wait expired (code %d)", herr);
        return IGAPGPU_ERR_TIMEOUT;
      }
    }
  }
  if (do_res) {
    rc = launch_dirichlet_residual(c, RR);
    if (rc) return rc;
  }
  if (do_tan) {
    rc = launch_dirichlet_matrix(c, vals);
    if (rc) return rc;
  }
  return IGAPGPU_OK;
}

int launch_basis_tables(Context *c)
{
  for (int d = 0; d < 3; d++) {
    const int n = c->nelem[d] * c->nquad;
    basis_table_kernel<<<(n + 127) / 128, 128, 0, c->stream>>>(c->d_knots[d], c->nelem[d], c->d_xq,
                                                                c->nquad, c->d_tab[d], 1);
    basis_table_kernel<<<(n + 127) / 128, 128, 0, c->stream>>>(c->d_knots[d], c->nelem[d], c->d_xq,
                                                                c->nquad, c->d_tabn[d], 0);
    count_launch(2);
    IGAP_CHECK_LAUNCH();
  }
  return IGAPGPU_OK;
}

int launch_lingrad_dconst(Context *c)
{
  double *d_par = nullptr;
  IGAP_CUDA(cudaMalloc(&d_par, 9 * sizeof(double)));
  IGAP_CUDA(cudaMemcpyAsync(d_par, c->par, 9 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  lingrad_dconst_kernel<<<1, 32, 0, c->stream>>>(d_par, c->d_Dconst);
  count_launch();
  IGAP_CHECK_LAUNCH();
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  IGAP_CUDA(cudaFree(d_par));
  return IGAPGPU_OK;
}

int launch_pattern_cols(Context *c)
{
  const int64_t n = c->ndof;
  pattern_cols_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(
      c->d_rowptr, c->d_cols, n, c->nbasis[0], c->nbasis[1], c->nbasis[2], 0);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

int launch_neumann(Context *c, const double nfac[NFACE][2])
{
  if (!c->d_bct) {
    IGAP_CUDA(cudaMalloc(&c->d_bct, 36 * sizeof(int)));
    IGAP_CUDA(cudaMalloc(&c->d_neu, 36 * sizeof(double)));
  }
  int *d_bct = c->d_bct;
  double *d_neu = c->d_neu;
  IGAP_CUDA(cudaMemcpyAsync(d_bct, c->bc.bc_type, 36 * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  IGAP_CUDA(cudaMemcpyAsync(d_neu, c->bc.neumann, 36 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
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
    neumann_kernel<<<(n + 127) / 128, 128, 0, c->stream>>>(
        face, d_bct, d_neu, c->d_tabn[da], c->d_tabn[db], c->d_wq, c->nquad, c->nelem[da],
        c->nelem[db], c->nbasis[da], c->nbasis[db], sa, sb, sn, lay0, lay1, nfac[face][0],
        nfac[face][1], c->d_Fneu);
    count_launch();
    IGAP_CHECK_LAUNCH();
  }
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  return IGAPGPU_OK;
}

int launch_dirichlet_residual(Context *c, double *RR)
{
  if (c->n_dir == 0) return IGAPGPU_OK;
  dirichlet_residual_kernel<<<(unsigned)((c->n_dir + 255) / 256), 256, 0, c->stream>>>(
      c->d_dir_rows, c->d_dir_g, c->n_dir, c->d_Uhist, RR);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

__global__ void impose_dirichlet_kernel(const int64_t *rows, const double *g, int64_t n, double *U)
{
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) U[rows[t]] = g[t];
}

int launch_impose_dirichlet(Context *c, double *U)
{
  if (c->n_dir == 0) return IGAPGPU_OK;
  impose_dirichlet_kernel<<<(unsigned)((c->n_dir + 255) / 256), 256, 0, c->stream>>>(c->d_dir_rows, c->d_dir_g,
                                                                                     c->n_dir, U);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

int launch_dirichlet_matrix(Context *c, double *vals)
{
  if (c->porder == 3) return launch_dirichlet_matrix_p3(c, vals);
  if (c->n_dir == 0) return IGAPGPU_OK;
  dirichlet_matrix_kernel<<<(unsigned)((c->n_dir + 127) / 128), 128, 0, c->stream>>>(
      c->d_dir_rows, c->n_dir, c->d_rowptr, c->d_cols, c->nbasis[0], c->nbasis[1], c->nbasis[2],
      vals);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

}  // namespace igap

// --------------------------------------------------- scatter race check
// Every element adds 1 to each of its 81 x 81 CSR slots with a plain
// read-modify-write, colour by colour, as the element kernels scatter.  Two
// elements of one colour sharing a slot would lose updates and leave the slot
// below the number of elements whose support holds both of its control points.
namespace igap {
__global__ void slot_count_kernel(DevMesh m, int cx, int cy, int cz, int ncy, int ncz, double *counts)
{
  const int b = blockIdx.x;
  const int iz = b % ncz, iy = (b / ncz) % ncy, ix = b / (ncz * ncy);
  const int ex = cx + 3 * ix, ey = cy + 3 * iy, ez = cz + 3 * iz;
  const int nbv[3] = {m.nbasis[0], m.nbasis[1], m.nbasis[2]};
  for (int t = threadIdx.x; t < NE * NE; t += blockDim.x) {
    const int rr = t / NE, cc = t % NE;
    const int pb = rr / 3, d = rr % 3, pc = cc / 3, e = cc % 3;
    const int rx = ex + pb / 9, ry = ey + (pb / 3) % 3, rz = ez + pb % 3;
    const int sx = ex + pc / 9, sy = ey + (pc / 3) % 3, sz = ez + pc % 3;
    const int64_t cpb = ((int64_t)rx * nbv[1] + ry) * nbv[2] + rz;
    double *slot = counts + m.rowptr[3 * cpb + d] + 3 * stencil_pos(rx, ry, rz, sx, sy, sz, nbv) + e;
    *slot = *slot + 1.0;
  }
}
}  // namespace igap

extern "C" int igapgpu_debug_slot_counts(igapgpu_t c, double *counts)
{
  using namespace igap;
  if (!c || !counts) return IGAPGPU_ERR_ARG;
  if (c->batch || c->porder != P) {
    set_error("debug_slot_counts: quadratic single-lattice contexts only");
    return IGAPGPU_ERR_ARG;
  }
  const bool host = !is_device_ptr(counts);
  double *d = counts;
  if (host && cudaMalloc(&d, sizeof(double) * (size_t)c->nnz) != cudaSuccess) {
    cudaGetLastError();
    set_error("debug_slot_counts: allocation failed");
    return IGAPGPU_ERR_NOMEM;
  }
  cudaError_t e = cudaMemsetAsync(d, 0, sizeof(double) * (size_t)c->nnz, c->stream);
  const DevMesh m = c->devmesh();
  for (int cx = 0; cx < 3 && e == cudaSuccess; cx++)
    for (int cy = 0; cy < 3 && e == cudaSuccess; cy++)
      for (int cz = 0; cz < 3 && e == cudaSuccess; cz++) {
        const int ncx = (c->nelem[0] - cx + 2) / 3, ncy = (c->nelem[1] - cy + 2) / 3,
                  ncz = (c->nelem[2] - cz + 2) / 3;
        if (ncx * ncy * ncz <= 0) continue;
        slot_count_kernel<<<ncx * ncy * ncz, 256, 0, c->stream>>>(m, cx, cy, cz, ncy, ncz, d);
        count_launch();
        e = cudaGetLastError();
      }
  if (e == cudaSuccess && host)
    e = cudaMemcpyAsync(counts, d, sizeof(double) * (size_t)c->nnz, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (host) cudaFree(d);
  if (e != cudaSuccess) {
    set_error("debug_slot_counts: CUDA error %s", cudaGetErrorString(e));
    return IGAPGPU_ERR_CUDA;
  }
  return IGAPGPU_OK;
}

// ------------------------------------------------------- FP64 peak probe
namespace igap {
__global__ void fp64_peak_kernel(double *out, int iters)
{
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
  double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
  const double b = 0.999999, cc = 1e-12;
  for (int i = 0; i < iters; i++) {
    a0 = fma(a0, b, cc); a1 = fma(a1, b, cc); a2 = fma(a2, b, cc); a3 = fma(a3, b, cc);
    a4 = fma(a4, b, cc); a5 = fma(a5, b, cc); a6 = fma(a6, b, cc); a7 = fma(a7, b, cc);
  }
  if (a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7 == 1234.5) out[0] = 1.0;
}

__global__ void fp32_peak_kernel(double *out, int iters)
{
  float a0 = threadIdx.x * 1e-6f, a1 = a0 + 1e-6f, a2 = a0 + 2e-6f, a3 = a0 + 3e-6f;
  float a4 = a0 + 4e-6f, a5 = a0 + 5e-6f, a6 = a0 + 6e-6f, a7 = a0 + 7e-6f;
  const float b = 0.9999f, cc = 1e-7f;
  for (int i = 0; i < iters; i++) {
    a0 = fmaf(a0, b, cc); a1 = fmaf(a1, b, cc); a2 = fmaf(a2, b, cc); a3 = fmaf(a3, b, cc);
    a4 = fmaf(a4, b, cc); a5 = fmaf(a5, b, cc); a6 = fmaf(a6, b, cc); a7 = fmaf(a7, b, cc);
  }
  if (a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7 == 1234.5f) out[0] = 1.0;
}

// FMA throughput of a register-only kernel (8 independent chains a thread,
// 8 CTAs of 256 threads per SM), in TFLOP/s.
template <typename K>
static int measure_peak(K kern, int iters, double *tflops)
{
  int dev = 0, nsm = 0;
  IGAP_CUDA(cudaGetDevice(&dev));
  IGAP_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  double *d = nullptr;
  IGAP_CUDA(cudaMalloc(&d, sizeof(double)));
  cudaEvent_t e0, e1;
  IGAP_CUDA(cudaEventCreate(&e0));
  IGAP_CUDA(cudaEventCreate(&e1));
  const int blocks = nsm * 8, threads = 256;
  kern<<<blocks, threads>>>(d, 64);  // warm-up
  IGAP_CUDA(cudaEventRecord(e0));
  kern<<<blocks, threads>>>(d, iters);
  IGAP_CUDA(cudaEventRecord(e1));
  count_launch(2);
  IGAP_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  IGAP_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  return IGAPGPU_OK;
}
}  // namespace igap

extern "C" int igapgpu_measure_fp64_peak(double *tflops)
{
  if (!tflops) return IGAPGPU_ERR_ARG;
  return igap::measure_peak(igap::fp64_peak_kernel, 1 << 14, tflops);
}

extern "C" int igapgpu_measure_fp32_peak(double *tflops)
{
  if (!tflops) return IGAPGPU_ERR_ARG;
  return igap::measure_peak(igap::fp32_peak_kernel, 1 << 18, tflops);
}

// Runs wait_selftest_kernel on a zeroed counter: target 0 (satisfied at once)
// or 1 (never reached, the wait expires after `limit` polls).  *status gets the
// device error word: 0, or 3 for an expired wait.
extern "C" int igapgpu_wait_selftest(int target, unsigned int limit, int *status)
{
  using namespace igap;
  if (!status || target < 0 || target > 1 || limit > (1u << 24)) {
    set_error("wait self-test: target must be 0 or 1, limit at most 2^24 polls");
    return IGAPGPU_ERR_ARG;
  }
  int *d = nullptr;
  IGAP_CUDA(cudaMalloc(&d, 2 * sizeof(int)));
  cudaError_t e = cudaMemset(d, 0, 2 * sizeof(int));
  if (e == cudaSuccess) {
    wait_selftest_kernel<<<2, 64>>>(d, target, limit, d + 1);
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(status, d + 1, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) {
    set_error("wait self-test: %s", cudaGetErrorString(e));
    return IGAPGPU_ERR_CUDA;
  }
  return IGAPGPU_OK;
}
