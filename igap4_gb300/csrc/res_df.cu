// Residual of the linear strain-gradient law on the FP32 pipe in double-FP32
// arithmetic (the split-precision and FP64-quality modes; the FP64 mode keeps
// the FP64 element kernel).
//
// The residual is the reference's element loop (src/assmcore_iga.c:209-258:
// interpolate the state's first and second derivatives at every Gauss
// point, evaluate the law, project on every basis function) with the linear
// law of laws.cuh (lingrad_residual_dev), element by element:
//   u_dk(q) = sum_b N_bk(q) u_bd                 (k: 3 first, 6 second derivatives)
//   rr_dk(q) = w_q (D u)_dk(q)                   (the law's stress slots)
//   R_bd = sum_q sum_k N_bk(q) rr_dk(q)
// On this GPU the FP64 pipe is the bottleneck of that loop (about 1/64 of the
// FP32 rate), so every product and sum runs on float pairs (df32.cuh): the
// derivatives N_bk and weights come from a pair cache built once from the
// FP64 geometry cache, the state is split into pairs once per assembly, the
// two contractions are compensated dot products (Dot2) and the law is pair
// arithmetic.  Measured against the FP64 kernel: about 1e-14 relative.
//
// Layout and work split: one thread per Gauss point (a warp holds 32 points
// of one element), the pair cache point-minor ([element][value][point]), so
// that a warp's loads are contiguous; a point's projection partials are
// summed over the element's points through shared memory; the element sums
// go to a per-element buffer, and a gather kernel adds them per DOF in a fixed
// order (deterministic, no atomics).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

#include "common.cuh"
#include "element.cuh"
#include "df32.cuh"
#include "gram_common.cuh"

namespace igap {

constexpr int RP_V = NB * 9 + 1;  // pair-cache values per point: 27 x 9 derivatives, weight
constexpr int RD_THREADS = 128;

struct DfLaw {
  float2 lam, mu, l2;
};

// FP64 -> pair on the FP64 pipe (cache build and state split only)
__device__ __forceinline__ float2 split_pair(double x)
{
  const float h = __double2float_rn(x);
  return make_float2(h, __double2float_rn(x - (double)h));
}

__global__ void res_pair_cache_kernel(const double *__restrict__ geo, int npts, int64_t nelem,
                                      float2 *__restrict__ pc)
{
  const int64_t n = nelem * npts * RP_V;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int q = (int)(i % npts);
    const int64_t t = i / npts;
    const int v = (int)(t % RP_V);
    const int64_t e = t / RP_V;
    const double *g = geo + (e * npts + q) * GEO_STRIDE;
    pc[i] = split_pair(v < NB * 9 ? g[NDD * (v / 9) + 1 + v % 9] : g[NB * NDD]);
  }
}

__global__ void state_pair_kernel(const double *__restrict__ U, int64_t n, float2 *__restrict__ up)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    up[i] = split_pair(U[i]);
}

__device__ __forceinline__ constexpr int hs6(int i, int m)
{
  return i < m ? (i == 0 ? m : (i == 1 ? 2 + m : 5)) : (m == 0 ? i : (m == 1 ? 2 + i : 5));
}

__device__ __forceinline__ float2 twice(float2 a) { return make_float2(2.f * a.x, 2.f * a.y); }

// The linear law of lingrad_residual_dev in pair arithmetic.  ud[9d + k]:
// derivatives of displacement component d (k 0..2 gradient, 3..8 Hessian
// xx, xy, xz, yy, yz, zz); rr[9d + k]: the weighted stress slots.
__device__ __forceinline__ void lin_law_df(const float2 *ud, float2 wt, const DfLaw &L, float2 *rr)
{
  const float2 ldiv = df_mul(L.lam, df_add(df_add(ud[0], ud[9 + 1]), ud[18 + 2]));
#pragma unroll
  for (int d = 0; d < 3; d++)
#pragma unroll
    for (int i = 0; i < 3; i++) {
      float2 s = df_mul(L.mu, df_add(ud[9 * d + i], ud[9 * i + d]));
      if (d == i) s = df_add(s, ldiv);
      rr[9 * d + i] = df_mul(wt, s);
    }
  float2 Dm[3];  // derivatives of the divergence
#pragma unroll
  for (int m = 0; m < 3; m++)
    Dm[m] = df_add(df_add(ud[3 + hs6(0, m)], ud[9 + 3 + hs6(1, m)]), ud[18 + 3 + hs6(2, m)]);
  const float2 wl2 = df_mul(wt, L.l2);
#pragma unroll
  for (int d = 0; d < 3; d++)
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int m = i; m < 3; m++) {
        // slot (i, m): T_d[i][m] (+ T_d[m][i] off the diagonal), with
        // T_d[i][m] = mu (H_d(i,m) + H_i(d,m)) + lam delta_di Dm[m]
        float2 t;
        if (i == m) {
          t = df_mul(L.mu, df_add(ud[9 * d + 3 + hs6(i, i)], ud[9 * i + 3 + hs6(d, i)]));
          if (d == i) t = df_add(t, df_mul(L.lam, Dm[i]));
        } else {
          const float2 h = df_add(twice(ud[9 * d + 3 + hs6(i, m)]),
                                  df_add(ud[9 * i + 3 + hs6(d, m)], ud[9 * m + 3 + hs6(d, i)]));
          t = df_mul(L.mu, h);
          if (d == i) t = df_add(t, df_mul(L.lam, Dm[m]));
          if (d == m) t = df_add(t, df_mul(L.lam, Dm[i]));
        }
        rr[9 * d + 3 + hs6(i, m)] = df_mul(wl2, t);
      }
}

// Loads of the pair cache with an L2 eviction-priority hint: the
// interpolation pass marks its lines evict-last (the projection pass reads
// them again), the projection pass evict-first.
__device__ __forceinline__ uint64_t l2_policy_last()
{
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_policy_first()
{
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ float2 ld_pair(const float2 *p, uint64_t pol)
{
  float2 v;
  asm("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(p), "l"(pol));
  return v;
}

// NW warps per element (npts <= 32 NW), RD_THREADS / (32 NW) elements per CTA.
// rel[e][3b + d]: the element's residual pairs.  The interpolation loads the
// next basis function's derivatives ahead; the projection visits the basis
// functions in the reverse order of the interpolation, so that the lines read
// last are read again first (with the eviction hints, 7.9 -> 6.8 ms per
// residual at 128x32x32; fewer CTAs per SM for more L2 reuse measured slower).
template <int NW>
__global__ void __launch_bounds__(RD_THREADS) res_df_kernel(const float2 *__restrict__ pc,
                                                            const float2 *__restrict__ up, int npts,
                                                            int64_t nelem, int ne1, int ne2, int nb1, int nb2,
                                                            DfLaw L, float2 *__restrict__ rel)
{
  constexpr int NWARP = RD_THREADS / 32, EPB = NWARP / NW;
  __shared__ float2 su[EPB][NE];
  __shared__ float2 red[NWARP][32][27];
  __shared__ float2 part[EPB][NW][NE];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int le = warp / NW, wq = warp % NW;
  const int64_t e0 = (int64_t)blockIdx.x * EPB;
  for (int t = tid; t < EPB * NE; t += RD_THREADS) {
    const int l = t / NE, i = t % NE, b = i / 3, d = i % 3;
    const int64_t ee = e0 + l;
    float2 v = make_float2(0.f, 0.f);
    if (ee < nelem) {
      const int ez = (int)(ee % ne2), ey = (int)((ee / ne2) % ne1);
      const int64_t ex = ee / ((int64_t)ne1 * ne2);
      const int64_t cp = ((ex + b / 9) * nb1 + (ey + (b / 3) % 3)) * nb2 + (ez + b % 3);
      v = __ldg(up + 3 * cp + d);
    }
    su[l][i] = v;
  }
  __syncthreads();
  const int64_t e = e0 + le;
  const int q = 32 * wq + lane;
  const bool act = e < nelem && q < npts;
  const float2 *p = pc + (act ? ((e * RP_V) * npts + q) : 0);
  const uint64_t pol1 = l2_policy_last(), pol2 = l2_policy_first();
  float2 rr[27];
  {
    float s[27], c[27];
#pragma unroll
    for (int i = 0; i < 27; i++) s[i] = c[i] = 0.f;
    float2 wt = make_float2(0.f, 0.f);
    if (act) {
      float2 n[9];
#pragma unroll
      for (int k = 0; k < 9; k++) n[k] = ld_pair(p + (size_t)k * npts, pol1);
#pragma unroll 1
      for (int b = 0; b < NB; b++) {
        float2 nn[9];  // the next basis function's derivatives, loaded ahead
        const int bn = b + 1 < NB ? b + 1 : b;
#pragma unroll
        for (int k = 0; k < 9; k++) nn[k] = ld_pair(p + (size_t)(9 * bn + k) * npts, pol1);
        const float2 u0 = su[le][3 * b], u1 = su[le][3 * b + 1], u2 = su[le][3 * b + 2];
#pragma unroll
        for (int k = 0; k < 9; k++) {
          dot2(s[k], c[k], n[k], u0);
          dot2(s[9 + k], c[9 + k], n[k], u1);
          dot2(s[18 + k], c[18 + k], n[k], u2);
        }
#pragma unroll
        for (int k = 0; k < 9; k++) n[k] = nn[k];
      }
      wt = __ldg(p + (size_t)(NB * 9) * npts);
    }
    float2 ud[27];
#pragma unroll
    for (int i = 0; i < 27; i++) ud[i] = dot2_pair(s[i], c[i]);
    lin_law_df(ud, wt, L, rr);
  }
  // projection: block j of 9 basis functions at a time, summed over the
  // warp's points through red[warp]
#pragma unroll 1
  for (int jj = 0; jj < 3; jj++) {
    const int j = 2 - jj;
#pragma unroll 1
    for (int bi = 0; bi < 9; bi++) {
      const int bb = 8 - bi;
      const int b = 9 * j + bb;
      float2 n[9];
#pragma unroll
      for (int k = 0; k < 9; k++)
        n[k] = act ? ld_pair(p + (size_t)(9 * b + k) * npts, pol2) : make_float2(0.f, 0.f);
#pragma unroll
      for (int d = 0; d < 3; d++) {
        float s = 0.f, c = 0.f;
#pragma unroll
        for (int k = 0; k < 9; k++) dot2(s, c, n[k], rr[9 * d + k]);
        red[warp][lane][3 * bb + d] = dot2_pair(s, c);
      }
    }
    __syncwarp();
    if (lane < 27) {
      float2 t = red[warp][0][lane];
#pragma unroll 4
      for (int l = 1; l < 32; l++) t = df_add(t, red[warp][l][lane]);
      part[le][wq][27 * j + lane] = t;
    }
    __syncwarp();
  }
  __syncthreads();
  for (int t = tid; t < EPB * NE; t += RD_THREADS) {
    const int l = t / NE, i = t % NE;
    if (e0 + l >= nelem) continue;
    float2 v = part[l][0][i];
#pragma unroll
    for (int w = 1; w < NW; w++) v = df_add(v, part[l][w][i]);
    rel[(e0 + l) * NE + i] = v;
  }
}

// RR[dof] += the sum of its elements' residual pairs, elements in a fixed order.
__global__ void res_gather_kernel(const float2 *__restrict__ rel, int ne0, int ne1, int ne2, int nb0, int nb1,
                                  int nb2, double *__restrict__ RR)
{
  const int64_t ndof = 3 * (int64_t)nb0 * nb1 * nb2;
  for (int64_t dof = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; dof < ndof;
       dof += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cp = dof / 3;
    const int d = (int)(dof % 3);
    const int iz = (int)(cp % nb2), iy = (int)((cp / nb2) % nb1), ix = (int)(cp / ((int64_t)nb1 * nb2));
    float2 s = make_float2(0.f, 0.f);
    for (int ex = max(ix - P, 0); ex <= min(ix, ne0 - 1); ex++)
      for (int ey = max(iy - P, 0); ey <= min(iy, ne1 - 1); ey++)
        for (int ez = max(iz - P, 0); ez <= min(iz, ne2 - 1); ez++) {
          const int64_t el = ((int64_t)ex * ne1 + ey) * ne2 + ez;
          const int b = (ix - ex) * 9 + (iy - ey) * 3 + (iz - ez);
          s = df_add(s, __ldg(rel + el * NE + 3 * b + d));
        }
    RR[dof] += (double)s.x + (double)s.y;
  }
}

// ------------------------------------------------------ batched instances
// The linear law of lin_law_df with one output slot per lane and no divergent
// branches: slot (d, k), lane 9d + k, is
//   w_k sc (mu (f u[A] + u[B] + u[C]) + lam (u[E] + u[F]))
// over the point's derivatives u[0..26] with u[27] = 0, u[28] the divergence
// and u[29 + m] its derivative m.  First-gradient slot i: A = 9d + i,
// B = 9i + d, f = 1, E the divergence if d = i.  Hessian slot (i, m):
// A = H_d(i,m) with f = 2, B = H_i(d,m), C = H_m(d,i), E = D_m if d = i,
// F = D_i if d = m, weight w l^2; a diagonal slot (i = m) counts every term
// twice and is halved (sc = 1/2, exact), so that each slot repeats the pair
// operations of lin_law_df.
// The slot of a lane packed in an int2: x = A | B << 8 | C << 16 | E << 24,
// y = F | second << 8 | diagonal << 9.
__device__ __forceinline__ int2 law_slot(int lane)
{
  int A = 27, B = 27, C = 27, E = 27, F = 27, second = 0, diag = 0;
  if (lane < 27) {
    const int d = lane / 9, k = lane % 9;
    if (k < 3) {
      A = 9 * d + k;
      B = 9 * k + d;
      if (d == k) E = 28;
    } else {
      const int sl = k - 3;
      const int i = sl < 3 ? 0 : (sl < 5 ? 1 : 2), m = sl < 3 ? sl : (sl < 5 ? sl - 2 : 2);
      A = 9 * d + 3 + hs6(i, m);
      B = 9 * i + 3 + hs6(d, m);
      C = 9 * m + 3 + hs6(d, i);
      second = 1;
      diag = i == m;
      if (d == i) E = 29 + m;
      if (d == m) F = 29 + i;
    }
  }
  return make_int2(A | B << 8 | C << 16 | E << 24, F | second << 8 | diag << 9);
}

__device__ __forceinline__ float2 law_slot_eval(const float2 *u, int2 s, float2 wt, float2 wl2, const DfLaw &L)
{
  const bool second = (s.y >> 8) & 1;
  const float f = second ? 2.f : 1.f, sc = (s.y >> 9) & 1 ? 0.5f : 1.f;
  const float2 a = u[s.x & 255];
  const float2 h = df_add(make_float2(f * a.x, f * a.y), df_add(u[(s.x >> 8) & 255], u[(s.x >> 16) & 255]));
  float2 t = df_add(df_mul(L.mu, h), df_mul(L.lam, df_add(u[(s.x >> 24) & 255], u[s.y & 255])));
  t = make_float2(sc * t.x, sc * t.y);
  return df_mul(second ? wl2 : wt, t);
}

// lanes 28..31: the divergence of u and its three derivatives, as lin_law_df sums them
__device__ __forceinline__ float2 law_divergence(const float2 *u, int j)
{
  if (j == 0) return df_add(df_add(u[0], u[9 + 1]), u[18 + 2]);
  const int m = j - 1;
  return df_add(df_add(u[3 + hs6(0, m)], u[9 + 3 + hs6(1, m)]), u[18 + 3 + hs6(2, m)]);
}

__device__ __forceinline__ int find_inst(const int64_t *__restrict__ off, int ninst, int64_t x)
{
  int lo = 0, hi = ninst;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

// The linear-law residual of every element of a batch (instances with their
// own meshes and law parameters) in double-FP32 arithmetic.  A CTA per
// element, a warp per Gauss point (8 points per warp): the point's 243
// physical derivatives and weight are read from the instance's FP64
// geometry cache and split into pairs on the integer pipe as they are read
// (the batch keeps no pair cache: 125 KB per element would not fit beside its
// other caches); lanes 0..26 interpolate one derivative of u each and
// evaluate one stress slot each; the projection gives each lane 3 of the 81
// outputs, accumulated over the warp's points, then over the 8 warps.  Each
// warp loads the next point's geometry into registers before it works on the
// current one, so that the DRAM latency hides behind the contractions; the
// element's instance comes from a per-element table (one load, not a search).
constexpr int RB_THREADS = 256, RB_WARPS = RB_THREADS / 32, RB_LD = (RP_V + 31) / 32;
__device__ __forceinline__ int rb_geo_index(int v) { return v < NB * 9 ? NDD * (v / 9) + 1 + v % 9 : NB * NDD; }

__global__ void __launch_bounds__(RB_THREADS, 4) res_df_batch_kernel(const DevMesh *__restrict__ meshes,
                                                                     const DevLaw *__restrict__ laws,
                                                                     const int64_t *__restrict__ eoff,
                                                                     const int *__restrict__ einst,
                                                                     const double *__restrict__ U,
                                                                     float2 *__restrict__ rel)
{
  __shared__ float2 su[NE];
  __shared__ float2 sR[RB_WARPS][RP_V];
  __shared__ float2 sU[RB_WARPS][32], sRR[RB_WARPS][27];
  __shared__ float2 part[RB_WARPS][NE];
  __shared__ DfLaw sL;
  __shared__ int2 sslot[32];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t g = blockIdx.x;
  const int inst = __ldg(einst + g);
  const DevMesh &m = meshes[inst];
  const int ne1 = m.nelem[1], ne2 = m.nelem[2], nb1 = m.nbasis[1], nb2 = m.nbasis[2], npts = m.npts;
  const int e = (int)(g - __ldg(eoff + inst));  // element within its instance
  const double *gel = m.geo + (int64_t)e * npts * GEO_STRIDE;
  double gv[RB_LD];
  if (warp < npts) {
#pragma unroll
    for (int i = 0; i < RB_LD; i++) {
      const int v = lane + 32 * i;
      gv[i] = v < RP_V ? __ldg(gel + (int64_t)warp * GEO_STRIDE + rb_geo_index(v)) : 0.0;
    }
  }
  const int ez = e % ne2, ey = (e / ne2) % ne1, ex = e / (ne1 * ne2);
  for (int t = tid; t < NE; t += RB_THREADS) {
    const int b = t / 3, d = t % 3;
    const int64_t cp = ((int64_t)(ex + b / 9) * nb1 + (ey + (b / 3) % 3)) * nb2 + (ez + b % 3);
    su[t] = f64_to_pair(__ldg(U + m.dof_off + 3 * cp + d));
  }
  if (tid == 0) {
    const double *par = laws[inst].par;
    sL.lam = split_pair(par[0]);
    sL.mu = split_pair(par[1]);
    sL.l2 = split_pair(par[2] * par[2]);
  }
  if (lane == 27) sU[warp][27] = make_float2(0.f, 0.f);
  if (tid < 32) sslot[tid] = law_slot(tid);
  __syncthreads();
  const DfLaw L = sL;
  float ps[3] = {0.f, 0.f, 0.f}, pc[3] = {0.f, 0.f, 0.f};
  for (int q = warp; q < npts; q += RB_WARPS) {
#pragma unroll
    for (int i = 0; i < RB_LD; i++) {
      const int v = lane + 32 * i;
      if (v < RP_V) sR[warp][v] = f64_to_pair(gv[i]);
    }
    const int qn = q + RB_WARPS;
    if (qn < npts) {
#pragma unroll
      for (int i = 0; i < RB_LD; i++) {
        const int v = lane + 32 * i;
        if (v < RP_V) gv[i] = __ldg(gel + (int64_t)qn * GEO_STRIDE + rb_geo_index(v));
      }
    }
    __syncwarp();
    if (lane < 27) {  // u_dk, lane = 9d + k
      const int d = lane / 9, k = lane % 9;
      float s = 0.f, c = 0.f;
#pragma unroll 9
      for (int b = 0; b < NB; b++) dot2(s, c, sR[warp][9 * b + k], su[3 * b + d]);
      sU[warp][lane] = dot2_pair(s, c);
    }
    __syncwarp();
    if (lane >= 28) sU[warp][lane] = law_divergence(sU[warp], lane - 28);
    __syncwarp();
    if (lane < 27) {
      const float2 wt = sR[warp][NB * 9];
      sRR[warp][lane] = law_slot_eval(sU[warp], sslot[lane], wt, df_mul(wt, L.l2), L);
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int o = lane + 32 * j;
      if (o < NE) {
        const int b = o / 3, d = o % 3;
#pragma unroll
        for (int k = 0; k < 9; k++) dot2(ps[j], pc[j], sR[warp][9 * b + k], sRR[warp][9 * d + k]);
      }
    }
    __syncwarp();
  }
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int o = lane + 32 * j;
    if (o < NE) part[warp][o] = dot2_pair(ps[j], pc[j]);
  }
  __syncthreads();
  for (int t = tid; t < NE; t += RB_THREADS) {
    float2 v = part[0][t];
#pragma unroll
    for (int w = 1; w < RB_WARPS; w++) v = df_add(v, part[w][t]);
    rel[g * NE + t] = v;
  }
}

// RR[dof] += the sum of the element residual pairs of the dof's instance, in
// a fixed element order.
__global__ void res_gather_batch_kernel(const float2 *__restrict__ rel, const DevMesh *__restrict__ meshes,
                                        const int64_t *__restrict__ doff, const int64_t *__restrict__ eoff,
                                        int ninst, int64_t ndof, double *__restrict__ RR)
{
  for (int64_t dof = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; dof < ndof;
       dof += (int64_t)gridDim.x * blockDim.x) {
    const int inst = find_inst(doff, ninst, dof);
    const DevMesh &m = meshes[inst];
    const int ne0 = m.nelem[0], ne1 = m.nelem[1], ne2 = m.nelem[2], nb1 = m.nbasis[1], nb2 = m.nbasis[2];
    const int64_t loc = dof - __ldg(doff + inst), cp = loc / 3, e0 = __ldg(eoff + inst);
    const int d = (int)(loc % 3);
    const int iz = (int)(cp % nb2), iy = (int)((cp / nb2) % nb1), ix = (int)(cp / ((int64_t)nb1 * nb2));
    float2 s = make_float2(0.f, 0.f);
    for (int ex = max(ix - P, 0); ex <= min(ix, ne0 - 1); ex++)
      for (int ey = max(iy - P, 0); ey <= min(iy, ne1 - 1); ey++)
        for (int ez = max(iz - P, 0); ez <= min(iz, ne2 - 1); ez++) {
          const int64_t el = e0 + ((int64_t)ex * ne1 + ey) * ne2 + ez;
          const int b = (ix - ex) * 9 + (iy - ey) * 3 + (iz - ez);
          s = df_add(s, __ldg(rel + el * NE + 3 * b + d));
        }
    RR[dof] += (double)s.x + (double)s.y;
  }
}

int launch_res_df_batch(Context *c, const DevMesh *meshes, const DevLaw *laws, const int64_t *eoff,
                        const int *einst, const int64_t *doff, int ninst, int64_t nel, float2 *rel, double *RR)
{
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (c->prof) {
    IGAP_CUDA(cudaEventCreate(&e0));
    IGAP_CUDA(cudaEventCreate(&e1));
    IGAP_CUDA(cudaEventRecord(e0, c->stream));
  }
  res_df_batch_kernel<<<(unsigned)nel, RB_THREADS, 0, c->stream>>>(meshes, laws, eoff, einst, c->d_Uhist, rel);
  count_launch();
  IGAP_CHECK_LAUNCH();
  if (c->prof) {
    IGAP_CUDA(cudaEventRecord(e1, c->stream));
    c->prof_ev[0].emplace_back(e0, e1);
    c->prof_launches[0]++;
    c->prof_elements[0] += nel;
  }
  res_gather_batch_kernel<<<152 * 8, 256, 0, c->stream>>>(rel, meshes, doff, eoff, ninst, c->ndof, RR);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

// ------------------------------------------------- the reference's laws
// gradelast / gradelasttime in the tensor-core modes (law outputs of every
// point precomputed, a thread per point, FP64 law): the two contractions
// around the law on float pairs.
//  * law_in_df_kernel: the law's inputs (src/assmcore_iga.c:209-229 and the
//    transient segment of the law kernel), from nodal combinations of the
//    history levels formed once per assembly in FP64 and split into pairs:
//    static m = sum_b R_bk u0; transient, at the derivative slots,
//    m = sum_b R_bk (u1 + u2) / 2 and delta = sum_b R_bk (u0 - u2) / 2, at the
//    value slots (inertia and damping) damp/(2 dt) sum_b R_b (u0 - u2) +
//    rho/dt^2 sum_b R_b ((u0 + u2) - 2 u1).  The differences are taken on the
//    nodal values in FP64 before the interpolation, so that the second
//    difference of the inertia term carries no cancellation of interpolated
//    values.  Output per point p: lin[64 p + slot] (m, 30 slots),
//    lin[64 p + 30 + slot] (delta), lin[64 p + 60] the weight.
//  * res_law_df_kernel: R_bd = sum_q sum_k N_bk(q) rr_dk(q) over the 10 slots
//    (value included) from the law outputs (FP64, [element][slot][point]),
//    element pairs to rel, res_gather_kernel adds them per DOF.
// Both read the FP64 geometry cache and split it into pairs as they read it
// (one CTA per element, a warp per Gauss point, the next point's values
// loaded before the current point's contractions).
constexpr int LI_THREADS = 256, LI_WARPS = LI_THREADS / 32, LI_NV = NB * NDD, LI_LD = (LI_NV + 1 + 31) / 32;

__global__ void law_state_pair_kernel(const double *__restrict__ U, int64_t ndof, int transient,
                                      float2 *__restrict__ up)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ndof; i += (int64_t)gridDim.x * blockDim.x) {
    const double u0 = U[i];
    if (!transient) {
      up[i] = split_pair(u0);
      continue;
    }
    const double u1 = U[ndof + i], u2 = U[2 * ndof + i];
    up[i] = split_pair(u1 + u2);
    up[ndof + i] = split_pair(u0 - u2);
    up[2 * ndof + i] = split_pair((u0 + u2) - 2.0 * u1);
  }
}

__device__ __forceinline__ double pair_to_f64(float2 a) { return f32_to_f64(a.x) + f32_to_f64(a.y); }

template <bool TR>
__global__ void __launch_bounds__(LI_THREADS, 4)
    law_in_df_kernel(const double *__restrict__ geo, const float2 *__restrict__ up, int64_t ndof, int npts,
                     int ne1, int ne2, int nb1, int nb2, float2 cdamp, float2 crho, double *__restrict__ lin)
{
  __shared__ float2 sc[TR ? 3 : 1][NE];
  __shared__ float2 sR[LI_WARPS][LI_NV];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t e = blockIdx.x;
  const double *gel = geo + e * npts * GEO_STRIDE;
  double gv[LI_LD];
  if (warp < npts) {
#pragma unroll
    for (int i = 0; i < LI_LD; i++) {
      const int v = lane + 32 * i;
      gv[i] = v <= LI_NV ? __ldg(gel + (int64_t)warp * GEO_STRIDE + v) : 0.0;
    }
  }
  const int ez = (int)(e % ne2), ey = (int)((e / ne2) % ne1);
  const int64_t ex = e / ((int64_t)ne1 * ne2);
  for (int t = tid; t < (TR ? 3 : 1) * NE; t += LI_THREADS) {
    const int c = t / NE, i = t % NE, b = i / 3, d = i % 3;
    const int64_t cp = ((ex + b / 9) * nb1 + (ey + (b / 3) % 3)) * nb2 + (ez + b % 3);
    sc[c][i] = __ldg(up + c * ndof + 3 * cp + d);
  }
  __syncthreads();
  for (int q = warp; q < npts; q += LI_WARPS) {
    double *o = lin + (e * npts + q) * 64;
#pragma unroll
    for (int i = 0; i < LI_LD; i++) {
      const int v = lane + 32 * i;
      if (v < LI_NV) sR[warp][v] = f64_to_pair(gv[i]);
      if (v == LI_NV) o[60] = gv[i];  // the point's weight, as cached
    }
    const int qn = q + LI_WARPS;
    if (qn < npts) {
#pragma unroll
      for (int i = 0; i < LI_LD; i++) {
        const int v = lane + 32 * i;
        if (v <= LI_NV) gv[i] = __ldg(gel + (int64_t)qn * GEO_STRIDE + v);
      }
    }
    __syncwarp();
    if (lane < 30) {
      const int d = lane / NDD, k = lane % NDD;
      // transient: value slots take (u0 - u2, second difference), the others
      // (u1 + u2, u0 - u2)
      const float2 *sa = sc[TR && k == 0 ? 1 : 0];
      const float2 *sb = sc[TR ? (k == 0 ? 2 : 1) : 0];
      float s1 = 0.f, c1 = 0.f, s2 = 0.f, c2 = 0.f;
#pragma unroll 9
      for (int b = 0; b < NB; b++) {
        const float2 n = sR[warp][NDD * b + k];
        dot2(s1, c1, n, sa[3 * b + d]);
        if (TR) dot2(s2, c2, n, sb[3 * b + d]);
      }
      const float2 A = dot2_pair(s1, c1);
      if (!TR) {
        o[lane] = pair_to_f64(A);
      } else {
        const float2 B = dot2_pair(s2, c2);
        if (k == 0) {
          o[lane] = pair_to_f64(df_add(df_mul(cdamp, A), df_mul(crho, B)));
          o[30 + lane] = 0.0;
        } else {
          o[lane] = pair_to_f64(make_float2(0.5f * A.x, 0.5f * A.y));
          o[30 + lane] = pair_to_f64(make_float2(0.5f * B.x, 0.5f * B.y));
        }
      }
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(LI_THREADS, 4)
    res_law_df_kernel(const double *__restrict__ geo, const double *__restrict__ preR, int npts,
                      float2 *__restrict__ rel)
{
  __shared__ float2 sR[LI_WARPS][LI_NV];
  __shared__ float2 srr[30 * 64];  // [slot][point]
  __shared__ float2 part[LI_WARPS][NE];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t e = blockIdx.x;
  const double *gel = geo + e * npts * GEO_STRIDE;
  double gv[LI_LD];
  if (warp < npts) {
#pragma unroll
    for (int i = 0; i < LI_LD; i++) {
      const int v = lane + 32 * i;
      gv[i] = v < LI_NV ? __ldg(gel + (int64_t)warp * GEO_STRIDE + v) : 0.0;
    }
  }
  const double *rr = preR + e * 30 * npts;
  for (int t = tid; t < 30 * npts; t += LI_THREADS) srr[t] = f64_to_pair(__ldg(rr + t));
  __syncthreads();
  float ps[3] = {0.f, 0.f, 0.f}, pc[3] = {0.f, 0.f, 0.f};
  for (int q = warp; q < npts; q += LI_WARPS) {
#pragma unroll
    for (int i = 0; i < LI_LD; i++) {
      const int v = lane + 32 * i;
      if (v < LI_NV) sR[warp][v] = f64_to_pair(gv[i]);
    }
    const int qn = q + LI_WARPS;
    if (qn < npts) {
#pragma unroll
      for (int i = 0; i < LI_LD; i++) {
        const int v = lane + 32 * i;
        if (v < LI_NV) gv[i] = __ldg(gel + (int64_t)qn * GEO_STRIDE + v);
      }
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int o = lane + 32 * j;
      if (o < NE) {
        const int b = o / 3, d = o % 3;
#pragma unroll
        for (int k = 0; k < NDD; k++) dot2(ps[j], pc[j], sR[warp][NDD * b + k], srr[(NDD * d + k) * npts + q]);
      }
    }
    __syncwarp();
  }
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int o = lane + 32 * j;
    if (o < NE) part[warp][o] = dot2_pair(ps[j], pc[j]);
  }
  __syncthreads();
  for (int t = tid; t < NE; t += LI_THREADS) {
    float2 v = part[0][t];
#pragma unroll
    for (int w = 1; w < LI_WARPS; w++) v = df_add(v, part[w][t]);
    rel[e * NE + t] = v;
  }
}

static float2 host_pair(double x)
{
  const float h = (float)x;
  return make_float2(h, (float)(x - (double)h));
}

// Builds the pair cache once (linear law, quadratic, single lattice, FP64
// geometry cache present, memory allows; IGAPGPU_RES_DF=0 turns it off).
int ensure_res_pairs(Context *c)
{
  if (c->rpc_state >= 0) return IGAPGPU_OK;
  c->rpc_state = 0;
  const char *env = getenv("IGAPGPU_RES_DF");
  if (env && env[0] == '0') return IGAPGPU_OK;
  if (!c->d_geo || c->batch || c->porder != 2) return IGAPGPU_OK;
  const int npts = c->nquad * c->nquad * c->nquad;
  if (npts > 64) return IGAPGPU_OK;
  if (c->law == IGAPGPU_LAW_GRADELAST || (c->law == IGAPGPU_LAW_GRADELASTTIME && c->torder >= 2)) {
    // the reference's laws: the law-input buffer, the nodal combinations and
    // the element pairs (the law outputs come from the precomputed-law path)
    const int ncomb = c->law == IGAPGPU_LAW_GRADELASTTIME ? 3 : 1;
    const size_t lbytes = (size_t)c->nelem_total * npts * 64 * sizeof(double);
    const size_t rbytes = (size_t)c->nelem_total * NE * sizeof(float2);
    const size_t ubytes = (size_t)ncomb * c->ndof * sizeof(float2);
    size_t freeb = 0, totb = 0;
    IGAP_CUDA(cudaMemGetInfo(&freeb, &totb));
    if (lbytes + rbytes + ubytes + ((size_t)4 << 30) > freeb / 2) return IGAPGPU_OK;
    if (cudaMalloc(&c->d_lin, lbytes) != cudaSuccess || cudaMalloc(&c->d_rel, rbytes) != cudaSuccess ||
        cudaMalloc(&c->d_upair, ubytes) != cudaSuccess) {
      cudaGetLastError();
      if (c->d_lin) cudaFree(c->d_lin);
      if (c->d_rel) cudaFree(c->d_rel);
      if (c->d_upair) cudaFree(c->d_upair);
      c->d_lin = nullptr;
      c->d_rel = c->d_upair = nullptr;
      return IGAPGPU_OK;
    }
    c->rpc_state = 2;
    return IGAPGPU_OK;
  }
  if (c->law != IGAPGPU_LAW_LINGRAD) return IGAPGPU_OK;
  const size_t bytes = (size_t)c->nelem_total * npts * RP_V * sizeof(float2);
  const size_t rbytes = (size_t)c->nelem_total * NE * sizeof(float2);
  const size_t ubytes = (size_t)c->ndof * sizeof(float2);
  size_t freeb = 0, totb = 0;
  IGAP_CUDA(cudaMemGetInfo(&freeb, &totb));
  if (bytes + rbytes + ubytes + ((size_t)4 << 30) > freeb) return IGAPGPU_OK;
  if (cudaMalloc(&c->d_rpc, bytes) != cudaSuccess || cudaMalloc(&c->d_rel, rbytes) != cudaSuccess ||
      cudaMalloc(&c->d_upair, ubytes) != cudaSuccess) {
    cudaGetLastError();
    if (c->d_rpc) cudaFree(c->d_rpc);
    if (c->d_rel) cudaFree(c->d_rel);
    if (c->d_upair) cudaFree(c->d_upair);
    c->d_rpc = c->d_rel = c->d_upair = nullptr;
    return IGAPGPU_OK;
  }
  res_pair_cache_kernel<<<152 * 16, 256, 0, c->stream>>>(c->d_geo, npts, c->nelem_total, c->d_rpc);
  count_launch();
  IGAP_CHECK_LAUNCH();
  c->rpc_state = 1;
  return IGAPGPU_OK;
}

// RR += element residuals of the linear law from the pair cache.
int launch_res_df(Context *c, double *RR)
{
  const int npts = c->nquad * c->nquad * c->nquad;
  const DfLaw L = {host_pair(c->par[0]), host_pair(c->par[1]), host_pair(c->par[2] * c->par[2])};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (c->prof) {
    IGAP_CUDA(cudaEventCreate(&e0));
    IGAP_CUDA(cudaEventCreate(&e1));
  }
  state_pair_kernel<<<152 * 4, 256, 0, c->stream>>>(c->d_Uhist, c->ndof, c->d_upair);
  count_launch();
  IGAP_CHECK_LAUNCH();
  if (c->prof) IGAP_CUDA(cudaEventRecord(e0, c->stream));
  const int64_t ne = c->nelem_total;
  if (npts <= 32) {
    constexpr int EPB = RD_THREADS / 32;
    res_df_kernel<1><<<(unsigned)((ne + EPB - 1) / EPB), RD_THREADS, 0, c->stream>>>(
        c->d_rpc, c->d_upair, npts, ne, c->nelem[1], c->nelem[2], c->nbasis[1], c->nbasis[2], L, c->d_rel);
  } else {
    constexpr int EPB = RD_THREADS / 64;
    res_df_kernel<2><<<(unsigned)((ne + EPB - 1) / EPB), RD_THREADS, 0, c->stream>>>(
        c->d_rpc, c->d_upair, npts, ne, c->nelem[1], c->nelem[2], c->nbasis[1], c->nbasis[2], L, c->d_rel);
  }
  count_launch();
  IGAP_CHECK_LAUNCH();
  if (c->prof) {
    IGAP_CUDA(cudaEventRecord(e1, c->stream));
    c->prof_ev[0].emplace_back(e0, e1);
    c->prof_launches[0]++;
    c->prof_elements[0] += ne;
  }
  res_gather_kernel<<<152 * 4, 256, 0, c->stream>>>(c->d_rel, c->nelem[0], c->nelem[1], c->nelem[2],
                                                   c->nbasis[0], c->nbasis[1], c->nbasis[2], RR);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

// The law's inputs at every point from pair interpolation (the reference's
// laws in the tensor-core modes; before the law kernel).
int launch_law_in_df(Context *c)
{
  const int npts = c->nquad * c->nquad * c->nquad;
  const bool tr = c->law == IGAPGPU_LAW_GRADELASTTIME;
  law_state_pair_kernel<<<152 * 4, 256, 0, c->stream>>>(c->d_Uhist, c->ndof, tr ? 1 : 0, c->d_upair);
  count_launch();
  IGAP_CHECK_LAUNCH();
  const double damp = c->par[6], rho = c->par[5], dt = c->par[7];
  const float2 cd = tr ? host_pair(damp / (2.0 * dt)) : make_float2(0.f, 0.f);
  const float2 cr = tr ? host_pair(rho / (dt * dt)) : make_float2(0.f, 0.f);
  const unsigned grid = (unsigned)c->nelem_total;
  if (tr)
    law_in_df_kernel<true><<<grid, LI_THREADS, 0, c->stream>>>(c->d_geo, c->d_upair, c->ndof, npts, c->nelem[1],
                                                               c->nelem[2], c->nbasis[1], c->nbasis[2], cd, cr,
                                                               c->d_lin);
  else
    law_in_df_kernel<false><<<grid, LI_THREADS, 0, c->stream>>>(c->d_geo, c->d_upair, c->ndof, npts, c->nelem[1],
                                                                c->nelem[2], c->nbasis[1], c->nbasis[2], cd, cr,
                                                                c->d_lin);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

// RR += element residuals of the reference's laws from the precomputed law
// outputs (projection on pairs, gather per DOF).
int launch_res_law_df(Context *c, const double *preR, double *RR)
{
  const int npts = c->nquad * c->nquad * c->nquad;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (c->prof) {
    IGAP_CUDA(cudaEventCreate(&e0));
    IGAP_CUDA(cudaEventCreate(&e1));
    IGAP_CUDA(cudaEventRecord(e0, c->stream));
  }
  res_law_df_kernel<<<(unsigned)c->nelem_total, LI_THREADS, 0, c->stream>>>(c->d_geo, preR, npts, c->d_rel);
  count_launch();
  IGAP_CHECK_LAUNCH();
  if (c->prof) {
    IGAP_CUDA(cudaEventRecord(e1, c->stream));
    c->prof_ev[0].emplace_back(e0, e1);
    c->prof_launches[0]++;
    c->prof_elements[0] += c->nelem_total;
  }
  res_gather_kernel<<<152 * 4, 256, 0, c->stream>>>(c->d_rel, c->nelem[0], c->nelem[1], c->nelem[2],
                                                   c->nbasis[0], c->nbasis[1], c->nbasis[2], RR);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

}  // namespace igap
