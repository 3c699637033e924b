// Split-precision tangent assembly on the tensor cores (tcgen05, TF32x3).
//
// For one element the tangent block of the assembly loop,
//   K[(b,d),(c,e)] = sum_q sum_{k,l} R_q[b,k] w_q D_q[(d,k),(e,l)] R_q[c,l]
// (src/assmcore_iga.c:722-750), is evaluated as one GEMM per element
//   K^T[(d,c,e), b] = sum_{(q,k)} A[(d,c,e),(q,k)] B[b,(q,k)]
//   A[(d,c,e),(q,k)] = sum_l w_q D_q[(d,k),(e,l)] R_q[c,l]      (stage 1, FP32 CUDA cores)
//   B[b,(q,k)]       = R_q[b,k]
// with the 243 rows (d,c,e) in two M=128 tiles, N = 32 >= 27 columns b, and
// the reduction over 64 points x 10 derivative slots in chunks of K = 40
// (8 points x 5 slots).  Each operand is split into TF32 hi + lo parts and
// the three products hi.hi + hi.lo + lo.hi accumulate in FP32 in tensor
// memory; the epilogue reads TMEM and adds into the FP64 CSR values.
// The residual is not touched here (the FP64 element kernel computes it).
//
// One persistent CTA per SM walks the elements of one colour, so the CSR
// scatter is conflict-free as in the FP64 kernel.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdlib.h>

#include "common.cuh"
#include "element.cuh"
#include "df32.cuh"
#include "tcgen05.cuh"

namespace igap {

namespace {
constexpr int TC_THREADS = 256;
constexpr int KCH = 40;                    // K per chunk: 8 points x 5 slots
constexpr int NKT = KCH / 8;               // tf32 MMA K-steps per chunk (K = 8 each)
constexpr int A_TILE = 128 * 8 * 4;        // one (K-step, M-tile) block: 4096 B
constexpr int A_PIECE = NKT * 2 * A_TILE;  // 40960 B
constexpr int B_TILE = 32 * 8 * 4;         // 1024 B
constexpr int B_PIECE = NKT * B_TILE;      // 5120 B
constexpr uint32_t WAIT_LIMIT = 1u << 26;  // bounded polls of an mbarrier
constexpr uint32_t TMEM_COLS = 64;

// bounded acquire-wait until *p >= target (batched queue dependencies)
__device__ __forceinline__ bool tc_wait_count_ge(const int *p, int target)
{
  for (uint32_t i = 0; i < (1u << 24); i++) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    if (v >= target) return true;
    __nanosleep(128);
  }
  return false;
}

using tc::kmajor_off;
}  // namespace

struct TcSmem {
  unsigned char A[2 * A_PIECE];  // [piece][kstep][mtile][block]
  unsigned char B[2 * B_PIECE];  // [piece][kstep][block]
  uint64_t mbar;
  uint32_t taddr;
  int abort;
  ElemData E;
  PointScratch Pt[PW];
  double R[PW][NB * NDD];
  float Rf[PW][NB * NDD];
  float Dwf[PW][900];
  int64_t rowp[NE];          // CSR row offsets of the element's 81 rows (b,d)
  float wtf[PW];             // quadrature weights (constant-tangent path)
  float Dc[900];             // constant tangent (FP32) of the linear law
  int64_t base;              // batched launch: first queue item of this fetch
};

// ------------------------------------------------------------ self-test
// D (128 x 32) = A (128 x 16) . B (32 x 16)^T with small integers;
// variant 0: TF32, two K-steps, LBO = 128 / SBO = 256; variant 1: the same
// with LBO and SBO swapped; variant 2: BF16 (kind::f16), one K = 16 step,
// core matrices of 8 rows x 8 values (16 B), LBO = 128 / SBO = 256.
__global__ void tc_selftest_kernel(int variant, float *out, int *err)
{
  __shared__ __align__(1024) float sA[2][128 * 8];
  __shared__ __align__(1024) float sB[2][32 * 8];
  __shared__ uint64_t mbar;
  __shared__ uint32_t taddr_s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    tc::tmem_alloc(&taddr_s, 32);
    tc::tmem_relinquish();
  }
  if (tid == 0) tc::mbar_init(&mbar, 1);
  __nv_bfloat16 *hA = reinterpret_cast<__nv_bfloat16 *>(sA[0]), *hB = reinterpret_cast<__nv_bfloat16 *>(sB[0]);
  for (int i = tid; i < 128 * 16; i += blockDim.x) {
    const int r = i / 16, kk = i % 16;
    const float a = (float)(((r * 3 + kk * 5) % 7) - 3);
    if (variant == 2)
      hA[(r >> 3) * 128 + (kk >> 3) * 64 + (r & 7) * 8 + (kk & 7)] = __float2bfloat16_rn(a);
    else
      sA[kk / 8][kmajor_off(r, kk % 8) / 4] = a;
  }
  for (int i = tid; i < 32 * 16; i += blockDim.x) {
    const int n = i / 16, kk = i % 16;
    const float b = (float)(((n * 2 + kk * 3) % 5) - 2);
    if (variant == 2)
      hB[(n >> 3) * 128 + (kk >> 3) * 64 + (n & 7) * 8 + (kk & 7)] = __float2bfloat16_rn(b);
    else
      sB[kk / 8][kmajor_off(n, kk % 8) / 4] = b;
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = taddr_s;
  const uint32_t lbo = variant == 0 ? 128 : 256, sbo = variant == 0 ? 256 : 128;
  if (tid == 0) {
    if (variant == 2) {
      tc::mma_bf16(taddr, tc::smem_desc(tc::smem_u32(sA[0]), 128, 256), tc::smem_desc(tc::smem_u32(sB[0]), 128, 256),
                   tc::instr_desc(1, 128, 32), 0u);
    } else {
      for (int kt = 0; kt < 2; kt++)
        tc::mma_tf32(taddr, tc::smem_desc(tc::smem_u32(sA[kt]), lbo, sbo),
                     tc::smem_desc(tc::smem_u32(sB[kt]), lbo, sbo), tc::instr_desc(2, 128, 32), kt > 0);
    }
    tc::mma_commit(&mbar);
  }
  if (!tc::mbar_wait(&mbar, 0, WAIT_LIMIT)) atomicExch(err, 1);
  tc::fence_after_sync();
  if (warp < 4) {
    uint32_t v[32];
    tc::tmem_ld_32x32b_x32(taddr + ((uint32_t)(warp * 32) << 16), v);
    for (int j = 0; j < 32; j++) out[(warp * 32 + lane) * 32 + j] = __uint_as_float(v[j]);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, 32);
}

// ------------------------------------------------------ split tangent
// One element on the tensor cores: phase A (FP32 basis and tangent
// integrand), stage 1 and B operands in shared memory, tcgen05 MMAs into
// TMEM, epilogue scatter into the CSR values.  `commits` counts the MMA
// commits of the CTA (mbarrier phase).  Returns false when a bounded wait
// expired (S.abort set).  COH: the CSR read-modify-write bypasses L1.
// PRE (law outputs of every point precomputed in FP32, FP64 geometry cache):
// each warp loads its point's basis and law outputs of the next chunk into
// registers while the current chunk's stage 1 and MMAs run (the same values
// as point_setup reads, so the tangent is bit-identical).
constexpr int PF_R = (NB * NDD + 31) / 32, PF_D = (900 + 31) / 32;

template <int LAWK>
__device__ __forceinline__ void tc_prefetch(double (&gR)[PF_R], float (&gD)[PF_D], const DevMesh &m,
                                            const DevLaw &L, int64_t eg, int q, int lane)
{
  const bool valid = q < m.npts;
  const double *g = m.geo + (eg * m.npts + (valid ? q : 0)) * GEO_STRIDE;
  const float *dsrc = L.preDf + eg * 900 * (int64_t)m.npts + (valid ? q : 0);
#pragma unroll
  for (int t = 0; t < PF_R; t++) {
    const int i = lane + 32 * t;
    gR[t] = (valid && i < NB * NDD) ? __ldg(g + i) : 0.0;
  }
#pragma unroll
  for (int t = 0; t < PF_D; t++) {
    const int i = lane + 32 * t;
    gD[t] = (valid && i < 900) ? __ldg(dsrc + (int64_t)i * m.npts) : 0.f;
  }
}

template <int LAWK, bool COH, bool PRE = false>
__device__ __forceinline__ bool tc_element(TcSmem &S, LawSmem<LAWK> &LS, const DevMesh &m, const DevLaw &L,
                                           int ex, int ey, int ez, bool const_d,
                                           const double *__restrict__ Uhist, double *__restrict__ vals,
                                           uint32_t taddr, uint32_t idesc, uint32_t a_base, uint32_t b_base,
                                           uint32_t &commits)
{
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nh = L.nhist;
  const int nb1 = m.nbasis[1], nb2 = m.nbasis[2];
  const int nbv[3] = {m.nbasis[0], nb1, nb2};
  const int nchunk = (m.npts + PW - 1) / PW;
  load_element(S.E, m, nh, Uhist, ex, ey, ez, tid, TC_THREADS);
  if (tid < NE) {
    const int b = tid / 3, dd = tid % 3;
    const int64_t cpb = ((int64_t)(ex + b / 9) * nb1 + (ey + (b / 3) % 3)) * nb2 + (ez + b % 3);
    S.rowp[tid] = __ldg(m.rowptr + 3 * cpb + dd);
  }
  __syncthreads();
  bool first = true;
  [[maybe_unused]] double gR[PRE ? PF_R : 1];
  [[maybe_unused]] float gD[PRE ? PF_D : 1];
  [[maybe_unused]] const int64_t eg = ((int64_t)ex * m.nelem[1] + ey) * m.nelem[2] + ez;
  if constexpr (PRE) tc_prefetch<LAWK>(gR, gD, m, L, eg, warp, lane);
  for (int ch = 0; ch < nchunk; ch++) {
    // phase A: 8 points, one warp each
    if constexpr (PRE) {
#pragma unroll
      for (int t = 0; t < PF_R; t++) {
        const int i = lane + 32 * t;
        if (i < NB * NDD) S.Rf[warp][i] = f64_to_pair(gR[t]).x;
      }
#pragma unroll
      for (int t = 0; t < PF_D; t++) {
        const int i = lane + 32 * t;
        if (i < 900) S.Dwf[warp][i] = gD[t];
      }
      if (ch + 1 < nchunk) tc_prefetch<LAWK>(gR, gD, m, L, eg, (ch + 1) * PW + warp, lane);
    } else if (const_d) {  // FP32 cached basis and weight; the tangent is constant
      const int q = ch * PW + warp;
      if (q < m.npts) {
        const int64_t eg = ((int64_t)ex * m.nelem[1] + ey) * m.nelem[2] + ez;
        const float *g = m.geof + (eg * m.npts + q) * GEO_STRIDE;
        for (int i = lane; i < NB * NDD; i += 32) S.Rf[warp][i] = __ldg(g + i);
        if (lane == 0) S.wtf[warp] = __ldg(g + NB * NDD);
      } else {
        for (int i = lane; i < NB * NDD; i += 32) S.Rf[warp][i] = 0.f;
        if (lane == 0) S.wtf[warp] = 0.f;
      }
    } else {  // FP64 geometry, FP32 tangent integrand
      point_setup<LAWK, false, true, float>(S.E, S.Pt[warp], LS, m, L, ex, ey, ez, warp,
                                            ch * PW + warp, lane, S.R[warp], nullptr, S.Dwf[warp]);
      // FP32 basis for the TF32 split, converted on the integer pipe
      for (int i = lane; i < NB * NDD; i += 32) S.Rf[warp][i] = f64_to_pair(S.R[warp][i]).x;
    }
    __syncthreads();
    for (int kg = 0; kg < 2; kg++) {
      // the previous chunk's MMAs must be done before A/B are overwritten
      if (commits > 0) {
        if (!tc::mbar_wait(&S.mbar, (commits - 1) & 1, WAIT_LIMIT)) S.abort = 1;
      }
      __syncthreads();
      if (S.abort) return false;
      // stage 1 (rows (d,c,e)) and B (rows b); columns kk = kq*8 + pt.
      // Loop order: 4 points at a time (R rows in registers), then the 5
      // derivative slots of this group; float4 stores of 4 points.
      if (tid < 243 && const_d) {
        // A = w_q * sum_l D[(d,k),(e,l)] R_q[c,l] with the constant D row
        // loaded once for the 4 points of a half
        const int d = tid / 81, c = (tid % 81) / 3, e = tid % 3;
        const int r = tid, mt = r >> 7;
        for (int half = 0; half < 2; half++) {
          float rc[4][NDD], wq[4];
#pragma unroll
          for (int j = 0; j < 4; j++) {
            wq[j] = S.wtf[half * 4 + j];
#pragma unroll
            for (int l = 0; l < NDD; l++) rc[j][l] = S.Rf[half * 4 + j][NDD * c + l];
          }
          for (int kq = 0; kq < 5; kq++) {
            const int k = kg * 5 + kq;
            float dr[NDD];
#pragma unroll
            for (int l = 0; l < NDD; l++) dr[l] = S.Dc[30 * (10 * d + k) + 10 * e + l];
            float4 hi, lo;
            float *ph = &hi.x, *pl = &lo.x;
#pragma unroll
            for (int j = 0; j < 4; j++) {
              float sacc = 0.f;
#pragma unroll
              for (int l = 0; l < NDD; l++) sacc = fmaf(dr[l], rc[j][l], sacc);
              sacc *= wq[j];
              const float h = tc::to_tf32(sacc);
              ph[j] = h;
              pl[j] = tc::to_tf32(sacc - h);
            }
            const uint32_t off = (uint32_t)((kq * 2 + mt) * A_TILE) + kmajor_off(r & 127, half * 4);
            *reinterpret_cast<float4 *>(S.A + off) = hi;
            *reinterpret_cast<float4 *>(S.A + A_PIECE + off) = lo;
          }
        }
      } else if (tid < 243) {
        const int d = tid / 81, c = (tid % 81) / 3, e = tid % 3;
        const int r = tid, mt = r >> 7;
        for (int half = 0; half < 2; half++) {
          float rc[4][NDD];
#pragma unroll
          for (int j = 0; j < 4; j++)
#pragma unroll
            for (int l = 0; l < NDD; l++) rc[j][l] = S.Rf[half * 4 + j][NDD * c + l];
          for (int kq = 0; kq < 5; kq++) {
            const int k = kg * 5 + kq;
            float4 hi, lo;
            float *ph = &hi.x, *pl = &lo.x;
#pragma unroll
            for (int j = 0; j < 4; j++) {
              const float *drow = S.Dwf[half * 4 + j] + 30 * (10 * d + k) + 10 * e;
              float sacc = 0.f;
#pragma unroll
              for (int l = 0; l < NDD; l++) sacc = fmaf(drow[l], rc[j][l], sacc);
              const float h = tc::to_tf32(sacc);
              ph[j] = h;
              pl[j] = tc::to_tf32(sacc - h);
            }
            const uint32_t off = (uint32_t)((kq * 2 + mt) * A_TILE) + kmajor_off(r & 127, half * 4);
            *reinterpret_cast<float4 *>(S.A + off) = hi;
            *reinterpret_cast<float4 *>(S.A + A_PIECE + off) = lo;
          }
        }
      }
      if (tid < NB) {
        const int b = tid;
        for (int kq = 0; kq < 5; kq++) {
          const int k = kg * 5 + kq;
          for (int half = 0; half < 2; half++) {
            float4 hi, lo;
            float *ph = &hi.x, *pl = &lo.x;
            for (int j = 0; j < 4; j++) {
              const float s = S.Rf[half * 4 + j][NDD * b + k];
              const float h = tc::to_tf32(s);
              ph[j] = h;
              pl[j] = tc::to_tf32(s - h);
            }
            const uint32_t off = (uint32_t)(kq * B_TILE) + kmajor_off(b, half * 4);
            *reinterpret_cast<float4 *>(S.B + off) = hi;
            *reinterpret_cast<float4 *>(S.B + B_PIECE + off) = lo;
          }
        }
      }
      tc::fence_proxy_async();
      tc::fence_before_sync();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
        for (int kt = 0; kt < NKT; kt++)
          for (int mt = 0; mt < 2; mt++)
            for (int pp = 0; pp < 3; pp++) {  // hi.hi, hi.lo, lo.hi
              const int pa = (pp == 2) ? 1 : 0, pb = (pp == 1) ? 1 : 0;
              const uint64_t ad = tc::smem_desc(a_base + pa * A_PIECE + (kt * 2 + mt) * A_TILE, 128, 256);
              const uint64_t bd = tc::smem_desc(b_base + pb * B_PIECE + kt * B_TILE, 128, 256);
              const uint32_t acc = (first && kt == 0 && pp == 0) ? 0u : 1u;
              tc::mma_tf32(taddr + (uint32_t)(mt * 32), ad, bd, idesc, acc);
            }
        tc::mma_commit(&S.mbar);
      }
      commits++;
      first = false;
    }
    __syncthreads();  // Rf / Dwf of this chunk are no longer read after the next wait
  }
  // epilogue: wait for the element's last MMAs, read TMEM, scatter
  if (!tc::mbar_wait(&S.mbar, (commits - 1) & 1, WAIT_LIMIT)) S.abort = 1;
  tc::fence_after_sync();
  __syncthreads();
  if (S.abort) return false;
  {
    // warp w reads tile (w / 4), TMEM lane quarter (w % 4)
    const int mt = warp >> 2, quarter = warp & 3;
    uint32_t v[32];
    tc::tmem_ld_32x32b_x32(taddr + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(mt * 32), v);
    const int r = mt * 128 + quarter * 32 + lane;
    if (r < 243) {
      const int d = r / 81, c = (r % 81) / 3, e = r % 3;
      const int sx = ex + c / 9, sy = ey + (c / 3) % 3, sz = ez + c % 3;
      for (int bi = 0; bi < 3; bi++) {  // 9 rows b at a time: loads first, then stores
        int64_t slot[9];
        double old[9];
#pragma unroll
        for (int t = 0; t < 9; t++) {
          const int b = 9 * bi + t;
          const int rx = ex + bi, ry = ey + t / 3, rz = ez + t % 3;
          slot[t] = S.rowp[3 * b + d] + 3 * stencil_pos(rx, ry, rz, sx, sy, sz, nbv) + e;
        }
#pragma unroll
        for (int t = 0; t < 9; t++) old[t] = COH ? __ldcg(vals + slot[t]) : vals[slot[t]];
#pragma unroll
        for (int t = 0; t < 9; t++) vals[slot[t]] = old[t] + (double)__uint_as_float(v[9 * bi + t]);
      }
    }
  }
  return true;
}

// TMEM allocation, mbarrier, zero padding rows (243..255 of A, 27..31 of B
// stay zero for the whole kernel).
__device__ __forceinline__ void tc_setup(TcSmem &S)
{
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    tc::tmem_alloc(&S.taddr, TMEM_COLS);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&S.mbar, 1);
    S.abort = 0;
  }
  for (int i = tid; i < (int)(sizeof(S.A) / 4); i += TC_THREADS) reinterpret_cast<float *>(S.A)[i] = 0.f;
  for (int i = tid; i < (int)(sizeof(S.B) / 4); i += TC_THREADS) reinterpret_cast<float *>(S.B)[i] = 0.f;
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
}

__device__ __forceinline__ void tc_teardown(TcSmem &S, uint32_t taddr, int *err)
{
  tc::fence_before_sync();
  __syncthreads();
  if (S.abort && threadIdx.x == 0) atomicCAS(err, 0, 2);
  if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(taddr, TMEM_COLS);
}

// One persistent CTA per SM walks the elements of one colour.
template <int LAWK, bool PRE>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_tangent_kernel(DevMesh m, DevLaw L, int cx, int cy, int cz, int ncx, int ncy, int ncz,
                      const double *__restrict__ Uhist, double *__restrict__ vals, int *err)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcSmem &S = *reinterpret_cast<TcSmem *>(smem_raw);
  LawSmem<LAWK> &LS = *reinterpret_cast<LawSmem<LAWK> *>(smem_raw + sizeof(TcSmem));
  const int tid = threadIdx.x;
  tc_setup(S);
  const uint32_t taddr = S.taddr;
  const uint32_t idesc = tc::instr_desc(2, 128, 32);
  const uint32_t a_base = tc::smem_u32(S.A), b_base = tc::smem_u32(S.B);
  uint32_t commits = 0;  // commits issued so far (uniform across the CTA)
  const int nelem_c = ncx * ncy * ncz;
  // constant sparse tangent (linear law) with the FP32 geometry cache
  const bool const_d = (LAWK == 0) && m.geof != nullptr && L.Dconst != nullptr;
  if (const_d)
    for (int i = tid; i < 900; i += TC_THREADS) S.Dc[i] = (float)L.Dconst[i];
  __syncthreads();
  for (int ei = blockIdx.x; ei < nelem_c; ei += gridDim.x) {
    const int iz = ei % ncz, iy = (ei / ncz) % ncy, ix = ei / (ncz * ncy);
    if (!tc_element<LAWK, false, PRE>(S, LS, m, L, cx + 3 * ix, cy + 3 * iy, cz + 3 * iz, const_d, Uhist, vals,
                                      taddr, idesc, a_base, b_base, commits))
      break;
    tc::fence_before_sync();
    __syncthreads();
  }
  tc_teardown(S, taddr, err);
}

// Batched launch: elements come from the colour-major queue of a batch (see
// element_batch_kernel); mesh and law of the current instance live in shared
// memory.
template <int LAWK>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_batch_kernel(BatchArgs ba, const double *__restrict__ Uhist, double *__restrict__ vals)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcSmem &S = *reinterpret_cast<TcSmem *>(smem_raw);
  LawSmem<LAWK> &LS = *reinterpret_cast<LawSmem<LAWK> *>(smem_raw + sizeof(TcSmem));
  const int tid = threadIdx.x;
  tc_setup(S);
  const uint32_t taddr = S.taddr;
  const uint32_t idesc = tc::instr_desc(2, 128, 32);
  const uint32_t a_base = tc::smem_u32(S.A), b_base = tc::smem_u32(S.B);
  uint32_t commits = 0;
  bool const_d = false;
  int cur = -1;
  DevMesh m;  // current instance, in registers
  DevLaw L;
  int64_t next = 0;  // queue position of the following fetch, reserved one fetch ahead
  if (tid == 0) next = atomicAdd(ba.head, ba.grab);
  for (;;) {
    if (tid == 0) S.base = next;
    __syncthreads();
    const int64_t base = S.base;
    __syncthreads();
    if (base >= ba.nitems || S.abort) break;
    if (tid == 0) next = atomicAdd(ba.head, ba.grab);
    const int64_t end = base + ba.grab < ba.nitems ? base + ba.grab : ba.nitems;
    bool ok = true;
    for (int64_t it = base; it < end && ok; it++) {
      const BatchItem w = ba.items[it];
      if (w.inst != cur) {
        __syncthreads();  // the previous instance's constant tangent is no longer read
        m = ba.meshes[w.inst];
        L = ba.laws[w.inst];
        cur = w.inst;
        const_d = (LAWK == 0) && m.geof != nullptr && L.Dconst != nullptr;
        if (const_d)
          for (int i = tid; i < 900; i += TC_THREADS) S.Dc[i] = (float)L.Dconst[i];
      }
      if (tid == 0 && w.col > 0) {
        if (!tc_wait_count_ge(ba.done + w.inst, ba.need[27 * w.inst + w.col])) {
          S.abort = 1;
          atomicExch(ba.err, 3);
        }
      }
      __syncthreads();
      if (S.abort) {
        ok = false;
        break;
      }
      ok = tc_element<LAWK, true>(S, LS, m, L, w.ex, w.eyz >> 16, w.eyz & 0xffff, const_d, Uhist, vals,
                                  taddr, idesc, a_base, b_base, commits);
      if (!ok) break;
      tc::fence_before_sync();
      __syncthreads();
      if (tid == 0)  // release at GPU scope after the barrier (see release_add)
        asm volatile("fence.acq_rel.gpu;\n\tred.relaxed.gpu.global.add.s32 [%0], 1;" ::"l"(ba.done + w.inst) : "memory");
    }
    if (!ok) break;
  }
  tc_teardown(S, taddr, ba.err);
}

template <int LAWK>
static int run_tc(Context *c, const DevLaw &L, double *vals)
{
  const DevMesh m = c->devmesh();
  const size_t smem = sizeof(TcSmem) + sizeof(LawSmem<LAWK>) + 1024;
  // precomputed FP32 law outputs: the prefetching form (IGAPGPU_TC_PREFETCH=0
  // keeps the point_setup form)
  const char *pf = getenv("IGAPGPU_TC_PREFETCH");
  const bool pre = LAWK != 0 && m.geo && L.preR && L.preDf && !(pf && pf[0] == '0');
  auto kern = pre ? tc_tangent_kernel<LAWK, LAWK != 0> : tc_tangent_kernel<LAWK, false>;
  static bool attr[2] = {false, false};
  if (!attr[pre]) {
    IGAP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr[pre] = true;
  }
  int dev = 0, nsm = 0;
  IGAP_CUDA(cudaGetDevice(&dev));
  IGAP_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
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
        const int nel = ncx * ncy * ncz;
        if (nel <= 0) continue;
        const int grid = nel < nsm ? nel : nsm;
        kern<<<grid, TC_THREADS, smem, c->stream>>>(m, L, cx, cy, cz, ncx, ncy, ncz, c->d_Uhist, vals,
                                                    c->d_err);
        count_launch();
        IGAP_CHECK_LAUNCH();
        if (c->prof) {
          c->prof_launches[1]++;
          c->prof_elements[1] += nel;
        }
      }
  if (c->prof) {
    IGAP_CUDA(cudaEventRecord(e1, c->stream));
    c->prof_ev[1].emplace_back(e0, e1);
  }
  return IGAPGPU_OK;
}

template <int LAWK>
static int run_tc_batch(Context *c, const BatchArgs &a, int grid, const double *Uhist, double *vals)
{
  const size_t smem = sizeof(TcSmem) + sizeof(LawSmem<LAWK>) + 1024;
  auto kern = tc_batch_kernel<LAWK>;
  static bool attr = false;
  if (!attr) {
    IGAP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  kern<<<grid, TC_THREADS, smem, c->stream>>>(a, Uhist, vals);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

int launch_tc_batch(Context *c, const BatchArgs &a, int law, int grid, const double *Uhist, double *vals)
{
  if (law == IGAPGPU_LAW_LINGRAD) return run_tc_batch<0>(c, a, grid, Uhist, vals);
  if (law == IGAPGPU_LAW_GRADELAST) return run_tc_batch<1>(c, a, grid, Uhist, vals);
  if (law == IGAPGPU_LAW_GRADELASTTIME) return run_tc_batch<2>(c, a, grid, Uhist, vals);
  set_error("unknown law %d", law);
  return IGAPGPU_ERR_LAW;
}

int launch_tc_tangent(Context *c, double *vals, const DevLaw &L)
{
  if (c->law == IGAPGPU_LAW_LINGRAD && c->d_geof && !getenv("IGAPGPU_TC_DENSE")) return launch_tc_gram(c, vals);
  if (c->law == IGAPGPU_LAW_LINGRAD) return run_tc<0>(c, L, vals);
  if (c->law == IGAPGPU_LAW_GRADELAST) return run_tc<1>(c, L, vals);
  if (c->law == IGAPGPU_LAW_GRADELASTTIME) return run_tc<2>(c, L, vals);
  set_error("unknown law %d", c->law);
  return IGAPGPU_ERR_LAW;
}

}  // namespace igap

using namespace igap;

extern "C" int igapgpu_tc_selftest(int variant, float *out)
{
  float *d_out = nullptr;
  int *d_err = nullptr;
  IGAP_CUDA(cudaMalloc(&d_out, sizeof(float) * 128 * 32));
  IGAP_CUDA(cudaMalloc(&d_err, sizeof(int)));
  IGAP_CUDA(cudaMemset(d_err, 0, sizeof(int)));
  tc_selftest_kernel<<<1, 128>>>(variant, d_out, d_err);
  count_launch();
  IGAP_CHECK_LAUNCH();
  int herr = 0;
  IGAP_CUDA(cudaMemcpy(out, d_out, sizeof(float) * 128 * 32, cudaMemcpyDeviceToHost));
  IGAP_CUDA(cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost));
  cudaFree(d_out);
  cudaFree(d_err);
  if (herr) {
    set_error("tcgen05 self-test: mbarrier wait timed out");
    return IGAPGPU_ERR_TIMEOUT;
  }
  return IGAPGPU_OK;
}
