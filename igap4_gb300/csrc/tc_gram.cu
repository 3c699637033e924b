// Split-precision tangent of the linear isotropic strain-gradient law on the
// tensor cores, in Gram form.
//
// For this law the tangent block of basis functions b, c is
//   K[(b,d),(c,e)] = lam G[(b,d),(c,e)] + mu G[(b,e),(c,d)] + delta_de mu sum_i G[(b,i),(c,i)]
// with the Gram matrix (rows (b,i), columns (c,j), i,j = 0..2)
//   G[(b,i),(c,j)] = sum_q w_q ( dN_b/dx_i dN_c/dx_j + ell^2 sum_m d2N_b/dx_i dx_m d2N_c/dx_j dx_m ),
// the same sum as the assembly loop's R^T D R (src/assmcore_iga.c:722-750)
// with this law's constant D.  Per element that is one GEMM
//   G = A . B^T,  A[(b,i), k] = w_q [dN_b/dx_i | ell^2 d2N_b/dx_i dx_m],
//                 B[(c,j), k] = [dN_c/dx_j | d2N_c/dx_j dx_m],
// M = 81 rows (one 128-row tile), N = 81 columns (96), K = 64 points x (1 + 3)
// = 256, processed in chunks of 8 points (K = 32 = 4 tf32 K-steps).  A and B
// come straight from the FP32 geometry cache: each chunk's 8 point rows
// (8 x 1088 contiguous bytes) are fetched by a bulk asynchronous copy one
// chunk ahead, the operands are split into TF32 hi + lo, and hi.hi + hi.lo +
// lo.hi accumulate in FP32 in tensor memory (tcgen05.mma kind::tf32).  The
// operand buffers are double buffered: chunk n+1 is built while the MMAs of
// chunk n run.  The epilogue stages G in shared memory, forms K and adds it
// into the FP64 CSR values.  Every mbarrier wait is bounded.
#include <cuda_runtime.h>
#include <stdlib.h>

#include "common.cuh"
#include "element.cuh"
#include "tcgen05.cuh"
#include "gram_common.cuh"

namespace igap {

namespace {
constexpr int G_THREADS = 256;
constexpr int GROWS = 81;                    // (b,i) rows / (c,j) columns
constexpr int GN = 96;                       // MMA N (>= 81, multiple of 16)
constexpr int GKS = 4;                       // K-steps per chunk (K = 32)
constexpr int GA_TILE = 128 * 8 * 4;         // one K-step of A: 4096 B
constexpr int GB_TILE = GN * 8 * 4;          // one K-step of B: 3072 B
constexpr int GA_PIECE = GKS * GA_TILE;      // 16384 B (hi or lo)
constexpr int GB_PIECE = GKS * GB_TILE;      // 12288 B
constexpr int PT_FLOATS = GEO_STRIDE;        // 272 floats per cached point
constexpr uint32_t G_WAIT_LIMIT = 1u << 26;
constexpr uint32_t G_TMEM_COLS = 128;
constexpr int GPAD = 84;                     // row stride of the staged Gram matrix


__device__ __forceinline__ bool tc_wait_ge(const int *p, int target)
{
  for (uint32_t i = 0; i < (1u << 24); i++) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    if (v >= target) return true;
    __nanosleep(128);
  }
  return false;
}
}  // namespace

// K[(b,d),(c,e)] = lam G[(b,d),(c,e)] + mu G[(b,e),(c,d)] + delta_de mu tr G_bc
// for every (b,d), (c,e) (6,561 slots, each once per element), added into the
// FP64 CSR values by fire-and-forget reductions at L2: no load latency and no
// FP64 add on the SM.  Within a colour no two elements share a slot and the
// colours are ordered, so every slot still receives its contributions in
// colour order (the same sums, bit for bit, as a read-modify-write).
template <typename PosT>
__device__ __forceinline__ void gram_scatter(const float *G, const int64_t *rowp, const PosT *pos, const DevLaw &L,
                                             double *__restrict__ vals, int first = -1, int nthreads = G_THREADS)
{
  const float lam = (float)L.par[0], mu = (float)L.par[1];
  for (int t = first < 0 ? (int)threadIdx.x : first; t < NE * NE; t += nthreads) {
    const int rr = t / NE, cc = t - NE * rr;
    const int b = rr / 3, d = rr - 3 * b, c = cc / 3, e = cc - 3 * c;
    float kk = lam * G[(3 * b + d) * GPAD + 3 * c + e] + mu * G[(3 * b + e) * GPAD + 3 * c + d];
    if (d == e)
      kk += mu * (G[(3 * b) * GPAD + 3 * c] + G[(3 * b + 1) * GPAD + 3 * c + 1] + G[(3 * b + 2) * GPAD + 3 * c + 2]);
    double *dst = vals + rowp[rr] + 3 * (int)pos[NB * b + c] + e;
    asm volatile("red.relaxed.gpu.global.add.f64 [%0], %1;" ::"l"(dst), "d"(f32_to_f64(kk)) : "memory");
  }
}

struct TcgSmem {
  unsigned char A[2 * GA_PIECE];     // [hi, lo][K-step][4096 B]; the Gram matrix is staged here after the MMAs
  unsigned char B[2 * GB_PIECE];     // [hi, lo][K-step][3072 B]
  float Rf[2][PW * PT_FLOATS];       // [buffer] 8 cached point rows
  int pos[NB * NB];                  // stencil position of column point c in the row of point b
  int64_t rowp[NE];
  uint64_t mbar_mma;
  uint64_t mbar_cp[2];
  uint32_t taddr;
  int abort;
  int64_t base;
};
static_assert(GROWS * GPAD * 4 <= 2 * GA_PIECE, "the staged Gram matrix fits in the A buffer");

// Barrier phase bookkeeping of one CTA (uniform across its threads).
struct TcgState {
  uint32_t mma_n;     // commits issued to mbar_mma
  uint32_t cp_n[2];   // copies issued to mbar_cp[b]
};

// Operand tasks of one thread, fixed for the whole kernel: task j covers
// 4 consecutive K slots of one row of A or B in one K-step.  dst: byte offset
// in its operand (bit 31 set for B), 0xffffffff if the thread has no task j;
// code: per slot the source float in the chunk's point rows (12 bits), the
// point (3 bits), whether it is a Hessian slot (1 bit).
constexpr int NTASK = (2 * GROWS * GKS * 2 + G_THREADS - 1) / G_THREADS;  // 6
struct TcgTasks {
  uint32_t dst[NTASK];
  uint64_t code[NTASK];
};

__device__ __forceinline__ void tcg_make_tasks(TcgTasks &T)
{
#pragma unroll
  for (int j = 0; j < NTASK; j++) {
    const int t = threadIdx.x + j * G_THREADS;
    if (t >= 2 * GROWS * GKS * 2) {
      T.dst[j] = 0xffffffffu;
      T.code[j] = 0;
      continue;
    }
    const int mat = t / (GROWS * GKS * 2), u = t % (GROWS * GKS * 2);
    const int r = u % GROWS, ks = (u / GROWS) % GKS, half = u / (GROWS * GKS);
    const int bsf = r / 3, i = r % 3;
    T.dst[j] = (uint32_t)(ks * (mat == 0 ? GA_TILE : GB_TILE)) + tc::kmajor_off(r, half * 4) |
               (mat ? 0x80000000u : 0u);
    uint64_t code = 0;
    for (int jj = 0; jj < 4; jj++) {
      const int k = ks * 8 + half * 4 + jj;
      int p, idx, hess;
      if (k < PW) {  // gradient part: one slot per point
        p = k;
        idx = 1 + i;
        hess = 0;
      } else {       // Hessian part: three slots per point
        p = (k - PW) / 3;
        idx = 4 + hess_slot(i, (k - PW) % 3);
        hess = 1;
      }
      const uint64_t cj = (uint64_t)(p * PT_FLOATS + NDD * bsf + idx) | ((uint64_t)p << 12) | ((uint64_t)hess << 15);
      code |= cj << (16 * jj);
    }
    T.code[j] = code;
  }
}

__device__ __forceinline__ void tcg_issue_copy(TcgSmem &S, TcgState &st, const float *gsrc, int npts, int ch)
{
  const int rb = ch & 1;
  const int q0 = ch * PW;
  const int nv = npts - q0 < PW ? npts - q0 : PW;
  if (threadIdx.x == 0) {
    tc::fence_proxy_async();
    tc::mbar_arrive_expect_tx(&S.mbar_cp[rb], (uint32_t)(nv * PT_FLOATS * 4));
    tc::bulk_g2s(S.Rf[rb], gsrc + (size_t)q0 * PT_FLOATS, (uint32_t)(nv * PT_FLOATS * 4), &S.mbar_cp[rb]);
  }
  st.cp_n[rb]++;
}

// One element.  Returns false when a bounded wait expired (S.abort set).
template <bool COH>
__device__ __forceinline__ bool tcg_element(TcgSmem &S, TcgState &st, const TcgTasks &T, const DevMesh &m,
                                            const DevLaw &L, int ex, int ey, int ez, double *__restrict__ vals,
                                            uint32_t taddr, uint32_t a_base, uint32_t b_base)
{
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nb1 = m.nbasis[1], nb2 = m.nbasis[2];
  const int nbv[3] = {m.nbasis[0], nb1, nb2};
  const int npts = m.npts;
  const int nchunk = (npts + PW - 1) / PW;
  const int64_t eg = ((int64_t)ex * m.nelem[1] + ey) * m.nelem[2] + ez;
  const float *gsrc = m.geof + eg * npts * PT_FLOATS;
  const float l2 = (float)(L.par[2] * L.par[2]);
  const uint32_t idesc = tc::instr_desc(2, 128, GN);
  tcg_issue_copy(S, st, gsrc, npts, 0);
  if (tid < NE) {
    const int b = tid / 3, dd = tid % 3;
    const int64_t cpb = ((int64_t)(ex + b / 9) * nb1 + (ey + (b / 3) % 3)) * nb2 + (ez + b % 3);
    S.rowp[tid] = __ldg(m.rowptr + 3 * cpb + dd);
  }
  for (int t = tid; t < NB * NB; t += G_THREADS) {
    const int b = t / NB, c = t % NB;
    S.pos[t] = (int)stencil_pos(ex + b / 9, ey + (b / 3) % 3, ez + b % 3, ex + c / 9, ey + (c / 3) % 3,
                                ez + c % 3, nbv);
  }
  for (int ch = 0; ch < nchunk; ch++) {
    const int rb = ch & 1;
    if (ch + 1 < nchunk) tcg_issue_copy(S, st, gsrc, npts, ch + 1);  // its buffer was last read by chunk ch-1
    bool ok = tc::mbar_wait(&S.mbar_cp[rb], (st.cp_n[rb] - 1) & 1, G_WAIT_LIMIT);
    // the operands are single buffered: the previous MMAs must be done
    if (ok && st.mma_n > 0) ok = tc::mbar_wait(&S.mbar_mma, (st.mma_n - 1) & 1, G_WAIT_LIMIT);
    if (!ok) S.abort = 1;
    __syncthreads();
    if (S.abort) return false;
    const float *R = S.Rf[rb];
    const int q0 = ch * PW;
#pragma unroll
    for (int j = 0; j < NTASK; j++) {
      const uint32_t dst = T.dst[j];
      if (dst == 0xffffffffu) continue;
      const bool isB = (dst >> 31) != 0;
      float4 hi, lo;
      float *ph = &hi.x, *pl = &lo.x;
#pragma unroll
      for (int jj = 0; jj < 4; jj++) {
        const uint32_t code = (uint32_t)(T.code[j] >> (16 * jj)) & 0xffffu;
        const int src = (int)(code & 4095u), p = (int)((code >> 12) & 7u);
        float v = 0.f;
        if (q0 + p < npts) {
          v = R[src];
          if (!isB) v *= ((code >> 15) ? l2 : 1.f) * R[p * PT_FLOATS + NB * NDD];  // A carries w_q (and ell^2)
        }
        const float h = tc::to_tf32(v);
        ph[jj] = h;
        pl[jj] = tc::to_tf32(v - h);
      }
      unsigned char *base = isB ? S.B : S.A;
      const int piece = isB ? GB_PIECE : GA_PIECE;
      const uint32_t off = dst & 0x7fffffffu;
      *reinterpret_cast<float4 *>(base + off) = hi;
      *reinterpret_cast<float4 *>(base + piece + off) = lo;
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      for (int ks = 0; ks < GKS; ks++)
        for (int pp = 0; pp < 3; pp++) {  // hi.hi, hi.lo, lo.hi
          const int pa = (pp == 2) ? 1 : 0, pb = (pp == 1) ? 1 : 0;
          const uint64_t ad = tc::smem_desc(a_base + (uint32_t)(pa * GA_PIECE + ks * GA_TILE), 128, 256);
          const uint64_t bd = tc::smem_desc(b_base + (uint32_t)(pb * GB_PIECE + ks * GB_TILE), 128, 256);
          tc::mma_tf32(taddr, ad, bd, idesc, (ch == 0 && ks == 0 && pp == 0) ? 0u : 1u);
        }
      tc::mma_commit(&S.mbar_mma);
    }
    st.mma_n++;
  }
  // epilogue: the last commit covers every MMA of the element
  if (!tc::mbar_wait(&S.mbar_mma, (st.mma_n - 1) & 1, G_WAIT_LIMIT)) S.abort = 1;
  tc::fence_after_sync();
  __syncthreads();
  if (S.abort) return false;
  float *G = reinterpret_cast<float *>(S.A);  // operands are no longer read
  {
    // warp w reads TMEM lane quarter (w % 4), columns [32 (w / 4), +32) and, for
    // w < 4, also [64, 96)
    const int quarter = warp & 3;
    const int r = quarter * 32 + lane;
    for (int cb = warp >> 2; cb < 3; cb += 2) {
      uint32_t v[32];
      tc::tmem_ld_32x32b_x32(taddr + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(cb * 32), v);
      if (r < GROWS)
#pragma unroll
        for (int j = 0; j < 32; j++)
          if (cb * 32 + j < GROWS) G[r * GPAD + cb * 32 + j] = __uint_as_float(v[j]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  gram_scatter(G, S.rowp, S.pos, L, vals);
  return true;
}

__device__ __forceinline__ void tcg_setup(TcgSmem &S)
{
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    tc::tmem_alloc(&S.taddr, G_TMEM_COLS);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&S.mbar_mma, 1);
    for (int b = 0; b < 2; b++) tc::mbar_init(&S.mbar_cp[b], 1);
    S.abort = 0;
  }
  // padding rows 81..95 of B stay zero for the whole kernel; rows 81..127 of A
  // only feed accumulator rows that are never read
  for (int i = tid; i < (int)(sizeof(S.A) / 4); i += G_THREADS) reinterpret_cast<float *>(S.A)[i] = 0.f;
  for (int i = tid; i < (int)(sizeof(S.B) / 4); i += G_THREADS) reinterpret_cast<float *>(S.B)[i] = 0.f;
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
}

// Teardown: on an abort, wait (bounded) for copies still in flight before the
// CTA's shared memory is released; then free TMEM.
__device__ __forceinline__ void tcg_teardown(TcgSmem &S, const TcgState &st, int *err)
{
  tc::fence_before_sync();
  __syncthreads();
  if (S.abort) {
    for (int b = 0; b < 2; b++)
      if (st.cp_n[b] > 0) tc::mbar_wait(&S.mbar_cp[b], (st.cp_n[b] - 1) & 1, G_WAIT_LIMIT);
    if (st.mma_n > 0) tc::mbar_wait(&S.mbar_mma, (st.mma_n - 1) & 1, G_WAIT_LIMIT);
    if (threadIdx.x == 0) atomicCAS(err, 0, 2);
  }
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(S.taddr, G_TMEM_COLS);
}

__global__ void __launch_bounds__(G_THREADS, 2)
    tcg_kernel(DevMesh m, DevLaw L, int cx, int cy, int cz, int ncx, int ncy, int ncz, double *__restrict__ vals,
               int *err)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcgSmem &S = *reinterpret_cast<TcgSmem *>(smem_raw);
  tcg_setup(S);
  const uint32_t taddr = S.taddr, a_base = tc::smem_u32(S.A), b_base = tc::smem_u32(S.B);
  TcgState st = {0, {0, 0}};
  TcgTasks T;
  tcg_make_tasks(T);
  const int nelem_c = ncx * ncy * ncz;
  for (int ei = blockIdx.x; ei < nelem_c; ei += gridDim.x) {
    const int iz = ei % ncz, iy = (ei / ncz) % ncy, ix = ei / (ncz * ncy);
    if (!tcg_element<false>(S, st, T, m, L, cx + 3 * ix, cy + 3 * iy, cz + 3 * iz, vals, taddr, a_base, b_base))
      break;
    tc::fence_before_sync();
    __syncthreads();
  }
  tcg_teardown(S, st, err);
}

// Batched: elements from the colour-major queue (see element_batch_kernel).
__global__ void __launch_bounds__(G_THREADS, 2) tcg_batch_kernel(BatchArgs ba, double *__restrict__ vals)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcgSmem &S = *reinterpret_cast<TcgSmem *>(smem_raw);
  const int tid = threadIdx.x;
  tcg_setup(S);
  const uint32_t taddr = S.taddr, a_base = tc::smem_u32(S.A), b_base = tc::smem_u32(S.B);
  TcgState st = {0, {0, 0}};
  TcgTasks T;
  tcg_make_tasks(T);
  int cur = -1;
  DevMesh m;
  DevLaw L;
  int64_t next = 0;
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
    for (int64_t it = base; it < end; it++) {
      const BatchItem w = ba.items[it];
      if (w.inst != cur) {
        m = ba.meshes[w.inst];
        L = ba.laws[w.inst];
        cur = w.inst;
      }
      if (tid == 0 && w.col > 0) {
        if (!tc_wait_ge(ba.done + w.inst, ba.need[27 * w.inst + w.col])) {
          S.abort = 1;
          atomicExch(ba.err, 3);
        }
      }
      __syncthreads();
      if (S.abort) {
        ok = false;
        break;
      }
      ok = tcg_element<true>(S, st, T, m, L, w.ex, w.eyz >> 16, w.eyz & 0xffff, vals, taddr, a_base, b_base);
      if (!ok) break;
      tc::fence_before_sync();
      __syncthreads();
      if (tid == 0)  // release at GPU scope after the barrier
        asm volatile("fence.acq_rel.gpu;\n\tred.relaxed.gpu.global.add.s32 [%0], 1;" ::"l"(ba.done + w.inst)
                     : "memory");
    }
    if (!ok) break;
  }
  tcg_teardown(S, st, ba.err);
}

// ------------------------------------------------- cached-operand variant
// With the point weight split symmetrically, the Gram matrix is S S^T,
//   S[(b,i), (q,0)]   = sqrt(w_q) dN_b/dx_i,
//   S[(b,i), (q,1+m)] = sqrt(w_q) ell d2N_b/dx_i dx_m,
// which depends only on the geometry and ell.  It is built once per context
// in FP32, already in the MMA operand layout: per element and chunk of 8
// points, 4 K-steps of 11 row groups (rows 0..87, rows 81..87 zero) of
// 8 rows x 32 B.  Each chunk is then one bulk copy; the kernel only splits it
// into TF32 hi + lo, and the same shared-memory tile is both MMA operands.
// An MMA of M = 128 (N = 96) rows reads past row 87 into the next K-step's
// rows: those products land in accumulator rows (columns) >= 88, never read.
constexpr int S_RG = 11;                                     // row groups with rows 0..87
constexpr int S_KS_BYTES = S_RG * 256;                       // 2816: one K-step
constexpr int S_CH_BYTES = GKS * S_KS_BYTES;                 // 11264: one chunk of 8 points
constexpr int S_OP_BYTES = (GKS - 1) * S_KS_BYTES + 128 * 32; // 12544: the last K-step's M = 128 read stays inside
// copy stages x CTAs per SM: 2 x 3 (default; measured 6.9 ms per tangent at
// 128x32x32) or 4 x 2 (IGAPGPU_TCS_CTAS=2; 8.0 ms)

// out[e][chunk][K-step][row group][K half][row][4]; bad = 1 when a point
// weight is not positive (the symmetric split needs sqrt(w)).
__global__ void gram_operand_kernel(const double *__restrict__ geo, int npts, int nchunk, int64_t nelem, double ell,
                                    float *__restrict__ out, int *__restrict__ bad)
{
  constexpr int CHF = S_CH_BYTES / 4, KSF = S_KS_BYTES / 4;
  const int64_t per_elem = (int64_t)nchunk * CHF;
  const int64_t total = nelem * per_elem;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / per_elem;
    int u = (int)(t - e * per_elem);
    const int ch = u / CHF;
    u -= ch * CHF;
    const int ks = u / KSF;
    u -= ks * KSF;
    const int rg = u / 64, half = (u % 64) / 32, r8 = (u % 32) / 4, f = u % 4;
    const int r = rg * 8 + r8, kk = ks * 8 + half * 4 + f;
    float v = 0.f;
    if (r < GROWS) {
      const int b = r / 3, i = r % 3;
      int p, slot;
      bool hess;
      if (kk < PW) {
        p = kk;
        slot = 1 + i;
        hess = false;
      } else {
        p = (kk - PW) / 3;
        slot = 4 + hess_slot(i, (kk - PW) % 3);
        hess = true;
      }
      const int q = ch * PW + p;
      if (q < npts) {
        const double *g = geo + (e * npts + q) * GEO_STRIDE;
        const double w = g[NB * NDD];
        if (w > 0.0)
          v = (float)(sqrt(w) * (hess ? ell : 1.0) * g[NDD * b + slot]);
        else
          atomicExch(bad, 1);
      }
    }
    out[t] = v;
  }
}

template <int NS>
struct TcsSmem {
  unsigned char op[2][2][S_OP_BYTES];  // [buffer][hi, lo]; the Gram matrix is staged here after the MMAs
  unsigned char val[NS][S_CH_BYTES];   // bulk-copy stages
  unsigned char pos[NB * NB];          // stencil position (< 125) of column point c in the row of point b
  int64_t rowp[NE];
  uint64_t mbar_cp[NS];
  uint64_t mbar_mma[2];
  uint32_t taddr;
  int abort;
  int64_t base;
};
static_assert(GROWS * GPAD * 4 <= 2 * 2 * S_OP_BYTES, "the staged Gram matrix fits in the operand buffers");
static_assert((2 * P + 1) * (2 * P + 1) * (2 * P + 1) <= 256, "stencil positions fit in a byte");

// Pipeline counters of one CTA (uniform across its threads): the chunk
// stream runs over the CTA's elements; copies are issued up to NS chunks
// ahead of the chunk being consumed, across element boundaries when the next
// element is known.
template <int NS>
struct TcsState {
  uint32_t cp_n[NS];    // copies issued per stage
  uint32_t mma_n[2];    // commits per operand buffer
  uint32_t issued, consumed, elem_start;
};

template <int NS>
__device__ __forceinline__ void tcs_issue(TcsSmem<NS> &S, TcsState<NS> &st, const unsigned char *src)
{
  const int sg = (int)(st.issued % NS);
  if (threadIdx.x == 0) {
    tc::fence_proxy_async();
    tc::mbar_arrive_expect_tx(&S.mbar_cp[sg], (uint32_t)S_CH_BYTES);
    tc::bulk_g2s(S.val[sg], src, (uint32_t)S_CH_BYTES, &S.mbar_cp[sg]);
  }
  st.cp_n[sg]++;
  st.issued++;
}

// One element from its cached operands esrc (nsrc: the next element of this
// CTA, prefetched, or null).  Returns false when a bounded wait expired.
template <int NS, bool COH>
__device__ __forceinline__ bool tcs_element(TcsSmem<NS> &S, TcsState<NS> &st, const DevMesh &m, const DevLaw &L, int ex,
                                            int ey, int ez, const unsigned char *esrc, const unsigned char *nsrc,
                                            double *__restrict__ vals, uint32_t taddr, uint32_t op_base)
{
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nb1 = m.nbasis[1], nb2 = m.nbasis[2];
  const int nbv[3] = {m.nbasis[0], nb1, nb2};
  const uint32_t nchunk = (uint32_t)((m.npts + PW - 1) / PW);
  const uint32_t idesc = tc::instr_desc(2, 128, GN);
  if (tid < NE) {
    const int b = tid / 3, dd = tid % 3;
    const int64_t cpb = ((int64_t)(ex + b / 9) * nb1 + (ey + (b / 3) % 3)) * nb2 + (ez + b % 3);
    S.rowp[tid] = __ldg(m.rowptr + 3 * cpb + dd);
  }
  for (int t = tid; t < NB * NB; t += G_THREADS) {
    const int b = t / NB, c = t % NB;
    S.pos[t] = (unsigned char)stencil_pos(ex + b / 9, ey + (b / 3) % 3, ez + b % 3, ex + c / 9, ey + (c / 3) % 3,
                                ez + c % 3, nbv);
  }
  for (uint32_t c = 0; c < nchunk; c++) {
    while (st.issued - st.consumed < (uint32_t)NS) {  // stages freed by the chunks already split
      const uint32_t k = st.issued - st.elem_start;
      if (k < nchunk)
        tcs_issue(S, st, esrc + (size_t)k * S_CH_BYTES);
      else if (nsrc && k < 2 * nchunk)
        tcs_issue(S, st, nsrc + (size_t)(k - nchunk) * S_CH_BYTES);
      else
        break;
    }
    const int sg = (int)(st.consumed % NS), ob = (int)(st.consumed & 1);
    bool ok = tc::mbar_wait(&S.mbar_cp[sg], (st.cp_n[sg] - 1) & 1, G_WAIT_LIMIT);
    // operand buffer ob was last read by the MMAs of the chunk before the previous one
    if (ok && st.mma_n[ob] > 0) ok = tc::mbar_wait(&S.mbar_mma[ob], (st.mma_n[ob] - 1) & 1, G_WAIT_LIMIT);
    // each thread waits for itself; a wait that expired is acted on after the barrier
    if (!ok) S.abort = 1;
    {
      const float4 *src = reinterpret_cast<const float4 *>(S.val[sg]);
      float4 *hi = reinterpret_cast<float4 *>(S.op[ob][0]);
      float4 *lo = reinterpret_cast<float4 *>(S.op[ob][1]);
      for (int i = tid; i < S_CH_BYTES / 16; i += G_THREADS) {
        const float4 v = src[i];
        float4 h, l;
        h.x = tc::to_tf32(v.x);
        h.y = tc::to_tf32(v.y);
        h.z = tc::to_tf32(v.z);
        h.w = tc::to_tf32(v.w);
        l.x = tc::to_tf32(v.x - h.x);
        l.y = tc::to_tf32(v.y - h.y);
        l.z = tc::to_tf32(v.z - h.z);
        l.w = tc::to_tf32(v.w - h.w);
        hi[i] = h;
        lo[i] = l;
      }
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    if (S.abort) return false;
    if (tid == 0) {
      tc::fence_after_sync();
      const uint32_t hb = op_base + (uint32_t)(ob * 2 * S_OP_BYTES), lb = hb + (uint32_t)S_OP_BYTES;
      for (int ks = 0; ks < GKS; ks++)
        for (int pp = 0; pp < 3; pp++) {  // hi.hi, hi.lo, lo.hi
          const uint32_t a = (pp == 2 ? lb : hb) + (uint32_t)(ks * S_KS_BYTES);
          const uint32_t b = (pp == 1 ? lb : hb) + (uint32_t)(ks * S_KS_BYTES);
          tc::mma_tf32(taddr, tc::smem_desc(a, 128, 256), tc::smem_desc(b, 128, 256), idesc,
                       (c == 0 && ks == 0 && pp == 0) ? 0u : 1u);
        }
      tc::mma_commit(&S.mbar_mma[ob]);
    }
    st.mma_n[ob]++;
    st.consumed++;
  }
  st.elem_start += nchunk;
  // epilogue: the last commit covers every MMA of the element
  const int lob = (int)((st.consumed - 1) & 1);
  if (!tc::mbar_wait(&S.mbar_mma[lob], (st.mma_n[lob] - 1) & 1, G_WAIT_LIMIT)) S.abort = 1;
  tc::fence_after_sync();
  __syncthreads();
  if (S.abort) return false;
  float *G = reinterpret_cast<float *>(&S.op[0][0][0]);  // operands are no longer read
  {
    const int quarter = warp & 3;
    const int r = quarter * 32 + lane;
    for (int cb = warp >> 2; cb < 3; cb += 2) {
      uint32_t v[32];
      tc::tmem_ld_32x32b_x32(taddr + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(cb * 32), v);
      if (r < GROWS)
#pragma unroll
        for (int j = 0; j < 32; j++)
          if (cb * 32 + j < GROWS) G[r * GPAD + cb * 32 + j] = __uint_as_float(v[j]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  gram_scatter(G, S.rowp, S.pos, L, vals);
  return true;
}

template <int NS>
__device__ __forceinline__ void tcs_setup(TcsSmem<NS> &S)
{
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    tc::tmem_alloc(&S.taddr, G_TMEM_COLS);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int b = 0; b < 2; b++) tc::mbar_init(&S.mbar_mma[b], 1);
    for (int b = 0; b < NS; b++) tc::mbar_init(&S.mbar_cp[b], 1);
    S.abort = 0;
  }
  // the tail of each operand buffer past the split chunk (read only into
  // accumulator rows that are never read) stays zero
  for (int i = tid; i < (int)(sizeof(S.op) / 4); i += G_THREADS) reinterpret_cast<float *>(&S.op[0][0][0])[i] = 0.f;
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
}

// On an abort, waits (bounded) for the copies and MMAs in flight before the
// shared memory is released; then frees TMEM.
template <int NS>
__device__ __forceinline__ void tcs_teardown(TcsSmem<NS> &S, const TcsState<NS> &st, int *err)
{
  tc::fence_before_sync();
  __syncthreads();
  if (S.abort) {
    for (int b = 0; b < NS; b++)
      if (st.cp_n[b] > 0) tc::mbar_wait(&S.mbar_cp[b], (st.cp_n[b] - 1) & 1, G_WAIT_LIMIT);
    for (int b = 0; b < 2; b++)
      if (st.mma_n[b] > 0) tc::mbar_wait(&S.mbar_mma[b], (st.mma_n[b] - 1) & 1, G_WAIT_LIMIT);
    if (threadIdx.x == 0) atomicCAS(err, 0, 2);
  }
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(S.taddr, G_TMEM_COLS);
}

template <int NS, int MINB>
__global__ void __launch_bounds__(G_THREADS, MINB)
    tcs_kernel(DevMesh m, DevLaw L, int cx, int cy, int cz, int ncx, int ncy, int ncz, double *__restrict__ vals,
               int *err)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcsSmem<NS> &S = *reinterpret_cast<TcsSmem<NS> *>(smem_raw);
  tcs_setup(S);
  const uint32_t taddr = S.taddr, op_base = tc::smem_u32(&S.op[0][0][0]);
  TcsState<NS> st = {};
  const int nelem_c = ncx * ncy * ncz;
  const size_t ebytes = (size_t)((m.npts + PW - 1) / PW) * S_CH_BYTES;
  const unsigned char *cache = reinterpret_cast<const unsigned char *>(m.gop);
  auto src_of = [&](int ei, int &ex, int &ey, int &ez) {
    const int iz = ei % ncz, iy = (ei / ncz) % ncy, ix = ei / (ncz * ncy);
    ex = cx + 3 * ix;
    ey = cy + 3 * iy;
    ez = cz + 3 * iz;
    const int64_t eg = ((int64_t)ex * m.nelem[1] + ey) * m.nelem[2] + ez;
    return cache + (size_t)eg * ebytes;
  };
  for (int ei = blockIdx.x; ei < nelem_c; ei += gridDim.x) {
    int ex, ey, ez, nx, ny, nz;
    const unsigned char *esrc = src_of(ei, ex, ey, ez);
    const unsigned char *nsrc = ei + (int)gridDim.x < nelem_c ? src_of(ei + gridDim.x, nx, ny, nz) : nullptr;
    if (!tcs_element<NS, false>(S, st, m, L, ex, ey, ez, esrc, nsrc, vals, taddr, op_base)) break;
    tc::fence_before_sync();
    __syncthreads();
  }
  tcs_teardown(S, st, err);
}

// Batched: elements from the colour-major queue (see element_batch_kernel);
// copies prefetch within an element only.
template <int NS, int MINB>
__global__ void __launch_bounds__(G_THREADS, MINB) tcs_batch_kernel(BatchArgs ba, double *__restrict__ vals)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcsSmem<NS> &S = *reinterpret_cast<TcsSmem<NS> *>(smem_raw);
  const int tid = threadIdx.x;
  tcs_setup(S);
  const uint32_t taddr = S.taddr, op_base = tc::smem_u32(&S.op[0][0][0]);
  TcsState<NS> st = {};
  int cur = -1;
  DevMesh m;
  DevLaw L;
  int64_t next = 0;
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
    for (int64_t it = base; it < end; it++) {
      const BatchItem w = ba.items[it];
      if (w.inst != cur) {
        m = ba.meshes[w.inst];
        L = ba.laws[w.inst];
        cur = w.inst;
      }
      if (tid == 0 && w.col > 0) {
        if (!tc_wait_ge(ba.done + w.inst, ba.need[27 * w.inst + w.col])) {
          S.abort = 1;
          atomicExch(ba.err, 3);
        }
      }
      __syncthreads();
      if (S.abort) {
        ok = false;
        break;
      }
      const int ey = w.eyz >> 16, ez = w.eyz & 0xffff;
      const int64_t eg = ((int64_t)w.ex * m.nelem[1] + ey) * m.nelem[2] + ez;
      const unsigned char *esrc = reinterpret_cast<const unsigned char *>(m.gop) +
                                  (size_t)eg * ((m.npts + PW - 1) / PW) * S_CH_BYTES;
      ok = tcs_element<NS, true>(S, st, m, L, w.ex, ey, ez, esrc, nullptr, vals, taddr, op_base);
      if (!ok) break;
      tc::fence_before_sync();
      __syncthreads();
      if (tid == 0)  // release at GPU scope after the barrier
        asm volatile("fence.acq_rel.gpu;\n\tred.relaxed.gpu.global.add.s32 [%0], 1;" ::"l"(ba.done + w.inst)
                     : "memory");
    }
    if (!ok) break;
  }
  tcs_teardown(S, st, ba.err);
}


// ------------------------------------------------ warp-specialised variant
// The cached-operand tangent with its stages on separate warps, so that the
// copies, the TF32 split, the MMAs and the scatter of different chunks and
// elements overlap inside one CTA (two CTAs per SM, two TMEM accumulators):
//   warp 0 (one thread): bulk copies of the chunk stream into W_NS stages,
//   warps 2-3: TF32 split of a staged chunk into a free operand buffer,
//   warp 1 (one thread): the 12 MMAs of a chunk into the element's accumulator,
//   warps 4-7: epilogue of the previous element (TMEM -> G -> K -> L2 reductions).
// Hand-offs are mbarriers (full/empty per copy stage, opfull/opempty per
// operand buffer, accfull/accempty per accumulator); every wait is bounded and
// gives up early once another role has aborted.
constexpr int W_NS = 2;
constexpr uint32_t W_TMEM_COLS = 256;  // two accumulators of 128 columns

struct TcwSmem {
  unsigned char op[2][2][S_OP_BYTES];  // [buffer][hi, lo]
  unsigned char val[W_NS][S_CH_BYTES]; // copy stages
  float G[GROWS * GPAD];               // epilogue staging
  unsigned char pos[NB * NB];
  int64_t rowp[NE];
  uint64_t full[W_NS], empty[W_NS], opfull[2], opempty[2], accfull[2], accempty[2];
  uint32_t cp_n[W_NS], ope_n[2], accf_n[2];  // issue counts for the teardown
  uint32_t taddr;
  int abort;
};

__device__ __forceinline__ void mbar_arrive(uint64_t *mbar)
{
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(mbar)) : "memory");
}

// Bounded wait that also returns (false) once another role set the abort flag.
__device__ __forceinline__ bool tcw_wait(uint64_t *mbar, uint32_t parity, volatile int *abort)
{
  const uint32_t addr = tc::smem_u32(mbar);
  for (uint32_t it = 0; it < G_WAIT_LIMIT; it++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
    if ((it & 255u) == 255u && *abort) return false;
  }
  return false;
}

__global__ void __launch_bounds__(G_THREADS, 2)
    tcw_kernel(DevMesh m, DevLaw L, int cx, int cy, int cz, int ncx, int ncy, int ncz, double *__restrict__ vals,
               int *err)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcwSmem &S = *reinterpret_cast<TcwSmem *>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  volatile int *abort = &S.abort;
  if (warp == 0) {
    tc::tmem_alloc(&S.taddr, W_TMEM_COLS);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < W_NS; i++) {
      tc::mbar_init(&S.full[i], 1);
      tc::mbar_init(&S.empty[i], 64);
      S.cp_n[i] = 0;
    }
    for (int i = 0; i < 2; i++) {
      tc::mbar_init(&S.opfull[i], 64);
      tc::mbar_init(&S.opempty[i], 1);
      tc::mbar_init(&S.accfull[i], 1);
      tc::mbar_init(&S.accempty[i], 128);
      S.ope_n[i] = S.accf_n[i] = 0;
    }
    S.abort = 0;
  }
  for (int i = tid; i < (int)(sizeof(S.op) / 4); i += G_THREADS) reinterpret_cast<float *>(&S.op[0][0][0])[i] = 0.f;
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = S.taddr;
  const int nelem_c = ncx * ncy * ncz;
  const int nmine = (int)blockIdx.x < nelem_c ? (nelem_c - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  const uint32_t nchunk = (uint32_t)((m.npts + PW - 1) / PW);
  const size_t ebytes = (size_t)nchunk * S_CH_BYTES;
  auto element = [&](int j, int &ex, int &ey, int &ez) {
    const int ei = (int)blockIdx.x + j * (int)gridDim.x;
    const int iz = ei % ncz, iy = (ei / ncz) % ncy, ix = ei / (ncz * ncy);
    ex = cx + 3 * ix;
    ey = cy + 3 * iy;
    ez = cz + 3 * iz;
    return ((int64_t)ex * m.nelem[1] + ey) * m.nelem[2] + ez;
  };
  if (warp == 0) {
    if (lane == 0) {  // producer
      const unsigned char *cache = reinterpret_cast<const unsigned char *>(m.gop);
      uint32_t s = 0, cpn[W_NS] = {};
      bool ok = true;
      for (int j = 0; j < nmine && ok; j++) {
        int ex, ey, ez;
        const unsigned char *src = cache + (size_t)element(j, ex, ey, ez) * ebytes;
        for (uint32_t c = 0; c < nchunk; c++, s++) {
          const int st = (int)(s % W_NS);
          if (s >= (uint32_t)W_NS && !tcw_wait(&S.empty[st], ((s / W_NS) - 1) & 1, abort)) {
            ok = false;
            break;
          }
          tc::mbar_arrive_expect_tx(&S.full[st], (uint32_t)S_CH_BYTES);
          tc::bulk_g2s(S.val[st], src + (size_t)c * S_CH_BYTES, (uint32_t)S_CH_BYTES, &S.full[st]);
          cpn[st]++;
        }
      }
      if (!ok) S.abort = 1;
      for (int i = 0; i < W_NS; i++) S.cp_n[i] = cpn[i];
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      const uint32_t idesc = tc::instr_desc(2, 128, GN);
      const uint32_t op_base = tc::smem_u32(&S.op[0][0][0]);
      uint32_t s = 0, open[2] = {0, 0}, accn[2] = {0, 0};
      bool ok = true;
      for (int j = 0; j < nmine && ok; j++) {
        const int a = j & 1;
        if (j >= 2 && !tcw_wait(&S.accempty[a], ((uint32_t)(j / 2) - 1) & 1, abort)) {
          ok = false;
          break;
        }
        tc::fence_after_sync();
        const uint32_t dacc = taddr + (uint32_t)(a * 128);
        for (uint32_t c = 0; c < nchunk; c++, s++) {
          const int b = (int)(s & 1);
          if (!tcw_wait(&S.opfull[b], (s / 2) & 1, abort)) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const uint32_t hb = op_base + (uint32_t)(b * 2 * S_OP_BYTES), lb = hb + (uint32_t)S_OP_BYTES;
          for (int ks = 0; ks < GKS; ks++)
            for (int pp = 0; pp < 3; pp++) {  // hi.hi, hi.lo, lo.hi
              const uint32_t ad = (pp == 2 ? lb : hb) + (uint32_t)(ks * S_KS_BYTES);
              const uint32_t bd = (pp == 1 ? lb : hb) + (uint32_t)(ks * S_KS_BYTES);
              tc::mma_tf32(dacc, tc::smem_desc(ad, 128, 256), tc::smem_desc(bd, 128, 256), idesc,
                           (c == 0 && ks == 0 && pp == 0) ? 0u : 1u);
            }
          tc::mma_commit(&S.opempty[b]);
          open[b]++;
        }
        if (!ok) break;
        tc::mma_commit(&S.accfull[a]);
        accn[a]++;
      }
      if (!ok) S.abort = 1;
      for (int i = 0; i < 2; i++) {
        S.ope_n[i] = open[i];
        S.accf_n[i] = accn[i];
      }
    }
  } else if (warp < 4) {  // TF32 split, 64 threads
    const int t = tid - 64;
    uint32_t s = 0;
    bool ok = true;
    for (int j = 0; j < nmine && ok; j++)
      for (uint32_t c = 0; c < nchunk; c++, s++) {
        const int st = (int)(s % W_NS), b = (int)(s & 1);
        if (!tcw_wait(&S.full[st], (s / W_NS) & 1, abort) ||
            (s >= 2 && !tcw_wait(&S.opempty[b], ((s / 2) - 1) & 1, abort))) {
          ok = false;
          break;
        }
        const float4 *src = reinterpret_cast<const float4 *>(S.val[st]);
        float4 *hi = reinterpret_cast<float4 *>(S.op[b][0]);
        float4 *lo = reinterpret_cast<float4 *>(S.op[b][1]);
        for (int i = t; i < S_CH_BYTES / 16; i += 64) {
          const float4 v = src[i];
          float4 h, l;
          h.x = tc::to_tf32(v.x);
          h.y = tc::to_tf32(v.y);
          h.z = tc::to_tf32(v.z);
          h.w = tc::to_tf32(v.w);
          l.x = tc::to_tf32(v.x - h.x);
          l.y = tc::to_tf32(v.y - h.y);
          l.z = tc::to_tf32(v.z - h.z);
          l.w = tc::to_tf32(v.w - h.w);
          hi[i] = h;
          lo[i] = l;
        }
        tc::fence_proxy_async();  // the MMAs read the operands through the async proxy
        mbar_arrive(&S.empty[st]);
        mbar_arrive(&S.opfull[b]);
      }
    if (!ok) S.abort = 1;
  } else {  // epilogue, 128 threads: warp & 3 is the TMEM lane quarter
    const int t = tid - 128, quarter = warp & 3;
    const int nb1 = m.nbasis[1], nb2 = m.nbasis[2];
    const int nbv[3] = {m.nbasis[0], nb1, nb2};
    bool ok = true;
    for (int j = 0; j < nmine && ok; j++) {
      const int a = j & 1;
      int ex, ey, ez;
      element(j, ex, ey, ez);
      if (t < NE) {
        const int b = t / 3, dd = t % 3;
        const int64_t cpb = ((int64_t)(ex + b / 9) * nb1 + (ey + (b / 3) % 3)) * nb2 + (ez + b % 3);
        S.rowp[t] = __ldg(m.rowptr + 3 * cpb + dd);
      }
      for (int i = t; i < NB * NB; i += 128) {
        const int b = i / NB, c = i % NB;
        S.pos[i] = (unsigned char)stencil_pos(ex + b / 9, ey + (b / 3) % 3, ez + b % 3, ex + c / 9,
                                              ey + (c / 3) % 3, ez + c % 3, nbv);
      }
      // the four epilogue warps take the same decision (a named-barrier OR):
      // a thread that gave up must not leave the others at a named barrier
      const uint32_t got = tcw_wait(&S.accfull[a], ((uint32_t)j / 2) & 1, abort) ? 1u : 0u;
      uint32_t any_failed;
      asm volatile(
          "{\n\t.reg .pred p, q;\n\t"
          "setp.eq.u32 p, %1, 0;\n\t"
          "bar.red.or.pred q, 1, 128, p;\n\t"
          "selp.u32 %0, 1, 0, q;\n\t}\n"
          : "=r"(any_failed)
          : "r"(got)
          : "memory");
      if (any_failed) {
        ok = false;
        break;
      }
      tc::fence_after_sync();
      const int r = quarter * 32 + lane;
      for (int cb = 0; cb < 3; cb++) {
        uint32_t v[32];
        tc::tmem_ld_32x32b_x32(taddr + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(a * 128 + cb * 32), v);
        if (r < GROWS)
#pragma unroll
          for (int jj = 0; jj < 32; jj++)
            if (cb * 32 + jj < GROWS) S.G[r * GPAD + cb * 32 + jj] = __uint_as_float(v[jj]);
      }
      tc::fence_before_sync();
      mbar_arrive(&S.accempty[a]);
      asm volatile("bar.sync 1, 128;" ::: "memory");  // G, rowp, pos of the element complete
      gram_scatter(S.G, S.rowp, S.pos, L, vals, t, 128);
      asm volatile("bar.sync 1, 128;" ::: "memory");  // before the next element overwrites them
    }
    if (!ok) S.abort = 1;
  }
  tc::fence_before_sync();
  __syncthreads();
  if (S.abort) {
    if (tid == 0) {
      for (int i = 0; i < W_NS; i++)
        if (S.cp_n[i] > 0) tc::mbar_wait(&S.full[i], (S.cp_n[i] - 1) & 1, G_WAIT_LIMIT);
      for (int i = 0; i < 2; i++) {
        if (S.ope_n[i] > 0) tc::mbar_wait(&S.opempty[i], (S.ope_n[i] - 1) & 1, G_WAIT_LIMIT);
        if (S.accf_n[i] > 0) tc::mbar_wait(&S.accfull[i], (S.accf_n[i] - 1) & 1, G_WAIT_LIMIT);
      }
      atomicCAS(err, 0, 2);
    }
  }
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, W_TMEM_COLS);
}

// ------------------------------------------------------------- launches
static size_t tcg_smem() { return sizeof(TcgSmem) + 1024; }
template <int NS>
static size_t tcs_smem() { return sizeof(TcsSmem<NS>) + 1024; }

// 3 CTAs per SM with 2 copy stages (default), or 2 CTAs per SM with 4
static int tcs_ctas_per_sm()
{
  const char *env = getenv("IGAPGPU_TCS_CTAS");
  return (env && env[0] == '2') ? 2 : 3;
}

int ensure_gram_operands(Context *c)
{
  if (c->gop_state >= 0 || c->law != IGAPGPU_LAW_LINGRAD || !c->d_geo) return IGAPGPU_OK;
  const char *env = getenv("IGAPGPU_TC_GRAM_CACHE");
  c->gop_state = 0;
  if (env && env[0] == '0') return IGAPGPU_OK;
  const int npts = c->nquad * c->nquad * c->nquad, nchunk = (npts + PW - 1) / PW;
  const size_t bytes = (size_t)c->nelem_total * nchunk * S_CH_BYTES;
  size_t freeb = 0, totb = 0;
  IGAP_CUDA(cudaMemGetInfo(&freeb, &totb));
  if (bytes + ((size_t)4 << 30) > freeb) return IGAPGPU_OK;  // the plain Gram kernel stays in use
  if (cudaMalloc(&c->d_gop, bytes) != cudaSuccess) {
    cudaGetLastError();
    c->d_gop = nullptr;
    return IGAPGPU_OK;
  }
  int *d_bad = nullptr;
  if (cudaMalloc(&d_bad, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(c->d_gop);
    c->d_gop = nullptr;
    return IGAPGPU_OK;
  }
  int bad = 0;
  cudaError_t e = cudaMemsetAsync(d_bad, 0, sizeof(int), c->stream);
  int dev = 0, nsm = 0;
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) {
    gram_operand_kernel<<<nsm * 16, 256, 0, c->stream>>>(c->d_geo, npts, nchunk, c->nelem_total, c->par[2],
                                                         c->d_gop, d_bad);
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_bad);
  if (e != cudaSuccess) {
    cudaFree(c->d_gop);
    c->d_gop = nullptr;
    set_error("gram operands: CUDA error %s", cudaGetErrorString(e));
    return IGAPGPU_ERR_CUDA;
  }
  if (bad) {  // a non-positive point weight: keep the plain Gram kernel
    cudaFree(c->d_gop);
    c->d_gop = nullptr;
    return IGAPGPU_OK;
  }
  c->gop_state = 1;
  return IGAPGPU_OK;
}

// One persistent launch per colour of a Gram-form tangent kernel: `kern`
// with `smem` dynamic shared memory and `ctas` CTAs per SM (fewer when the
// colour has fewer elements), timed as one tensor-core kernel group when
// profiling is on.  `attr_set` (one per kernel, owned by the caller) records
// that the kernel's shared-memory limit was raised, once, before any graph
// capture can reach this call.
template <typename Kern>
static int launch_colours(Context *c, Kern kern, size_t smem, int ctas, double *vals, bool &attr_set)
{
  const DevMesh m = c->devmesh();
  const DevLaw L = c->devlaw();
  if (!attr_set) {
    IGAP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
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
        const int grid = nel < ctas * nsm ? nel : ctas * nsm;
        kern<<<grid, G_THREADS, smem, c->stream>>>(m, L, cx, cy, cz, ncx, ncy, ncz, vals, c->d_err);
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

template <int NS, int MINB>
static int launch_tc_gop_cfg(Context *c, double *vals)
{
  static bool attr = false;
  return launch_colours(c, tcs_kernel<NS, MINB>, tcs_smem<NS>(), MINB, vals, attr);
}

static int launch_tc_gop_ws(Context *c, double *vals)
{
  static bool attr = false;
  return launch_colours(c, tcw_kernel, sizeof(TcwSmem) + 1024, 2, vals, attr);
}

// The warp-specialised kernel by default (6.3 ms per tangent at 128x32x32
// against 7.0 ms for the single-role kernel); IGAPGPU_TCS_WS=0 selects the
// single-role kernel (the batched path always uses its queue variant).
static int launch_tc_gop(Context *c, double *vals)
{
  const char *ws = getenv("IGAPGPU_TCS_WS");
  if (!(ws && ws[0] == '0')) return launch_tc_gop_ws(c, vals);
  return tcs_ctas_per_sm() == 3 ? launch_tc_gop_cfg<2, 3>(c, vals) : launch_tc_gop_cfg<4, 2>(c, vals);
}

int launch_tc_gram(Context *c, double *vals)
{
  if (c->d_gop) return launch_tc_gop(c, vals);
  static bool attr = false;
  return launch_colours(c, tcg_kernel, tcg_smem(), 2, vals, attr);  // two CTAs per SM
}

int launch_tc_gram_batch(Context *c, const BatchArgs &a, int nsm, double *vals, bool cached)
{
  if (cached) {
    const bool three = tcs_ctas_per_sm() == 3;
    auto kern = three ? tcs_batch_kernel<2, 3> : tcs_batch_kernel<4, 2>;
    const size_t sm = three ? tcs_smem<2>() : tcs_smem<4>();
    static bool attr_s[2] = {false, false};
    if (!attr_s[three]) {
      IGAP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      attr_s[three] = true;
    }
    kern<<<(three ? 3 : 2) * nsm, G_THREADS, sm, c->stream>>>(a, vals);  // persistent CTAs per SM
    count_launch();
    IGAP_CHECK_LAUNCH();
    return IGAPGPU_OK;
  }
  static bool attr = false;
  if (!attr) {
    IGAP_CUDA(cudaFuncSetAttribute(tcg_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)tcg_smem()));
    attr = true;
  }
  tcg_batch_kernel<<<2 * nsm, G_THREADS, tcg_smem(), c->stream>>>(a, vals);  // two persistent CTAs per SM
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

}  // namespace igap
