// Learned Newton predictor: a 3-D convolutional network on the control-point
// lattice, with hand-written forward, backward and Adam kernels.
//
// Layout: activations [B][nx][ny][nz][C] (channels last, the DOF order of
// U: 3*cp + d), weights [Co][27][Ci] with tap t = 9*(dx+1) + 3*(dy+1) + (dz+1),
// zero padding at the lattice boundary.  Layers 9->32->32->32->3, ReLU after
// the first three.  Storage type T is float (used for gradient checks) or
// bfloat16 (training and inference); every product accumulates in FP32.
// Master weights and Adam moments are FP32.
// No counterpart in the reference (an addition to its solver path).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "common.cuh"
#include "tcgen05.cuh"

namespace igap {

constexpr int NL = 4;
static const int kCin[NL] = {9, 32, 32, 32};
static const int kCout[NL] = {32, 32, 32, 3};

template <typename T> __device__ __forceinline__ float ld(const T *p);
template <> __device__ __forceinline__ float ld<float>(const float *p) { return *p; }
template <> __device__ __forceinline__ float ld<__nv_bfloat16>(const __nv_bfloat16 *p) { return __bfloat162float(*p); }
template <typename T> __device__ __forceinline__ T cvt(float x);
template <> __device__ __forceinline__ float cvt<float>(float x) { return x; }
template <> __device__ __forceinline__ __nv_bfloat16 cvt<__nv_bfloat16>(float x) { return __float2bfloat16_rn(x); }

struct Lattice {
  int nx, ny, nz;
  int64_t P;  // points per sample
};

__device__ __forceinline__ bool nbr(const Lattice &L, int64_t p, int t, int64_t &q)
{
  const int iz = (int)(p % L.nz), iy = (int)((p / L.nz) % L.ny), ix = (int)(p / ((int64_t)L.ny * L.nz));
  const int jx = ix + t / 9 - 1, jy = iy + (t / 3) % 3 - 1, jz = iz + t % 3 - 1;
  if (jx < 0 || jx >= L.nx || jy < 0 || jy >= L.ny || jz < 0 || jz >= L.nz) return false;
  q = ((int64_t)jx * L.ny + jy) * L.nz + jz;
  return true;
}

// out[b,p,co] = act(bias[co] + sum_t sum_ci W[co,t,ci] in[b,p+t,ci])
template <typename T>
__global__ void conv_fwd(const T *__restrict__ in, int Ci, const T *__restrict__ W, const float *__restrict__ bias,
                         T *__restrict__ out, int Co, Lattice L, int B, int relu)
{
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t total = (int64_t)B * L.P * Co;
  if (idx >= total) return;
  const int co = (int)(idx % Co);
  const int64_t bp = idx / Co;
  const int b = (int)(bp / L.P);
  const int64_t p = bp % L.P;
  float acc = bias[co];
  for (int t = 0; t < 27; t++) {
    int64_t q;
    if (!nbr(L, p, t, q)) continue;
    const T *x = in + ((int64_t)b * L.P + q) * Ci;
    const T *w = W + ((int64_t)co * 27 + t) * Ci;
    for (int ci = 0; ci < Ci; ci++) acc = fmaf(ld(w + ci), ld(x + ci), acc);
  }
  if (relu && acc < 0.f) acc = 0.f;
  out[idx] = cvt<T>(acc);
}

// dZ = dA * [A > 0] (ReLU), in place on dA (FP32)
template <typename T>
__global__ void relu_bwd(float *dA, const T *A, int64_t n)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && !(ld(A + i) > 0.f)) dA[i] = 0.f;
}

// dIn[b,p,ci] = sum_t sum_co W[co,t,ci] dZ[b,p-t,co]
template <typename T>
__global__ void conv_bwd_data(const float *__restrict__ dZ, int Co, const T *__restrict__ W, float *__restrict__ dIn,
                              int Ci, Lattice L, int B)
{
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t total = (int64_t)B * L.P * Ci;
  if (idx >= total) return;
  const int ci = (int)(idx % Ci);
  const int64_t bp = idx / Ci;
  const int b = (int)(bp / L.P);
  const int64_t p = bp % L.P;
  float acc = 0.f;
  for (int t = 0; t < 27; t++) {
    int64_t q;
    if (!nbr(L, p, 26 - t, q)) continue;  // q = p - offset(t)
    const float *dz = dZ + ((int64_t)b * L.P + q) * Co;
    for (int co = 0; co < Co; co++) acc = fmaf(ld(W + ((int64_t)co * 27 + t) * Ci + ci), dz[co], acc);
  }
  dIn[idx] = acc;
}

// dW[co,t,ci] += sum_{b,p} dZ[b,p,co] in[b,p+t,ci]; db[co] += sum dZ[b,p,co]
// one block per (co, t); threads: 32 input channels x 8 point lanes
template <typename T>
__global__ void __launch_bounds__(256) conv_bwd_weight(const float *__restrict__ dZ, int Co, const T *__restrict__ in,
                                                       int Ci, float *__restrict__ dW, float *__restrict__ db,
                                                       Lattice L, int B)
{
  __shared__ float red[8][33];
  const int co = blockIdx.x / 27, t = blockIdx.x % 27;
  const int ci = threadIdx.x & 31, pl = threadIdx.x >> 5;
  const int64_t NP = (int64_t)B * L.P;
  float acc = 0.f, accb = 0.f;
  for (int64_t bp = pl; bp < NP; bp += 8) {
    const int b = (int)(bp / L.P);
    const int64_t p = bp % L.P;
    const float g = dZ[bp * Co + co];
    if (t == 13 && ci == 0) accb += g;
    if (g == 0.f || ci >= Ci) continue;
    int64_t q;
    if (!nbr(L, p, t, q)) continue;
    acc = fmaf(g, ld(in + ((int64_t)b * L.P + q) * Ci + ci), acc);
  }
  red[pl][ci] = acc;
  if (ci == 0) red[pl][32] = accb;
  __syncthreads();
  if (threadIdx.x < 32 && ci < Ci) {
    float s = 0.f;
    for (int k = 0; k < 8; k++) s += red[k][ci];
    dW[((int64_t)co * 27 + t) * Ci + ci] += s;
  }
  __syncthreads();
  if (threadIdx.x == 0 && t == 13) {
    // bias: the ci==0 lanes of each point lane accumulated accb
    float s = 0.f;
    for (int k = 0; k < 8; k++) s += red[k][32];
    db[co] += s;
  }
}

// ------------------------------------------- tensor-core convolution (tcgen05)
// The 32 -> 32 channel layers as an implicit GEMM on the tensor cores:
// for a tile of 128 consecutive lattice points of one sample,
//   D[p][n] = sum_t sum_k A_t[p][k] B_t[n][k],  A_t[p][k] = in[p + o(t)][k]
// (zero where the neighbour is outside the lattice), one tcgen05.mma
// kind::f16 (BF16 inputs, FP32 accumulation in tensor memory, M128 N32 K16)
// per tap and 16 input channels: 54 MMAs per tile.  Forward: B_t[co][ci] =
// W[co][t][ci], output BF16 with bias and ReLU.  Data gradient: the same
// product of dZ (BF16) with B_t[ci][co] = W[co][26 - t][ci] (o(26 - t) =
// -o(t)), output FP32.  Operands in shared memory in the K-major no-swizzle
// layout (core matrices of 8 rows x 16 B, LBO 128 B, SBO 256 B): the weights
// of all 27 taps once per CTA (persistent over tiles), the neighbour rows of
// one tap double buffered: the threads load tap t + 1 (16-byte loads of the
// channels-last rows, the lattice boundary masked) while the tensor core
// multiplies tap t.  Every mbarrier wait is bounded.
constexpr int CT_THREADS = 128;
constexpr int CT_TAP_A = 2 * 16 * 256;   // one tap's A tile: 2 K-steps x 16 row groups x 256 B
constexpr int CT_TAP_B = 2 * 4 * 256;    // one tap's B tile: 2 K-steps x 4 row groups x 256 B
constexpr uint32_t CT_WAIT_LIMIT = 1u << 24;

struct ConvTcSmem {
  unsigned char A[2][CT_TAP_A];
  unsigned char B[27][CT_TAP_B];
  uint64_t done[2];
  uint32_t taddr;
};

// Byte offset of BF16 element (row r, k in [0, 16)) inside one K-step block.
__device__ __forceinline__ uint32_t ct_off(int r, int k)
{
  return (uint32_t)((r >> 3) * 256 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// The B operand of every tap for one layer and mode, [27][n][k] (BF16):
// forward Wk[t][co][ci] = W[co][t][ci]; data gradient Wk[t][ci][co] =
// W[co][26 - t][ci].
__global__ void conv_tc_weights_kernel(const __nv_bfloat16 *__restrict__ W, __nv_bfloat16 *__restrict__ Wk, int mode)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 27 * 32 * 32) return;
  const int t = i / 1024, n = (i / 32) % 32, k = i % 32;
  Wk[i] = mode == 0 ? W[((int64_t)n * 27 + t) * 32 + k] : W[((int64_t)k * 27 + (26 - t)) * 32 + n];
}

// MODE 0: forward (out BF16, bias, ReLU); MODE 1: data gradient (out FP32).
// Thread r of the CTA owns row r of every tile (its lattice coordinates are
// computed once per tile) and loads that row's neighbour (64 B) for every tap,
// one tap ahead of the one it stores.
template <int MODE>
__global__ void __launch_bounds__(CT_THREADS) conv_tc_kernel(const __nv_bfloat16 *__restrict__ in,
                                                             const __nv_bfloat16 *__restrict__ Wk,
                                                             const float *__restrict__ bias, void *__restrict__ out,
                                                             Lattice L, int B, int relu, int *err)
{
  extern __shared__ __align__(1024) unsigned char ct_raw[];
  ConvTcSmem &S = *reinterpret_cast<ConvTcSmem *>(ct_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    tc::tmem_alloc(&S.taddr, 32);
    tc::tmem_relinquish();
  }
  // weights of every tap: B_t[n][k], K-major (2 K-steps of 16 per tap), 16 B at a time
  for (int i = tid; i < 27 * 32 * 4; i += CT_THREADS) {
    const int t = i / 128, n = (i / 4) % 32, j = i % 4;
    const uint4 w = __ldg(reinterpret_cast<const uint4 *>(Wk + ((int64_t)t * 32 + n) * 32) + j);
    *reinterpret_cast<uint4 *>(S.B[t] + (j >> 1) * 1024 + ct_off(n, (j & 1) * 8)) = w;
  }
  if (tid == 0) {
    tc::mbar_init(&S.done[0], 1);
    tc::mbar_init(&S.done[1], 1);
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = S.taddr;
  const uint32_t idesc = tc::instr_desc(1, 128, 32);
  const int64_t tiles_per_sample = (L.P + 127) / 128, ntiles = tiles_per_sample * B;
  const int64_t syz = (int64_t)L.ny * L.nz;
  uint32_t use0 = 0, use1 = 0;  // commits issued on each buffer
  bool ok = true;
  for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int b = (int)(tile / tiles_per_sample);
    const int64_t p0 = (tile % tiles_per_sample) * 128;
    const int64_t p = p0 + tid;  // this thread's row
    const bool rowv = p < L.P;
    const int iz = (int)(p % L.nz), iy = (int)((p / L.nz) % L.ny), ix = (int)(p / syz);
    const uint4 *src = reinterpret_cast<const uint4 *>(in + ((int64_t)b * L.P + p) * 32);
    // this row's neighbour for tap t (zero outside the lattice)
    auto load_tap = [&](int t, uint4 *x) {
      const int dx = t / 9 - 1, dy = (t / 3) % 3 - 1, dz = t % 3 - 1;
      const bool v = rowv && (unsigned)(ix + dx) < (unsigned)L.nx && (unsigned)(iy + dy) < (unsigned)L.ny &&
                     (unsigned)(iz + dz) < (unsigned)L.nz;
      const int64_t off = ((int64_t)dx * L.ny + dy) * L.nz + dz;  // rows
#pragma unroll
      for (int j16 = 0; j16 < 4; j16++) x[j16] = v ? __ldg(src + off * 4 + j16) : make_uint4(0u, 0u, 0u, 0u);
    };
    uint4 cur[4];
    load_tap(0, cur);
    for (int t = 0; t < 27 && ok; t++) {
      const int buf = t & 1;
      const uint32_t used = buf ? use1 : use0;
      if (used > 0 && !tc::mbar_wait(&S.done[buf], (used - 1) & 1, CT_WAIT_LIMIT)) {
        ok = false;
        break;
      }
      unsigned char *a = S.A[buf];
#pragma unroll
      for (int j16 = 0; j16 < 4; j16++)
        *reinterpret_cast<uint4 *>(a + (j16 >> 1) * 4096 + ct_off(tid, (j16 & 1) * 8)) = cur[j16];
      if (t + 1 < 27) load_tap(t + 1, cur);  // in flight across the barrier and the MMA issue
      tc::fence_proxy_async();
      tc::fence_before_sync();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
        const uint32_t abase = tc::smem_u32(S.A[buf]), bbase = tc::smem_u32(S.B[t]);
        for (int ks = 0; ks < 2; ks++) {
          const uint64_t ad = tc::smem_desc(abase + (uint32_t)ks * 4096u, 128, 256);
          const uint64_t bd = tc::smem_desc(bbase + (uint32_t)ks * 1024u, 128, 256);
          tc::mma_bf16(taddr, ad, bd, idesc, (t > 0 || ks > 0) ? 1u : 0u);
        }
        tc::mma_commit(&S.done[buf]);
      }
      if (buf) use1++;
      else use0++;
    }
    if (!ok) break;
    // the last tap's commit (buffer 0) covers every MMA of the tile
    if (!tc::mbar_wait(&S.done[0], (use0 - 1) & 1, CT_WAIT_LIMIT)) {
      ok = false;
      break;
    }
    tc::fence_after_sync();
    uint32_t r[32];
    tc::tmem_ld_32x32b_x32(taddr + ((uint32_t)(warp * 32) << 16), r);
    const int64_t pw = p0 + warp * 32 + lane;  // TMEM lane = row = this thread's row
    if (pw < L.P) {
      if constexpr (MODE == 0) {
        uint32_t pk[16];
#pragma unroll
        for (int n = 0; n < 32; n += 2) {
          float a0 = __uint_as_float(r[n]) + bias[n], a1 = __uint_as_float(r[n + 1]) + bias[n + 1];
          if (relu) {
            a0 = fmaxf(a0, 0.f);
            a1 = fmaxf(a1, 0.f);
          }
          const __nv_bfloat162 h = __floats2bfloat162_rn(a0, a1);
          pk[n / 2] = *reinterpret_cast<const uint32_t *>(&h);
        }
        uint4 *o = reinterpret_cast<uint4 *>((__nv_bfloat16 *)out + ((int64_t)b * L.P + pw) * 32);
#pragma unroll
        for (int q4 = 0; q4 < 4; q4++) o[q4] = make_uint4(pk[4 * q4], pk[4 * q4 + 1], pk[4 * q4 + 2], pk[4 * q4 + 3]);
      } else {
        float4 *o = reinterpret_cast<float4 *>((float *)out + ((int64_t)b * L.P + pw) * 32);
#pragma unroll
        for (int q4 = 0; q4 < 8; q4++)
          o[q4] = make_float4(__uint_as_float(r[4 * q4]), __uint_as_float(r[4 * q4 + 1]),
                              __uint_as_float(r[4 * q4 + 2]), __uint_as_float(r[4 * q4 + 3]));
      }
    }
    tc::fence_before_sync();  // the next tile's first MMA overwrites the accumulator
  }
  if (!ok && tid == 0) {
    atomicCAS(err, 0, 2);
    // let MMAs still in flight finish before the tensor memory is freed
    if (use0 > 0) tc::mbar_wait(&S.done[0], (use0 - 1) & 1, CT_WAIT_LIMIT);
    if (use1 > 0) tc::mbar_wait(&S.done[1], (use1 - 1) & 1, CT_WAIT_LIMIT);
  }
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, 32);
}

// Weight gradient on the tensor cores: dW[co][t][ci] += sum_p dZ[p][co] X[p + o(t)][ci]
// as D[(tl, ci)][co] = sum_p A[(tl, ci)][p] Z[co][p] for groups of TPG =
// 128 / CI taps (4 taps of 32 channels, or 14 taps of the 9 input features
// per M = 128 rows, row tl * CI + ci), K = the 128 points of a tile, N = 32
// output channels: 8 MMAs (K16) per group and tile, one TMEM accumulator of
// 32 columns per group for the whole run of the CTA (persistent over tiles);
// at the end the CTA adds its sums into dW with FP32 reductions.  Thread p of
// the CTA owns point p of each tile: it loads the point's output gradient
// (64 B) and its neighbours' features (16-byte loads for 32 channels) and
// writes them transposed (K-major, the points along K).
template <int CI, int CO>
struct WgradCfg {
  static constexpr int TPG = 128 / CI;
  static constexpr int NG = (27 + TPG - 1) / TPG;
  static constexpr int NPAD = CO <= 16 ? 16 : 32;  // N of the MMA (multiple of 16)
  static constexpr uint32_t COLS = NG * NPAD <= 32 ? 32 : (NG * NPAD <= 64 ? 64 : (NG * NPAD <= 128 ? 128 : 256));
};
// The transposed operands are written 2 bytes at a time by consecutive points
// (consecutive K): with the packed layout (LBO 128 B, SBO 256 B, K-steps 4 KB
// apart) those stores hit four words of four banks, a four-way conflict.  The
// strides below spread one warp's 32 points over 16 banks (LBO 144 B, SBO
// 288 B, K-steps 32 B past a multiple of 128 B); they are plain descriptor
// strides of the K-major no-swizzle layout.
constexpr int WG_LBO = 144, WG_SBO = 288;
constexpr int WG_KS_A = 16 * WG_SBO + 32;  // one K-step of A (128 rows)
constexpr int WG_KS_Z = 4 * WG_SBO + 32;   // one K-step of Z (up to 32 rows)
constexpr int WG_TAP_A = 8 * WG_KS_A;      // A of one group: 8 K-steps
constexpr int WG_Z = 8 * WG_KS_Z;

struct WgradSmem {
  unsigned char A[2][WG_TAP_A];
  unsigned char Z[WG_Z];
  uint64_t done[2];
  uint32_t taddr;
};

__device__ __forceinline__ uint32_t wg_off(int m, int k, int ks_bytes)
{
  return (uint32_t)((k >> 4) * ks_bytes + (m >> 3) * WG_SBO + ((k >> 3) & 1) * WG_LBO + (m & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ void st_bf16(unsigned char *base, uint32_t off, uint32_t bits)
{
  asm volatile("st.shared.b16 [%0], %1;" ::"r"(tc::smem_u32(base + off)), "h"((unsigned short)bits) : "memory");
}

// Weight gradient on the tensor cores: dW[co][t][ci] += sum_p dZ[p][co] X[p + o(t)][ci]
// as D[(tl, ci)][co] = sum_p A[(tl, ci)][p] Z[co][p] for groups of TPG =
// 128 / CI taps (4 taps of 32 channels, or 14 taps of the 9 input features
// per M = 128 rows, row tl * CI + ci), K = the 128 points of a tile, N = the
// output channels (32, or 3 padded to 16): 8 MMAs (K16) per group and tile,
// one TMEM accumulator per group for the whole run of the CTA (persistent
// over tiles); at the end the CTA adds its sums into dW with FP32
// reductions.  Thread p of the CTA owns point p of each tile: it loads the
// point's output gradient and its neighbours' features and writes them
// transposed (K-major, the points along K).
template <int CI, int CO>
__global__ void __launch_bounds__(CT_THREADS) conv_tc_wgrad_kernel(const __nv_bfloat16 *__restrict__ X,
                                                                   const __nv_bfloat16 *__restrict__ dZh,
                                                                   float *__restrict__ gW, Lattice L, int B,
                                                                   int *err)
{
  using C = WgradCfg<CI, CO>;
  extern __shared__ __align__(1024) unsigned char wg_raw[];
  WgradSmem &S = *reinterpret_cast<WgradSmem *>(wg_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    tc::tmem_alloc(&S.taddr, C::COLS);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&S.done[0], 1);
    tc::mbar_init(&S.done[1], 1);
  }
  for (int co = CO; co < C::NPAD; co++) st_bf16(S.Z, wg_off(co, tid, WG_KS_Z), 0u);  // padding rows of Z
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = S.taddr;
  const uint32_t idesc = tc::instr_desc(1, 128, C::NPAD);
  const int64_t tiles_per_sample = (L.P + 127) / 128, ntiles = tiles_per_sample * B;
  const int64_t syz = (int64_t)L.ny * L.nz;
  uint32_t use0 = 0, use1 = 0, nuse = 0;
  bool ok = true, first = true;
  for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int b = (int)(tile / tiles_per_sample);
    const int64_t p = (tile % tiles_per_sample) * 128 + tid;
    const bool rowv = p < L.P;
    const int iz = (int)(p % L.nz), iy = (int)((p / L.nz) % L.ny), ix = (int)(p / syz);
    // Z is read by every group's MMAs of the previous tile: wait for the last one
    if (nuse > 0) {
      const int lb = (nuse - 1) & 1;
      const uint32_t used = lb ? use1 : use0;
      if (!tc::mbar_wait(&S.done[lb], (used - 1) & 1, CT_WAIT_LIMIT)) {
        ok = false;
        break;
      }
    }
    if constexpr (CO == 32) {
      const uint4 *zr = reinterpret_cast<const uint4 *>(dZh + ((int64_t)b * L.P + p) * 32);
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const uint4 z = rowv ? __ldg(zr + j) : make_uint4(0u, 0u, 0u, 0u);
        const uint32_t w4[4] = {z.x, z.y, z.z, z.w};
#pragma unroll
        for (int h = 0; h < 8; h++)
          st_bf16(S.Z, wg_off(8 * j + h, tid, WG_KS_Z), (w4[h >> 1] >> (16 * (h & 1))) & 0xffffu);
      }
    } else {
      const unsigned short *zr = reinterpret_cast<const unsigned short *>(dZh + ((int64_t)b * L.P + p) * CO);
#pragma unroll
      for (int co = 0; co < CO; co++) st_bf16(S.Z, wg_off(co, tid, WG_KS_Z), rowv ? __ldg(zr + co) : 0u);
    }
    for (int g = 0; g < C::NG && ok; g++, nuse++) {
      const int buf = nuse & 1;
      const uint32_t used = buf ? use1 : use0;
      if (used > 0 && !tc::mbar_wait(&S.done[buf], (used - 1) & 1, CT_WAIT_LIMIT)) {
        ok = false;
        break;
      }
      unsigned char *a = S.A[buf];
      for (int tl = 0; tl < C::TPG; tl++) {
        const int t = g * C::TPG + tl;
        const int dx = t / 9 - 1, dy = (t / 3) % 3 - 1, dz = t % 3 - 1;
        const bool v = t < 27 && rowv && (unsigned)(ix + dx) < (unsigned)L.nx &&
                       (unsigned)(iy + dy) < (unsigned)L.ny && (unsigned)(iz + dz) < (unsigned)L.nz;
        const int64_t q = (int64_t)b * L.P + p + ((int64_t)dx * L.ny + dy) * L.nz + dz;
        if constexpr (CI == 32) {
          const uint4 *xr = reinterpret_cast<const uint4 *>(X + q * 32);
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const uint4 x = v ? __ldg(xr + j) : make_uint4(0u, 0u, 0u, 0u);
            const uint32_t w4[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
            for (int h = 0; h < 8; h++)
              st_bf16(a, wg_off(tl * 32 + 8 * j + h, tid, WG_KS_A), (w4[h >> 1] >> (16 * (h & 1))) & 0xffffu);
          }
        } else {
          const unsigned short *xr = reinterpret_cast<const unsigned short *>(X + q * CI);
#pragma unroll
          for (int ci = 0; ci < CI; ci++) st_bf16(a, wg_off(tl * CI + ci, tid, WG_KS_A), v ? __ldg(xr + ci) : 0u);
        }
      }
      for (int m = C::TPG * CI; m < 128; m++) st_bf16(a, wg_off(m, tid, WG_KS_A), 0u);  // rows past the group
      tc::fence_proxy_async();
      tc::fence_before_sync();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
        const uint32_t abase = tc::smem_u32(a), zbase = tc::smem_u32(S.Z);
        for (int ks = 0; ks < 8; ks++) {
          const uint64_t ad = tc::smem_desc(abase + (uint32_t)(ks * WG_KS_A), WG_LBO, WG_SBO);
          const uint64_t zd = tc::smem_desc(zbase + (uint32_t)(ks * WG_KS_Z), WG_LBO, WG_SBO);
          tc::mma_bf16(taddr + (uint32_t)(g * C::NPAD), ad, zd, idesc, (!first || ks > 0) ? 1u : 0u);
        }
        tc::mma_commit(&S.done[buf]);
      }
      if (buf) use1++;
      else use0++;
    }
    first = false;
  }
  // the last commit covers every MMA of the CTA
  if (ok && nuse > 0) {
    const int lb = (nuse - 1) & 1;
    const uint32_t used = lb ? use1 : use0;
    if (!tc::mbar_wait(&S.done[lb], (used - 1) & 1, CT_WAIT_LIMIT)) ok = false;
  }
  if (ok && nuse > 0) {
    tc::fence_after_sync();
    const int m = warp * 32 + lane;  // TMEM lane = row (tl, ci)
    for (int g = 0; g < C::NG; g++) {
      uint32_t r[32];  // the group's NPAD columns (and the next group's, unused)
      tc::tmem_ld_32x32b_x32(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)(g * C::NPAD), r);
      const int t = g * C::TPG + m / CI, ci = m % CI;
      if (m < C::TPG * CI && t < 27)
#pragma unroll
        for (int co = 0; co < CO; co++) atomicAdd(gW + ((int64_t)co * 27 + t) * CI + ci, __uint_as_float(r[co]));
    }
  }
  if (!ok && tid == 0) {
    atomicCAS(err, 0, 2);
    if (use0 > 0) tc::mbar_wait(&S.done[0], (use0 - 1) & 1, CT_WAIT_LIMIT);
    if (use1 > 0) tc::mbar_wait(&S.done[1], (use1 - 1) & 1, CT_WAIT_LIMIT);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, C::COLS);
}

// db[co] += sum over the points of dZ[p][co] (FP32)
__global__ void bias_grad_kernel(const float *__restrict__ dZ, int Co, int64_t NP, float *__restrict__ db)
{
  __shared__ float sh[8][33];
  const int co = threadIdx.x & 31, pl = threadIdx.x >> 5;
  float s = 0.f;
  if (co < Co)
    for (int64_t p = (int64_t)blockIdx.x * 8 + pl; p < NP; p += (int64_t)gridDim.x * 8) s += dZ[p * Co + co];
  sh[pl][co] = s;
  __syncthreads();
  if (threadIdx.x < 32 && co < Co) {
    float t = 0.f;
    for (int k = 0; k < 8; k++) t += sh[k][co];
    atomicAdd(db + co, t);
  }
}

// dZ (FP32, masked by ReLU') -> BF16 copy for the tensor-core data gradient
__global__ void to_bf16_kernel(const float *src, __nv_bfloat16 *dst, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = __float2bfloat16_rn(src[i]);
}

// loss = mean (y - target)^2 over n values; dY = 2 (y - target) / n
template <typename T>
__global__ void mse_kernel(const T *y, const float *target, float *dY, float *loss, int64_t n)
{
  __shared__ float sh[32];
  float s = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float d = ld(y + i) - target[i];
    dY[i] = 2.f * d / (float)n;
    s += d * d;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (int)(blockDim.x / 32) ? sh[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) atomicAdd(loss, s / (float)n);
  }
}

template <typename T>
__global__ void adam_kernel(float *w, float *m, float *v, const float *g, T *wt, int n, float lr, float b1,
                            float b2, float eps, float c1, float c2)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  if (wt) wt[i] = cvt<T>(wi);
}

template <typename T>
__global__ void cast_kernel(const float *src, T *dst, int64_t n)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = cvt<T>(src[i]);
}
template <typename T>
__global__ void uncast_kernel(const T *src, float *dst, int64_t n)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = ld(src + i);
}

}  // namespace igap

using namespace igap;

// ------------------------------------------------------------------ ABI
struct igapgpu_net {
  int storage;  // 0 float, 1 bf16
  Lattice L;
  int bmax;
  int64_t woff[NL + 1], boff[NL + 1];
  int64_t nw, nb;
  float *W = nullptr, *bias = nullptr;        // FP32 master
  void *Wt = nullptr;                         // storage-type weights
  float *gW = nullptr, *gb = nullptr;         // gradients
  float *mW = nullptr, *vW = nullptr, *mb = nullptr, *vb = nullptr;
  void *act[NL + 1] = {};                     // activations (storage type), act[0] = input
  float *dA = nullptr, *dB = nullptr;         // gradient scratch [bmax*P*32]
  float *target = nullptr, *loss = nullptr;
  __nv_bfloat16 *dZh = nullptr;               // BF16 copy of a layer's output gradient [bmax*P*32]
  __nv_bfloat16 *Wk = nullptr;                // one layer's weights arranged per tap [27][32][32]
  int *err = nullptr;                         // device error word of the tensor-core convolutions
  int step = 0;
  cudaStream_t stream = nullptr;
};

namespace {
// The tensor-core convolution for the 32 -> 32 layers of a BF16 network
// (IGAPGPU_NET_TC=0 keeps the scalar kernels, for comparisons).
bool use_tc(const igapgpu_net *n, int l)
{
  const char *e = getenv("IGAPGPU_NET_TC");
  return n->storage == 1 && kCin[l] == 32 && kCout[l] == 32 && !(e && e[0] == '0');
}

template <int MODE>
int launch_conv_tc(igapgpu_net *n, const __nv_bfloat16 *in, const __nv_bfloat16 *W, const float *bias, void *out,
                   int B, int relu)
{
  conv_tc_weights_kernel<<<(27 * 32 * 32 + 255) / 256, 256, 0, n->stream>>>(W, n->Wk, MODE);
  count_launch();
  static bool attr[2] = {false, false};
  const size_t smem = sizeof(ConvTcSmem) + 1024;
  if (!attr[MODE]) {
    IGAP_CUDA(cudaFuncSetAttribute(conv_tc_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr[MODE] = true;
  }
  int dev = 0, nsm = 0;
  IGAP_CUDA(cudaGetDevice(&dev));
  IGAP_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int64_t ntiles = (n->L.P + 127) / 128 * B;
  const int grid = (int)(ntiles < (int64_t)nsm * 3 ? ntiles : (int64_t)nsm * 3);
  conv_tc_kernel<MODE><<<grid, CT_THREADS, smem, n->stream>>>(in, n->Wk, bias, out, n->L, B, relu, n->err);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

// the weight gradient of every layer (9 or 32 inputs, 32 or 3 outputs)
bool use_tc_wgrad(const igapgpu_net *n, int l)
{
  const char *e = getenv("IGAPGPU_NET_TC");
  return n->storage == 1 && (kCout[l] == 32 || kCout[l] == 3) && (kCin[l] == 32 || kCin[l] == 9) &&
         !(e && e[0] == '0');
}

template <int CI, int CO>
int launch_wgrad_tc(igapgpu_net *n, const __nv_bfloat16 *X, float *gW, int B)
{
  static bool attr = false;
  const size_t smem = sizeof(WgradSmem) + 1024;
  if (!attr) {
    IGAP_CUDA(cudaFuncSetAttribute(conv_tc_wgrad_kernel<CI, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
    attr = true;
  }
  int dev = 0, nsm = 0;
  IGAP_CUDA(cudaGetDevice(&dev));
  IGAP_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int64_t ntiles = (n->L.P + 127) / 128 * B;
  const int grid = (int)(ntiles < (int64_t)nsm * 2 ? ntiles : (int64_t)nsm * 2);
  conv_tc_wgrad_kernel<CI, CO><<<grid, CT_THREADS, smem, n->stream>>>(X, n->dZh, gW, n->L, B, n->err);
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

// error word of the tensor-core convolutions (synchronises)
int check_err(igapgpu_net *n)
{
  int h = 0;
  IGAP_CUDA(cudaMemcpyAsync(&h, n->err, sizeof(int), cudaMemcpyDeviceToHost, n->stream));
  IGAP_CUDA(cudaStreamSynchronize(n->stream));
  if (h) {
    IGAP_CUDA(cudaMemsetAsync(n->err, 0, sizeof(int), n->stream));
    set_error("tensor-core convolution: a bounded mbarrier wait expired (code %d)", h);
    return IGAPGPU_ERR_TIMEOUT;
  }
  return IGAPGPU_OK;
}

template <typename T>
int net_forward_t(igapgpu_net *n, int B)
{
  const Lattice L = n->L;
  for (int l = 0; l < NL; l++) {
    if (use_tc(n, l)) {
      const int r = launch_conv_tc<0>(n, (const __nv_bfloat16 *)n->act[l], (const __nv_bfloat16 *)n->Wt + n->woff[l],
                                      n->bias + n->boff[l], n->act[l + 1], B, l < NL - 1);
      if (r) return r;
      continue;
    }
    const int64_t tot = (int64_t)B * L.P * kCout[l];
    conv_fwd<T><<<(unsigned)((tot + 255) / 256), 256, 0, n->stream>>>(
        (const T *)n->act[l], kCin[l], (const T *)n->Wt + n->woff[l], n->bias + n->boff[l], (T *)n->act[l + 1],
        kCout[l], L, B, l < NL - 1);
    count_launch();
  }
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

template <typename T>
int net_backward_t(igapgpu_net *n, int B)
{
  // dA holds dLoss/d(output) on entry (FP32, [B][P][3])
  const Lattice L = n->L;
  float *dcur = n->dA, *dnext = n->dB;
  for (int l = NL - 1; l >= 0; l--) {
    const int64_t nout = (int64_t)B * L.P * kCout[l];
    if (l < NL - 1) {
      relu_bwd<T><<<(unsigned)((nout + 255) / 256), 256, 0, n->stream>>>(dcur, (const T *)n->act[l + 1], nout);
      count_launch();
    }
    // the BF16 copy of the output gradient feeds both tensor-core products
    const bool tcw = use_tc_wgrad(n, l), tcd = l > 0 && use_tc(n, l);
    if (tcw || tcd) {
      to_bf16_kernel<<<152 * 8, 256, 0, n->stream>>>(dcur, n->dZh, nout);
      count_launch();
    }
    if (tcw) {
      const __nv_bfloat16 *xin = (const __nv_bfloat16 *)n->act[l];
      float *gw = n->gW + n->woff[l];
      const int r = kCin[l] == 9   ? launch_wgrad_tc<9, 32>(n, xin, gw, B)
                    : kCout[l] == 3 ? launch_wgrad_tc<32, 3>(n, xin, gw, B)
                                    : launch_wgrad_tc<32, 32>(n, xin, gw, B);
      if (r) return r;
      bias_grad_kernel<<<152 * 4, 256, 0, n->stream>>>(dcur, kCout[l], (int64_t)B * L.P, n->gb + n->boff[l]);
      count_launch();
    } else {
      conv_bwd_weight<T><<<kCout[l] * 27, 256, 0, n->stream>>>(dcur, kCout[l], (const T *)n->act[l], kCin[l],
                                                                 n->gW + n->woff[l], n->gb + n->boff[l], L, B);
      count_launch();
    }
    if (l > 0) {
      const int64_t nin = (int64_t)B * L.P * kCin[l];
      if (tcd) {
        const int r = launch_conv_tc<1>(n, n->dZh, (const __nv_bfloat16 *)n->Wt + n->woff[l], nullptr, dnext, B, 0);
        if (r) return r;
      } else {
        conv_bwd_data<T><<<(unsigned)((nin + 255) / 256), 256, 0, n->stream>>>(dcur, kCout[l], (const T *)n->Wt + n->woff[l],
                                                                               dnext, kCin[l], L, B);
        count_launch();
      }
      float *tmp = dcur;
      dcur = dnext;
      dnext = tmp;
    }
  }
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

size_t tsize(int storage) { return storage ? sizeof(__nv_bfloat16) : sizeof(float); }
}  // namespace

extern "C" {

int igapgpu_net_create(igapgpu_net **out, int nx, int ny, int nz, int batch_max, int storage)
{
  if (!out || nx < 1 || ny < 1 || nz < 1 || batch_max < 1 || (storage != 0 && storage != 1)) {
    set_error("net_create: bad arguments");
    return IGAPGPU_ERR_ARG;
  }
  igapgpu_net *n = new igapgpu_net();
  n->storage = storage;
  n->L.nx = nx;
  n->L.ny = ny;
  n->L.nz = nz;
  n->L.P = (int64_t)nx * ny * nz;
  n->bmax = batch_max;
  n->woff[0] = n->boff[0] = 0;
  for (int l = 0; l < NL; l++) {
    n->woff[l + 1] = n->woff[l] + (int64_t)kCout[l] * 27 * kCin[l];
    n->boff[l + 1] = n->boff[l] + kCout[l];
  }
  n->nw = n->woff[NL];
  n->nb = n->boff[NL];
  const size_t ts = tsize(storage);
  const int64_t maxact = (int64_t)batch_max * n->L.P * 32;
  bool ok = cudaMalloc(&n->W, sizeof(float) * n->nw) == cudaSuccess &&
            cudaMalloc(&n->bias, sizeof(float) * n->nb) == cudaSuccess &&
            cudaMalloc(&n->Wt, ts * n->nw) == cudaSuccess &&
            cudaMalloc(&n->gW, sizeof(float) * n->nw) == cudaSuccess &&
            cudaMalloc(&n->gb, sizeof(float) * n->nb) == cudaSuccess &&
            cudaMalloc(&n->mW, sizeof(float) * n->nw) == cudaSuccess &&
            cudaMalloc(&n->vW, sizeof(float) * n->nw) == cudaSuccess &&
            cudaMalloc(&n->mb, sizeof(float) * n->nb) == cudaSuccess &&
            cudaMalloc(&n->vb, sizeof(float) * n->nb) == cudaSuccess &&
            cudaMalloc(&n->dA, sizeof(float) * maxact) == cudaSuccess &&
            cudaMalloc(&n->dB, sizeof(float) * maxact) == cudaSuccess &&
            cudaMalloc(&n->target, sizeof(float) * batch_max * n->L.P * 3) == cudaSuccess &&
            cudaMalloc(&n->loss, sizeof(float)) == cudaSuccess &&
            cudaMalloc(&n->err, sizeof(int)) == cudaSuccess &&
            (storage == 0 || (cudaMalloc(&n->dZh, sizeof(__nv_bfloat16) * maxact) == cudaSuccess &&
                              cudaMalloc(&n->Wk, sizeof(__nv_bfloat16) * 27 * 32 * 32) == cudaSuccess));
  for (int l = 0; l <= NL && ok; l++) {
    const int C = l == 0 ? kCin[0] : kCout[l - 1];
    ok = cudaMalloc(&n->act[l], ts * (size_t)batch_max * n->L.P * C) == cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    set_error("net_create: device allocation failed");
    return IGAPGPU_ERR_NOMEM;
  }
  cudaMemset(n->err, 0, sizeof(int));
  cudaMemset(n->mW, 0, sizeof(float) * n->nw);
  cudaMemset(n->vW, 0, sizeof(float) * n->nw);
  cudaMemset(n->mb, 0, sizeof(float) * n->nb);
  cudaMemset(n->vb, 0, sizeof(float) * n->nb);
  *out = n;
  return IGAPGPU_OK;
}

int igapgpu_net_destroy(igapgpu_net *n)
{
  if (!n) return IGAPGPU_OK;
  void *bufs[] = {n->W, n->bias, n->Wt, n->gW, n->gb, n->mW, n->vW, n->mb, n->vb, n->dA, n->dB, n->target, n->loss,
                  n->dZh, n->Wk, n->err};
  for (void *p : bufs)
    if (p) cudaFree(p);
  for (int l = 0; l <= NL; l++)
    if (n->act[l]) cudaFree(n->act[l]);
  delete n;
  return IGAPGPU_OK;
}

int64_t igapgpu_net_num_params(igapgpu_net *n) { return n ? n->nw + n->nb : 0; }

int igapgpu_net_set_stream(igapgpu_net *n, void *s)
{
  if (!n) return IGAPGPU_ERR_ARG;
  n->stream = (cudaStream_t)s;
  return IGAPGPU_OK;
}

// params: host FP32 array, weights (layer by layer [Co][27][Ci]) then biases
int igapgpu_net_set_params(igapgpu_net *n, const float *params)
{
  if (!n || !params) return IGAPGPU_ERR_ARG;
  IGAP_CUDA(cudaMemcpy(n->W, params, sizeof(float) * n->nw, cudaMemcpyHostToDevice));
  IGAP_CUDA(cudaMemcpy(n->bias, params + n->nw, sizeof(float) * n->nb, cudaMemcpyHostToDevice));
  if (n->storage)
    cast_kernel<__nv_bfloat16><<<(unsigned)((n->nw + 255) / 256), 256, 0, n->stream>>>(n->W, (__nv_bfloat16 *)n->Wt, n->nw);
  else
    cast_kernel<float><<<(unsigned)((n->nw + 255) / 256), 256, 0, n->stream>>>(n->W, (float *)n->Wt, n->nw);
  count_launch();
  IGAP_CHECK_LAUNCH();
  IGAP_CUDA(cudaStreamSynchronize(n->stream));
  n->step = 0;
  return IGAPGPU_OK;
}

int igapgpu_net_get_params(igapgpu_net *n, float *params)
{
  if (!n || !params) return IGAPGPU_ERR_ARG;
  IGAP_CUDA(cudaStreamSynchronize(n->stream));
  IGAP_CUDA(cudaMemcpy(params, n->W, sizeof(float) * n->nw, cudaMemcpyDeviceToHost));
  IGAP_CUDA(cudaMemcpy(params + n->nw, n->bias, sizeof(float) * n->nb, cudaMemcpyDeviceToHost));
  return IGAPGPU_OK;
}

// grads: host FP32, same layout as params (accumulated since the last zeroing)
int igapgpu_net_get_grads(igapgpu_net *n, float *grads)
{
  if (!n || !grads) return IGAPGPU_ERR_ARG;
  IGAP_CUDA(cudaStreamSynchronize(n->stream));
  IGAP_CUDA(cudaMemcpy(grads, n->gW, sizeof(float) * n->nw, cudaMemcpyDeviceToHost));
  IGAP_CUDA(cudaMemcpy(grads + n->nw, n->gb, sizeof(float) * n->nb, cudaMemcpyDeviceToHost));
  return IGAPGPU_OK;
}

// in: device FP32 [B][P][9]; out: device FP32 [B][P][3]
int igapgpu_net_forward(igapgpu_net *n, const float *in, float *out, int B)
{
  if (!n || !in || !out || B < 1 || B > n->bmax) {
    set_error("net_forward: bad arguments (batch %d, max %d)", B, n ? n->bmax : 0);
    return IGAPGPU_ERR_ARG;
  }
  const int64_t nin = (int64_t)B * n->L.P * 9, nout = (int64_t)B * n->L.P * 3;
  int r;
  if (n->storage) {
    cast_kernel<__nv_bfloat16><<<(unsigned)((nin + 255) / 256), 256, 0, n->stream>>>(in, (__nv_bfloat16 *)n->act[0], nin);
    count_launch();
    if ((r = net_forward_t<__nv_bfloat16>(n, B))) return r;
    uncast_kernel<__nv_bfloat16><<<(unsigned)((nout + 255) / 256), 256, 0, n->stream>>>((const __nv_bfloat16 *)n->act[NL], out, nout);
    count_launch();
    IGAP_CHECK_LAUNCH();
    return check_err(n);
  } else {
    cast_kernel<float><<<(unsigned)((nin + 255) / 256), 256, 0, n->stream>>>(in, (float *)n->act[0], nin);
    count_launch();
    if ((r = net_forward_t<float>(n, B))) return r;
    uncast_kernel<float><<<(unsigned)((nout + 255) / 256), 256, 0, n->stream>>>((const float *)n->act[NL], out, nout);
  }
  count_launch();
  IGAP_CHECK_LAUNCH();
  return IGAPGPU_OK;
}

// Forward + MSE loss against target (device FP32 [B][P][3]) + backward;
// gradients are zeroed first.  lr > 0 also applies one Adam step.
// loss_out: host float (synchronises).
int igapgpu_net_train_step(igapgpu_net *n, const float *in, const float *target, int B, float lr,
                           float *loss_out)
{
  if (!n || !in || !target || B < 1 || B > n->bmax) {
    set_error("net_train_step: bad arguments");
    return IGAPGPU_ERR_ARG;
  }
  const int64_t nout = (int64_t)B * n->L.P * 3;
  IGAP_CUDA(cudaMemsetAsync(n->gW, 0, sizeof(float) * n->nw, n->stream));
  IGAP_CUDA(cudaMemsetAsync(n->gb, 0, sizeof(float) * n->nb, n->stream));
  IGAP_CUDA(cudaMemsetAsync(n->loss, 0, sizeof(float), n->stream));
  const int64_t nin = (int64_t)B * n->L.P * 9;
  int r;
  if (n->storage) {
    cast_kernel<__nv_bfloat16><<<(unsigned)((nin + 255) / 256), 256, 0, n->stream>>>(in, (__nv_bfloat16 *)n->act[0], nin);
    count_launch();
    if ((r = net_forward_t<__nv_bfloat16>(n, B))) return r;
    mse_kernel<__nv_bfloat16><<<152, 256, 0, n->stream>>>((const __nv_bfloat16 *)n->act[NL], target, n->dA, n->loss, nout);
    count_launch();
    if ((r = net_backward_t<__nv_bfloat16>(n, B))) return r;
  } else {
    cast_kernel<float><<<(unsigned)((nin + 255) / 256), 256, 0, n->stream>>>(in, (float *)n->act[0], nin);
    count_launch();
    if ((r = net_forward_t<float>(n, B))) return r;
    mse_kernel<float><<<152, 256, 0, n->stream>>>((const float *)n->act[NL], target, n->dA, n->loss, nout);
    count_launch();
    if ((r = net_backward_t<float>(n, B))) return r;
  }
  if (lr > 0.f) {
    n->step++;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.f - powf(b1, (float)n->step), c2 = 1.f - powf(b2, (float)n->step);
    if (n->storage) {
      adam_kernel<__nv_bfloat16><<<(unsigned)((n->nw + 255) / 256), 256, 0, n->stream>>>(
          n->W, n->mW, n->vW, n->gW, (__nv_bfloat16 *)n->Wt, (int)n->nw, lr, b1, b2, eps, c1, c2);
      adam_kernel<__nv_bfloat16><<<(unsigned)((n->nb + 255) / 256), 256, 0, n->stream>>>(
          n->bias, n->mb, n->vb, n->gb, (__nv_bfloat16 *)nullptr, (int)n->nb, lr, b1, b2, eps, c1, c2);
    } else {
      adam_kernel<float><<<(unsigned)((n->nw + 255) / 256), 256, 0, n->stream>>>(
          n->W, n->mW, n->vW, n->gW, (float *)n->Wt, (int)n->nw, lr, b1, b2, eps, c1, c2);
      adam_kernel<float><<<(unsigned)((n->nb + 255) / 256), 256, 0, n->stream>>>(
          n->bias, n->mb, n->vb, n->gb, (float *)nullptr, (int)n->nb, lr, b1, b2, eps, c1, c2);
    }
    count_launch(2);
  }
  IGAP_CHECK_LAUNCH();
  if (loss_out) {
    IGAP_CUDA(cudaMemcpyAsync(loss_out, n->loss, sizeof(float), cudaMemcpyDeviceToHost, n->stream));
    IGAP_CUDA(cudaStreamSynchronize(n->stream));
    if (n->storage) return check_err(n);
  }
  return IGAPGPU_OK;
}

}  // extern "C"
