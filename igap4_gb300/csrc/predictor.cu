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
#include <string.h>

#include "common.cuh"

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
  int step = 0;
  cudaStream_t stream = nullptr;
};

namespace {
template <typename T>
int net_forward_t(igapgpu_net *n, int B)
{
  const Lattice L = n->L;
  for (int l = 0; l < NL; l++) {
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
    conv_bwd_weight<T><<<kCout[l] * 27, 256, 0, n->stream>>>(dcur, kCout[l], (const T *)n->act[l], kCin[l],
                                                               n->gW + n->woff[l], n->gb + n->boff[l], L, B);
    count_launch();
    if (l > 0) {
      const int64_t nin = (int64_t)B * L.P * kCin[l];
      conv_bwd_data<T><<<(unsigned)((nin + 255) / 256), 256, 0, n->stream>>>(dcur, kCout[l], (const T *)n->Wt + n->woff[l],
                                                                             dnext, kCin[l], L, B);
      count_launch();
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
            cudaMalloc(&n->loss, sizeof(float)) == cudaSuccess;
  for (int l = 0; l <= NL && ok; l++) {
    const int C = l == 0 ? kCin[0] : kCout[l - 1];
    ok = cudaMalloc(&n->act[l], ts * (size_t)batch_max * n->L.P * C) == cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    set_error("net_create: device allocation failed");
    return IGAPGPU_ERR_NOMEM;
  }
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
  void *bufs[] = {n->W, n->bias, n->Wt, n->gW, n->gb, n->mW, n->vW, n->mb, n->vb, n->dA, n->dB, n->target, n->loss};
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
  }
  return IGAPGPU_OK;
}

}  // extern "C"
