// FP64 2-norm that allocates no device memory.
//
// igapgpu_norm2 (krylov.cu) keeps its per-block partial sums in a buffer the
// library obtains from cudaMalloc when a context is created.  Some callers
// cannot provide that: a host application whose pool allocator already owns
// the device memory (PyTorch's caching allocator, a PETSc device pool), so an
// extra cudaMalloc fails or escapes the pool's accounting, and code paths that
// must not allocate or free device memory because cudaMalloc / cudaFree can
// synchronise the whole device.  For them igapgpu_norm2_noalloc keeps its
// scratch in a fixed array compiled into the library instead.
//
// The scratch array is a file-scope __device__ variable: it exists on every
// GPU on which the library's module is loaded and stays there until the
// process exits.  In host code its name is only a host-side stand-in, not a
// device address, so the device address is looked up once per device with
// cudaGetSymbolAddress (with that device current) and passed to the kernels.
// That lookup happens in the first call on each device.
#include <cuda_runtime.h>
#include <mutex>

#include "common.cuh"

namespace igap {
namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_ITEMS = 16;
constexpr int64_t NA_CHUNK = (int64_t)NA_THREADS * NA_ITEMS;   // elements per partial sum
constexpr int NA_MAX_PARTIALS = 8192;                           // 64 KiB of partial sums
constexpr int64_t NA_MAX_N = NA_CHUNK * NA_MAX_PARTIALS;        // 33,554,432 elements
constexpr int NA_MAX_DEVICES = 64;

}  // namespace

// Partial sums [0, NA_MAX_PARTIALS) and the result slot [NA_MAX_PARTIALS].
static __device__ __align__(256) double g_norm2_scratch[NA_MAX_PARTIALS + 1];

// One partial sum of squares per chunk of NA_CHUNK elements; the chunking
// does not depend on the GPU, so the result is the same on every device.
__global__ void __launch_bounds__(NA_THREADS) na_partial_kernel(const double *__restrict__ x, int64_t n,
                                                                double *__restrict__ partials)
{
  __shared__ double sh[NA_THREADS / 32];
  const int64_t base = (int64_t)blockIdx.x * NA_CHUNK;
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < NA_ITEMS; i++) {
    const int64_t k = base + (int64_t)i * NA_THREADS + threadIdx.x;
    if (k < n) s = fma(x[k], x[k], s);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < NA_THREADS / 32 ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
  }
}

__global__ void __launch_bounds__(1024) na_final_kernel(const double *__restrict__ partials, int np,
                                                        double *__restrict__ out)
{
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += partials[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (int)(blockDim.x / 32) ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[0] = sqrt(s);
  }
}

// Device address of g_norm2_scratch, looked up once per device.
static double *g_scratch_addr[NA_MAX_DEVICES];
static std::mutex g_scratch_mu;

static int scratch_address(double **p)
{
  int dev = 0;
  IGAP_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= NA_MAX_DEVICES) {
    set_error("norm2_noalloc: device ordinal %d out of range", dev);
    return IGAPGPU_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void *a = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&a, g_norm2_scratch);
    if (e != cudaSuccess || !a) {
      cudaGetLastError();
      set_error("norm2_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                cudaGetErrorString(e));
      return IGAPGPU_ERR_CUDA;
    }
    g_scratch_addr[dev] = static_cast<double *>(a);
  }
  *p = g_scratch_addr[dev];
  return IGAPGPU_OK;
}

}  // namespace igap

using namespace igap;

extern "C" int igapgpu_norm2_noalloc(const double *x, int64_t n, double *out, void *stream)
{
  if (!out || (n > 0 && !x) || n < 0) {
    set_error("norm2_noalloc: null pointer or negative size");
    return IGAPGPU_ERR_ARG;
  }
  if (n > NA_MAX_N) {
    set_error("norm2_noalloc: n = %lld exceeds the maximum of %lld elements "
              "(fixed scratch of %d partial sums); use igapgpu_norm2",
              (long long)n, (long long)NA_MAX_N, NA_MAX_PARTIALS);
    return IGAPGPU_ERR_ARG;
  }
  if (n > 0 && !is_device_ptr(x)) {
    set_error("norm2_noalloc: x must be device memory (staging host data would allocate)");
    return IGAPGPU_ERR_ARG;
  }
  double *scratch = nullptr;
  int r = scratch_address(&scratch);
  if (r) return r;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int np = (int)((n + NA_CHUNK - 1) / NA_CHUNK);
  if (np > 0) {
    na_partial_kernel<<<np, NA_THREADS, 0, s>>>(x, n, scratch);
    count_launch();
    IGAP_CHECK_LAUNCH();
  }
  const bool out_dev = is_device_ptr(out);
  double *dst = out_dev ? out : scratch + NA_MAX_PARTIALS;
  na_final_kernel<<<1, 1024, 0, s>>>(scratch, np, dst);
  count_launch();
  IGAP_CHECK_LAUNCH();
  if (!out_dev) {
    IGAP_CUDA(cudaMemcpyAsync(out, dst, sizeof(double), cudaMemcpyDeviceToHost, s));
    IGAP_CUDA(cudaStreamSynchronize(s));
  }
  return IGAPGPU_OK;
}
