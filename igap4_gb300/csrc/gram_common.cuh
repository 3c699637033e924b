// Helpers shared by the Gram-form tensor-core tangents of the linear law
// (tc_gram.cu: TF32x3 split precision; tc_ozaki.cu: FP64-quality BF16 slices).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace igap {

// Index of the Hessian component (i, m) among the 6 stored second
// derivatives: (0,0)0 (0,1)1 (0,2)2 (1,1)3 (1,2)4 (2,2)5.
__device__ __forceinline__ int hess_slot(int i, int m)
{
  const int a = i < m ? i : m, b = i < m ? m : i;
  return a == 0 ? b : (a == 1 ? 2 + b : 5);
}

// float -> double on the integer pipe (bit-exact with the conversion for
// normal numbers and zeros; subnormals, infinities and NaN take the
// conversion instruction): FP64 work is scarce on this GPU.
static __device__ __noinline__ double f32_to_f64_rare(float f) { return (double)f; }

__device__ __forceinline__ double f32_to_f64(float f)
{
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xffu;
  if ((b & 0x7fffffffu) == 0u) return __hiloint2double((int)(b & 0x80000000u), 0);
  if (__builtin_expect(e == 0u || e == 0xffu, 0)) return f32_to_f64_rare(f);
  const uint32_t hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3);
  return __hiloint2double((int)hi, (int)(b << 29));
}

static __device__ __noinline__ double f32_to_f64_scaled_rare(float f, int sh) { return ldexp((double)f, sh); }

// f * 2^sh as a double, the scaling folded into the exponent on the integer
// pipe (exact); |sh| small enough that the result stays a normal double.
// Zeros stay on the integer pipe; subnormal, infinite and NaN inputs take an
// out-of-line call (the FP64 pipe only there).
__device__ __forceinline__ double f32_to_f64_scaled(float f, int sh)
{
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xffu;
  if ((b & 0x7fffffffu) == 0u) return __hiloint2double((int)(b & 0x80000000u), 0);
  if (__builtin_expect(e == 0u || e == 0xffu, 0)) return f32_to_f64_scaled_rare(f, sh);
  const uint32_t hi = (b & 0x80000000u) | ((uint32_t)((int)e + 896 + sh) << 20) | ((b & 0x7fffffu) >> 3);
  return __hiloint2double((int)hi, (int)(b << 29));
}

}  // namespace igap
