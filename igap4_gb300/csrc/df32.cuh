// Error-free transformations and double-FP32 ("double-float") arithmetic on
// the FP32 pipe.  A value is carried as an unevaluated pair hi + lo of floats
// (|lo| <= ulp(hi) / 2 after renormalisation): 48 significant bits, about
// 3.6e-15 relative, with the FP32 exponent range.  FP64 arithmetic on this
// GPU runs at about 1/64 of the FP32 rate, so FP64-accurate contractions go
// through these pairs instead.
//
// Methods: Knuth's two-sum, Dekker's fast two-sum, the fused-multiply-add
// two-product, and the compensated dot product "Dot2" of Ogita, Rump and
// Oishi (SIAM J. Sci. Comput. 26, 2005): the running sum s gathers the
// rounded products, c gathers the exact rounding errors of every product
// and every addition, and s + c is as accurate as the dot product evaluated
// in twice the working precision.  Every operation is spelled with the
// round-to-nearest intrinsics so that the compiler cannot contract or
// reassociate it.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace igap {

__device__ __forceinline__ float two_sum(float a, float b, float &e)
{
  const float s = __fadd_rn(a, b), bv = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bv)), __fsub_rn(b, bv));
  return s;
}

__device__ __forceinline__ float two_prod(float a, float b, float &e)
{
  const float p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
  return p;
}

// |a| >= |b| (or a == 0)
__device__ __forceinline__ float2 fast_two_sum(float a, float b)
{
  const float s = __fadd_rn(a, b);
  return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ float2 df_add(float2 a, float2 b)
{
  float e;
  const float s = two_sum(a.x, b.x, e);
  return fast_two_sum(s, __fadd_rn(e, __fadd_rn(a.y, b.y)));
}

__device__ __forceinline__ float2 df_mul(float2 a, float2 b)
{
  float e;
  const float p = two_prod(a.x, b.x, e);
  e = __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, e));
  return fast_two_sum(p, e);
}

// One Dot2 term: (s, c) += a * b for pairs a, b (the lo * lo product,
// 2^-48 relative, is left out).
__device__ __forceinline__ void dot2(float &s, float &c, float2 a, float2 b)
{
  float ep, es;
  const float p = two_prod(a.x, b.x, ep);
  ep = __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, ep));
  s = two_sum(s, p, es);
  c = __fadd_rn(c, __fadd_rn(es, ep));
}

// The pair of a Dot2 accumulator.
__device__ __forceinline__ float2 dot2_pair(float s, float c) { return fast_two_sum(s, c); }

static __device__ __noinline__ float2 f64_to_pair_rare(double x)
{
  const float h = __double2float_rn(x);
  return make_float2(h, __double2float_rn(x - (double)h));
}

// x = hi + lo to 2^-48 |x| on the integer pipe: hi is x truncated to 24
// significant bits (exponent and top mantissa bits moved into a float), lo
// the remaining 29 mantissa bits converted and scaled by 2^(e - 52).  Zeros
// stay on the integer pipe; |x| outside [2^-74, 2^127), subnormal and
// non-finite values take the out-of-line FP64 path.
__device__ __forceinline__ float2 f64_to_pair(double x)
{
  const uint32_t hw = (uint32_t)__double2hiint(x), lw = (uint32_t)__double2loint(x);
  const uint32_t ef = (hw >> 20) & 0x7ffu;  // biased exponent, e = ef - 1023
  if (__builtin_expect(ef - 949u > 200u, 0)) {
    if ((hw & 0x7fffffffu) == 0u && lw == 0u) return make_float2(__uint_as_float(hw & 0x80000000u), 0.f);
    return f64_to_pair_rare(x);
  }
  const uint32_t sg = hw & 0x80000000u;
  const float h = __uint_as_float(sg | ((ef - 896u) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
  const float l = __fmul_rn(__uint2float_rn(lw & 0x1fffffffu), __uint_as_float((ef - 948u) << 23));
  return make_float2(h, __uint_as_float(__float_as_uint(l) | sg));
}

}  // namespace igap
