// nsp_cvt.cuh -- double <-> float conversions on the integer pipe.
//
// On GB300 the hardware conversion instructions between FP64 and FP32 issue on the
// FP64 pipe (one warp instruction per 64 cycles per SM sub-partition), the bound of
// the linear pass.  These routines assemble the result from the bit fields with
// integer instructions only (no hardware fallback, which the compiler may predicate
// rather than branch around): double -> float rounds to nearest even, float ->
// double is exact, Inf and NaN are kept (NaN as the quiet NaN of its sign), and
// magnitudes below 2^-126, the float denormal range, flush to a signed zero -- the
// mixed form's FP32 values carry nothing there that the FP64 state needs.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace nsp {

__host__ __device__ __forceinline__ uint32_t f64_to_f32_bits(uint64_t b) {
  const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
  const uint32_t sign = hi & 0x80000000u, e = (hi >> 20) & 0x7FFu;
  if (e < 897u) return sign;  // below 2^-126: zero, double denormals, float denormal range
  if (e == 0x7FFu) return sign | ((((hi & 0xFFFFFu) | lo) != 0u) ? 0x7FC00000u : 0x7F800000u);  // NaN, Inf
  if (e > 1150u) return sign | 0x7F800000u;  // 2^128 and beyond: Inf
  uint32_t f = ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);  // exponent rebias 1023 -> 127
  const uint32_t rest = lo & 0x1FFFFFFFu;                                  // the 29 dropped mantissa bits
  f += (rest > 0x10000000u) || (rest == 0x10000000u && (f & 1u));          // ties to even; may carry to Inf
  return sign | f;
}

__host__ __device__ __forceinline__ uint64_t f32_to_f64_bits(uint32_t u) {
  const uint32_t sign = u & 0x80000000u, e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
  if (e == 0u) return (uint64_t)sign << 32;  // zero; float denormals flush
  const uint32_t eh = e == 0xFFu ? 0x7FFu : e + 896u;  // Inf/NaN keep the all-ones exponent
  return ((uint64_t)(sign | (eh << 20) | (m >> 3)) << 32) | (uint64_t)(m << 29);
}

#ifdef __CUDACC__
__device__ __forceinline__ float f64_to_f32(double x) {
  return __uint_as_float(f64_to_f32_bits((uint64_t)__double_as_longlong(x)));
}
__device__ __forceinline__ double f32_to_f64(float x) {
  return __longlong_as_double((long long)f32_to_f64_bits(__float_as_uint(x)));
}
#endif

}  // namespace nsp
