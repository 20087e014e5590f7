// nsp_cvt.cuh -- double <-> float conversions on the integer pipe.
//
// On GB300 the hardware conversion instructions between FP64 and FP32 issue on the
// FP64 pipe (one warp instruction per 64 cycles per SM sub-partition), the bound of
// the linear pass.  These routines produce the same bits with a handful of integer
// instructions for the common range and fall back to the hardware conversion only
// for the rare remainder (float denormals, overflow, Inf/NaN).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace nsp {

// Round-to-nearest-even double -> float, bit-identical to __double2float_rn.
__host__ __device__ __forceinline__ uint32_t f64_to_f32_bits(uint64_t b, bool& fallback) {
  const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
  const uint32_t sign = hi & 0x80000000u;
  const uint32_t e = (hi >> 20) & 0x7FFu;
  fallback = false;
  if (e == 0) return sign;  // zero and double denormals round to a signed zero
  if (e < 897u || e > 1150u) { fallback = true; return 0; }  // |x| < 2^-126 or >= 2^128, Inf, NaN
  uint32_t f = ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);  // exponent rebias 1023 -> 127
  const uint32_t rest = lo & 0x1FFFFFFFu;                                  // the 29 dropped mantissa bits
  f += (rest > 0x10000000u) || (rest == 0x10000000u && (f & 1u));          // ties to even; may carry to Inf
  return sign | f;
}

// Exact float -> double.
__host__ __device__ __forceinline__ uint64_t f32_to_f64_bits(uint32_t u, bool& fallback) {
  const uint32_t sign = u & 0x80000000u, e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
  fallback = false;
  if (e == 0) {
    if (m == 0) return (uint64_t)sign << 32;
    fallback = true;  // float denormal
    return 0;
  }
  if (e == 0xFFu) { fallback = true; return 0; }
  const uint32_t hi = sign | ((e + 896u) << 20) | (m >> 3);
  return ((uint64_t)hi << 32) | (uint64_t)(m << 29);
}

#ifdef __CUDACC__
__device__ __forceinline__ float f64_to_f32(double x) {
  bool fb;
  const uint32_t r = f64_to_f32_bits((uint64_t)__double_as_longlong(x), fb);
  return fb ? __double2float_rn(x) : __uint_as_float(r);
}
__device__ __forceinline__ double f32_to_f64(float x) {
  bool fb;
  const uint64_t r = f32_to_f64_bits(__float_as_uint(x), fb);
  return fb ? (double)x : __longlong_as_double((long long)r);
}

// The same for arithmetic whose inputs and results below 2^-126 may be taken as zero:
// those flush to a signed zero instead of taking the hardware conversion.
__device__ __forceinline__ float f64_to_f32_ftz(double x) {
  const uint32_t hi = (uint32_t)__double2hiint(x);
  if (((hi >> 20) & 0x7FFu) < 897u) return __uint_as_float(hi & 0x80000000u);
  return f64_to_f32(x);
}
__device__ __forceinline__ double f32_to_f64_ftz(float x) {
  const uint32_t u = __float_as_uint(x);
  if (((u >> 23) & 0xFFu) == 0u) return __longlong_as_double((long long)((uint64_t)(u & 0x80000000u) << 32));
  return f32_to_f64(x);
}
#endif

}  // namespace nsp
