// nsp_df.cuh -- double-float arithmetic for the mixed form's banded solves.
//
// A value is the unevaluated sum hi + lo of two FP32 numbers with hi = fl(hi + lo),
// about 48 significant bits.  On GB300 the FP64 pipe issues one warp instruction per
// 64 cycles per SM sub-partition and the FP32 pipe one per cycle, so a multiply-add in
// this form (about 12 FP32 instructions) costs a fifth of an FP64 one.  The exponent
// range is FP32's: magnitudes below 2^-126 carry no precision, which the mixed form's
// increments, made in FP32, do not have anyway.
//
// Built from error-free transforms: Knuth's two-sum (TAOCP vol. 2, 4.2.2), the FMA
// two-product (Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci.
// Comput. 26, 2005), with the cross terms of Dekker's product ("A floating-point
// technique for extending the available precision", Numer. Math. 18, 1971).  The _rn
// intrinsics keep the compiler from contracting or reassociating them.
#pragma once
#include <cuda_runtime.h>

namespace nsp {

struct __align__(8) dfloat {
  float hi, lo;
};

__device__ __forceinline__ dfloat df_make(float x) { return dfloat{x, 0.f}; }

// (s, t) renormalised to hi = fl(s + t), lo = the rest, by Dekker's fast two-sum: exact
// when |s| >= |t|.  Here t only ever holds the accumulated rounding terms of the values
// summed into s (a few ulps of the largest of them), so where cancellation leaves
// |s| < |t| the result's error is an ulp of t, about 2^-48 of those values -- the
// form's own accuracy -- for half the operations of the full two-sum.
__device__ __forceinline__ dfloat df_norm(float s, float t) {
  const float h = __fadd_rn(s, t);
  return dfloat{h, __fsub_rn(t, __fsub_rn(h, s))};
}

// s + t -= a b: the high product leaves s exactly by two-sum, its rounding error and
// the cross terms a.hi b.lo + a.lo b.hi go into t (the lo.lo term is below 2^-48).
__device__ __forceinline__ void df_sub_prod(float& s, float& t, const dfloat& a, const dfloat& b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  // two-sum of s and -p: u = s - p, w = u - s, error = (s - (u - w)) + (-p - w)
  const float u = __fsub_rn(s, p), w = __fsub_rn(u, s);
  const float r = __fsub_rn(__fsub_rn(s, __fsub_rn(u, w)), __fadd_rn(p, w));
  t = __fsub_rn(__fadd_rn(t, r), e);
  s = u;
}

// s + t += a b (df_sub_prod with the product's sign flipped).
__device__ __forceinline__ void df_add_prod(float& s, float& t, const dfloat& a, const dfloat& b) {
  df_sub_prod(s, t, dfloat{-a.hi, -a.lo}, b);
}

// a + b: two-sum of the high parts, the low parts and the error summed, renormalised.
__device__ __forceinline__ dfloat df_add(const dfloat& a, const dfloat& b) {
  const float s = __fadd_rn(a.hi, b.hi), v = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
  return df_norm(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dfloat df_neg(const dfloat& a) { return dfloat{-a.hi, -a.lo}; }
__device__ __forceinline__ dfloat df_sub(const dfloat& a, const dfloat& b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ dfloat df_mul(const dfloat& a, const dfloat& b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_norm(p, e);
}

}  // namespace nsp
