// nsp_state.cuh -- device access to a member's transform input (shared by the
// FFT and tensor-core transform kernels).
#pragma once
#include <cuda_runtime.h>

#include "nsp_fft.cuh"
#include "nsp_internal.h"

namespace nsp {

// Source field of a member: the state in the predictor phase, the iterate in corrector phases.
__device__ __forceinline__ const double2* member_source(const Tables& tb, const Bufs& bf, const Ctl* ctl, int mloc,
                                                        const double2* src_override, bool& skip) {
  skip = false;
  if (src_override) return src_override;
  int ph = ctl->phase[tb.mem0 + mloc];
  if (ph < 0) { skip = true; return nullptr; }
  int which = (ph == 0) ? ctl->parity : (ctl->parity ^ 1);
  return (which ? bf.U[1] : bf.U[0]) + (size_t)mloc * 3 * tb.S;  // (a select keeps bf out of local memory)
}

// Scalars and 1/r of the tables in the working precision (FP32 copies for T = float).
template <typename T> __device__ __forceinline__ T tb_kts(const Tables& tb) {
  if constexpr (sizeof(T) == 4) return tb.kts32; else return tb.kts;
}
template <typename T> __device__ __forceinline__ T tb_kzs(const Tables& tb) {
  if constexpr (sizeof(T) == 4) return tb.kzs32; else return tb.kzs;
}
template <typename T> __device__ __forceinline__ T tb_inv_norm(const Tables& tb) {
  if constexpr (sizeof(T) == 4) return tb.inv_norm32; else return tb.inv_norm;
}
template <typename T> __device__ __forceinline__ T tb_rinv(const Tables& tb, int i) {
  if constexpr (sizeof(T) == 4) return tb.rinv32[i]; else return tb.rinv[i];
}

// Transform input in the working precision: the FP64 state, or its FP32 mirror.
template <typename T> struct StateIn;
template <> struct StateIn<double> {
  const double2* p;
  __device__ __forceinline__ cpx<double> ld(size_t h) const { double2 a = p[h]; return mk<double>(a.x, a.y); }
};
template <> struct StateIn<float> {
  const float2* p;
  __device__ __forceinline__ cpx<float> ld(size_t h) const { float2 a = __ldg(p + h); return mk<float>(a.x, a.y); }
};
template <typename T> __device__ __forceinline__ const T* dtab(const Tables& tb);
template <> __device__ __forceinline__ const double* dtab<double>(const Tables& tb) { return tb.D; }
template <> __device__ __forceinline__ const float* dtab<float>(const Tables& tb) { return tb.D32; }

template <typename T>
__device__ __forceinline__ StateIn<T> member_input(const Tables& tb, const Bufs& bf, const Ctl* ctl, int mloc,
                                                  const double2* src, const float2* src32) {
  StateIn<T> s;
  int which = 0;
  if (!src) {
    int ph = ctl->phase[tb.mem0 + mloc];
    which = (ph == 0) ? ctl->parity : (ctl->parity ^ 1);
  }
  if constexpr (sizeof(T) == 8) s.p = src ? src : (which ? bf.U[1] : bf.U[0]) + (size_t)mloc * 3 * tb.S;
  else s.p = src ? src32 : (which ? bf.U32[1] : bf.U32[0]) + (size_t)mloc * 3 * tb.S;
  return s;
}

// FP32 radial-derivative mirror of the member's transform input (mixed form, member
// state only; explicit fields have none and the kernels apply the stencil themselves).
__device__ __forceinline__ const float2* member_dr32(const Tables& tb, const Bufs& bf, const Ctl* ctl, int mloc,
                                                    const double2* src) {
  if (src || !bf.DR32[0]) return nullptr;
  const int ph = ctl->phase[tb.mem0 + mloc];
  const int which = (ph == 0) ? ctl->parity : (ctl->parity ^ 1);
  return (which ? bf.DR32[1] : bf.DR32[0]) + (size_t)mloc * 3 * tb.S;
}

// d_r of one FP32 line value at level i (derivr_k, mod_radialFD.cu:10-30): the
// 7-point parity stencil in FP32, terms in row order.  Shared by the linear pass
// (which writes the DR32 mirror) and the transform kernels, so both give the same bits.
template <typename LOAD>
__device__ __forceinline__ float2 dr32_line(const float* Dr, int left, int len, LOAD ld) {
  float vx = 0.f, vy = 0.f;
  for (int j = 0; j < len; j++) {
    const float de = __ldg(Dr + j);
    const float2 a = ld(left + j);
    vx += de * a.x;
    vy += de * a.y;
  }
  return make_float2(vx, vy);
}

}  // namespace nsp
