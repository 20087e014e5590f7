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

// ---- the mean flow of the mixed form's nonlinear term
// The mixed form evaluates -(u.grad)u with the mean flow -- W(r) = Re u_theta(m=0,k_z=0)
// and U(r) = Re u_z(0,0) -- taken out of the transform input, and adds the terms that
// contain it afterwards, mode by mode.  With u' = u minus that mean flow (the mean u_r,
// zero after every pass, stays in the transforms), the terms of -(u.grad)u with a factor
// W, U, W' or U' are, for mode (m, k_z) with a = m W / r + k_z U:
//   N_r:     -i a u'_r + 2 W u'_theta / r        (+ W^2 / r at mode (0,0))
//   N_theta: -i a u'_theta - (W' + W / r) u'_r
//   N_z:     -i a u'_z - U' u'_r
// (at mode (0,0) u'_theta = u'_z = 0 and u'_r is the mean u_r).  No product of the mean
// with a retained mode leaves the retained modes, so these are exactly the terms the
// dealiased transforms would give.  Taking the mean flow out matters because the
// transforms then carry the perturbation only: a base flow of order 1 over a
// perturbation of order 1e-3 otherwise sets the transforms' rounding (and the tensor
// cores' accumulation) at 1e-3 of the perturbation's scale, and the mean mode of N --
// a sum over theta that cancels to the perturbation's square -- inherits it.
//
// True for the transform input fields whose mean mode is taken out: u_theta, u_z and
// their radial derivatives (fields 1, 2, 4, 5 of the inverse transforms' 9).
__device__ __forceinline__ bool mean_field(int f) { return f == 1 || f == 2 || f == 4 || f == 5; }

struct Mean32 {
  float W, U, Wp, Up, rinv;
};
// The mean flow at level i of a member's FP32 transform input (U32: its 3 components; DR32:
// their radial derivatives, or null: the 7-point parity stencil, u_theta odd and u_z even
// at m = 0).
// The mean flow at level i as the theta-inverse recorded it (Bufs::MEAN of a member: NR rows).
__device__ __forceinline__ Mean32 mean_flow32_rec(const Tables& tb, const float* mean, int i) {
  const float* m = mean + (size_t)i * MEAN_N;
  Mean32 o;
  o.W = m[MEAN_W];
  o.U = m[MEAN_U];
  o.Wp = m[MEAN_WP];
  o.Up = m[MEAN_UP];
  o.rinv = tb.rinv32[i];
  return o;
}
__device__ __forceinline__ Mean32 mean_flow32(const Tables& tb, const float2* U32, const float2* DR32, int i) {
  const long long S = tb.S;
  const size_t h = (size_t)i * tb.NTNZ;
  Mean32 o;
  o.W = U32[S + h].x;
  o.U = U32[2 * S + h].x;
  o.rinv = tb.rinv32[i];
  if (DR32) {
    o.Wp = DR32[S + h].x;
    o.Up = DR32[2 * S + h].x;
  } else {
    const int NR = tb.NR, left = max(0, i - IW), right = min(i + IW, NR - 1), len = right + 1 - left, i0 = i + IW - right;
    const size_t NTNZ = tb.NTNZ;
    o.Wp = dr32_line(tb.D32 + STEN * NR + STEN * i + i0, left, len,
                     [&](int row) { return U32[S + (size_t)row * NTNZ]; }).x;
    o.Up = dr32_line(tb.D32 + STEN * i + i0, left, len, [&](int row) { return U32[2 * S + (size_t)row * NTNZ]; }).x;
  }
  return o;
}
// The mean-flow terms of component c of N at mode (m, l): kt = k_theta m, kz = k_z of l;
// ur, ut, uz the transform input's values at the mode (ut = uz = 0 at mode (0,0), where
// only the real part of u_r -- the mean radial velocity the transforms see -- counts).
__device__ __forceinline__ float2 mean_terms32(const Mean32& mf, int c, bool zero_mode, float kt, float kz,
                                               float2 ur, float2 ut, float2 uz) {
  if (zero_mode) ur.y = 0.f;
  const float a = fmaf(kt * mf.W, mf.rinv, kz * mf.U);
  if (c == 0) {
    const float w2 = 2.f * mf.W * mf.rinv;
    float2 v = make_float2(fmaf(a, ur.y, w2 * ut.x), fmaf(-a, ur.x, w2 * ut.y));
    if (zero_mode) v.x += mf.W * mf.W * mf.rinv;
    return v;
  }
  const float b = c == 1 ? fmaf(mf.W, mf.rinv, mf.Wp) : mf.Up;
  const float2 q = c == 1 ? ut : uz;
  return make_float2(fmaf(a, q.y, -b * ur.x), fmaf(-a, q.x, -b * ur.y));
}

}  // namespace nsp
