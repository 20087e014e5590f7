// nsp_linear.cu -- the linear part of the predictor and corrector, one CTA per
// block of LM (m, k_z) mode lines of one member: all FP64 in the plain FP64 form;
// double-float, FP32 and FP64 in the mixed form (DFS and INC below).
//
// One launch replaces the ~28 launches of predictor()/corrector()
// (mod_integrate.cu:164-228): decoupleForward/Backward (mod_utils.cu:30-59),
// addRHS_k (mod_integrate.cu:43-59), addLaplacian (mod_linear.cu:12-51,652-661),
// divergence (mod_radialFD.cu:67-96), write_bcon (mod_utils.cu:20-27), LUsolve_p
// and LUsolve_u x3 (mod_linear.cu:55-646), addGrad (mod_radialFD.cu:115-143),
// corBCon (mod_boundary.cu:269-278), modeZZ (mod_integrate.cu:63-68), adj_flux
// (mod_cublasflux.cu:90-103) and, in the corrector, the convergence measure
// mcor_k + iden_max (mod_integrate.cu:9-40, mod_cublasflux.cu:106-116) as a
// block max reduction and one atomicMax per CTA.
//
// The radial lines of the block's modes are staged in shared memory as
// [component][r][mode]; pointwise and stencil phases use all threads over
// (r, mode), the banded solves two threads per (component, mode) -- the real and
// imaginary parts -- sweeping r with the precomputed factors (read coalesced across
// modes; in the mixed form staged through a shared-memory ring).  The explicit
// Laplacian of u^n is applied from the state in global memory (FP64 form) or from a
// shared-memory tile of its FP32 mirror (mixed form), so a block holds 4 radial lines
// per mode.
#include <cstdio>

#include "nsp_bounds.cuh"
#include "nsp_cvt.cuh"
#include "nsp_df.cuh"
#include "nsp_fft.cuh"
#include "nsp_internal.h"
#include "nsp_state.cuh"

namespace nsp {


__device__ __forceinline__ double2 c2(double x, double y) { return make_double2(x, y); }

// x -= l * y for a complex line value (both parts) or one real part of it.
__device__ __forceinline__ void fms(double2& x, double l, const double2& y) { x.x -= l * y.x; x.y -= l * y.y; }
__device__ __forceinline__ void fms(double& x, double l, const double& y) { x -= l * y; }
__device__ __forceinline__ void scale(double2& x, double u) { x.x *= u; x.y *= u; }
__device__ __forceinline__ void scale(double& x, double u) { x *= u; }
__device__ __forceinline__ void fms(float& x, float l, const float& y) { x = fmaf(-l, y, x); }
__device__ __forceinline__ void scale(float& x, float u) { x *= u; }

// One forward-substitution row: x -= L(i-3) x_{i-3} + L(i-2) x_{i-2} + L(i-1) x_{i-1},
// in the reference's column order.  Factors of columns outside the band are stored
// as 0 (and the carried x start at 0), so edge rows need no branches.
template <typename V, typename L>
__device__ __forceinline__ void fwd_row(V& x, const L* l, V& xm1, V& xm2, V& xm3) {
  fms(x, l[0], xm3);
  fms(x, l[1], xm2);
  fms(x, l[2], xm1);
  xm3 = xm2; xm2 = xm1; xm1 = x;
}
// One backward row, farther neighbours first so that only one multiply-add and the
// pivot multiply wait on the row just finished: x = (x - U3 x3 - U2 x2 - U1 x1) / U_ii.
template <typename V, typename L>
__device__ __forceinline__ void bwd_row(V& x, const L* u, V& xp1, V& xp2, V& xp3) {
  fms(x, u[0], xp3);
  fms(x, u[1], xp2);
  fms(x, u[2], xp1);
  scale(x, u[3]);
  xp3 = xp2; xp2 = xp1; xp1 = x;
}

// The same rows in double-float (nsp_df.cuh): one part of a line, factors split the same way.
__device__ __forceinline__ void fwd_row(dfloat& x, const dfloat* l, dfloat& xm1, dfloat& xm2, dfloat& xm3) {
  float s = x.hi, t = x.lo;
  df_sub_prod(s, t, l[0], xm3);
  df_sub_prod(s, t, l[1], xm2);
  df_sub_prod(s, t, l[2], xm1);
  x = df_norm(s, t);
  xm3 = xm2; xm2 = xm1; xm1 = x;
}
// The mixed form's factor tables hold U'(i, i+j) = U(i, i+j) / U_ii (split_fac_k), so a
// backward row is x = y / U_ii - U'3 x3 - U'2 x2 - U'1 x1: the division of y, which is
// known early, stays off the dependency chain.
__device__ __forceinline__ void bwd_row(dfloat& x, const dfloat* u, dfloat& xp1, dfloat& xp2, dfloat& xp3) {
  const dfloat y = df_mul(x, u[3]);
  float s = y.hi, t = y.lo;
  df_sub_prod(s, t, u[0], xp3);
  df_sub_prod(s, t, u[1], xp2);
  df_sub_prod(s, t, u[2], xp1);
  x = df_norm(s, t);
  xp3 = xp2; xp2 = xp1; xp1 = x;
}
__device__ __forceinline__ void bwd_row(float& x, const float* u, float& xp1, float& xp2, float& xp3) {
  x *= u[3];
  x = fmaf(-u[0], xp3, x);
  x = fmaf(-u[1], xp2, x);
  x = fmaf(-u[2], xp1, x);
  xp3 = xp2; xp2 = xp1; xp1 = x;
}

__device__ __forceinline__ double ldf(const double* p) { return __ldg(p); }
__device__ __forceinline__ float ldf(const float* p) { return __ldg(p); }
__device__ __forceinline__ dfloat ldf(const dfloat* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return dfloat{v.x, v.y};
}

// Forward + backward substitution of one mode line held in X[i*ld] (i = 0..NR-1):
// V = double2 solves the complex line, V = double one of its parts (the factors are
// real, so the real and imaginary parts are independent solves and two threads can
// share a line), V = dfloat one part in double-float with the factors F = dfloat.
// Factor rows are fetched four at a time so that their L2 latencies overlap.
template <typename V, typename F>
__device__ __forceinline__ void solve_line(V* X, int ld, const F* __restrict__ f, int NTNZ, int NR) {
  const size_t rs = (size_t)NFAC * NTNZ;  // row stride of the factor table
  V xm1{}, xm2{}, xm3{};
  int i = 0;
  for (; i + 4 <= NR; i += 4) {
    F l[4][3];
    V b[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const F* fr = f + (i + r) * rs;
      l[r][0] = ldf(fr); l[r][1] = ldf(fr + NTNZ); l[r][2] = ldf(fr + 2 * NTNZ);
      b[r] = X[(i + r) * ld];
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      fwd_row(b[r], l[r], xm1, xm2, xm3);
      X[(i + r) * ld] = b[r];
    }
  }
  for (; i < NR; i++) {
    const F* fr = f + i * rs;
    F l[3] = {ldf(fr), ldf(fr + NTNZ), ldf(fr + 2 * NTNZ)};
    V x = X[i * ld];
    fwd_row(x, l, xm1, xm2, xm3);
    X[i * ld] = x;
  }
  V xp1{}, xp2{}, xp3{};
  i = NR - 1;
  for (; i >= 3; i -= 4) {
    F u[4][4];
    V b[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const F* fr = f + (i - r) * rs;
      u[r][0] = ldf(fr + 6 * NTNZ); u[r][1] = ldf(fr + 5 * NTNZ);
      u[r][2] = ldf(fr + 4 * NTNZ); u[r][3] = ldf(fr + 3 * NTNZ);
      b[r] = X[(i - r) * ld];
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      bwd_row(b[r], u[r], xp1, xp2, xp3);
      X[(i - r) * ld] = b[r];
    }
  }
  for (; i >= 0; i--) {
    const F* fr = f + i * rs;
    F u[4] = {ldf(fr + 6 * NTNZ), ldf(fr + 5 * NTNZ), ldf(fr + 4 * NTNZ), ldf(fr + 3 * NTNZ)};
    V x = X[i * ld];
    bwd_row(x, u, xp1, xp2, xp3);
    X[i * ld] = x;
  }
}

// 8-byte asynchronous copies global -> shared (cp.async), their groups and waits.
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];\n" ::"l"(p)); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Depth of the factor ring of the double-float solves, in batches of four rows, and of
// the increment pass's pressure ring, which lives in its lines' free upper halves.
constexpr int RING_B = 3;
constexpr int RING_DEEP = 8;
// Shared memory of one kind's ring: [RING_B][4 rows][4 slots][LM] double-float factors.
constexpr size_t ring_bytes(int LM) { return (size_t)RING_B * 16 * LM * sizeof(dfloat); }
// Dynamic shared memory of a linear-pass block beyond its 4 radial lines (mixed form): the
// pressure solve's ring, and with the pressure line, which is dead by then, the three
// Helmholtz solves' rings.
// The same space holds, in the predictor's first stage, the block's tile of the FP32
// mirror of u^n (3 lines of float2) that its explicit stencil reads.
inline size_t ring_extra(int NR, int LM) {
  const size_t pl = sizeof(double2) * (size_t)NR * LM, r = ring_bytes(LM);
  const size_t rings = 3 * r > pl + r ? 3 * r - pl : r, tile = 3 * sizeof(float2) * (size_t)NR * LM;
  return tile > pl + rings ? tile - pl : rings;
}

// solve_line<V, V> (V = dfloat: double-float; V = float: FP32, the increment pass's
// Helmholtz solves) with the factor rows staged through a shared-memory ring:
// the copies of batch b + RB - 1 are in flight while batch b computes, so the rows
// wait on shared memory instead of L2.  The two threads of a line (part 0 and 1, adjacent
// lanes, both calling) share the copies -- part 0 fetches slots 0-1, part 1 slots 2-3 --
// and meet at __syncwarp(pair) after each wait and before a slot is refilled.  Slots:
// forward L(i-3), L(i-2), L(i-1); backward U(i+3), U(i+2), U(i+1), 1/U_ii.  Rows past the
// last full batch read the table directly.  RB: ring depth in batches; RS: element
// stride of the ring (2: the free upper halves of line slots that hold FP32 pairs).
template <int LM, int RB, int RS, typename V>
__device__ __forceinline__ void solve_line_ring(V* X, int ld, const V* __restrict__ f, int NTNZ, int NR,
                                                V* ring, int mm, int part, unsigned pair) {
  const size_t rs = (size_t)NFAC * NTNZ;
  const int nb = NR / 4;
  auto at = [&](int b, int e) { return ring + (((b % RB) * 16 + e) * LM + mm) * RS; };
  auto issue = [&](int b, bool fwd) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int row = fwd ? 4 * b + r : NR - 1 - 4 * b - r;
#pragma unroll
      for (int q = 0; q < 2; q++) {
        const int slot = 2 * part + q, e = fwd ? slot : 6 - slot;
        if (!fwd || slot < 3) {
          if constexpr (sizeof(V) == 8) cp_async8(at(b, r * 4 + slot), f + row * rs + (size_t)e * NTNZ);
          else cp_async4(at(b, r * 4 + slot), f + row * rs + (size_t)e * NTNZ);
        }
      }
    }
  };
  V xm1{}, xm2{}, xm3{};
#pragma unroll
  for (int b = 0; b < RB - 1; b++) {
    if (b < nb) issue(b, true);
    cp_async_commit();
  }
  for (int b = 0; b < nb; b++) {
    if (b + RB - 1 < nb) issue(b + RB - 1, true);
    cp_async_commit();
    cp_async_wait<RB - 1>();
    __syncwarp(pair);
    V l[4][3], x[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
#pragma unroll
      for (int j = 0; j < 3; j++) l[r][j] = *at(b, r * 4 + j);
      x[r] = X[(4 * b + r) * ld];
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      fwd_row(x[r], l[r], xm1, xm2, xm3);
      X[(4 * b + r) * ld] = x[r];
    }
    __syncwarp(pair);
  }
  for (int i = 4 * nb; i < NR; i++) {
    const V* fr = f + i * rs;
    V l[3] = {ldf(fr), ldf(fr + NTNZ), ldf(fr + 2 * NTNZ)};
    V x = X[i * ld];
    fwd_row(x, l, xm1, xm2, xm3);
    X[i * ld] = x;
  }
  V xp1{}, xp2{}, xp3{};
#pragma unroll
  for (int b = 0; b < RB - 1; b++) {
    if (b < nb) issue(b, false);
    cp_async_commit();
  }
  for (int b = 0; b < nb; b++) {
    if (b + RB - 1 < nb) issue(b + RB - 1, false);
    cp_async_commit();
    cp_async_wait<RB - 1>();
    __syncwarp(pair);
    V u[4][4], x[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
#pragma unroll
      for (int j = 0; j < 4; j++) u[r][j] = *at(b, r * 4 + j);
      x[r] = X[(NR - 1 - 4 * b - r) * ld];
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      bwd_row(x[r], u[r], xp1, xp2, xp3);
      X[(NR - 1 - 4 * b - r) * ld] = x[r];
    }
    __syncwarp(pair);
  }
  for (int i = NR - 1 - 4 * nb; i >= 0; i--) {
    const V* fr = f + i * rs;
    V u[4] = {ldf(fr + 6 * NTNZ), ldf(fr + 5 * NTNZ), ldf(fr + 4 * NTNZ), ldf(fr + 3 * NTNZ)};
    V x = X[i * ld];
    bwd_row(x, u, xp1, xp2, xp3);
    X[i * ld] = x;
  }
  cp_async_wait<0>();  // (only empty groups can be left)
  __syncwarp(pair);
}

// The low half of a line slot holds an FP32 pair in the increment passes.
__device__ __forceinline__ float2& f32slot(double2* a, int e) { return reinterpret_cast<float2*>(a)[2 * e]; }
// The mixed passes hold a line slot as two double-float parts (re.hi, re.lo, im.hi,
// im.lo) -- the predictor from its right-hand side to its correction, the increment
// passes around their banded solves: the same 16 bytes, so a solve addresses one part
// where the FP64 pass addresses one double.
__device__ __forceinline__ float4& dfslot(double2* a, int e) { return reinterpret_cast<float4*>(a)[e]; }
__device__ __forceinline__ void put_df(double2* a, int e, float x, float y) { dfslot(a, e) = make_float4(x, 0.f, y, 0.f); }
// An FP64 value split into double-float: hi = fl32(x), lo = fl32(x - hi) (x - hi exact).
__device__ __forceinline__ float2 split_df(double x) {
  const float hi = f64_to_f32(x);
  return make_float2(hi, f64_to_f32(x - f32_to_f64(hi)));
}
__device__ __forceinline__ void put_df(double2* a, int e, double2 v) {
  const float2 x = split_df(v.x), y = split_df(v.y);
  dfslot(a, e) = make_float4(x.x, x.y, y.x, y.y);
}
__device__ __forceinline__ void put_df(double2* a, int e, dfloat x, dfloat y) {
  dfslot(a, e) = make_float4(x.hi, x.lo, y.hi, y.lo);
}
__device__ __forceinline__ dfloat df_re(const float4& v) { return dfloat{v.x, v.y}; }
__device__ __forceinline__ dfloat df_im(const float4& v) { return dfloat{v.z, v.w}; }
__device__ __forceinline__ dfloat ld_df(const float2* p) {
  const float2 v = __ldg(p);
  return dfloat{v.x, v.y};
}
// A double-float slot's value in FP64 (the widenings on the integer pipe, one FP64 add).
__device__ __forceinline__ double2 df_value(double2* a, int e) {
  const float4 v = dfslot(a, e);
  return make_double2(f32_to_f64(v.x) + f32_to_f64(v.y), f32_to_f64(v.z) + f32_to_f64(v.w));
}

// At least 1024 threads per SM resident (4 radial lines of 48 points x 16 modes
// is 49 KB of shared memory, 55 KB with the mixed form's factor rings, so four
// 256-thread blocks fit): 64 registers.
//
// INC (mixed form, corrector passes): the pass is affine in its right-hand side, so
// iterate i+1 is iterate i plus the linear part of the pass applied to
// (d_im/2) (N_i - N_{i-1}):
//   u_{i+1} = u_i + (d_im/2) L(N_i - N_{i-1}),
// L = divergence, pressure solve, gradient, Helmholtz solves, influence correction
// and the flux correction without its Qdes term (equal to the full pass in exact
// arithmetic).  The increment is small next to u, so its divergence and gradient
// stencils, influence correction, mode (0,0) constraints and flux fix run in FP32, its
// Helmholtz solves in FP32 (well-conditioned operators), its pressure solve in
// double-float (condition numbers up to ~1e6); only the update of u is FP64.  N_{i-1}
// is kept in RHSW32 (the predictor stores N(u^n) there in the mixed form).  Without INC
// the kernel is the full pass, and in the mixed form it takes only the predictor.
//
// DFS (mixed form, both passes): FP64-class arithmetic in double-float (nsp_df.cuh),
// about 48 bits, with the factors, stencils and correction profiles split the same way:
// on GB300 an FP64 instruction costs 64 times an FP32 one's issue.  The predictor splits
// u^n once, runs its stencils, solves and corrections in double-float and sums the
// result back to FP64 when it stores the state.
template <int LM, int NTH, bool INC, bool DFS>
__global__ void __launch_bounds__(NTH, NTH >= 1024 ? 1 : ((1024 / NTH) < 2 ? 2 : (1024 / NTH)))
    linear_k(Tables tb, Bufs bf, Ctl* ctl) {
  const int mloc = blockIdx.y, gm = tb.mem0 + mloc;
  if (!NSP_IN_BOUNDS(tb, mloc, tb.nmem, BC_LIN_MEMBER) || !NSP_IN_BOUNDS(tb, gm, ctl->nmem, BC_LIN_MEMBER)) return;
  const int ph = ctl->phase[gm];
  if (ph < 0) return;
  if (INC ? ph == 0 : (ph > 0 && bf.U32[0] != nullptr)) return;  // the other kernel's pass
  const bool pred = !INC && ph == 0;
  const int par = ctl->parity;
  const int NR = tb.NR, NT = tb.NT, NZ = tb.NZ, NTNZ = tb.NTNZ;
  const long long S = tb.S;
  const int k0 = blockIdx.x * LM;
  const int LN = NR * LM;
  extern __shared__ double2 sm[];
  double2* R = sm;           // [3][NR][LM] right-hand side, then the new velocity
  double2* P = sm + 3 * LN;  // [NR][LM] divergence, then the pressure
  // DFS: the solves' factor rings (solve_line_ring), the pressure's after the lines, the
  // Helmholtz solves' from the pressure line on (dead by then)
  dfloat* ringD = reinterpret_cast<dfloat*>(sm + 4 * LN);
  dfloat* ringF = reinterpret_cast<dfloat*>(P);
  __shared__ double2 dvs[LM];
  __shared__ float2 dvs32[LM];  // increment passes: the same in FP32
  __shared__ unsigned long long wnum[NTH / 32], wden[NTH / 32];
  __shared__ double skt[LM], skz[LM];  // k_theta, k_z of the block's modes
  __shared__ double snkz2[LM], snkt2[LM], shdk[LM];  // -k_z^2, -k_theta^2, -c_ex k_theta (predictor)
  __shared__ int spar[LM];             // |m| mod 2 (selects the parity tables)
  __shared__ bool sdrop[LM];           // theta Nyquist slot or l = NZ-1: modes the transforms drop
  __shared__ float skt32[LM], skz32[LM];  // k_theta, k_z in FP32 (increment passes)
  __shared__ dfloat skt_df[LM], skz_df[LM];  // the same in double-float (mixed predictor)
  __shared__ float4 dvs_df[LM];              // the wall divergence in double-float (mixed predictor)
  __shared__ float snkz2_32[LM], snkt2_32[LM], shdk32[LM];  // FP32 copies (mixed predictor)
  __shared__ int bad;
  // (selects instead of indexing the parameter arrays by a run-time value, which
  // would copy them to local memory)
  const double2* Un = (par ? bf.U[1] : bf.U[0]) + (size_t)mloc * 3 * S;
  double2* Ui = (par ? bf.U[0] : bf.U[1]) + (size_t)mloc * 3 * S;
  float2* U32i = par ? bf.U32[0] : bf.U32[1];
  float2* Ui32 = U32i ? U32i + (size_t)mloc * 3 * S : nullptr;  // mixed form
  float2* DR32i = par ? bf.DR32[0] : bf.DR32[1];
  float2* Udr32 = DR32i ? DR32i + (size_t)mloc * 3 * S : nullptr;  // mixed form: d_r of the FP32 mirror
  const double2* Nn = bf.N ? bf.N + (size_t)mloc * 3 * S : nullptr;  // FP64 form
  double2* Rw = bf.RHSW ? bf.RHSW + (size_t)mloc * 3 * S : nullptr;
  // mixed form: N and N_{i-1} in FP32, the FP64 line Re N_z(0,0) apart (bf.NF, bf.RW00)
  const float2* N32n = bf.N32 ? bf.N32 + (size_t)mloc * 3 * S : nullptr;
  float2* Rw32 = bf.RHSW32 ? bf.RHSW32 + (size_t)mloc * 3 * S : nullptr;
  // The member's operator parameter set (its Re): LU factors, correction profiles,
  // explicit Laplacian, flux profile and scalars.
  const int ps = member_set(tb, mloc);
  const double* fac = tb.fac + (size_t)ps * 4 * NR * NFAC * NTNZ;
  const double2* Vp = tb.V + (size_t)ps * 3 * S;
  const double* Luc = tb.Luc + (size_t)ps * 2 * STEN * NR;
  const double* ucp = tb.uc + (size_t)ps * NR;
  const double c_ex = tb.sscal[4 * ps], Qc = tb.sscal[4 * ps + 2];
  const int tid = threadIdx.x, nth = blockDim.x;
  if (tid == 0) bad = 0;
  if (tid < LM) {  // wavenumbers once per block instead of per point
    int k = k0 + tid, it = k / NZ, l = k - it * NZ, m = it < NT / 2 ? it : it - NT;
    const double kt = tb.kts * (double)m, kz = tb.kzs * (double)l;
    skt[tid] = kt;
    skz[tid] = kz;
    spar[tid] = abs(m) % 2;
    sdrop[tid] = it == NT / 2 || l == NZ - 1;
    snkz2[tid] = -kz * kz;
    snkt2[tid] = -kt * kt;
    shdk[tid] = -(0.5 * c_ex) * (2.0 * kt);
    skt32[tid] = f64_to_f32(kt);
    skz32[tid] = f64_to_f32(kz);
    if (DFS) {
      const float2 a = split_df(kt), b = split_df(kz);
      skt_df[tid] = dfloat{a.x, a.y};
      skz_df[tid] = dfloat{b.x, b.y};
    }
    snkz2_32[tid] = f64_to_f32(snkz2[tid]);
    snkt2_32[tid] = f64_to_f32(snkt2[tid]);
    shdk32[tid] = f64_to_f32(shdk[tid]);
  }
  __syncthreads();

  // Every line from the right-hand side to the Helmholtz solutions is carried at
  // half scale (exact: a power of two through linear operations), so the +/- <->
  // r/theta conversions need no multiply by 1/2.
  //
  // The explicit part of the right-hand side, e = u^n/dt + (1-d_im)/Re L+- u^n
  // (addLaplacian, mod_linear.cu:12-51), is the same in the predictor and in every
  // corrector of a step.  The predictor computes it once and stores
  // rhsw' = (1-d_im) N(u^n) + e, in r/theta form and at half scale; a corrector's
  // right-hand side is then d_im N(u_i) + rhsw' (addRHS_k + addLaplacian), with no
  // stencil, no +/- conversion and no read of u^n.  (The mixed form's increment
  // passes need no rhsw': its predictor stores N(u^n) there instead.)
  if (pred) {
    // e = u^n/dt + (1-d_im)/Re (L_r - k_z^2 - m^2/r^2 [-1/r^2 -+ 2m/r^2]) u^n on the +/- lines
    // (addLaplacian), evaluated in r/theta form: with dd+- the two diagonals,
    // s = (dd+ + dd-)/2 and d = (dd+ - dd-)/2,
    //   e_r = L u_r + s u_r + i d u_t,   e_theta = L u_t + s u_t - i d u_r.
    // Luc holds the stencil pre-scaled by 1/2, so e comes out at half scale; u^n is
    // read straight from global memory (the stencil's rows are served by L1).
    // Then, at half scale: rhs = N + e, rhsw' = (1-d_im) N + e.
    const double hc = 0.5 * c_ex, hidt = 0.5 * tb.inv_dt, hw = 0.5 * tb.one_m_dim;
    const float2* U32n = par ? bf.U32[1] : bf.U32[0];
    const float2* Un32 = U32n ? U32n + (size_t)mloc * 3 * S : nullptr;  // mixed form: FP32 mirror of u^n
    const float* Luc32 = tb.Luc32 + (size_t)ps * 2 * STEN * NR;
    dfloat hidt_df{0.f, 0.f};
    // mixed: the block's tile of the FP32 mirror of u^n, [3][NR][LM], in the pressure line
    // and ring space (free until stage C), loaded coalesced; the stencil reads it there.
    float2* T32 = reinterpret_cast<float2*>(P);
    if constexpr (DFS) {
      const float2 a = split_df(hidt);
      hidt_df = dfloat{a.x, a.y};
      for (int e = tid; e < 3 * LN; e += nth) {
        const int c = e / LN, q = e - c * LN, ii = q / LM, k = k0 + q - ii * LM;
        T32[e] = k < NTNZ ? __ldg(Un32 + (size_t)c * S + (size_t)ii * NTNZ + k) : make_float2(0.f, 0.f);
      }
      __syncthreads();
    }
    for (int p = tid; p < LN; p += nth) {
      int i = p / LM, mm = p - i * LM, k = k0 + mm;
      if (k >= NTNZ) {
        for (int c = 0; c < 3; c++) R[c * LN + p] = c2(0, 0);
        continue;
      }
      int par_m = spar[mm];
      int left = max(0, i - IW), right = min(i + IW, NR - 1), len = right + 1 - left, i0 = i + IW - right;
      const int lo = (1 - par_m) * STEN * NR + STEN * i + i0;  // u_r, u_theta rows (odd flag)
      const int le = par_m * STEN * NR + STEN * i + i0;        // u_z rows
      const size_t h = (size_t)i * NTNZ + k;
      if (!NSP_IN_BOUNDS(tb, h, S, BC_LIN_POINT) || !NSP_IN_BOUNDS(tb, lo + len - 1, 2 * STEN * NR, BC_LIN_TAP) ||
          !NSP_IN_BOUNDS(tb, le + len - 1, 2 * STEN * NR, BC_LIN_TAP) ||
          !NSP_IN_BOUNDS(tb, (size_t)(left + len - 1) * NTNZ + k, S, BC_LIN_TAP))
        continue;
      if (DFS && k != 0) {  // (DFS: the mixed predictor)
        // mixed form: everything but u^n/dt in FP32 on the FP32 mirror of u^n -- the
        // stencil sums and the diagonal terms ((1-d_im)/Re times the Laplacian) and N/2
        // (exact in FP32: the FP32 transforms' values) -- then one FP64 multiply-add
        // per value adds u^n/dt.  The mean mode (k = 0) stays in FP64: its Laplacian is
        // steady, so FP32 rounding there would add up step after step.
        float2 fr = make_float2(0.f, 0.f), ft = fr, fz = fr;
        for (int j = 0; j < len; j++) {
          const float a = __ldg(Luc32 + lo + j), b = __ldg(Luc32 + le + j);
          const int e = (left + j) * LM + mm;
          const float2 vr = T32[e], vt = T32[LN + e], vz = T32[2 * LN + e];
          fr.x = fmaf(a, vr.x, fr.x); fr.y = fmaf(a, vr.y, fr.y);
          ft.x = fmaf(a, vt.x, ft.x); ft.y = fmaf(a, vt.y, ft.y);
          fz.x = fmaf(b, vz.x, fz.x); fz.y = fmaf(b, vz.y, fz.y);
        }
        const float ri = tb.rinv32[i], ir2f = ri * ri, hcf = f64_to_f32(hc);
        const float basef = fmaf(snkt2_32[mm], ir2f, snkz2_32[mm]);  // -k_z^2 - k_theta^2 / r^2
        const float hzf = hcf * basef, hsf = hcf * (basef - ir2f), hdf = shdk32[mm] * ir2f;
        // N(u^n) in FP32 (the transforms' values are exact in FP32) plus the mean-flow terms
        // (nsp_state.cuh), from the same FP32 values of u^n the explicit stencil uses
        float2 nf[3];
#pragma unroll
        for (int c = 0; c < 3; c++) nf[c] = N32n[c * S + h];
        {
          const float2 fur = T32[p], fut = T32[LN + p], fuz = T32[2 * LN + p];
          fr.x += fmaf(hsf, fur.x, -hdf * fut.y);
          fr.y += fmaf(hsf, fur.y, hdf * fut.x);
          ft.x += fmaf(hsf, fut.x, hdf * fur.y);
          ft.y += fmaf(hsf, fut.y, -hdf * fur.x);
          fz.x += hzf * fuz.x;
          fz.y += hzf * fuz.y;
          if (!sdrop[mm]) {
            const Mean32 mf = mean_flow32_rec(tb, bf.MEAN + (size_t)mloc * NR * MEAN_N, i);
#pragma unroll
            for (int c = 0; c < 3; c++) {
              const float2 ml = mean_terms32(mf, c, false, skt32[mm], skz32[mm], fur, fut, fuz);
              nf[c].x += ml.x;
              nf[c].y += ml.y;
            }
          }
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
          Rw32[c * S + h] = nf[c];  // full N(u^n) for the first increment pass
          const float2 f = c == 0 ? fr : (c == 1 ? ft : fz);
          const float gx = fmaf(0.5f, nf[c].x, f.x), gy = fmaf(0.5f, nf[c].y, f.y);
          // widening on the integer pipe (the hardware conversion issues on the FP64 pipe)
          const double2 u = Un[c * S + h];
          if constexpr (DFS) {  // u^n/(2dt) + g in double-float: u^n split, the product and the sum exact
            const float2 ux = split_df(u.x), uy = split_df(u.y);
            float sx = 0.f, tx = 0.f, sy = 0.f, ty = 0.f;
            df_add_prod(sx, tx, hidt_df, dfloat{ux.x, ux.y});
            df_add_prod(sy, ty, hidt_df, dfloat{uy.x, uy.y});
            put_df(R, c * LN + p, df_add(df_norm(sx, tx), df_make(gx)), df_add(df_norm(sy, ty), df_make(gy)));
          } else {
            R[c * LN + p] = c2(fma(hidt, u.x, f32_to_f64(gx)), fma(hidt, u.y, f32_to_f64(gy)));
          }
        }
        continue;
      }
      // the diagonals from the per-mode tables: 4 FP64 operations per point
      const double ir2 = tb.rinv2[i];
      const double base = fma(snkt2[mm], ir2, snkz2[mm]);  // -k_z^2 - k_theta^2 / r^2
      const double hz = fma(hc, base, hidt);                // diagonal of the u_z line / 2
      const double hs = fma(-hc, ir2, hz);                  // s/2 = hc (base - 1/r^2) + 1/(2 dt)
      const double hd = shdk[mm] * ir2;                     // d/2 = -hc 2 k_theta / r^2
      double2 lr = c2(0, 0), lt = c2(0, 0), lz = c2(0, 0);
      for (int j = 0; j < len; j++) {
        double a = __ldg(Luc + lo + j), b = __ldg(Luc + le + j);
        size_t hj = (size_t)(left + j) * NTNZ + k;
        double2 vr = Un[hj], vt = Un[S + hj], vz = Un[2 * S + hj];
        lr.x += a * vr.x; lr.y += a * vr.y;
        lt.x += a * vt.x; lt.y += a * vt.y;
        lz.x += b * vz.x; lz.y += b * vz.y;
      }
      const double2 ur = Un[h], ut = Un[S + h], uz = Un[2 * S + h];
      double2 er = c2(lr.x + hs * ur.x - hd * ut.y, lr.y + hs * ur.y + hd * ut.x);
      double2 et = c2(lt.x + hs * ut.x + hd * ur.y, lt.y + hs * ut.y - hd * ur.x);
      double2 ez = c2(lz.x + hz * uz.x, lz.y + hz * uz.y);
      double2 nr, nt, nz;
      if constexpr (DFS) {  // mixed form (mode (0,0)): N in FP32 plus the FP64 wall forcing on Re N_z
        const float2 a = N32n[h], b = N32n[S + h], z = N32n[2 * S + h];
        nr = c2(f32_to_f64(a.x), f32_to_f64(a.y));
        nt = c2(f32_to_f64(b.x), f32_to_f64(b.y));
        nz = c2(f32_to_f64(z.x) + bf.NF[mloc], f32_to_f64(z.y));
      } else {
        nr = Nn[h]; nt = Nn[S + h]; nz = Nn[2 * S + h];
      }
      if (Un32) {  // mixed form, mode (0,0): the mean flow's own terms (nsp_state.cuh)
        const float* mean = bf.MEAN + (size_t)mloc * NR * MEAN_N;
        const Mean32 mf = mean_flow32_rec(tb, mean, i);
        const float2 vr = make_float2(mean[(size_t)i * MEAN_N + MEAN_V], 0.f), zero = make_float2(0.f, 0.f);
        nr.x = f32_to_f64(f64_to_f32(nr.x) + mean_terms32(mf, 0, true, 0.f, 0.f, vr, zero, zero).x);
        nt.x = f32_to_f64(f64_to_f32(nt.x) + mean_terms32(mf, 1, true, 0.f, 0.f, vr, zero, zero).x);
        nz.x += (double)mean_terms32(mf, 2, true, 0.f, 0.f, vr, zero, zero).x;  // (nz: FP64 wall forcing)
      }
      const double2 r0 = c2(0.5 * nr.x + er.x, 0.5 * nr.y + er.y), r1 = c2(0.5 * nt.x + et.x, 0.5 * nt.y + et.y),
                    r2 = c2(0.5 * nz.x + ez.x, 0.5 * nz.y + ez.y);
      if constexpr (DFS) {  // (mode (0,0) of the mixed predictor)
        put_df(R, p, r0); put_df(R, LN + p, r1); put_df(R, 2 * LN + p, r2);
      } else {
        R[p] = r0; R[LN + p] = r1; R[2 * LN + p] = r2;
      }
      if constexpr (DFS) {  // mixed form: N(u^n) for the first increment pass (all FP32 numbers but Re N_z)
        Rw32[h] = make_float2(f64_to_f32(nr.x), f64_to_f32(nr.y));
        Rw32[S + h] = make_float2(f64_to_f32(nt.x), f64_to_f32(nt.y));
        Rw32[2 * S + h] = make_float2(0.f, f64_to_f32(nz.y));
        bf.RW00[(size_t)mloc * NR + i] = nz.x;
      } else {
        Rw[h] = c2(hw * nr.x + er.x, hw * nr.y + er.y);
        Rw[S + h] = c2(hw * nt.x + et.x, hw * nt.y + et.y);
        Rw[2 * S + h] = c2(hw * nz.x + ez.x, hw * nz.y + ez.y);
      }
    }
  } else if constexpr (INC) {
    // B'. N_i - N_{i-1} in FP32, into the FP32 halves of the line slots; RHSW32 takes N_i.
    // N_i is the transforms' output plus the mean-flow terms (nsp_state.cuh), from u_i's
    // FP32 mirror -- the transforms' input, at this block's own points -- and the mean
    // flow the theta-inverse recorded.  Both are stored as FP32 numbers (the transforms'
    // values and the FP32 sums of the previous pass), except Re N_z(0,0), which carries
    // the FP64 wall forcing: its difference is taken in FP64 from N32 + NF and RW00.
    constexpr int UB = 2;  // points per thread whose loads are issued together (RHSW is also stored)
    const float* mean = bf.MEAN + (size_t)mloc * NR * MEAN_N;
    for (int pb = tid; pb < LN; pb += UB * nth) {
      float2 n[UB][3], q[UB][3], w[UB][3];
#pragma unroll
      for (int u = 0; u < UB; u++) {
        const int p = pb + u * nth, i = p / LM, k = k0 + p - i * LM;
        const bool ok = p < LN && k < NTNZ && NSP_IN_BOUNDS(tb, (size_t)i * NTNZ + k, S, BC_LIN_POINT);
        const size_t h = ok ? (size_t)i * NTNZ + k : 0;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          n[u][c] = ok ? N32n[c * S + h] : make_float2(0.f, 0.f);
          q[u][c] = ok ? Rw32[c * S + h] : make_float2(0.f, 0.f);
          w[u][c] = ok ? Ui32[c * S + h] : make_float2(0.f, 0.f);
        }
      }
#pragma unroll
      for (int u = 0; u < UB; u++) {
        const int p = pb + u * nth, i = p / LM, mm = p - i * LM, k = k0 + mm;
        if (p >= LN) continue;
        const bool ok = k < NTNZ && (!kBoundsCheck || (size_t)i * NTNZ + k < (size_t)S);
        const size_t h = (size_t)i * NTNZ + k;
        float2 ml[3] = {};
        if (ok && !sdrop[mm]) {
          const Mean32 mf = mean_flow32_rec(tb, mean, i);
          if (k == 0) {  // mode (0,0): u'_theta = u'_z = 0, and only the mean u_r counts
            w[u][0] = make_float2(mean[(size_t)i * MEAN_N + MEAN_V], 0.f);
            w[u][1] = w[u][2] = make_float2(0.f, 0.f);
          }
#pragma unroll
          for (int c = 0; c < 3; c++) ml[c] = mean_terms32(mf, c, k == 0, skt32[mm], skz32[mm], w[u][0], w[u][1], w[u][2]);
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
          float2 d;
          if (c == 2 && k == 0) {  // Re N_z(0,0) in FP64: the FP32 value plus the wall forcing
            const double nx = f32_to_f64(n[u][c].x) + bf.NF[mloc] + (double)ml[c].x;
            double* rw = bf.RW00 + (size_t)mloc * NR + i;
            d = make_float2(f64_to_f32(nx - *rw), n[u][c].y - q[u][c].y);
            *rw = nx;
            Rw32[2 * S + h] = make_float2(0.f, n[u][c].y);
          } else {
            const float nx = n[u][c].x + ml[c].x, ny = n[u][c].y + ml[c].y;
            if (ok) Rw32[c * S + h] = make_float2(nx, ny);
            d = make_float2(nx - q[u][c].x, ny - q[u][c].y);
          }
          f32slot(R, c * LN + p) = d;  // zero where k >= NTNZ
        }
      }
    }
  } else {
    // A+B. rhs/2 = (d_im/2) N(u_i) + rhsw'/2, straight in r/theta form.  U points per
    // thread have their loads issued together (measured best at 1 here: more spills).
    const double hd = 0.5 * tb.d_im;
    constexpr int U = 1;
    for (int pb = tid; pb < LN; pb += U * nth) {
      double2 n[U][3], w[U][3];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int p = pb + u * nth, i = p / LM, k = k0 + p - i * LM;
        const bool ok = p < LN && k < NTNZ && NSP_IN_BOUNDS(tb, (size_t)i * NTNZ + k, S, BC_LIN_POINT);
        const size_t h = ok ? (size_t)i * NTNZ + k : 0;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          n[u][c] = ok ? Nn[c * S + h] : c2(0, 0);
          w[u][c] = ok ? Rw[c * S + h] : c2(0, 0);
        }
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int p = pb + u * nth;
        if (p < LN) {
#pragma unroll
          for (int c = 0; c < 3; c++) R[c * LN + p] = c2(hd * n[u][c].x + w[u][c].x, hd * n[u][c].y + w[u][c].y);
        }
      }
    }
  }
  __syncthreads();

  // C. divergence of rhs into P; wall row = 0 (write_bcon).
  for (int p = tid; p < LN; p += nth) {
    int i = p / LM, mm = p - i * LM, k = k0 + mm;
    double2 d = c2(0, 0);
    if constexpr (INC) {  // FP32 on the increment, into double-float for the solve
      float sx = 0.f, sy = 0.f;
      if (k < NTNZ && i < NR - 1) {
        const int left = max(0, i - IW), right = min(i + IW, NR - 1), len = right + 1 - left, i0 = i + IW - right;
        const float* Dr = tb.Ddiv32 + (1 - spar[mm]) * STEN * NR + STEN * i + i0;
        for (int j = 0; j < len; j++) {
          const float de = __ldg(Dr + j);
          const float2 a = f32slot(R, (left + j) * LM + mm);
          sx = fmaf(de, a.x, sx);
          sy = fmaf(de, a.y, sy);
        }
        const float kti = skt32[mm] * tb.rinv32[i], kz = skz32[mm];
        const float2 rt = f32slot(R, LN + p), rz = f32slot(R, 2 * LN + p);
        sx -= kti * rt.y; sy += kti * rt.x;
        sx -= kz * rz.y; sy += kz * rz.x;
      }
      put_df(P, p, sx, sy);
      continue;
    } else if constexpr (DFS) {  // mixed predictor: the same stencil in double-float
      float sx = 0.f, tx = 0.f, sy = 0.f, ty = 0.f;
      if (k < NTNZ && i < NR - 1) {
        const int left = max(0, i - IW), right = min(i + IW, NR - 1), len = right + 1 - left, i0 = i + IW - right;
        const float2* Dr = tb.Ddivdf + (1 - spar[mm]) * STEN * NR + STEN * i + i0;
        for (int j = 0; j < len; j++) {
          const dfloat de = ld_df(Dr + j);
          const float4 a = dfslot(R, (left + j) * LM + mm);
          df_add_prod(sx, tx, de, df_re(a));
          df_add_prod(sy, ty, de, df_im(a));
        }
        const dfloat kti = df_mul(skt_df[mm], ld_df(tb.rinvdf + i)), kz = skz_df[mm];
        const float4 rt = dfslot(R, LN + p), rz = dfslot(R, 2 * LN + p);
        df_sub_prod(sx, tx, kti, df_im(rt)); df_add_prod(sy, ty, kti, df_re(rt));
        df_sub_prod(sx, tx, kz, df_im(rz)); df_add_prod(sy, ty, kz, df_re(rz));
      }
      put_df(P, p, df_norm(sx, tx), df_norm(sy, ty));
      continue;
    } else if (k < NTNZ && i < NR - 1) {
      double kt = skt[mm], kz = skz[mm];
      int left = max(0, i - IW), right = min(i + IW, NR - 1), len = right + 1 - left, i0 = i + IW - right;
      int tab = 1 - spar[mm];
      // d_r u_r + u_r / r in one stencil: Ddiv is D with 1/r_i added to the centre weight
      const double* Dr = tb.Ddiv + tab * STEN * NR + STEN * i + i0;
      double sx = 0.0, sy = 0.0;
      for (int j = 0; j < len; j++) {
        double de = __ldg(Dr + j);
        double2 a = R[(left + j) * LM + mm];
        sx += de * a.x;
        sy += de * a.y;
      }
      double kti = kt * tb.rinv[i];
      double2 rt = R[LN + p], rz = R[2 * LN + p];
      sx -= kti * rt.y; sy += kti * rt.x;
      sx -= kz * rz.y; sy += kz * rz.x;
      d = c2(sx, sy);
    }
    P[p] = d;
  }
  __syncthreads();

  // D. pressure Poisson solve, one thread per mode.
  // (two threads per mode line: real and imaginary parts; every lane of the warp busy)
  // The last factor a solve reads of kind c, mode k: row NR-1, entry 6.
  auto fac_ok = [&](int c, int k) {
    return NSP_IN_BOUNDS(tb, ((size_t)c * NR + NR - 1) * NFAC * NTNZ + 6 * (size_t)NTNZ + k,
                         (size_t)4 * NR * NFAC * NTNZ, BC_LIN_FACTOR);
  };
  // Increment passes: the warps that wait through the solves first prefetch into L2 the
  // rows of u_i that stage I reads (128-byte lines of 8 complex values; the first value
  // of each line clamped into the row).
  if constexpr (INC) {
    if (tid >= 2 * LM) {
      constexpr int LPR = (LM + 7) / 8;  // lines per row segment
      for (int e = tid - 2 * LM; e < 3 * NR * LPR; e += nth - 2 * LM) {
        const int c = e / (NR * LPR), q = e - c * NR * LPR, i = q / LPR, k = min(k0 + 8 * (q - i * LPR), NTNZ - 1);
        prefetch_l2(Ui + (size_t)c * S + (size_t)i * NTNZ + k);
      }
    }
  }
  // Mixed form: the pressure solve in double-float (nsp_df.cuh), the factors split the same way.
  const dfloat* facdf = reinterpret_cast<const dfloat*>(tb.facdf) + (size_t)ps * 4 * NR * NFAC * NTNZ;
  if (tid < 2 * LM) {
    const int mm = tid >> 1, part = tid & 1;
    if (k0 + mm < NTNZ && fac_ok(3, k0 + mm)) {
      dfloat* X = reinterpret_cast<dfloat*>(P + mm) + part;
      const dfloat* fp = facdf + 3 * (size_t)NR * NFAC * NTNZ + k0 + mm;
      const unsigned pair = 3u << ((tid & 31) & ~1);
      if constexpr (INC) {
        // the increment pass's lines hold FP32 pairs here: a deep ring in their slots'
        // free upper halves (3 NR LM entries, RING_DEEP x 16 LM needed)
        if (3 * NR >= 16 * RING_DEEP)
          solve_line_ring<LM, RING_DEEP, 2>(X, 2 * LM, fp, NTNZ, NR, reinterpret_cast<dfloat*>(R) + 1, mm, part, pair);
        else
          solve_line_ring<LM, RING_B, 1>(X, 2 * LM, fp, NTNZ, NR, ringD, mm, part, pair);
      } else if constexpr (DFS)
        solve_line_ring<LM, RING_B, 1>(X, 2 * LM, fp, NTNZ, NR, ringD, mm, part, pair);
      else
        solve_line(reinterpret_cast<double*>(P + mm) + part, 2 * LM, fac + 3 * (size_t)NR * NFAC * NTNZ + k0 + mm,
                   NTNZ, NR);
    }
  }
  __syncthreads();
  if constexpr (INC) {  // the pressure increment to FP32 (hi = fl(hi + lo)), in place
    for (int p = tid; p < LN; p += nth) {
      const float4 a = dfslot(P, p);
      f32slot(P, p) = make_float2(a.x, a.z);
    }
    __syncthreads();
  }

  // E. rhs -= grad p, r/theta -> +/-, wall rows = 0.
  for (int p = tid; p < LN; p += nth) {
    int i = p / LM, mm = p - i * LM, k = k0 + mm;
    if (k >= NTNZ) continue;
    double2 up = c2(0, 0), um = c2(0, 0), rz = c2(0, 0);
    if constexpr (INC) {  // FP32 on the increment; each thread reads its own slots and the P taps
      if (i < NR - 1) {
        const int left = max(0, i - IW), right = min(i + IW, NR - 1), len = right + 1 - left, i0 = i + IW - right;
        const float* Dr = tb.D32 + spar[mm] * STEN * NR + STEN * i + i0;
        float2 rr = f32slot(R, p);
        for (int j = 0; j < len; j++) {
          const float de = __ldg(Dr + j);
          const float2 a = f32slot(P, (left + j) * LM + mm);
          rr.x = fmaf(-de, a.x, rr.x);
          rr.y = fmaf(-de, a.y, rr.y);
        }
        const float kti = skt32[mm] * tb.rinv32[i], kz = skz32[mm];
        const float2 pp = f32slot(P, p);
        float2 rt = f32slot(R, LN + p), fz = f32slot(R, 2 * LN + p);
        rt.x += kti * pp.y; rt.y -= kti * pp.x;
        fz.x += kz * pp.y; fz.y -= kz * pp.x;
        put_df(R, p, rr.x - rt.y, rr.y + rt.x);
        put_df(R, LN + p, rr.x + rt.y, rr.y - rt.x);
        put_df(R, 2 * LN + p, fz.x, fz.y);
        continue;
      }
    } else if constexpr (DFS) {  // mixed predictor: the same in double-float
      const dfloat z{0.f, 0.f};
      dfloat upx = z, upy = z, umx = z, umy = z, rzx = z, rzy = z;
      if (i < NR - 1) {
        const int left = max(0, i - IW), right = min(i + IW, NR - 1), len = right + 1 - left, i0 = i + IW - right;
        const float2* Dr = tb.Ddf + spar[mm] * STEN * NR + STEN * i + i0;
        const float4 r0 = dfslot(R, p);
        float sx = r0.x, tx = r0.y, sy = r0.z, ty = r0.w;  // rr - d_r p
        for (int j = 0; j < len; j++) {
          const dfloat de = ld_df(Dr + j);
          const float4 a = dfslot(P, (left + j) * LM + mm);
          df_sub_prod(sx, tx, de, df_re(a));
          df_sub_prod(sy, ty, de, df_im(a));
        }
        const dfloat rrx = df_norm(sx, tx), rry = df_norm(sy, ty);
        const dfloat kti = df_mul(skt_df[mm], ld_df(tb.rinvdf + i)), kz = skz_df[mm];
        const float4 pp = dfslot(P, p), rt = dfslot(R, LN + p), rz = dfslot(R, 2 * LN + p);
        float a0 = rt.x, b0 = rt.y, a1 = rt.z, b1 = rt.w;  // rt.x += kti pp.y, rt.y -= kti pp.x
        df_add_prod(a0, b0, kti, df_im(pp));
        df_sub_prod(a1, b1, kti, df_re(pp));
        const dfloat rtx = df_norm(a0, b0), rty = df_norm(a1, b1);
        a0 = rz.x; b0 = rz.y; a1 = rz.z; b1 = rz.w;  // rz.x += kz pp.y, rz.y -= kz pp.x
        df_add_prod(a0, b0, kz, df_im(pp));
        df_sub_prod(a1, b1, kz, df_re(pp));
        rzx = df_norm(a0, b0);
        rzy = df_norm(a1, b1);
        upx = df_sub(rrx, rty); upy = df_add(rry, rtx);
        umx = df_add(rrx, rty); umy = df_sub(rry, rtx);
      }
      put_df(R, p, upx, upy); put_df(R, LN + p, umx, umy); put_df(R, 2 * LN + p, rzx, rzy);
      continue;
    } else if (i < NR - 1) {
      double kt = skt[mm], kz = skz[mm];
      int left = max(0, i - IW), right = min(i + IW, NR - 1), len = right + 1 - left, i0 = i + IW - right;
      int tab = spar[mm];
      const double* Dr = tb.D + tab * STEN * NR + STEN * i + i0;
      double2 rr = R[p];  // rr - d_r p, accumulated straight into the multiply-adds
      for (int j = 0; j < len; j++) {
        double de = __ldg(Dr + j);
        double2 a = P[(left + j) * LM + mm];
        rr.x -= de * a.x;
        rr.y -= de * a.y;
      }
      double kti = kt * tb.rinv[i];
      double2 pp = P[p], rt = R[LN + p];
      rz = R[2 * LN + p];
      rt.x += kti * pp.y; rt.y -= kti * pp.x;
      rz.x += kz * pp.y; rz.y -= kz * pp.x;
      up = c2(rr.x - rt.y, rr.y + rt.x);
      um = c2(rr.x + rt.y, rr.y - rt.x);
    }
    R[p] = up; R[LN + p] = um; R[2 * LN + p] = rz;
  }
  __syncthreads();

  // F. Helmholtz solves for u+, u-, u_z, on the warps after the pressure solve's: a
  // block's four solves then run on four different warps, and so on four different SM
  // sub-partitions (warp w of a block on sub-partition (base + w) mod 4), each taking its
  // share of the FP64 pipe.
  constexpr int F0 = ((2 * LM + 31) / 32) * 32 + 6 * LM <= NTH ? ((2 * LM + 31) / 32) * 32 : 0;
  if (tid >= F0 && tid < F0 + 6 * LM) {
    const int tf = tid - F0;
    const int c = tf / (2 * LM), rem = tf - c * 2 * LM, mm = rem >> 1, part = rem & 1;
    if (k0 + mm < NTNZ && fac_ok(c, k0 + mm)) {
      if constexpr (INC)  // FP32 on the hi parts (lo stays 0): an increment of a well-conditioned operator;
                          // FP32 factors, so twice the batches in a ring of the same bytes
        solve_line_ring<LM, 2 * RING_B, 1>(reinterpret_cast<float*>(R + c * LN + mm) + 2 * part, 4 * LM,
                            tb.fac32 + (size_t)ps * 4 * NR * NFAC * NTNZ + (size_t)c * NR * NFAC * NTNZ + k0 + mm,
                            NTNZ, NR, reinterpret_cast<float*>(ringF) + (size_t)c * 2 * RING_B * 16 * LM, mm, part,
                            3u << ((tid & 31) & ~1));
      else if constexpr (DFS)
        solve_line_ring<LM, RING_B, 1>(reinterpret_cast<dfloat*>(R + c * LN + mm) + part, 2 * LM,
                            facdf + (size_t)c * NR * NFAC * NTNZ + k0 + mm, NTNZ, NR,
                            ringF + (size_t)c * RING_B * 16 * LM, mm, part, 3u << ((tid & 31) & ~1));
      else
        solve_line(reinterpret_cast<double*>(R + c * LN + mm) + part, 2 * LM,
                   fac + (size_t)c * NR * NFAC * NTNZ + k0 + mm, NTNZ, NR);
    }
  }
  __syncthreads();

  // G1. wall divergence of the (half-scale) solution, in r/theta form, per mode: FP64;
  // the mixed predictor in double-float, the increment passes in FP32 (their lines hold
  // FP32 values after the solves).
  if (tid < LM) {
    int mm = tid, k = k0 + mm;
    double2 dv = c2(0, 0);
    if constexpr (INC) {
      float sx = 0.f, sy = 0.f;
      if (k < NTNZ) {
        const float* Dw = tb.D32 + (1 - spar[mm]) * STEN * NR + STEN * (NR - 1) + IW;
        float2 urw = make_float2(0.f, 0.f), utw = urw;
        for (int j = 0; j <= IW; j++) {
          const int row = NR - 1 - IW + j;
          const float4 a = dfslot(R, row * LM + mm), b = dfslot(R, LN + row * LM + mm);
          const float2 ur = make_float2(0.5f * (a.x + b.x), 0.5f * (a.z + b.z));
          const float de = __ldg(Dw + j);
          sx = fmaf(de, ur.x, sx);
          sy = fmaf(de, ur.y, sy);
          if (j == IW) { urw = ur; utw = make_float2(0.5f * (a.z - b.z), -0.5f * (a.x - b.x)); }
        }
        const float uzx = dfslot(R, 2 * LN + (NR - 1) * LM + mm).x, uzy = dfslot(R, 2 * LN + (NR - 1) * LM + mm).z;
        const float kt = skt32[mm], kz = skz32[mm];
        sx += urw.x; sy += urw.y;
        sx += -kt * utw.y; sy += kt * utw.x;
        sx += -kz * uzy; sy += kz * uzx;
      }
      dvs32[mm] = make_float2(-sx, -sy);
    } else if constexpr (DFS) {
      float sx = 0.f, tx = 0.f, sy = 0.f, ty = 0.f;
      if (k < NTNZ) {
        const float2* Dw = tb.Ddf + (1 - spar[mm]) * STEN * NR + STEN * (NR - 1) + IW;
        dfloat urwx{0.f, 0.f}, urwy = urwx, utwx = urwx, utwy = urwx;
        for (int j = 0; j <= IW; j++) {
          const int row = NR - 1 - IW + j;
          const float4 a = dfslot(R, row * LM + mm), b = dfslot(R, LN + row * LM + mm);
          const dfloat s0 = df_add(df_re(a), df_re(b)), s1 = df_add(df_im(a), df_im(b));
          const dfloat urx{0.5f * s0.hi, 0.5f * s0.lo}, ury{0.5f * s1.hi, 0.5f * s1.lo};
          const dfloat de = ld_df(Dw + j);
          df_add_prod(sx, tx, de, urx);
          df_add_prod(sy, ty, de, ury);
          if (j == IW) {
            urwx = urx; urwy = ury;
            const dfloat d0 = df_sub(df_im(a), df_im(b)), d1 = df_sub(df_re(a), df_re(b));
            utwx = dfloat{0.5f * d0.hi, 0.5f * d0.lo};
            utwy = dfloat{-0.5f * d1.hi, -0.5f * d1.lo};
          }
        }
        const float4 z = dfslot(R, 2 * LN + (NR - 1) * LM + mm);
        const dfloat kt = skt_df[mm], kz = skz_df[mm];
        const dfloat one{1.f, 0.f};
        df_add_prod(sx, tx, one, urwx); df_add_prod(sy, ty, one, urwy);
        df_sub_prod(sx, tx, kt, utwy); df_add_prod(sy, ty, kt, utwx);
        df_sub_prod(sx, tx, kz, df_im(z)); df_add_prod(sy, ty, kz, df_re(z));
      }
      const dfloat dx = df_norm(sx, tx), dy = df_norm(sy, ty);
      dvs_df[mm] = make_float4(-dx.hi, -dx.lo, -dy.hi, -dy.lo);
    } else {
      if (k < NTNZ) {
        double kt = skt[mm], kz = skz[mm];
        int tab = 1 - spar[mm];
        const double* Dw = tb.D + tab * STEN * NR + STEN * (NR - 1) + IW;
        double sx = 0.0, sy = 0.0;
        double2 urw = c2(0, 0), utw = c2(0, 0);
        for (int j = 0; j <= IW; j++) {
          int row = NR - 1 - IW + j;
          const double2 a = R[row * LM + mm], b = R[LN + row * LM + mm];
          double2 ur = c2(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
          double de = __ldg(Dw + j);
          sx += de * ur.x;
          sy += de * ur.y;
          if (j == IW) { urw = ur; utw = c2(0.5 * (a.y - b.y), -0.5 * (a.x - b.x)); }
        }
        const double2 uzw = R[2 * LN + (NR - 1) * LM + mm];
        sx += urw.x; sy += urw.y;
        sx += -kt * utw.y; sy += kt * utw.x;
        sx += -kz * uzw.y; sy += kz * uzw.x;
        dv = c2(-sx, -sy);
      }
      dvs[mm] = dv;
    }
  }
  __syncthreads();

  // G2. u += (-div_wall) V (both at half scale), back to full-scale r/theta, mode (0,0) constraints.
  // Increment passes: in FP32 on the increment (the solves' results, their hi parts), into
  // the FP32 halves of the slots -- the increment needs FP32's relative precision, the update
  // of u in stage I stays FP64.  The mixed predictor: in double-float.
  if constexpr (INC) {
    const float2* Vp32 = tb.V32 + (size_t)ps * 3 * S;
    for (int p = tid; p < LN; p += nth) {
      const int i = p / LM, mm = p - i * LM, k = k0 + mm;
      if (k >= NTNZ) continue;
      const size_t hv = (size_t)i * NTNZ + k;
      if (!NSP_IN_BOUNDS(tb, hv, S, BC_LIN_POINT)) continue;
      const float4 a = dfslot(R, p), b = dfslot(R, LN + p), z = dfslot(R, 2 * LN + p);  // FP32: the hi parts
      float2 up = make_float2(a.x, a.z), um = make_float2(b.x, b.z), uz = make_float2(z.x, z.z);
      const float2 dv = dvs32[mm], v0 = Vp32[hv], v1 = Vp32[S + hv], v2 = Vp32[2 * S + hv];
      up.x += dv.x * v0.x - dv.y * v0.y; up.y += dv.x * v0.y + dv.y * v0.x;
      um.x += dv.x * v1.x - dv.y * v1.y; um.y += dv.x * v1.y + dv.y * v1.x;
      uz.x += dv.x * v2.x - dv.y * v2.y; uz.y += dv.x * v2.y + dv.y * v2.x;
      float2 ur = make_float2(up.x + um.x, up.y + um.y);
      float2 ut = make_float2(up.y - um.y, -(up.x - um.x));
      uz = make_float2(uz.x + uz.x, uz.y + uz.y);
      if (k == 0) { ur = make_float2(0.f, 0.f); ut.y = 0.f; uz.y = 0.f; }
      f32slot(R, p) = ur; f32slot(R, LN + p) = ut; f32slot(R, 2 * LN + p) = uz;
    }
  } else if constexpr (DFS) {  // mixed predictor: the same in double-float, with V split likewise
    const float4* Vd = reinterpret_cast<const float4*>(tb.Vdf) + (size_t)ps * 3 * S;
    for (int p = tid; p < LN; p += nth) {
      const int i = p / LM, mm = p - i * LM, k = k0 + mm;
      if (k >= NTNZ) continue;
      const size_t hv = (size_t)i * NTNZ + k;
      if (!NSP_IN_BOUNDS(tb, hv, S, BC_LIN_POINT)) continue;
      const float4 dv = dvs_df[mm];
      const dfloat dvx = df_re(dv), dvy = df_im(dv);
      // u + dv v, complex: x = u.x + dv.x v.x - dv.y v.y, y = u.y + dv.x v.y + dv.y v.x
      auto corr = [&](const float4& u, const float4& v, dfloat& ox, dfloat& oy) {
        float s0 = u.x, t0 = u.y;
        df_add_prod(s0, t0, dvx, df_re(v));
        df_sub_prod(s0, t0, dvy, df_im(v));
        ox = df_norm(s0, t0);
        s0 = u.z; t0 = u.w;
        df_add_prod(s0, t0, dvx, df_im(v));
        df_add_prod(s0, t0, dvy, df_re(v));
        oy = df_norm(s0, t0);
      };
      dfloat upx, upy, umx, umy, uzx, uzy;
      corr(dfslot(R, p), __ldg(Vd + hv), upx, upy);
      corr(dfslot(R, LN + p), __ldg(Vd + S + hv), umx, umy);
      corr(dfslot(R, 2 * LN + p), __ldg(Vd + 2 * S + hv), uzx, uzy);
      const dfloat zero{0.f, 0.f};
      dfloat urx = df_add(upx, umx), ury = df_add(upy, umy);
      const dfloat utx = df_sub(upy, umy);
      dfloat uty = df_neg(df_sub(upx, umx));
      uzx = dfloat{2.f * uzx.hi, 2.f * uzx.lo};
      uzy = dfloat{2.f * uzy.hi, 2.f * uzy.lo};
      if (k == 0) { urx = ury = zero; uty = zero; uzy = zero; }
      put_df(R, p, urx, ury); put_df(R, LN + p, utx, uty); put_df(R, 2 * LN + p, uzx, uzy);
    }
  } else for (int p = tid; p < LN; p += nth) {
    int i = p / LM, mm = p - i * LM, k = k0 + mm;
    if (k >= NTNZ) continue;
    double2 up = R[p], um = R[LN + p], uz = R[2 * LN + p];
    double2 dv = dvs[mm];
    size_t hv = (size_t)i * NTNZ + k;
    if (!NSP_IN_BOUNDS(tb, hv, S, BC_LIN_POINT)) continue;
    double2 v0 = Vp[hv], v1 = Vp[S + hv], v2 = Vp[2 * S + hv];
    up.x += dv.x * v0.x - dv.y * v0.y; up.y += dv.x * v0.y + dv.y * v0.x;
    um.x += dv.x * v1.x - dv.y * v1.y; um.y += dv.x * v1.y + dv.y * v1.x;
    uz.x += dv.x * v2.x - dv.y * v2.y; uz.y += dv.x * v2.y + dv.y * v2.x;
    double2 ur = c2(up.x + um.x, up.y + um.y);
    double2 ut = c2(up.y - um.y, -(up.x - um.x));
    uz = c2(uz.x + uz.x, uz.y + uz.y);
    if (k == 0) { ur = c2(0, 0); ut.y = 0.0; uz.y = 0.0; }
    R[p] = ur; R[LN + p] = ut; R[2 * LN + p] = uz;
  }
  __syncthreads();

  // H. constant mass flux on mode (0,0) (increment passes: on the FP32 increment, the
  // flux summed in FP64, no Qdes term).
  if (k0 == 0 && tid == 0) {
    double Q = 0.0;
    if constexpr (INC) {
      for (int i = 0; i < NR; i++) Q += tb.rdr[i] * f32_to_f64(f32slot(R, 2 * LN + i * LM).x);
      const double corr = -Q / Qc;
      for (int i = 0; i < NR; i++) f32slot(R, 2 * LN + i * LM).x += f64_to_f32(corr * ucp[i]);
    } else if constexpr (DFS) {  // the mixed predictor's double-float line, summed and corrected in FP64
      for (int i = 0; i < NR; i++) Q += tb.rdr[i] * df_value(R, 2 * LN + i * LM).x;
      const double corr = (tb.Qdes - Q) / Qc;
      for (int i = 0; i < NR; i++) {
        float4& v = dfslot(R, 2 * LN + i * LM);
        const float2 x = split_df(f32_to_f64(v.x) + f32_to_f64(v.y) + corr * ucp[i]);
        v.x = x.x;
        v.y = x.y;
      }
    } else {
      for (int i = 0; i < NR; i++) Q += tb.rdr[i] * R[2 * LN + i * LM].x;
      double corr = (tb.Qdes - Q) / Qc;
      for (int i = 0; i < NR; i++) R[2 * LN + i * LM].x += corr * ucp[i];
    }
  }
  __syncthreads();

  // I. store the new iterate; corrector: convergence measure against the previous one.
  // The maxima of squared magnitudes (>= +0, or NaN) are taken on their bit patterns
  // as unsigned integers, which order like the values, and the finiteness test reads
  // the exponent field: both on the integer pipe.
  unsigned long long lnum = 0ull, lden = 0ull;
  unsigned lnum32 = 0u, lden32 = 0u;  // increment passes: the same maxima as FP32 bits
  const double hdi = 0.5 * tb.d_im;   // increment passes: u_{i+1} = u_i + hdi * (the pass's result)
  bool nonfin = false;
  constexpr int UI = 2;  // points per thread whose previous-iterate loads are issued together
  for (int pb = tid; pb < LN; pb += UI * nth) {
    double2 o[UI][3];
    if (!pred) {
#pragma unroll
      for (int u = 0; u < UI; u++) {
        const int p = pb + u * nth, i = p / LM, k = k0 + p - i * LM;
        const bool ok = p < LN && k < NTNZ && NSP_IN_BOUNDS(tb, (size_t)i * NTNZ + k, S, BC_LIN_POINT);
        const size_t h = ok ? (size_t)i * NTNZ + k : 0;
#pragma unroll
        for (int c = 0; c < 3; c++) o[u][c] = ok ? Ui[c * S + h] : c2(0, 0);
      }
    }
#pragma unroll
    for (int u = 0; u < UI; u++) {
      const int p = pb + u * nth, i = p / LM, k = k0 + p - i * LM;
      if (p >= LN || k >= NTNZ) continue;
      const size_t h = (size_t)i * NTNZ + k;
      if (kBoundsCheck && h >= (size_t)S) continue;  // (recorded by the load loop above)
#pragma unroll
      for (int c = 0; c < 3; c++) {
        double2 v;
        if constexpr (INC) {
          // |increment|^2 and |u_i|^2 in FP32 (the measure only decides err > tol)
          const float2 f = f32slot(R, c * LN + p);
          const float ox = f64_to_f32(o[u][c].x), oy = f64_to_f32(o[u][c].y);
          lnum32 = max(lnum32, __float_as_uint(fmaf(f.x, f.x, f.y * f.y)));
          lden32 = max(lden32, __float_as_uint(fmaf(ox, ox, oy * oy)));
          v = c2(fma(hdi, f32_to_f64(f.x), o[u][c].x), fma(hdi, f32_to_f64(f.y), o[u][c].y));
        } else {
          v = DFS ? df_value(R, c * LN + p) : R[c * LN + p];
          if (!pred) {
            const double ex = o[u][c].x - v.x, ey = o[u][c].y - v.y;
            lnum = max(lnum, (unsigned long long)__double_as_longlong(ex * ex + ey * ey));
            lden = max(lden, (unsigned long long)__double_as_longlong(o[u][c].x * o[u][c].x + o[u][c].y * o[u][c].y));
          }
        }
        const unsigned EX = 0x7FF00000u;
        nonfin |= ((unsigned)__double2hiint(v.x) & EX) == EX || ((unsigned)__double2hiint(v.y) & EX) == EX;
        Ui[c * S + h] = v;
        if (Ui32) {
          const float2 f = make_float2(f64_to_f32(v.x), f64_to_f32(v.y));  // integer-pipe rounding
          Ui32[c * S + h] = f;
          reinterpret_cast<float2*>(R + c * LN + p)[0] = f;  // FP32 copy for the d_r mirror below
        }
      }
    }
  }
  if (nonfin) bad = 1;
  if constexpr (INC) {  // float -> double is exact and monotonic; the increment is hdi x the pass's result
    lnum = (unsigned long long)__double_as_longlong(f32_to_f64(__uint_as_float(lnum32)) * (hdi * hdi));
    lden = (unsigned long long)__double_as_longlong(f32_to_f64(__uint_as_float(lden32)));
  }
  if (!pred) {
    for (int o = 16; o > 0; o >>= 1) {
      lnum = max(lnum, __shfl_xor_sync(0xffffffffu, lnum, o));
      lden = max(lden, __shfl_xor_sync(0xffffffffu, lden, o));
    }
    if ((tid & 31) == 0) { wnum[tid >> 5] = lnum; wden[tid >> 5] = lden; }
  }
  __syncthreads();
  // J. mixed form: d_r of the new FP32 mirror (the theta-inverse's d_r u fields), with
  // the transform kernels' stencil, so that they read one value instead of 7 levels.
  if (Udr32) {
    const float2* F = reinterpret_cast<const float2*>(R);  // FP32 value of line entry e at F[2e]
    for (int p = tid; p < LN; p += nth) {
      const int i = p / LM, mm = p - i * LM, k = k0 + mm;
      if (k >= NTNZ) continue;
      const int left = max(0, i - IW), right = min(i + IW, NR - 1), len = right + 1 - left, i0 = i + IW - right;
      const size_t h = (size_t)i * NTNZ + k;
      if (!NSP_IN_BOUNDS(tb, h, S, BC_LIN_POINT)) continue;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const int tab = abs(spar[mm] - (c < 2 ? 1 : 0));
        const float* Dr = tb.D32 + tab * STEN * NR + STEN * i + i0;
        Udr32[c * S + h] = dr32_line(Dr, left, len, [&](int row) { return F[2 * (c * LN + row * LM + mm)]; });
      }
    }
  }
  if (tid == 0) {
    if (!pred) {
      unsigned long long a = 0ull, b = 0ull;
      for (int w = 0; w < nth / 32; w++) { a = max(a, wnum[w]); b = max(b, wden[w]); }
      atomicMax(ctl->num + gm, a);
      atomicMax(ctl->den + gm, b);
    }
    if (bad) atomicOr(ctl->status + gm, NSP_ERR_NONFINITE);
  }
}

// Per-member bookkeeping after each predictor/corrector pass; sets the graph's
// loop condition.  Single block.
__global__ void converge_k(Ctl* ctl, cudaGraphConditionalHandle h, int use_cond) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  const int nm = ctl->nmem;
  for (int m = threadIdx.x; m < nm; m += blockDim.x) {
    int ph = ctl->phase[m];
    if (ph == 0) {
      ph = 1;
      ctl->ite[m] = 0;
    } else if (ph > 0) {
      int it = ctl->ite[m] + 1;
      ctl->ite[m] = it;
      double num = __longlong_as_double((long long)ctl->num[m]);
      double den = __longlong_as_double((long long)ctl->den[m]);
      double err = num / den;
      ctl->err[m] = err;
      if (!isfinite(err)) atomicOr(ctl->status + m, NSP_ERR_NONFINITE);
      bool more = (it < ctl->maxit) && (err > ctl->tol);
      if (!more) {
        if (ctl->step < ctl->hist_cap) ctl->hist[(size_t)ctl->step * nm + m] = it;
        if (err > ctl->tol) ctl->unconv[m] += 1;  // stopped by maxit, not converged (one thread per m)
        ph = -1;
      } else {
        ph = ph + 1;
      }
    }
    ctl->num[m] = 0ull;
    ctl->den[m] = 0ull;
    ctl->phase[m] = ph;
    if (ph >= 0) any = 1;
  }
  __syncthreads();
  if (!any) {  // every member converged: the step is complete, roles of state and iterate swap
    for (int m = threadIdx.x; m < nm; m += blockDim.x) ctl->phase[m] = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!any && !ctl->hold) {
      ctl->parity ^= 1;
      ctl->step += 1;
    }
    ctl->any = any;
    if (use_cond) cudaGraphSetConditional(h, any ? 1u : 0u);
  }
}

__global__ void finish_step_k(Ctl* ctl) {
  ctl->parity ^= 1;
  ctl->step += 1;
}

// Divergence diagnostic of one member's state (div_k / divWall_k, mod_radialFD.cu:34-96):
// |d_r u_r + u_r/r + i m u_theta / r + i k_z u_z| per point, maximum over the interior
// rows into out[0] and over the wall row into out[1] (ordered bits, atomicMax).
__global__ void diag_div_k(Tables tb, const double2* __restrict__ U, unsigned long long* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int NR = tb.NR, NT = tb.NT, NZ = tb.NZ, NTNZ = tb.NTNZ;
  const long long S = tb.S;
  U += (size_t)blockIdx.z * 3 * S;  // member blockIdx.z of a batched launch
  out += 2 * blockIdx.z;
  double mi = 0.0, mw = 0.0;
  if (k < NTNZ) {
    const int it = k / NZ, l = k - it * NZ, m = it < NT / 2 ? it : it - NT;
    const double kt = tb.kts * (double)m, kz = tb.kzs * (double)l;
    const int tab = abs((abs(m) % 2) - 1);
    for (int i = 0; i < NR; i++) {
      const int left = max(0, i - IW), right = min(i + IW, NR - 1), len = right + 1 - left, i0 = i + IW - right;
      const double* Dr = tb.D + tab * STEN * NR + STEN * i + i0;
      double sx = 0.0, sy = 0.0;
      for (int j = 0; j < len; j++) {
        const double2 a = U[(size_t)(left + j) * NTNZ + k];
        sx += Dr[j] * a.x;
        sy += Dr[j] * a.y;
      }
      const size_t h = (size_t)i * NTNZ + k;
      const double ri = tb.rinv[i], kti = kt * ri;
      const double2 ur = U[h], ut = U[S + h], uz = U[2 * S + h];
      sx += ur.x * ri - kti * ut.y - kz * uz.y;
      sy += ur.y * ri + kti * ut.x + kz * uz.x;
      const double a = sqrt(sx * sx + sy * sy);
      if (i < NR - 1) mi = fmax(mi, a);
      else mw = fmax(mw, a);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    mi = fmax(mi, __shfl_xor_sync(0xffffffffu, mi, o));
    mw = fmax(mw, __shfl_xor_sync(0xffffffffu, mw, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out, (unsigned long long)__double_as_longlong(mi));
    atomicMax(out + 1, (unsigned long long)__double_as_longlong(mw));
  }
}

void launch_diag_div(const Tables& tb, const double2* U, unsigned long long* out, cudaStream_t st, int nmem) {
  diag_div_k<<<dim3((tb.NTNZ + 127) / 128, 1, nmem), 128, 0, st>>>(tb, U, out);
}

// Re u_z(m=0, k_z=0)(r_i) of nmem consecutive members -> out[member][NR].
__global__ void gather_mean_k(Tables tb, const double2* __restrict__ U, double* __restrict__ out, int nmem) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nmem * tb.NR) return;
  const int m = q / tb.NR, i = q - m * tb.NR;
  out[q] = U[((size_t)m * 3 + 2) * tb.S + (size_t)i * tb.NTNZ].x;
}

void launch_gather_mean(const Tables& tb, const double2* U, double* out, int nmem, cudaStream_t st) {
  gather_mean_k<<<(nmem * tb.NR + 127) / 128, 128, 0, st>>>(tb, U, out, nmem);
}

// Cross-section diagnostics of one member's state (wrt_qcr / wrt_ucr with q0kernel_k,
// u0kernel_k, q1kernel_k and intq, mod_io_nonlinear.cu:54-117, 572-660 and
// mod_cublasflux.cu:119-130): at every physical axial point z_n,
//   q(z_n) = sum_i rdr_i (1/NTP) sum_theta (u_r^2 + u_theta^2),   u(z_n) = the same with u_z^2.
// (The reference's periodic Simpson rule in theta with unit weights sums to the plain
// mean.)  The theta mean is taken by Parseval from the spectral coefficients: at
// (r_i, z_n), u(theta) = Re sum_m P_m e^{i m theta} with P_m = c_{m,0} + 2 sum_{l>0}
// c_{m,l} e^{i k_l z_n} (the reference's C2R extension), whose mean square is
// (Re P_0)^2 + 2 sum_{0<mu<NT/2} |(P_mu + conj P_-mu)/2|^2 + |P_-NT/2|^2 / 2.
// One thread per (level, z_n); per-level partials rdr_i * mean square go to
// part[2][NR][NZR], summed over i on the host in a fixed order.
__global__ void diag_cross_k(Tables tb, const double2* __restrict__ U, double* __restrict__ part) {
  const int i = blockIdx.y, n = blockIdx.x * blockDim.x + threadIdx.x;
  const int NT = tb.NT, NZ = tb.NZ, NZR = tb.NZR, NTNZ = tb.NTNZ;
  if (n >= NZR) return;
  const long long S = tb.S;
  U += (size_t)blockIdx.z * 3 * S;  // member blockIdx.z of a batched launch
  part += (size_t)blockIdx.z * 2 * tb.NR * NZR;
  double ms[3];
  for (int c = 0; c < 3; c++) {
    const double2* col = U + c * S + (size_t)i * NTNZ;
    // P of theta slot it at z_n
    auto P = [&](int it) {
      const double2* a = col + (size_t)it * NZ;
      double px = a[0].x, py = a[0].y;
      for (int l = 1; l < NZ; l++) {
        const double2 w = tb.tw_z[(size_t)l * n % NZR];  // exp(-2 pi i l n / NZR); E_l = conj(w)
        const double2 b = a[l];
        px += 2.0 * (b.x * w.x + b.y * w.y);
        py += 2.0 * (b.y * w.x - b.x * w.y);
      }
      return make_double2(px, py);
    };
    const double2 p0 = P(0);
    double s = p0.x * p0.x;
    for (int mu = 1; mu < NT / 2; mu++) {
      const double2 pp = P(mu), pm = P(NT - mu);
      const double qx = 0.5 * (pp.x + pm.x), qy = 0.5 * (pp.y - pm.y);
      s += 2.0 * (qx * qx + qy * qy);
    }
    const double2 pn = P(NT / 2);  // m = -NT/2, no +NT/2 partner
    s += 0.5 * (pn.x * pn.x + pn.y * pn.y);
    ms[c] = s;
  }
  const double w = tb.rdr[i];
  part[(size_t)i * NZR + n] = w * (ms[0] + ms[1]);
  part[(size_t)(tb.NR + i) * NZR + n] = w * ms[2];
}

void launch_diag_cross(const Tables& tb, const double2* U, double* part, cudaStream_t st, int nmem) {
  dim3 g((tb.NZR + 63) / 64, tb.NR, nmem);
  diag_cross_k<<<g, 64, 0, st>>>(tb, U, part);
}

// FP64 throughput probe: 8 independent multiply-add chains per thread, no memory
// traffic; the measured denominator of the FP64 roofline.
__global__ void fp64_peak_k(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = threadIdx.x + k;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = x[k] * a + b;
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

void launch_fp64_peak(double* out, int blocks, int threads, int iters, cudaStream_t st) {
  fp64_peak_k<<<blocks, threads, 0, st>>>(out, iters, 0.999999, 1e-7);
}

// kind 0..3: the FP64 solve; kind 4..7: the same operator's solve in double-float, as
// the increment passes run it (the right-hand side split into hi + lo, the solution
// returned as hi + lo in FP64).  One thread per mode line, or per part of one.
__global__ void lusolve_k(Tables tb, int kind, const double2* rhs, double2* sol) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  const size_t fo = (size_t)(kind & 3) * tb.NR * NFAC * tb.NTNZ;
  if (kind < 4) {
    if (k >= tb.NTNZ) return;
    for (int i = 0; i < tb.NR; i++) sol[(size_t)i * tb.NTNZ + k] = rhs[(size_t)i * tb.NTNZ + k];
    solve_line(sol + k, tb.NTNZ, tb.fac + fo + k, tb.NTNZ, tb.NR);
    return;
  }
  const int part = k & 1;
  k >>= 1;
  if (k >= tb.NTNZ) return;
  const double* in = reinterpret_cast<const double*>(rhs) + part;
  double* out = reinterpret_cast<double*>(sol) + part;
  dfloat* X = reinterpret_cast<dfloat*>(out);  // the double slots of this part hold the double-float values
  for (int i = 0; i < tb.NR; i++) {
    const size_t h = 2 * ((size_t)i * tb.NTNZ + k);
    const double x = in[h];
    const float hi = f64_to_f32(x);
    X[h] = dfloat{hi, f64_to_f32(x - f32_to_f64(hi))};
  }
  solve_line(X + 2 * (size_t)k, 2 * tb.NTNZ, reinterpret_cast<const dfloat*>(tb.facdf) + fo + k, tb.NTNZ, tb.NR);
  for (int i = 0; i < tb.NR; i++) {
    const size_t h = 2 * ((size_t)i * tb.NTNZ + k);
    const dfloat v = X[h];
    out[h] = f32_to_f64(v.hi) + f32_to_f64(v.lo);
  }
}

// Block shapes of the linear pass (modes per block, threads): the candidates of the
// setup-time autotuner.  Shared memory per block is 4 radial lines per mode.  Wide
// blocks (32, 64 modes) give the solve phases one or more full warps on every SM
// sub-partition; narrow ones more blocks per SM; 16 x 512 keeps 16-mode blocks at
// 1024 threads per SM where NR is large enough that two of them fill its shared memory.
#define NSP_LIN_SHAPES(X) \
  X(0, 16, 256) X(1, 8, 128) X(2, 8, 256) X(3, 4, 128) X(4, 12, 192) X(5, 12, 256) X(6, 24, 384) X(7, 32, 512) \
  X(8, 32, 256) X(9, 64, 512) X(10, 64, 1024) X(11, 16, 512)
struct LinShape { int LM, NTH; };
static const LinShape kLinShapes[LIN_VARIANTS] = {
#define NSP_LIN_ENTRY(v, lm, nth) {lm, nth},
    NSP_LIN_SHAPES(NSP_LIN_ENTRY)
#undef NSP_LIN_ENTRY
};

int linear_default_variant(int NR) { return NR <= 64 ? 0 : 2; }

void linear_shape(int v, int* LM, int* NTH) {
  *LM = kLinShapes[v].LM;
  *NTH = kLinShapes[v].NTH;
}

// Dynamic shared memory of a block: 4 radial lines, and the factor rings in the mixed form.
static size_t linear_smem(int v, int NR, bool mixed) {
  const int LM = kLinShapes[v].LM;
  return sizeof(double2) * 4 * (size_t)NR * LM + (mixed ? ring_extra(NR, LM) : 0);
}

bool linear_variant_fits(int v, int NR) {
  return v >= 0 && v < LIN_VARIANTS && linear_smem(v, NR, true) <= 200 * 1024;
}

void configure_linear_kernels() {
  const int big = 200 * 1024;
#define NSP_LIN_CFG(v, lm, nth)                                                                        \
  cudaFuncSetAttribute(linear_k<lm, nth, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big); \
  cudaFuncSetAttribute(linear_k<lm, nth, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);  \
  cudaFuncSetAttribute(linear_k<lm, nth, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);      \
  cudaFuncSetAttribute(linear_k<lm, nth, false, true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);  \
  cudaFuncSetAttribute(linear_k<lm, nth, true, true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  NSP_LIN_SHAPES(NSP_LIN_CFG)
#undef NSP_LIN_CFG
}

void launch_linear(const Tables& tb, const Bufs& bf, Ctl* dctl, cudaStream_t st, int which) {
  // The full pass, then in the mixed form the increment pass (correctors), each with
  // its own block shape; each returns at once in the other's passes.
  const bool mixed = bf.U32[0] != nullptr;
  for (int pass = 0; pass < 2; pass++) {
    if (mixed ? !(which & (pass ? LIN_CORR : LIN_PRED)) : (pass == 1 || which == 0)) continue;
    const int want = pass ? tb.lin_variant_inc : tb.lin_variant;
    const int v = linear_variant_fits(want, tb.NR) ? want : linear_default_variant(tb.NR);
    const LinShape s = kLinShapes[v];
    const dim3 grid((tb.NTNZ + s.LM - 1) / s.LM, tb.nmem);
    const size_t smem = linear_smem(v, tb.NR, mixed);
    switch (v) {
#define NSP_LIN_CASE(v, lm, nth)                                                          \
  case v:                                                                                \
    if (pass) linear_k<lm, nth, true, true><<<grid, nth, smem, st>>>(tb, bf, dctl);      \
    else if (mixed) linear_k<lm, nth, false, true><<<grid, nth, smem, st>>>(tb, bf, dctl); \
    else linear_k<lm, nth, false, false><<<grid, nth, smem, st>>>(tb, bf, dctl);         \
    break;
      NSP_LIN_SHAPES(NSP_LIN_CASE)
#undef NSP_LIN_CASE
      default: break;
    }
  }
}

void launch_converge(Ctl* dctl, int nmem, unsigned long long cond_handle, int use_cond, cudaStream_t st) {
  (void)nmem;
  converge_k<<<1, 256, 0, st>>>(dctl, (cudaGraphConditionalHandle)cond_handle, use_cond);
}

void launch_finish_step(Ctl* dctl, cudaStream_t st) { finish_step_k<<<1, 1, 0, st>>>(dctl); }

void launch_lusolve(const Tables& tb, int kind, const double2* rhs, double2* sol, cudaStream_t st) {
  const int n = kind < 4 ? tb.NTNZ : 2 * tb.NTNZ;
  lusolve_k<<<(n + 127) / 128, 128, 0, st>>>(tb, kind, rhs, sol);
}

}  // namespace nsp
