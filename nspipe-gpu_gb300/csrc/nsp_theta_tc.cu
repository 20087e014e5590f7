// nsp_theta_tc.cu -- the mixed form's azimuthal transforms as DFT-matrix GEMMs on
// the 5th-generation tensor cores (tcgen05, kind::tf32, accumulators in TMEM).
//
// The theta transforms of the nonlinear term (the 12 inverse and 3 forward
// transforms of nonlinear(), mod_io_nonlinear.cu:380-409 with mod_fft.cu:37-48)
// are short -- NTP = 3 NT / 2 points -- so each 128-line tile is multiplied by the
// real form of the DFT matrix instead of running a radix FFT:
//   inverse: [Re g; Im g](p)  = sum_it [[cos, -sin], [sin, cos]](phi) [Re c; Im c](it)
//            K = 2 NT inputs, N = 2 NTP outputs, phi = 2 pi m_it p / NTP;
//   forward: [Re n; Im n](it) = s sum_p [[cos, sin], [-sin, cos]](phi) [Re h; Im h](p)
//            K = 2 NTP inputs, N = 2 NT outputs, s = 1 / (NTP NZR) (normalize_k).
// The inverse tile is built in shared memory straight from the FP32 state mirror
// (u, the 7-point radial derivative d_r u and i m u / r, as nl_theta_inv does);
// the forward tile from the z stage's output H.  Outputs go to the same arrays as
// the FFT kernels' (G, and N with the retained-mode mask and wall forcing), so the
// z stage and the linear pass are unchanged.
//
// Precision (3xTF32): each FP32 operand x is split into hi (x rounded to TF32) and
// lo (the remainder, rounded to TF32); a tile accumulates lo*Bhi + hi*Blo + hi*Bhi
// in FP32, about 2^-21 relative per product instead of TF32's 2^-11.  The DFT matrix
// is split on the host from long-double values.
//
// Operands are K-major, unswizzled core matrices (nsp_tc.cuh); A = the data tile
// [128 lines][K], B = the DFT matrix [N][K], D = A B^T in 128 TMEM lanes x N
// columns, one line per lane, so the epilogue's stores are coalesced along l.
// Persistent CTAs (one per SM) copy the DFT image once with a bulk async copy and
// pipeline over tiles: tile j's operands (loaded into registers during the previous
// iteration) go to shared memory -> fence -> one thread of warp 0 issues 3 K/8 MMAs
// into TMEM accumulator j % 2 and commits to an mbarrier -> tile j+1's global loads
// are issued -> warps 1-15 each wait (bounded) for tile j-1's MMAs and drain its
// accumulator to global memory while tile j is on the tensor cores and tile j+1's
// loads are in flight.  Warp 0 takes no part in the drain, so the serial MMA issue is
// off the other warps' path.  Every wait is bounded: a CTA whose wait runs out records a fault in the
// control block, waits (bounded) for its MMAs and still frees its TMEM.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "nsp_bounds.cuh"
#include "nsp_cvt.cuh"
#include "nsp_fft.cuh"
#include "nsp_internal.h"
#include "nsp_state.cuh"
#include "nsp_tc.cuh"

namespace nsp {

namespace {

constexpr int TM = 128;             // lines per tile (the MMA's M)
constexpr int TC_THREADS = 512;     // 16 warps: fill by all; warp 0 issues the MMAs, warps 1-15 drain
constexpr int WAIT_LIMIT = 1 << 22; // try_wait polls before a wait is abandoned

// Issue lo*Bhi + hi*Blo + hi*Bhi over K (8 per instruction) and commit to bar.
template <int K, int N>
__device__ __forceinline__ void issue_3xtf32(uint32_t tmem, const unsigned char* ah, const unsigned char* al,
                                             const unsigned char* bh, const unsigned char* bl, uint64_t* bar) {
  constexpr uint32_t SBO = (K / 4) * 128;
  constexpr uint32_t ID = tc::idesc_tf32(TM, N);
  const uint32_t a_h = tc::saddr(ah), a_l = tc::saddr(al), b_h = tc::saddr(bh), b_l = tc::saddr(bl);
  tc::fence_after_sync();
#pragma unroll
  for (int s = 0; s < K / 8; s++)
    tc::mma_tf32(tmem, tc::desc(a_l + 256 * s, tc::LBO, SBO), tc::desc(b_h + 256 * s, tc::LBO, SBO), ID, s > 0);
#pragma unroll
  for (int s = 0; s < K / 8; s++)
    tc::mma_tf32(tmem, tc::desc(a_h + 256 * s, tc::LBO, SBO), tc::desc(b_l + 256 * s, tc::LBO, SBO), ID, 1);
#pragma unroll
  for (int s = 0; s < K / 8; s++)
    tc::mma_tf32(tmem, tc::desc(a_h + 256 * s, tc::LBO, SBO), tc::desc(b_h + 256 * s, tc::LBO, SBO), ID, 1);
  tc::commit(bar);
}

// Four consecutive K entries of one operand row (16 bytes at a 16-byte aligned core
// matrix offset): their TF32 hi and lo parts as two vector stores.
__device__ __forceinline__ void put_split4(unsigned char* ah, unsigned char* al, uint32_t off, const float* x) {
  float4 h, l;
  tc::split_tf32(x[0], h.x, l.x);
  tc::split_tf32(x[1], h.y, l.y);
  tc::split_tf32(x[2], h.z, l.z);
  tc::split_tf32(x[3], h.w, l.w);
  *reinterpret_cast<float4*>(ah + off) = h;
  *reinterpret_cast<float4*>(al + off) = l;
}

}  // namespace

// Accumulator drain: warps 1..15 (warp 0 issues the MMAs meanwhile).  A warp may read
// TMEM lane quarter warp % 4 only; quarter 0 has three draining warps (4, 8, 12), the
// others four (q, q+4, q+8, q+12), and each takes a contiguous share of the N columns in
// units of 8: [c0, c0 + nc).  False for warp 0.
template <int N>
__device__ __forceinline__ bool drain_share(int warp, int* q, int* c0, int* nc) {
  if (warp == 0) return false;
  *q = warp & 3;
  const int P = *q == 0 ? 3 : 4, p = *q == 0 ? (warp >> 2) - 1 : (warp >> 2);
  constexpr int U = N / 8;
  const int u0 = p * U / P, u1 = (p + 1) * U / P;
  *c0 = 8 * u0;
  *nc = 8 * (u1 - u0);
  return true;
}
template <int N> constexpr int drain_max() { return 8 * ((N / 8 + 2) / 3); }  // the largest share

// ------------------------------------------------------------------ tile jobs
// Inverse: line (f, level i, l) of a member, f = u_r, u_t, u_z, d_r u_r.., (i m / r) u_r..;
// K index it (Re) / NT + it (Im) over the NT stored modes.
template <int NT, int NTP> struct InvJob {
  static constexpr int K = 2 * NT, N = 2 * NTP, STAGES = 2;
  static constexpr int J = NT / 4;  // modes per thread in the fill
  static_assert(NT % 16 == 0, "the fill takes blocks of 4 modes, 4 blocks per round");
  __device__ static int columns(const Tables& tb) { return 9 * tb.NR * tb.NZ; }
  __device__ static const float* image(const Tables& tb) { return tb.dft_inv; }

  // Warp w fills lines 8w..8w+7; lane = line (lane % 8) x mode quarter (lane / 8); a
  // thread takes the blocks of 4 consecutive modes q, q+4, ... (q = its quarter), so
  // that each block is one 16-byte row of a core matrix (vector stores; a warp's
  // stores of one block cover 4 core matrices, conflict-free).  Every load of a
  // thread is independent of the others (one line, J modes, up to 7 levels).
  struct Regs { float vx[J], vy[J]; };  // one thread's share of a tile (line col, J modes)
  __device__ static int mode_of(int mq, int j) { return 4 * (mq + 4 * (j / 4)) + (j % 4); }

  // Global -> registers; the loop issues this for the next tile before draining the
  // previous one, so the loads are in flight during the epilogue.
  __device__ static void load(const Tables& tb, const Bufs& bf, const Ctl* ctl, int mloc, int t, const double2* src,
                              const float2* src32, Regs& rg) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int col = warp * 8 + (lane & 7), mq = lane >> 3;
    const int NR = tb.NR, NZ = tb.NZ, NTNZ = tb.NTNZ;
    const long long S = tb.S;
    const int g = t * TM + col;
    float* vx = rg.vx;
    float* vy = rg.vy;
#pragma unroll
    for (int j = 0; j < J; j++) { vx[j] = 0.f; vy[j] = 0.f; }
    if (g < columns(tb)) {
      const StateIn<float> U = member_input<float>(tb, bf, ctl, mloc, src, src32);
      const float2* DR = member_dr32(tb, bf, ctl, mloc, src);  // d_r mirror of the member state, if any
      const int i = g / (9 * NZ), rem = g - i * 9 * NZ, f = rem / NZ, l = rem - f * NZ;
      const int comp = f < 3 ? f : (f < 6 ? f - 3 : f - 6);
      const size_t base = (size_t)comp * S + l;
      // the largest index this line reads: level min(i + IW, NR - 1), mode NT - 1
      if (!NSP_IN_BOUNDS(tb, (size_t)min(i + IW, NR - 1) * NTNZ + base + (size_t)(NT - 1) * NZ, 3 * S, BC_THETA_IN))
        return;
      if (f >= 3 && f < 6 && DR) {  // d_r u from the mirror the linear pass wrote
#pragma unroll
        for (int j = 0; j < J; j++) {
          const float2 a = __ldg(DR + (size_t)i * NTNZ + base + (size_t)mode_of(mq, j) * NZ);
          vx[j] = a.x; vy[j] = a.y;
        }
      } else if (f < 3) {
#pragma unroll
        for (int j = 0; j < J; j++) {
          cpx<float> a = U.ld((size_t)i * NTNZ + base + (size_t)mode_of(mq, j) * NZ);
          vx[j] = a.x; vy[j] = a.y;
        }
      } else if (f < 6) {  // derivr_k (mod_radialFD.cu:10-30); |m| mod 2 = it mod 2 = j mod 2 here
        const int left = max(0, i - IW), right = min(i + IW, NR - 1), len = right + 1 - left, i0 = i + IW - right;
        const int odd = comp < 2 ? 1 : 0;  // u_r, u_theta take the odd table for even |m|
        const float* Dr0 = tb.D32 + abs(0 - odd) * STEN * NR + STEN * i + i0;  // even |m|
        const float* Dr1 = tb.D32 + abs(1 - odd) * STEN * NR + STEN * i + i0;  // odd |m|
#pragma unroll
        for (int r = 0; r < STEN; r++) {
          if (r < len) {
            const float de0 = __ldg(Dr0 + r), de1 = __ldg(Dr1 + r);
            const size_t row = (size_t)(left + r) * NTNZ + base;
#pragma unroll
            for (int j = 0; j < J; j++) {
              const float de = (j & 1) ? de1 : de0;
              cpx<float> a = U.ld(row + (size_t)mode_of(mq, j) * NZ);
              vx[j] += de * a.x;
              vy[j] += de * a.y;
            }
          }
        }
      } else {  // derivt_k (mod_deriv.cu:10-21) divided by r
        const float ktsf = tb.kts32, ri = tb.rinv32[i];
#pragma unroll
        for (int j = 0; j < J; j++) {
          const int it = mode_of(mq, j), m = it < NT / 2 ? it : it - NT;
          const float kt = (float)m * ktsf;
          cpx<float> a = U.ld((size_t)i * NTNZ + base + (size_t)it * NZ);
          vx[j] = -kt * a.y * ri;
          vy[j] = kt * a.x * ri;
        }
      }
      if (l == 0 && mq == 0) {  // mode (0,0) = mode_of(0, 0): the mean flow
        // recorded for the linear pass, which adds its terms (member steps; an explicit
        // field's terms are added by the forward transform) ...
        const int slot = f == 0 ? MEAN_V : f == 1 ? MEAN_W : f == 2 ? MEAN_U : f == 4 ? MEAN_WP : f == 5 ? MEAN_UP : -1;
        if (!src && slot >= 0) bf.MEAN[((size_t)mloc * NR + i) * MEAN_N + slot] = vx[0];
        if (mean_field(f)) {  // ... and kept out of the transforms
          vx[0] = 0.f;
          vy[0] = 0.f;
        }
      }
    }
  }

  // Registers -> the tile's operand stage (TF32 hi/lo split, core-matrix layout).
  __device__ static void store(const Regs& rg, unsigned char* ah, unsigned char* al) {
    constexpr uint32_t SBO = (K / 4) * 128;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int col = warp * 8 + (lane & 7), mq = lane >> 3;
#pragma unroll
    for (int j = 0; j < J; j += 4) {
      const int it = mode_of(mq, j);  // first of 4 consecutive modes
      put_split4(ah, al, tc::koff(col, it, SBO), rg.vx + j);
      put_split4(ah, al, tc::koff(col, NT + it, SBO), rg.vy + j);
    }
  }

  // A draining warp reads TMEM lanes 32 q.. (its lines) and columns [c0, c0 + nc).
  __device__ static void epilogue(const Tables& tb, const Bufs& bf, const Ctl*, int mloc, int t, const double2*,
                                  const float2*, double2*, uint32_t tacc) {
    int q, c0, nc;
    if (!drain_share<N>(threadIdx.x >> 5, &q, &c0, &nc)) return;
    constexpr int CM = drain_max<N>();
    const int col = q * 32 + (threadIdx.x & 31);
    float v[CM];
#pragma unroll
    for (int c8 = 0; c8 < CM; c8 += 8)
      if (c8 < nc) tc::tmem_ld8(tacc + ((uint32_t)(q * 32) << 16) + (uint32_t)(c0 + c8), v + c8);
    tc::tmem_wait_ld();
    const int NR = tb.NR, NZ = tb.NZ, g = t * TM + col;
    if (g >= columns(tb)) return;
    const int i = g / (9 * NZ), rem = g - i * 9 * NZ, f = rem / NZ, l = rem - f * NZ;
    cpx<float>* G = reinterpret_cast<cpx<float>*>(bf.G) + (size_t)mloc * 9 * NR * NTP * NZ;
    cpx<float>* Gl = G + (((size_t)f * NR + i) * NTP + (size_t)(c0 / 2)) * NZ + l;
    if (!NSP_IN_BOUNDS(tb, (((size_t)f * NR + i) * NTP + (size_t)((c0 + nc) / 2 - 1)) * NZ + l,
                       (size_t)9 * NR * NTP * NZ, BC_THETA_OUT))
      return;
#pragma unroll
    for (int j = 0; j < CM / 2; j++)
      if (2 * j < nc) Gl[(size_t)j * NZ] = mk<float>(v[2 * j], v[2 * j + 1]);
  }
};

// Forward: line (component c, level i, l) of the z stage's output H; K index p (Re) /
// NTP + p (Im) over the NTP physical points; outputs the NT retained theta modes.
template <int NT, int NTP> struct FwdJob {
  static constexpr int K = 2 * NTP, N = 2 * NT, STAGES = 1;
  static constexpr int J = NTP / 4;
  static_assert(NTP % 16 == 0, "the fill takes blocks of 4 points, 4 blocks per round");
  __device__ static int columns(const Tables& tb) { return 3 * tb.NR * tb.NZ; }
  __device__ static const float* image(const Tables& tb) { return tb.dft_fwd; }

  struct Regs { cpx<float> h[J]; };
  // blocks of 4 consecutive points per thread, as the inverse's modes
  __device__ static int point_of(int pq, int j) { return 4 * (pq + 4 * (j / 4)) + (j % 4); }

  __device__ static void load(const Tables& tb, const Bufs& bf, const Ctl*, int mloc, int t, const double2*,
                              const float2*, Regs& rg) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int col = warp * 8 + (lane & 7), pq = lane >> 3;
    const int NR = tb.NR, NZ = tb.NZ, g = t * TM + col;
    cpx<float>* h = rg.h;
#pragma unroll
    for (int j = 0; j < J; j++) h[j] = mk<float>(0.f, 0.f);
    if (g < columns(tb)) {
      const int c = g / (NR * NZ), rem = g - c * NR * NZ, i = rem / NZ, l = rem - i * NZ;
      if (l < NZ - 1 && NSP_IN_BOUNDS(tb, (((size_t)c * NR + i) * NTP + NTP - 1) * NZ + l, (size_t)3 * NR * NTP * NZ,
                                      BC_THETA_IN)) {  // H holds the half spectrum l < NZ-1 (padBackward_k drops l = NZ-1)
        const cpx<float>* H = reinterpret_cast<const cpx<float>*>(bf.H) + (size_t)mloc * 3 * NR * NTP * NZ +
                              ((size_t)c * NR + i) * NTP * NZ + l;
#pragma unroll
        for (int j = 0; j < J; j++) h[j] = H[(size_t)point_of(pq, j) * NZ];
      }
    }
  }

  __device__ static void store(const Regs& rg, unsigned char* ah, unsigned char* al) {
    constexpr uint32_t SBO = (K / 4) * 128;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int col = warp * 8 + (lane & 7), pq = lane >> 3;
#pragma unroll
    for (int j = 0; j < J; j += 4) {
      const int p = point_of(pq, j);  // first of 4 consecutive points
      const float re[4] = {rg.h[j].x, rg.h[j + 1].x, rg.h[j + 2].x, rg.h[j + 3].x};
      const float im[4] = {rg.h[j].y, rg.h[j + 1].y, rg.h[j + 2].y, rg.h[j + 3].y};
      put_split4(ah, al, tc::koff(col, p, SBO), re);
      put_split4(ah, al, tc::koff(col, NTP + p, SBO), im);
    }
  }

  __device__ static void epilogue(const Tables& tb, const Bufs& bf, const Ctl* ctl, int mloc, int t,
                                  const double2* src, const float2* src32, double2* dst, uint32_t tacc) {
    int q, c0, nc;
    if (!drain_share<N>(threadIdx.x >> 5, &q, &c0, &nc)) return;
    constexpr int CM = drain_max<N>();
    const int col = q * 32 + (threadIdx.x & 31);
    float v[CM];
#pragma unroll
    for (int c8 = 0; c8 < CM; c8 += 8)
      if (c8 < nc) tc::tmem_ld8(tacc + ((uint32_t)(q * 32) << 16) + (uint32_t)(c0 + c8), v + c8);
    tc::tmem_wait_ld();
    const int NR = tb.NR, NZ = tb.NZ, NTNZ = tb.NTNZ, g = t * TM + col;
    const long long S = tb.S;
    if (g >= columns(tb)) return;
    const int c = g / (NR * NZ), rem = g - c * NR * NZ, i = rem / NZ, l = rem - i * NZ;
    // Wall derivative of u_z(0,0) for the mean forcing (pressGrad_k, mod_radialFD.cu:100-111).
    double dwall = 0.0;
    if (c == 2 && l == 0 && c0 == 0) {
      bool skip;
      const double2* U = member_source(tb, bf, ctl, mloc, src, skip);
      const double* Dw = tb.D + STEN * (NR - 1) + IW;
      for (int j = 0; j <= IW; j++) dwall += Dw[j] * U[2 * S + (size_t)(NR - 1 - IW + j) * NTNZ].x;
    }
    if (!NSP_IN_BOUNDS(tb, c * S + (size_t)i * NTNZ + l + (size_t)((c0 + nc) / 2 - 1) * NZ, 3 * S, BC_THETA_OUT))
      return;
    if (!dst) {
      // a member's N: FP32 (its values are FP32 numbers), the wall forcing of Re N_z(0,0)
      // kept apart in FP64 -- the same at every level, written by level 0
      float2* N32 = bf.N32 + (size_t)mloc * 3 * S + c * S + (size_t)i * NTNZ + l;
      if (c == 2 && l == 0 && c0 == 0 && i == 0) bf.NF[mloc] = -(tb.sscal[4 * member_set(tb, mloc) + 1] * dwall);
#pragma unroll
      for (int j = 0; j < CM / 2; j++) {
        if (2 * j >= nc) break;
        const int it = c0 / 2 + j;
        N32[(size_t)it * NZ] = (it == NT / 2 || l == NZ - 1) ? make_float2(0.f, 0.f) : make_float2(v[2 * j], v[2 * j + 1]);
      }
      return;
    }
    double2* Nout = dst + c * S + (size_t)i * NTNZ + l;
    // An explicit field's mean-flow terms (nsp_state.cuh), from its FP32 copy; a member
    // state's are added by the linear pass.
    const float2* U32 = src ? src32 : nullptr;
    Mean32 mf{};
    if (U32) mf = mean_flow32(tb, U32, nullptr, i);
    const float2* Uq = U32 + (c == 2 ? 2 : 1) * S + (size_t)i * NTNZ + l;  // u_theta (N_r, N_theta) or u_z (N_z)
    const float2* Ur = U32 + (size_t)i * NTNZ + l;
    const float kzl = tb.kzs32 * (float)l;
#pragma unroll
    for (int j = 0; j < CM / 2; j++) {
      if (2 * j >= nc) break;
      const int it = c0 / 2 + j;
      float2 w = make_float2(v[2 * j], v[2 * j + 1]);
      if (U32 && it != NT / 2 && l != NZ - 1) {
        const bool zm = it == 0 && l == 0;
        const float2 ur = Ur[(size_t)it * NZ], uq = zm ? make_float2(0.f, 0.f) : Uq[(size_t)it * NZ];
        const float kt = (float)(it < NT / 2 ? it : it - NT) * tb.kts32;
        const float2 ml = mean_terms32(mf, c, zm, kt, kzl, ur, c < 2 ? uq : make_float2(0.f, 0.f),
                                       c == 2 ? uq : make_float2(0.f, 0.f));
        w.x += ml.x;
        w.y += ml.y;
      }
      double2 o = make_double2(f32_to_f64(w.x), f32_to_f64(w.y));  // exact, integer pipe
      if (it == NT / 2 || l == NZ - 1) o = make_double2(0.0, 0.0);  // padBackward_k's dropped modes
      if (c == 2 && it == 0 && l == 0) o.x -= tb.sscal[4 * member_set(tb, mloc) + 1] * dwall;  // 2/Re
      Nout[(size_t)it * NZ] = o;
    }
  }
};

// ------------------------------------------------------------------ pipelined tile loop
// One persistent CTA per SM.  Iteration j fills tile j into stage j % STAGES, issues
// its MMAs into TMEM accumulator j % 2 (one thread), then drains tile j-1's
// accumulator to global memory while the tensor cores work on tile j.  With one
// stage the fill of tile j first waits for tile j-1's MMAs (its operand buffer).
template <class JOB>
__global__ void __launch_bounds__(TC_THREADS, 1)
    theta_tc_k(Tables tb, Bufs bf, Ctl* ctl, const double2* src, const float2* src32, double2* dst) {
  constexpr int K = JOB::K, N = JOB::N, ST = JOB::STAGES;
  constexpr uint32_t A_BYTES = TM * K * 4, B_BYTES = N * K * 4;
  constexpr int ACC = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;  // TMEM columns per accumulator
  static_assert(TC_THREADS == 512 && K % 8 == 0 && N % 32 == 0 && N <= 256 && 2 * ACC <= 512, "tile shape");
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char* sB = smraw + ST * 2 * A_BYTES;  // [hi | lo] DFT image
  __shared__ __align__(8) uint64_t bar_b, bar_mma[ST];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fault;
  const int tid = threadIdx.x, warp = tid >> 5;

  if (warp == 0) tc::tmem_alloc(&tmem_slot, 2 * ACC);
  if (tid == 0) {
    s_fault = 0;
    tc::mbar_init(&bar_b, 1);
    for (int s = 0; s < ST; s++) tc::mbar_init(&bar_mma[s], 1);
    tc::mbar_fence_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  // Test hook: with bit 0 of ctl->inject the image copy is not issued, so nothing ever
  // arrives on bar_b and the (shortened) bounded wait below runs out -- the fault path.
  const bool inject = (ctl->inject & 1) != 0;
  const int limit = inject ? 4096 : WAIT_LIMIT;
  if (tid == 0 && !inject) {
    tc::mbar_arrive_expect_tx(&bar_b, 2 * B_BYTES);
    tc::bulk_g2s(sB, JOB::image(tb), 2 * B_BYTES, &bar_b);
  }
  const bool img_ok = __syncthreads_and(tc::mbar_wait(&bar_b, 0, limit)) != 0;
  const uint32_t tmem = tmem_slot;
  const int T = (JOB::columns(tb) + TM - 1) / TM;
  const int total = (src ? 1 : tb.nmem) * T;
  int issued = 0, drained = 0;  // MMA batches committed / seen complete
  int prev_m = 0, prev_t = 0;
  bool fault = !img_ok;

  // Wait (block-uniformly) until batch b has completed.
  auto wait_batch = [&](int b) -> bool {
    return __syncthreads_and(tc::mbar_wait(&bar_mma[b % ST], (uint32_t)((b / ST) & 1), limit)) != 0;
  };
  // This CTA's next tile at or after `from` whose member is active (uniform per CTA).
  auto next_tile = [&](int from) -> int {
    for (int tt = from; tt < total; tt += gridDim.x) {
      bool skip;
      member_source(tb, bf, ctl, tt / T, src, skip);
      if (!skip) return tt;
    }
    return total;
  };
  typename JOB::Regs rg;
  int tile = next_tile(blockIdx.x);
  if (tile < total) JOB::load(tb, bf, ctl, tile / T, tile % T, src, src32, rg);
  while (tile < total && !fault) {
    const int mloc = tile / T, t = tile - mloc * T;
    const int j = issued;
    if (ST == 1 && drained < j) {  // the single operand stage is busy until batch j-1 completes
      if (!wait_batch(j - 1)) { fault = true; break; }
      drained = j;
      tc::fence_after_sync();
    }
    unsigned char* ah = smraw + (j % ST) * 2 * A_BYTES;
    JOB::store(rg, ah, ah + A_BYTES);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) issue_3xtf32<K, N>(tmem + (uint32_t)((j & 1) * ACC), ah, ah + A_BYTES, sB, sB + B_BYTES, &bar_mma[j % ST]);
    issued = j + 1;
    // Next tile's loads now, so that they are in flight while the previous tile drains.
    const int nxt = next_tile(tile + gridDim.x);
    if (nxt < total) JOB::load(tb, bf, ctl, nxt / T, nxt % T, src, src32, rg);
    if (j > 0) {  // warps 1-15 drain the previous tile while warp 0 issues this one's MMAs
      bool ok = true;
      if (drained < j) {
        if (warp != 0) ok = tc::mbar_wait(&bar_mma[(j - 1) % ST], (uint32_t)(((j - 1) / ST) & 1), limit);
        if (!ok) s_fault = 1;  // made block-uniform after the barrier below
        drained = j;
      }
      tc::fence_after_sync();
      if (ok) JOB::epilogue(tb, bf, ctl, prev_m, prev_t, src, src32, dst, tmem + (uint32_t)(((j - 1) & 1) * ACC));
    }
    tc::fence_before_sync();
    __syncthreads();
    if (s_fault) {
      fault = true;
      break;
    }
    prev_m = mloc;
    prev_t = t;
    tile = nxt;
  }
  if (!fault && issued > 0) {
    if (wait_batch(issued - 1)) {
      drained = issued;
      tc::fence_after_sync();
      JOB::epilogue(tb, bf, ctl, prev_m, prev_t, src, src32, dst, tmem + (uint32_t)(((issued - 1) & 1) * ACC));
    } else {
      fault = true;
    }
  }
  // Teardown: an abandoned copy or MMA batch is given (bounded) time to land before
  // the CTA frees its TMEM and exits.
  if (!img_ok && !inject) tc::mbar_wait(&bar_b, 0, limit);
  if (drained < issued) tc::mbar_wait(&bar_mma[(issued - 1) % ST], (uint32_t)(((issued - 1) / ST) & 1), limit);
  if (fault && tid == 0) atomicOr(&ctl->fault, 1);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 2 * ACC);
  }
}

template <class JOB> constexpr size_t tc_smem() {
  return (size_t)JOB::STAGES * 2 * TM * JOB::K * 4 + 2 * (size_t)JOB::N * JOB::K * 4;
}

// ------------------------------------------------------------------ host side
#define NSP_TC_LIST(X) X(32, 48)

bool theta_tc_supported(int NT, int NTP) {
#define NSP_TC_HAS(a, b) if (NT == a && NTP == b) return true;
  NSP_TC_LIST(NSP_TC_HAS)
#undef NSP_TC_HAS
  return false;
}

// B-operand image of the DFT matrix: [hi | lo] x N rows x K, K-major core matrices.
std::vector<float> theta_dft_image(int NT, int NTP, bool inverse, double scale) {
  const int K = inverse ? 2 * NT : 2 * NTP, N = inverse ? 2 * NTP : 2 * NT;
  const uint32_t sbo = (uint32_t)(K / 4) * 128;
  std::vector<float> img(2 * (size_t)N * K, 0.0f);
  const long double two_pi = 6.283185307179586476925286766559L;
  for (int n = 0; n < N; n++)
    for (int k = 0; k < K; k++) {
      const int reim = n % 2;
      int it, p, part;
      if (inverse) { p = n / 2; it = k % NT; part = k / NT; }
      else { it = n / 2; p = k % NTP; part = k / NTP; }
      const int m = it < NT / 2 ? it : it - NT;
      const long e = (((long)m * p) % NTP + NTP) % NTP;  // exact angle index
      const long double ang = two_pi * (long double)e / (long double)NTP;
      const long double cs = cosl(ang), sn = sinl(ang);
      long double val;
      if (inverse) val = reim == 0 ? (part == 0 ? cs : -sn) : (part == 0 ? sn : cs);
      else val = (reim == 0 ? (part == 0 ? cs : sn) : (part == 0 ? -sn : cs)) * (long double)scale;
      // hi: val rounded to TF32; lo: the remainder rounded to TF32.
      float x = (float)val;
      uint32_t u;
      std::memcpy(&u, &x, 4);
      u = (u + 0x1000u) & 0xFFFFE000u;
      float hi;
      std::memcpy(&hi, &u, 4);
      float r = (float)(val - (long double)hi);
      std::memcpy(&u, &r, 4);
      u = (u + 0x1000u) & 0xFFFFE000u;
      float lo;
      std::memcpy(&lo, &u, 4);
      const size_t off = tc::koff(n, k, sbo) / 4;
      img[off] = hi;
      img[(size_t)N * K + off] = lo;
    }
  return img;
}

void configure_theta_tc_kernels() {
#define NSP_TC_CFG(a, b)                                                                            \
  cudaFuncSetAttribute(theta_tc_k<InvJob<a, b>>, cudaFuncAttributeMaxDynamicSharedMemorySize,       \
                       (int)tc_smem<InvJob<a, b>>());                                               \
  cudaFuncSetAttribute(theta_tc_k<FwdJob<a, b>>, cudaFuncAttributeMaxDynamicSharedMemorySize,       \
                       (int)tc_smem<FwdJob<a, b>>());
  NSP_TC_LIST(NSP_TC_CFG)
#undef NSP_TC_CFG
}

// Launch the inverse (dir 0) or forward (dir 1) tile GEMM over the group's members
// (or one explicit field); one persistent CTA per SM.
void launch_theta_tc(const Tables& tb, const Bufs& bf, Ctl* dctl, int dir, const double2* src, const float2* src32,
                     double2* dst, cudaStream_t st) {
  const int nm = src ? 1 : tb.nmem;
  const int C = (dir == 0 ? 9 : 3) * tb.NR * tb.NZ, T = (C + TM - 1) / TM;
  const int grid = std::max(1, std::min(nm * T, tb.nsm));
#define NSP_TC_LAUNCH(a, b)                                                                                    \
  if (tb.NT == a && tb.NTP == b) {                                                                             \
    if (dir == 0)                                                                                              \
      theta_tc_k<InvJob<a, b>><<<grid, TC_THREADS, tc_smem<InvJob<a, b>>(), st>>>(tb, bf, dctl, src, src32, dst); \
    else                                                                                                       \
      theta_tc_k<FwdJob<a, b>><<<grid, TC_THREADS, tc_smem<FwdJob<a, b>>(), st>>>(tb, bf, dctl, src, src32, dst); \
    return;                                                                                                    \
  }
  NSP_TC_LIST(NSP_TC_LAUNCH)
#undef NSP_TC_LAUNCH
}

}  // namespace nsp
