// nsp_transform.cu -- the 3/2-dealiased nonlinear term, one radial level at a time.
//
// Replaces nonlinear() (mod_io_nonlinear.cu:380-409): derivr x3, padForward x12,
// derivt/derivz x6, 12 batched 2-D Z2D and 3 D2Z cuFFT transforms
// (mod_fft.cu:37-48), calcNonlinear_k (:142-170), normalize (mod_utils.cu:10-17),
// padBackward x3 (:195-214) and pressGrad (mod_radialFD.cu:100-111).  Three
// kernels per evaluation:
//
//   nl_theta_inv  per (member, level, 16 (field, l) columns): builds the padded
//                 theta columns of u, d_r u (7-point stencil over levels, parity
//                 tables) and i m u / r straight from the spectral state and runs
//                 the length-NTP inverse FFTs -> G[f][level][theta_j][l] (9 fields);
//   nl_z          per (member, level, theta rows): forms the 12 Hermitian z
//                 spectra (d_z u = i k_z times the u columns of G), packs them
//                 two real fields per complex length-NZR inverse FFT, evaluates
//                 -(u.grad)u pointwise, packs the 3 products into complex forward
//                 FFTs and unpacks the half spectra l < NZ-1 -> H;
//   nl_theta_fwd  per (member, level, 16 (component, l) columns): length-NTP
//                 forward FFTs of H, scale by 1/(NTP*NZR), keep the retained modes
//                 (theta Nyquist and l = NZ-1 zeroed) and apply the wall-shear
//                 forcing to N_z(0,0).
//
// T = double gives the plain FP64 form; T = float the mixed form (the state is
// rounded to FP32 on load, the stencils and products run in FP32, N is written
// back in FP64).  Transform lengths used by the supported configurations are
// compile-time template arguments (all index arithmetic by constants); other
// 2^a 3^b lengths use the run-time FFT.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "nsp_bounds.cuh"
#include "nsp_cvt.cuh"
#include "nsp_fft.cuh"
#include "nsp_internal.h"
#include "nsp_state.cuh"

namespace nsp {

constexpr int MAXR = 4;   // register rounds of the run-time FFT
constexpr int LC = 16;    // theta columns per block
constexpr int TTH = 256;  // threads of the theta kernels
constexpr int ZTH = 256;  // threads of the z kernel
constexpr int Z2TH = 192; // threads of the two-pass z kernel (its passes run 192, 144, 384, 48, 36, 384 tasks)

template <typename T> __device__ __forceinline__ const typename vec2<T>::type* tw_t(const Tables& tb);
template <> __device__ __forceinline__ const double2* tw_t<double>(const Tables& tb) { return tb.tw_t; }
template <> __device__ __forceinline__ const float2* tw_t<float>(const Tables& tb) { return tb.tw_t32; }
template <typename T> __device__ __forceinline__ const typename vec2<T>::type* tw_z(const Tables& tb);
template <> __device__ __forceinline__ const double2* tw_z<double>(const Tables& tb) { return tb.tw_z; }
template <> __device__ __forceinline__ const float2* tw_z<float>(const Tables& tb) { return tb.tw_z32; }

template <typename T, int NTPC>
__device__ __forceinline__ void theta_fft(cpx<T>* buf, const Tables& tb, int sign) {
  if constexpr (NTPC > 0) {
    if (sign > 0) fft_ct<T, +1, NTPC, LC, LC, 1, true, TTH>(buf, tw_t<T>(tb));
    else fft_ct<T, -1, NTPC, LC, LC, 1, true, TTH>(buf, tw_t<T>(tb));
  } else {
    if (sign > 0) fft_batch<T, +1, MAXR, true>(buf, tb.pt, LC, LC, 1, tw_t<T>(tb));
    else fft_batch<T, -1, MAXR, true>(buf, tb.pt, LC, LC, 1, tw_t<T>(tb));
  }
}

// ---------------------------------------------------------------- theta inverse
template <typename T, int NTPC>
__global__ void __launch_bounds__(TTH) nl_theta_inv(Tables tb, Bufs bf, const Ctl* ctl, const double2* src_override,
                                                    const float2* src32_override) {
  const int mloc = blockIdx.z, i = blockIdx.y, c0 = blockIdx.x * LC;
  bool skip;
  member_source(tb, bf, ctl, mloc, src_override, skip);
  if (skip) return;
  const StateIn<T> U = member_input<T>(tb, bf, ctl, mloc, src_override, src32_override);
  extern __shared__ __align__(16) unsigned char smraw[];
  cpx<T>* buf = reinterpret_cast<cpx<T>*>(smraw);
  __shared__ int colf[LC], coll[LC];
  const int NR = tb.NR, NT = tb.NT, NZ = tb.NZ, NTNZ = tb.NTNZ;
  const int NTP = NTPC > 0 ? NTPC : tb.NTP;
  const long long S = tb.S;
  if (threadIdx.x < LC) {
    int c = c0 + threadIdx.x;
    colf[threadIdx.x] = c < 9 * NZ ? c / NZ : -1;
    coll[threadIdx.x] = c % NZ;
  }
  __syncthreads();
  const int left = max(0, i - IW), right = min(i + IW, NR - 1);
  const int len = right + 1 - left, i0 = i + IW - right;
  const T rinv = tb_rinv<T>(tb, i);
  const T ktsT = tb_kts<T>(tb);
  for (int idx = threadIdx.x; idx < NTP * LC; idx += TTH) {
    int p = idx / LC, lc = idx % LC;
    int f = colf[lc];
    int it = (p < NT / 2) ? p : (p >= NT ? p - NT / 2 : -1);
    cpx<T> v = mk<T>(0, 0);
    if (f >= 0 && it >= 0 &&
        NSP_IN_BOUNDS(tb, (size_t)right * NTNZ + (size_t)(f % 3) * S + (size_t)it * NZ + coll[lc], 3 * S, BC_THETA_IN)) {
      int comp = f % 3;
      size_t col = (size_t)comp * S + (size_t)it * NZ + coll[lc];
      if (f < 3) {
        v = U.ld((size_t)i * NTNZ + col);
      } else if (f < 6) {  // derivr_k, mod_radialFD.cu:10-30 (flag 1 for u_r, u_theta; 0 for u_z)
        int m = it < NT / 2 ? it : it - NT;
        int tab = abs((abs(m) % 2) - (comp < 2 ? 1 : 0));
        const T* Dr = dtab<T>(tb) + tab * STEN * NR + STEN * i + i0;
        T sx = 0, sy = 0;
        for (int j = 0; j < len; j++) {
          T de = __ldg(Dr + j);
          cpx<T> a = U.ld((size_t)(left + j) * NTNZ + col);
          sx += de * a.x;
          sy += de * a.y;
        }
        v = mk<T>(sx, sy);
      } else {  // derivt_k, mod_deriv.cu:10-21
        int m = it < NT / 2 ? it : it - NT;
        T kt = (sizeof(T) == 8) ? (T)(tb.kts * (double)m) : (T)m * ktsT;
        cpx<T> a = U.ld((size_t)i * NTNZ + col);
        v = mk<T>(-kt * a.y * rinv, kt * a.x * rinv);
      }
      // mixed form: the mean flow is recorded for the linear pass (member steps) and kept
      // out of the transforms; its terms are added by the linear pass, or for an explicit
      // field by nl_theta_fwd
      if (sizeof(T) == 4 && it == 0 && coll[lc] == 0) {
        const int slot = f == 0 ? MEAN_V : f == 1 ? MEAN_W : f == 2 ? MEAN_U : f == 4 ? MEAN_WP : f == 5 ? MEAN_UP : -1;
        if (!src_override && slot >= 0) bf.MEAN[((size_t)mloc * NR + i) * MEAN_N + slot] = (float)v.x;
        if (mean_field(f)) v = mk<T>(0, 0);
      }
    }
    buf[idx] = v;
  }
  __syncthreads();
  theta_fft<T, NTPC>(buf, tb, +1);
  cpx<T>* G = reinterpret_cast<cpx<T>*>(bf.G) + (size_t)mloc * 9 * NR * NTP * NZ;
  for (int idx = threadIdx.x; idx < NTP * LC; idx += TTH) {
    int p = idx / LC, lc = idx % LC;
    int f = colf[lc];
    if (f >= 0 && NSP_IN_BOUNDS(tb, (((size_t)f * NR + i) * NTP + p) * NZ + coll[lc], (size_t)9 * NR * NTP * NZ,
                                BC_THETA_OUT))
      G[(((size_t)f * NR + i) * NTP + p) * NZ + coll[lc]] = buf[idx];
  }
}

// ---------------------------------------------------------------- z stage
// Field order of the 12 physical arrays: u_r,u_t,u_z, dr u_r,dr u_t,dr u_z,
// dt u_r,dt u_t,dt u_z, dz u_r,dz u_t,dz u_z.  Pair t holds fields (2t, 2t+1).
template <typename T, int NZRC, int RPB>
__global__ void __launch_bounds__(ZTH) nl_z(Tables tb, Bufs bf, const Ctl* ctl, int standalone) {
  const int mloc = blockIdx.z, i = blockIdx.y, j0 = blockIdx.x * RPB;
  if (!standalone && ctl->phase[tb.mem0 + mloc] < 0) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  cpx<T>* Z = reinterpret_cast<cpx<T>*>(smraw);  // [RPB*6][NZR]
  const int NR = tb.NR, NZ = tb.NZ, NTP = tb.NTP;
  const int NZR = NZRC > 0 ? NZRC : tb.NZR;
  const cpx<T>* G = reinterpret_cast<const cpx<T>*>(bf.G) + (size_t)mloc * 9 * NR * NTP * NZ;
  cpx<T>* H = reinterpret_cast<cpx<T>*>(bf.H) + (size_t)mloc * 3 * NR * NTP * NZ;
  const T kzs = tb_kzs<T>(tb);
  // Hermitian-extended spectra, two real fields per complex transform.
  for (int idx = threadIdx.x; idx < RPB * 6 * NZR; idx += ZTH) {
    int q = idx % NZR, t = (idx / NZR) % 6, rr = idx / (6 * NZR);
    int j = j0 + rr;
    cpx<T> z = mk<T>(0, 0);
    int qq = -1;
    bool cj = false;
    if (q < NZ) qq = q;
    else if (q > NZR - NZ) { qq = NZR - q; cj = true; }
    if (j < NTP && qq >= 0) {
      cpx<T> ab[2];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        int fld = 2 * t + h;
        int src = fld < 9 ? fld : fld - 9;  // dz u_c comes from the u_c columns
        const size_t gi = (((size_t)src * NR + i) * NTP + j) * NZ + qq;
        cpx<T> g = NSP_IN_BOUNDS(tb, gi, (size_t)9 * NR * NTP * NZ, BC_Z_IN) ? G[gi] : mk<T>(0, 0);
        if (fld >= 9) {
          T kz = kzs * (T)qq;
          g = mk<T>(-kz * g.y, kz * g.x);
        }
        if (qq == 0) g.y = (T)0;  // C2R ignores Im of the k_z = 0 coefficient
        if (cj) g.y = -g.y;
        ab[h] = g;
      }
      z = mk<T>(ab[0].x - ab[1].y, ab[0].y + ab[1].x);
    }
    Z[(size_t)(rr * 6 + t) * NZR + q] = z;
  }
  __syncthreads();
  if constexpr (NZRC > 0) fft_ct<T, +1, NZRC, RPB * 6, 1, NZRC, false, ZTH>(Z, tw_z<T>(tb));
  else fft_batch<T, +1, MAXR, false>(Z, tb.pz, RPB * 6, 1, NZR, tw_z<T>(tb));
  // -(u.grad)u (calcNonlinear_k), packed for the forward transforms:
  // RPB 2: slot0 = (Nr0, Nt0), slot1 = (Nr1, Nt1), slot2 = (Nz0, Nz1); RPB 1: slot0 = (Nr, Nt), slot1 = (Nz, 0).
  const T rinv = tb_rinv<T>(tb, i);
  for (int n = threadIdx.x; n < NZR; n += ZTH) {
    T nr[RPB], nt[RPB], nz[RPB];
#pragma unroll
    for (int rr = 0; rr < RPB; rr++) {
      const cpx<T>* Zr = Z + (size_t)rr * 6 * NZR + n;
      cpx<T> a0 = Zr[0], a1 = Zr[NZR], a2 = Zr[2 * NZR], a3 = Zr[3 * NZR], a4 = Zr[4 * NZR], a5 = Zr[5 * NZR];
      T ur = a0.x, ut = a0.y, uz = a1.x;
      T drr = a1.y, drt = a2.x, drz = a2.y, dtr = a3.x, dtt = a3.y, dtz = a4.x, dzr = a4.y, dzt = a5.x, dzz = a5.y;
      T utr = ut * rinv;
      nr[rr] = -(ur * drr + ut * dtr + uz * dzr - ut * utr);
      nt[rr] = -(ur * drt + ut * dtt + uz * dzt + ur * utr);
      nz[rr] = -(ur * drz + ut * dtz + uz * dzz);
    }
    if (RPB == 2) {
      Z[n] = mk<T>(nr[0], nt[0]);
      Z[NZR + n] = mk<T>(nr[RPB - 1], nt[RPB - 1]);
      Z[2 * NZR + n] = mk<T>(nz[0], nz[RPB - 1]);
    } else {
      Z[n] = mk<T>(nr[0], nt[0]);
      Z[NZR + n] = mk<T>(nz[0], (T)0);
    }
  }
  __syncthreads();
  constexpr int NFWD = (RPB == 2) ? 3 : 2;
  if constexpr (NZRC > 0) fft_ct<T, -1, NZRC, NFWD, 1, NZRC, false, ZTH>(Z, tw_z<T>(tb));
  else fft_batch<T, -1, MAXR, false>(Z, tb.pz, NFWD, 1, NZR, tw_z<T>(tb));
  // Unpack: x = a + i b  ->  A_q = (X_q + conj X_{-q})/2,  B_q = (X_q - conj X_{-q})/(2i).
  const int NQ = NZ - 1;
  for (int idx = threadIdx.x; idx < RPB * 3 * NQ; idx += ZTH) {
    int q = idx % NQ, c = (idx / NQ) % 3, rr = idx / (3 * NQ);
    int j = j0 + rr;
    if (j >= NTP) continue;
    int slot;
    bool takeB;
    if (c < 2) { slot = rr; takeB = (c == 1); }
    else { slot = (RPB == 2) ? 2 : 1; takeB = (RPB == 2) && rr == 1; }
    const cpx<T>* X = Z + (size_t)slot * NZR;
    cpx<T> xq = X[q], xm = X[(NZR - q) % NZR];
    cpx<T> v = takeB ? mk<T>((T)0.5 * (xq.y + xm.y), (T)-0.5 * (xq.x - xm.x))
                     : mk<T>((T)0.5 * (xq.x + xm.x), (T)0.5 * (xq.y - xm.y));
    if (NSP_IN_BOUNDS(tb, (((size_t)c * NR + i) * NTP + j) * NZ + q, (size_t)3 * NR * NTP * NZ, BC_Z_OUT))
      H[(((size_t)c * NR + i) * NTP + j) * NZ + q] = v;
  }
}

// ---------------------------------------------------------------- z stage, two-pass
// The same z stage with each length-NZR transform split as NZR = N1 x N2 ("four-step"):
//   X[N2 k1 + k2] = sum_n1 w_N1^(n1 k1) [ w_NZR^(n1 k2) sum_n2 x[n1 + N1 n2] w_N2^(n2 k2) ],
// pass A: one thread per (transform, n1) runs the N2-point DFT in registers and
// applies the twiddle; pass B: one thread per (transform, k2) runs the N1-point DFT.
// Between the passes a padded [k2][n1] transpose buffer keeps shared memory free of
// bank conflicts; pass A of the inverse gathers the Hermitian spectra straight from
// G.  Two shared-memory round trips per transform instead of one per radix stage.

// exp(-2 pi i e / 96): every register sub-transform length used (4 .. 32) divides 96.
__constant__ float2 c_w96f[96];
__constant__ double2 c_w96d[96];
template <typename T> __device__ __forceinline__ cpx<T> w96(int e);
template <> __device__ __forceinline__ cpx<float> w96<float>(int e) { float2 w = c_w96f[e]; return mk<float>(w.x, w.y); }
template <> __device__ __forceinline__ cpx<double> w96<double>(int e) { double2 w = c_w96d[e]; return mk<double>(w.x, w.y); }

// In-register Stockham FFT of length N | 96 (every index a compile-time constant
// once unrolled, so the array stays in registers); natural order in and out.
template <typename T, int SIGN, int N, int S = 0, int NS = 1>
__device__ __forceinline__ void reg_fft(cpx<T>* v) {
  if constexpr (S < ct_nstages(N)) {
    constexpr int P = ct_radix(N, S), NB = N / P;
    static_assert(96 % (NS * P) == 0, "sub-transform length must divide 96");
    cpx<T> o[N];
#pragma unroll
    for (int j = 0; j < NB; j++) {
      const int k = j % NS;
      cpx<T> x[P];
#pragma unroll
      for (int q = 0; q < P; q++) x[q] = v[j + q * NB];
      if (NS > 1 && k > 0) {
#pragma unroll
        for (int q = 1; q < P; q++) {
          const cpx<T> w = w96<T>((q * k * (96 / (NS * P))) % 96);
          x[q] = cmulv(x[q], mk<T>(w.x, SIGN > 0 ? -w.y : w.y));
        }
      }
      dft<T, SIGN, P>(x);
#pragma unroll
      for (int q = 0; q < P; q++) o[(j / NS) * NS * P + k + q * NS] = x[q];
    }
#pragma unroll
    for (int n = 0; n < N; n++) v[n] = o[n];
    reg_fft<T, SIGN, N, S + 1, NS * P>(v);
  }
}

// Spectrum value n (0 <= n < NZR) of a packed pair of fields, Hermitian-extended:
// Ga / Gb are the fields' columns (d_z fields read the u columns and multiply by i k_z).
// Branch-free: the load index is clamped and the value selected.
template <typename T, int NZ, int NZR>
__device__ __forceinline__ cpx<T> z_pair_spec(const cpx<T>* Ga, const cpx<T>* Gb, bool dza, bool dzb, int n, T kzs) {
  const bool direct = n < NZ, mirror = n > NZR - NZ;
  const int qq = direct ? n : (mirror ? NZR - n : 0);
  cpx<T> a = Ga[qq], b = Gb[qq];
  const T kz = kzs * (T)qq;
  if (dza) a = mk<T>(-kz * a.y, kz * a.x);
  if (dzb) b = mk<T>(-kz * b.y, kz * b.x);
  // C2R ignores Im of the k_z = 0 coefficient; the mirrored half is the conjugate.
  const T sy = (qq == 0) ? (T)0 : (mirror ? (T)-1 : (T)1);
  a.y *= sy;
  b.y *= sy;
  const cpx<T> z = mk<T>(a.x - b.y, a.y + b.x);
  return (direct || mirror) ? z : mk<T>(0, 0);
}

// The same for an index range known to be all direct (MIRROR false: q = n) or all
// mirrored (MIRROR true: q = NZR - n, conjugated); q = 0 only where ZERO_OK.
template <typename T, bool MIRROR, bool ZERO_OK>
__device__ __forceinline__ cpx<T> z_pair_spec_in(const cpx<T>* Ga, const cpx<T>* Gb, bool dza, bool dzb, int qq, T kzs) {
  cpx<T> a = Ga[qq], b = Gb[qq];
  const T kz = kzs * (T)qq;
  if (dza) a = mk<T>(-kz * a.y, kz * a.x);
  if (dzb) b = mk<T>(-kz * b.y, kz * b.x);
  if (MIRROR) { a.y = -a.y; b.y = -b.y; }
  if (ZERO_OK && qq == 0) { a.y = (T)0; b.y = (T)0; }
  return mk<T>(a.x - b.y, a.y + b.x);
}

// Pitch (complex values) of a physical row of the two-pass z stage: the smallest
// value >= NZR that is 12 mod 16, so that the rows written by one warp in pass B
// (12 lanes per transform, 8-byte values) fall on disjoint bank ranges.
constexpr int z2_pitch(int nzr) { return nzr + (28 - nzr % 16) % 16; }

template <typename T, int NZRC, int N1, int N2, int R>
__global__ void __launch_bounds__(Z2TH) nl_z2(Tables tb, Bufs bf, const Ctl* ctl, int standalone) {
  static_assert(N1 * N2 == NZRC && R % 2 == 0 && NZRC % 3 == 0, "z split");
  constexpr int NZ = NZRC / 3 + 1;    // NZR = 3 (NZ - 1) (3/2 rule)
  constexpr int NQ = NZ - 1;          // retained z modes of the output
  constexpr int YP = N1 + 1;          // padded transpose row
  constexpr int YT = N2 * YP;         // one transform in the transpose buffer
  constexpr int PS = z2_pitch(NZRC);  // padded physical row (complex pairs)
  constexpr int NF = R + R / 2;       // forward transforms: (N_r, N_t) per row, (N_z, N_z) per row pair
  const int mloc = blockIdx.z, i = blockIdx.y, j0 = blockIdx.x * R;  // NTP % R == 0 (host check)
  if (!standalone && ctl->phase[tb.mem0 + mloc] < 0) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  cpx<T>* Y = reinterpret_cast<cpx<T>*>(smraw);  // [R*6][N2][N1+1]
  cpx<T>* Ph = Y + R * 6 * YT;                   // [R][6][PS]: physical field pairs (2t, 2t+1), then products
  const int NR = tb.NR, NTP = tb.NTP;
  const cpx<T>* G = reinterpret_cast<const cpx<T>*>(bf.G) + (size_t)mloc * 9 * NR * NTP * NZ;
  cpx<T>* H = reinterpret_cast<cpx<T>*>(bf.H) + (size_t)mloc * 3 * NR * NTP * NZ;
  const T kzs = tb_kzs<T>(tb);
  const auto* twz = tw_z<T>(tb);  // exp(-2 pi i e / NZR)
  const size_t fstride = (size_t)NR * NTP * NZ;

  // 1. inverse, pass A (spectra gathered from G)
  for (int task = threadIdx.x; task < R * 6 * N1; task += Z2TH) {
    const int n1 = task % N1, t = (task / N1) % 6, r = task / (6 * N1);
    const cpx<T>* Gi = G + ((size_t)i * NTP + j0 + r) * NZ;
    const int fa = 2 * t, fb = 2 * t + 1;  // d_z u_c (fields 9-11) comes from the u_c columns
    const cpx<T>* Ga = Gi + (size_t)(fa < 9 ? fa : fa - 9) * fstride;
    const cpx<T>* Gb = Gi + (size_t)(fb < 9 ? fb : fb - 9) * fstride;
    if (!NSP_IN_BOUNDS(tb, ((size_t)i * NTP + j0 + r) * NZ + NZ - 1, fstride, BC_Z_IN)) continue;
    cpx<T> x[N2];
#pragma unroll
    for (int n2 = 0; n2 < N2; n2++) {
      // The 16-wide range of n = n1 + N1 n2 is classified at compile time; only a
      // range that straddles a boundary of the Hermitian extension takes the general path.
      const int lo = N1 * n2, hi = lo + N1 - 1;
      if (hi < NZ) x[n2] = z_pair_spec_in<T, false, true>(Ga, Gb, fa >= 9, fb >= 9, n1 + lo, kzs);
      else if (lo > NZRC - NZ) x[n2] = z_pair_spec_in<T, true, false>(Ga, Gb, fa >= 9, fb >= 9, NZRC - n1 - lo, kzs);
      else if (lo >= NZ && hi <= NZRC - NZ) x[n2] = mk<T>(0, 0);  // dealiasing band: no load
      else x[n2] = z_pair_spec<T, NZ, NZRC>(Ga, Gb, fa >= 9, fb >= 9, n1 + lo, kzs);
    }
    reg_fft<T, +1, N2>(x);
    cpx<T>* Yt = Y + (r * 6 + t) * YT + n1;
#pragma unroll
    for (int k2 = 0; k2 < N2; k2++) {
      cpx<T> v = x[k2];
      if (k2 > 0) {
        const auto w = __ldg(twz + n1 * k2);
        v = cmulv(v, mk<T>(w.x, -w.y));
      }
      Yt[k2 * YP] = v;
    }
  }
  __syncthreads();
  // 2. inverse, pass B -> physical point z = N2 k1 + k2 of the pair (2t, 2t+1)
  for (int task = threadIdx.x; task < R * 6 * N2; task += Z2TH) {
    const int k2 = task % N2, t = (task / N2) % 6, r = task / (6 * N2);
    cpx<T> y[N1];
    const cpx<T>* Yt = Y + (r * 6 + t) * YT + k2 * YP;
#pragma unroll
    for (int n1 = 0; n1 < N1; n1++) y[n1] = Yt[n1];
    reg_fft<T, +1, N1>(y);
    cpx<T>* pz = Ph + (r * 6 + t) * PS + k2;
#pragma unroll
    for (int k1 = 0; k1 < N1; k1++) pz[N2 * k1] = y[k1];
  }
  __syncthreads();
  // 3. -(u.grad)u (calcNonlinear_k, mod_io_nonlinear.cu:142-170).  Pairs: (u_r,u_t) (u_z,dr u_r)
  // (dr u_t,dr u_z) (dt u_r,dt u_t) (dt u_z,dz u_r) (dz u_t,dz u_z).  Written back as
  // pair 0 = (N_r, N_t), pair 1 .x = N_z.
  const T rinv = tb_rinv<T>(tb, i);
  for (int task = threadIdx.x; task < R * NZRC; task += Z2TH) {
    const int z = task % NZRC, r = task / NZRC;
    cpx<T>* p = Ph + r * 6 * PS + z;
    const cpx<T> a0 = p[0], a1 = p[PS], a2 = p[2 * PS], a3 = p[3 * PS], a4 = p[4 * PS], a5 = p[5 * PS];
    const T ur = a0.x, ut = a0.y, uz = a1.x;
    const T drr = a1.y, drt = a2.x, drz = a2.y, dtr = a3.x, dtt = a3.y, dtz = a4.x, dzr = a4.y, dzt = a5.x, dzz = a5.y;
    const T utr = ut * rinv;
    p[0] = mk<T>(-(ur * drr + ut * dtr + uz * dzr - ut * utr), -(ur * drt + ut * dtt + uz * dzt + ur * utr));
    p[PS].x = -(ur * drz + ut * dtz + uz * dzz);
  }
  __syncthreads();
  // 4. forward, pass A: transform t < R is (N_r, N_t) of row t; t >= R packs N_z of rows 2(t-R), 2(t-R)+1.
  for (int task = threadIdx.x; task < NF * N1; task += Z2TH) {
    const int n1 = task % N1, t = task / N1;
    cpx<T> x[N2];
    if (t < R) {
      const cpx<T>* pa = Ph + t * 6 * PS + n1;
#pragma unroll
      for (int n2 = 0; n2 < N2; n2++) x[n2] = pa[N1 * n2];
    } else {
      const cpx<T>* pa = Ph + (2 * (t - R) * 6 + 1) * PS + n1;
      const cpx<T>* pb = pa + 6 * PS;
#pragma unroll
      for (int n2 = 0; n2 < N2; n2++) x[n2] = mk<T>(pa[N1 * n2].x, pb[N1 * n2].x);
    }
    reg_fft<T, -1, N2>(x);
    cpx<T>* Yt = Y + t * YT + n1;
#pragma unroll
    for (int k2 = 0; k2 < N2; k2++) {
      cpx<T> v = x[k2];
      if (k2 > 0) {
        const auto w = __ldg(twz + n1 * k2);
        v = cmulv(v, mk<T>(w.x, w.y));
      }
      Yt[k2 * YP] = v;
    }
  }
  __syncthreads();
  // 5. forward, pass B -> spectrum X[N2 k1 + k2] (natural order, over the physical buffer)
  cpx<T>* Xs = Ph;
  for (int task = threadIdx.x; task < NF * N2; task += Z2TH) {
    const int k2 = task % N2, t = task / N2;
    cpx<T> y[N1];
    const cpx<T>* Yt = Y + t * YT + k2 * YP;
#pragma unroll
    for (int n1 = 0; n1 < N1; n1++) y[n1] = Yt[n1];
    reg_fft<T, -1, N1>(y);
#pragma unroll
    for (int k1 = 0; k1 < N1; k1++) Xs[t * PS + N2 * k1 + k2] = y[k1];
  }
  __syncthreads();
  // 6. unpack x = a + i b: A_q = (X_q + conj X_-q)/2, B_q = (X_q - conj X_-q)/(2i); keep q < NZ-1.
  for (int task = threadIdx.x; task < R * 3 * NQ; task += Z2TH) {
    const int q = task % NQ, c = (task / NQ) % 3, r = task / (3 * NQ), j = j0 + r;
    const int slot = c < 2 ? r : R + r / 2;
    const bool takeB = c < 2 ? (c == 1) : (r & 1);
    const cpx<T>* X = Xs + slot * PS;
    const cpx<T> xq = X[q], xm = X[(NZRC - q) % NZRC];
    const cpx<T> v = takeB ? mk<T>((T)0.5 * (xq.y + xm.y), (T)-0.5 * (xq.x - xm.x))
                           : mk<T>((T)0.5 * (xq.x + xm.x), (T)0.5 * (xq.y - xm.y));
    if (NSP_IN_BOUNDS(tb, (((size_t)c * NR + i) * NTP + j) * NZ + q, 3 * fstride, BC_Z_OUT))
      H[(((size_t)c * NR + i) * NTP + j) * NZ + q] = v;
  }
}

// ---------------------------------------------------------------- theta forward
template <typename T, int NTPC>
__global__ void __launch_bounds__(TTH) nl_theta_fwd(Tables tb, Bufs bf, const Ctl* ctl, const double2* src_override,
                                                    const float2* src32_override, double2* dst_override) {
  const int mloc = blockIdx.z, i = blockIdx.y, c0 = blockIdx.x * LC;
  bool skip;
  const double2* U = member_source(tb, bf, ctl, mloc, src_override, skip);
  if (skip) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  cpx<T>* buf = reinterpret_cast<cpx<T>*>(smraw);
  __shared__ int colc[LC], coll[LC];
  const int NR = tb.NR, NT = tb.NT, NZ = tb.NZ, NTNZ = tb.NTNZ;
  const int NTP = NTPC > 0 ? NTPC : tb.NTP;
  const long long S = tb.S;
  if (threadIdx.x < LC) {
    int c = c0 + threadIdx.x;
    colc[threadIdx.x] = c < 3 * NZ ? c / NZ : -1;
    coll[threadIdx.x] = c % NZ;
  }
  __syncthreads();
  const cpx<T>* H = reinterpret_cast<const cpx<T>*>(bf.H) + (size_t)mloc * 3 * NR * NTP * NZ;
  double2* Nout = dst_override ? dst_override : (bf.N ? bf.N + (size_t)mloc * 3 * S : nullptr);  // (null: mixed, N32)
  for (int idx = threadIdx.x; idx < NTP * LC; idx += TTH) {
    int p = idx / LC, lc = idx % LC;
    int c = colc[lc], l = coll[lc];
    const size_t hi = (((size_t)c * NR + i) * NTP + p) * NZ + l;
    buf[idx] = (c >= 0 && l < NZ - 1 && NSP_IN_BOUNDS(tb, hi, (size_t)3 * NR * NTP * NZ, BC_THETA_IN)) ? H[hi]
                                                                                                : mk<T>(0, 0);
  }
  __syncthreads();
  theta_fft<T, NTPC>(buf, tb, -1);
  // Wall derivative of u_z(0,0) for the mean forcing (pressGrad_k).
  double dwall = 0.0;
  if (c0 <= 2 * NZ && c0 + LC > 2 * NZ) {
    const double* Dw = tb.D + STEN * (NR - 1) + IW;
    for (int j = 0; j <= IW; j++) dwall += Dw[j] * U[2 * S + (size_t)(NR - 1 - IW + j) * NTNZ].x;
  }
  const T scale = tb_inv_norm<T>(tb);
  // mixed form, explicit field: the mean-flow terms (nsp_state.cuh), from its FP32 copy
  const float2* U32 = nullptr;
  Mean32 mf{};
  if constexpr (sizeof(T) == 4) {
    if (src_override) {  // a member state's terms are added by the linear pass
      U32 = src32_override;
      mf = mean_flow32(tb, U32, nullptr, i);
    }
  }
  for (int idx = threadIdx.x; idx < NT * LC; idx += TTH) {
    int it = idx / LC, lc = idx % LC;
    int c = colc[lc], l = coll[lc];
    if (c < 0) continue;
    int p = it < NT / 2 ? it : NTP + it - NT;
    cpx<T> b = buf[p * LC + lc];
    double2 v;
    if constexpr (sizeof(T) == 8) {
      v = make_double2((double)b.x * tb.inv_norm, (double)b.y * tb.inv_norm);
    } else if (!dst_override) {
      // a member's N in the mixed form: FP32 (its values are FP32 numbers), the wall forcing
      // of Re N_z(0,0) kept apart in FP64 -- the same at every level, written by level 0
      const bool drop = it == NT / 2 || l == NZ - 1;
      const size_t e = c * S + (size_t)i * NTNZ + (size_t)it * NZ + l;
      if (c == 2 && it == 0 && l == 0 && i == 0) bf.NF[mloc] = -(tb.sscal[4 * member_set(tb, mloc) + 1] * dwall);
      if (NSP_IN_BOUNDS(tb, e, 3 * S, BC_THETA_OUT))
        bf.N32[(size_t)mloc * 3 * S + e] = drop ? make_float2(0.f, 0.f) : make_float2(b.x * scale, b.y * scale);
      continue;
    } else {
      float2 w = make_float2(b.x * scale, b.y * scale);
      if (U32 && it != NT / 2 && l != NZ - 1) {
        const bool zm = it == 0 && l == 0;
        const size_t hq = (size_t)i * NTNZ + (size_t)it * NZ + l;
        const float2 ur = U32[hq], uq = zm ? make_float2(0.f, 0.f) : U32[(c == 2 ? 2 : 1) * S + hq];
        const float kt = (float)(it < NT / 2 ? it : it - NT) * tb.kts32;
        const float2 ml = mean_terms32(mf, c, zm, kt, tb.kzs32 * (float)l, ur, c < 2 ? uq : make_float2(0.f, 0.f),
                                       c == 2 ? uq : make_float2(0.f, 0.f));
        w.x += ml.x;
        w.y += ml.y;
      }
      v = make_double2(f32_to_f64(w.x), f32_to_f64(w.y));  // exact, integer pipe
    }
    if (it == NT / 2 || l == NZ - 1) v = make_double2(0.0, 0.0);
    if (c == 2 && it == 0 && l == 0) v.x -= tb.sscal[4 * member_set(tb, mloc) + 1] * dwall;  // 2/Re
    if (NSP_IN_BOUNDS(tb, c * S + (size_t)i * NTNZ + (size_t)it * NZ + l, 3 * S, BC_THETA_OUT))
      Nout[c * S + (size_t)i * NTNZ + (size_t)it * NZ + l] = v;
  }
}

// ---------------------------------------------------------------- launcher
template <typename T, int NTPC>
static void launch_theta(const Tables& tb, const Bufs& bf, Ctl* dctl, const double2* src, const float2* src32,
                         double2* dst, cudaStream_t st, int mask, int nm) {
  size_t sm = sizeof(cpx<T>) * tb.NTP * LC;
  if (mask & 1) {
    dim3 g((9 * tb.NZ + LC - 1) / LC, tb.NR, nm);
    nl_theta_inv<T, NTPC><<<g, TTH, sm, st>>>(tb, bf, dctl, src, src32);
  }
  if (mask & 4) {
    dim3 g((3 * tb.NZ + LC - 1) / LC, tb.NR, nm);
    nl_theta_fwd<T, NTPC><<<g, TTH, sm, st>>>(tb, bf, dctl, src, src32, dst);
  }
}

template <typename T, int NZRC, int RPB>
static void launch_z(const Tables& tb, const Bufs& bf, Ctl* dctl, bool standalone, cudaStream_t st, int nm) {
  size_t sm = sizeof(cpx<T>) * 6 * RPB * tb.NZR;
  dim3 g((tb.NTP + RPB - 1) / RPB, tb.NR, nm);
  nl_z<T, NZRC, RPB><<<g, ZTH, sm, st>>>(tb, bf, dctl, standalone ? 1 : 0);
}

template <typename T, int NZRC, int N1, int N2, int R>
static constexpr size_t z2_smem() {
  return sizeof(cpx<T>) * ((size_t)R * 6 * N2 * (N1 + 1) + (size_t)R * 6 * z2_pitch(NZRC));
}

template <typename T, int NZRC, int N1, int N2, int R>
static void launch_z2(const Tables& tb, const Bufs& bf, Ctl* dctl, bool standalone, cudaStream_t st, int nm) {
  dim3 g((tb.NTP + R - 1) / R, tb.NR, nm);
  nl_z2<T, NZRC, N1, N2, R><<<g, Z2TH, z2_smem<T, NZRC, N1, N2, R>(), st>>>(tb, bf, dctl, standalone ? 1 : 0);
}

#define NSP_NTP_LIST(X) X(12) X(24) X(48) X(72) X(96) X(144) X(192)
#define NSP_NZR_LIST(X) X(24, 2) X(48, 2) X(96, 2) X(192, 2) X(384, 2) X(576, 1) X(768, 1)
// Two-pass z stage: (NZR, N1, N2, rows per block), the splits compiled for FP32 and for
// FP64 (whose shared memory, twice FP32's, limits it to NZR <= 384); the setup-time
// autotuner picks among them and the radix-stage kernel per shape.
#define NSP_Z2_LIST_F(X) X(24, 4, 6, 2) X(48, 8, 6, 2) X(96, 8, 12, 2) X(96, 12, 8, 2) X(192, 16, 12, 2) \
  X(192, 12, 16, 2) X(384, 16, 24, 2) X(384, 24, 16, 2) X(576, 24, 24, 2) X(768, 32, 24, 2) X(768, 24, 32, 2)
#define NSP_Z2_LIST_D(X) X(24, 4, 6, 2) X(48, 8, 6, 2) X(96, 8, 12, 2) X(192, 16, 12, 2) X(192, 12, 16, 2) \
  X(384, 16, 24, 2)

int z_variants(int NZR, int NTP, bool fp32) {
  int n = 0;
#define NSP_Z2_COUNT(len, a, b, r) n += (NZR == len && NTP % r == 0);
  if (fp32) { NSP_Z2_LIST_F(NSP_Z2_COUNT) } else { NSP_Z2_LIST_D(NSP_Z2_COUNT) }
#undef NSP_Z2_COUNT
  return n;
}

// The two-pass kernel where one is compiled for the length (the FP32 default, measured
// faster than the radix-stage kernel on the bench shape), else the radix-stage kernel.
int z_default_variant(int NZR, int NTP, bool fp32) {
  const char* e = getenv("NSP_Z2");
  if (e && e[0] == '0') return 0;
  return fp32 && z_variants(NZR, NTP, true) > 0 ? 1 : 0;
}

std::string z_variant_name(int NZR, int NTP, bool fp32, int v) {
  if (v <= 0) return "radix";
  int k = 0;
  std::string s = "radix";
#define NSP_Z2_NAME(len, a, b, r) \
  if (NZR == len && NTP % r == 0 && ++k == v) s = "two-pass " #a "x" #b;
  if (fp32) { NSP_Z2_LIST_F(NSP_Z2_NAME) } else { NSP_Z2_LIST_D(NSP_Z2_NAME) }
#undef NSP_Z2_NAME
  return s;
}

template <typename T>
static void launch_nl_t(const Tables& tb, const Bufs& bf, Ctl* dctl, const double2* src, const float2* src32,
                        double2* dst, cudaStream_t st, int mask) {
  int nm = src ? 1 : tb.nmem;
  const bool tc = sizeof(T) == 4 && tb.tc_theta;  // mixed form: theta transforms on the tensor cores
  if ((mask & 1) && tc) {
    launch_theta_tc(tb, bf, dctl, 0, src, src32, dst, st);
  } else if (mask & 1) {
    switch (tb.NTP) {
#define NSP_CASE_T(n) \
  case n: launch_theta<T, n>(tb, bf, dctl, src, src32, dst, st, 1, nm); break;
      NSP_NTP_LIST(NSP_CASE_T)
#undef NSP_CASE_T
      default: launch_theta<T, 0>(tb, bf, dctl, src, src32, dst, st, 1, nm);
    }
  }
  if (mask & 2) {
    bool done = false;
    // the group's z-stage variant: the k-th two-pass split of the length, or (0) radix
    if (tb.z_variant > 0) {
      int k = 0;
#define NSP_CASE_Z2(n, a, b, r)                                                      \
  if (!done && tb.NZR == n && tb.NTP % r == 0 && ++k == tb.z_variant) {             \
    launch_z2<T, n, a, b, r>(tb, bf, dctl, src != nullptr, st, nm);                  \
    done = true;                                                                     \
  }
      if constexpr (sizeof(T) == 4) { NSP_Z2_LIST_F(NSP_CASE_Z2) } else { NSP_Z2_LIST_D(NSP_CASE_Z2) }
#undef NSP_CASE_Z2
    }
    if (!done) {
      switch (tb.NZR) {
#define NSP_CASE_Z(n, r) \
  case n: launch_z<T, n, r>(tb, bf, dctl, src != nullptr, st, nm); break;
        NSP_NZR_LIST(NSP_CASE_Z)
#undef NSP_CASE_Z
        default: launch_z<T, 0, 1>(tb, bf, dctl, src != nullptr, st, nm);
      }
    }
  }
  if ((mask & 4) && tc) {
    launch_theta_tc(tb, bf, dctl, 1, src, src32, dst, st);
  } else if (mask & 4) {
    switch (tb.NTP) {
#define NSP_CASE_T(n) \
  case n: launch_theta<T, n>(tb, bf, dctl, src, src32, dst, st, 4, nm); break;
      NSP_NTP_LIST(NSP_CASE_T)
#undef NSP_CASE_T
      default: launch_theta<T, 0>(tb, bf, dctl, src, src32, dst, st, 4, nm);
    }
  }
}

int kernels_per_nonlinear() { return 3; }

template <typename T>
static void configure_t() {
  const int big = 200 * 1024;
#define NSP_CFG_T(n)                                                                            \
  cudaFuncSetAttribute(nl_theta_inv<T, n>, cudaFuncAttributeMaxDynamicSharedMemorySize, big); \
  cudaFuncSetAttribute(nl_theta_fwd<T, n>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  NSP_NTP_LIST(NSP_CFG_T)
  NSP_CFG_T(0)
#undef NSP_CFG_T
#define NSP_CFG_Z(n, r) cudaFuncSetAttribute(nl_z<T, n, r>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  NSP_NZR_LIST(NSP_CFG_Z)
  NSP_CFG_Z(0, 1)
#undef NSP_CFG_Z
}

void configure_transform_kernels() {
  configure_t<double>();
  configure_t<float>();
#define NSP_CFG_Z2F(n, a, b, r)                                                          \
  cudaFuncSetAttribute(nl_z2<float, n, a, b, r>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                       (int)z2_smem<float, n, a, b, r>());
  NSP_Z2_LIST_F(NSP_CFG_Z2F)
#undef NSP_CFG_Z2F
#define NSP_CFG_Z2D(n, a, b, r)                                                           \
  cudaFuncSetAttribute(nl_z2<double, n, a, b, r>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                       (int)z2_smem<double, n, a, b, r>());
  NSP_Z2_LIST_D(NSP_CFG_Z2D)
#undef NSP_CFG_Z2D
  // Twiddles of the register sub-transforms, exp(-2 pi i e / 96), from long double.
  float2 wf[96];
  double2 wd[96];
  for (int e = 0; e < 96; e++) {
    const long double a = -6.283185307179586476925286766559L * (long double)e / 96.0L;
    wd[e] = make_double2((double)cosl(a), (double)sinl(a));
    wf[e] = make_float2((float)cosl(a), (float)sinl(a));
  }
  cudaMemcpyToSymbol(c_w96f, wf, sizeof(wf));
  cudaMemcpyToSymbol(c_w96d, wd, sizeof(wd));
}

bool transform_supported(int NTP, int NZR) {
  bool ct_t = false, ct_z = false;
#define NSP_HAS_T(n) ct_t |= (NTP == n);
#define NSP_HAS_Z(n, r) ct_z |= (NZR == n);
  NSP_NTP_LIST(NSP_HAS_T)
  NSP_NZR_LIST(NSP_HAS_Z)
#undef NSP_HAS_T
#undef NSP_HAS_Z
  FftPlan pt, pz;
  make_plan(NTP, pt);
  make_plan(NZR, pz);
  return (ct_t || max_butterflies(pt, LC) <= MAXR * TTH) && (ct_z || max_butterflies(pz, 6) <= MAXR * ZTH);
}

void launch_nonlinear(const Tables& tb, const Bufs& bf, Ctl* dctl, bool mixed, const double2* src, double2* dst,
                      cudaStream_t st, int mask, const float2* src32) {
  if (mixed) launch_nl_t<float>(tb, bf, dctl, src, src32, dst, st, mask);
  else launch_nl_t<double>(tb, bf, dctl, src, nullptr, dst, st, mask);
}

__global__ void to_f32_k(const double2* __restrict__ src, float2* __restrict__ dst, long long n) {
  for (long long h = blockIdx.x * (long long)blockDim.x + threadIdx.x; h < n; h += (long long)gridDim.x * blockDim.x) {
    double2 a = src[h];
    dst[h] = make_float2(f64_to_f32(a.x), f64_to_f32(a.y));
  }
}

// FP32 mirror U32 and its radial derivative DR32 of a group's state (step start):
// the same conversion and stencil as the linear pass's stages I and J.  A block holds
// a tile of MR levels x MK modes of one member component (line), plus IW levels on
// either side, converted once into shared memory; the stencil reads the tile.  Lanes
// run along the modes (coalesced); lines are S = NR*NT*NZ < 2^31 values.
constexpr int MIR_K = 32, MIR_R = 24, MIR_T = 256;
__global__ void __launch_bounds__(MIR_T) mirror_k(Tables tb, const double2* __restrict__ U, float2* __restrict__ U32,
                                                  float2* __restrict__ DR32) {
  __shared__ float2 tile[(MIR_R + 2 * IW) * MIR_K];
  const int NR = tb.NR, NT = tb.NT, NZ = tb.NZ, NTNZ = tb.NTNZ;
  const int kx = threadIdx.x % MIR_K, ry = threadIdx.x / MIR_K;
  constexpr int RY = MIR_T / MIR_K;
  const int k = blockIdx.x * MIR_K + kx, r0 = blockIdx.y * MIR_R;
  const int lo = max(0, r0 - IW), hi = min(NR, r0 + MIR_R + IW), r1 = min(NR, r0 + MIR_R);
  const int it = k / NZ, m = it < NT / 2 ? it : it - NT, par_m = abs(m) % 2;
  for (int line = blockIdx.z; line < 3 * tb.nmem; line += gridDim.z) {
    const size_t base = (size_t)line * tb.S;
    __syncthreads();  // the previous line's tile has been read
    if (k < NTNZ)
      for (int r = lo + ry; r < hi; r += RY) {
        if (!NSP_IN_BOUNDS(tb, base + (size_t)r * NTNZ + k, (size_t)3 * tb.nmem * tb.S, BC_MIRROR)) break;
        const double2 a = U[base + (size_t)r * NTNZ + k];
        tile[(r - lo) * MIR_K + kx] = make_float2(f64_to_f32(a.x), f64_to_f32(a.y));
      }
    __syncthreads();
    if (k >= NTNZ) continue;
    const int tab = abs(par_m - (line % 3 < 2 ? 1 : 0));
    for (int i = r0 + ry; i < r1; i += RY) {
      const size_t h = base + (size_t)i * NTNZ + k;
      if (!NSP_IN_BOUNDS(tb, h, (size_t)3 * tb.nmem * tb.S, BC_MIRROR)) break;
      U32[h] = tile[(i - lo) * MIR_K + kx];
      const int left = max(0, i - IW), right = min(i + IW, NR - 1), len = right + 1 - left, i0 = i + IW - right;
      const float* Dr = tb.D32 + tab * STEN * NR + STEN * i + i0;
      DR32[h] = dr32_line(Dr, left, len, [&](int row) { return tile[(row - lo) * MIR_K + kx]; });
    }
  }
}

void launch_mirror(const Tables& tb, const double2* U, float2* U32, float2* DR32, cudaStream_t st) {
  const dim3 grid((unsigned)((tb.NTNZ + MIR_K - 1) / MIR_K), (unsigned)((tb.NR + MIR_R - 1) / MIR_R),
                  (unsigned)std::min(3 * tb.nmem, 65535));
  mirror_k<<<grid, MIR_T, 0, st>>>(tb, U, U32, DR32);
}

void launch_to_f32(const double2* src, float2* dst, long long n, cudaStream_t st) {
  int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
  to_f32_k<<<blocks, 256, 0, st>>>(src, dst, n);
}

// x = hi + lo with hi = fl32(x), lo = fl32(x - hi) (x - hi is exact in FP64): the
// double-float form of set-up tables, about 48 bits of x.
__global__ void split_df_k(const double* __restrict__ src, float2* __restrict__ dst, long long n) {
  for (long long h = blockIdx.x * (long long)blockDim.x + threadIdx.x; h < n; h += (long long)gridDim.x * blockDim.x) {
    const double x = src[h];
    const float hi = f64_to_f32(x);
    dst[h] = make_float2(hi, f64_to_f32(x - f32_to_f64(hi)));
  }
}

void launch_split_df(const double* src, float2* dst, long long n, cudaStream_t st) {
  int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
  split_df_k<<<blocks, 256, 0, st>>>(src, dst, n);
}

// The banded-LU factor tables [kk][NR][NFAC][NTNZ] in double-float and FP32 for the
// mixed form's solves, with the backward entries U(i, i+j) (entries 4..6) pre-divided by
// U_ii (times entry 3, 1/U_ii): a backward row is then x_i = y_i / U_ii - sum U'_ij x_j,
// the division applied to y_i off the row-to-row dependency chain.
__global__ void split_fac_k(const double* __restrict__ fac, float2* __restrict__ dfo, float* __restrict__ f32o,
                            long long n, int NTNZ) {
  for (long long h = blockIdx.x * (long long)blockDim.x + threadIdx.x; h < n; h += (long long)gridDim.x * blockDim.x) {
    const long long k = h % NTNZ, re = h / NTNZ, e = re % NFAC;
    double x = fac[h];
    if (e >= 4) x *= fac[(re - e + 3) * NTNZ + k];
    const float hi = f64_to_f32(x);
    dfo[h] = make_float2(hi, f64_to_f32(x - f32_to_f64(hi)));
    f32o[h] = hi;
  }
}

void launch_split_fac(const double* fac, float2* dfo, float* f32o, long long n, int NTNZ, cudaStream_t st) {
  int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
  split_fac_k<<<blocks, 256, 0, st>>>(fac, dfo, f32o, n, NTNZ);
}

}  // namespace nsp
