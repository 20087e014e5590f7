// nsp_transform.cu -- the 3/2-dealiased nonlinear term, one radial level at a time.
//
// Replaces nonlinear() (mod_io_nonlinear.cu:380-409): derivr x3, padForward x12,
// derivt/derivz x6, 12 batched 2-D Z2D and 3 D2Z cuFFT transforms
// (mod_fft.cu:37-48), calcNonlinear_k (:142-170), normalize (mod_utils.cu:10-17),
// padBackward x3 (:195-214) and pressGrad (mod_radialFD.cu:100-111).  Three
// kernels per evaluation:
//
//   nl_theta_inv  per (member, level, l-chunk): builds the padded theta columns
//                 of u, d_r u (7-point stencil over levels, parity tables) and
//                 i m u / r straight from the spectral state and runs the
//                 length-NTP inverse FFTs -> G[f][level][theta_j][l] (9 fields);
//   nl_z          per (member, level, theta rows): forms the 12 Hermitian z
//                 spectra (d_z u = i k_z times the u columns of G), packs them
//                 two real fields per complex length-NZR inverse FFT, evaluates
//                 -(u.grad)u pointwise, packs the 3 products into complex forward
//                 FFTs and unpacks the half spectra l < NZ-1 -> H;
//   nl_theta_fwd  per (member, level, l-chunk): length-NTP forward FFTs of H,
//                 scale by 1/(NTP*NZR), keep the retained modes (theta Nyquist and
//                 l = NZ-1 zeroed) and apply the wall-shear forcing to N_z(0,0).
//
// T = double gives the plain FP64 form; T = float the mixed form (the state,
// d_r u and i m u / r are formed in FP64 and rounded to FP32 on load; N is
// written back in FP64).
#include <cstdio>

#include "nsp_fft.cuh"
#include "nsp_internal.h"

namespace nsp {

constexpr int MAXR = 4;

template <typename T> __device__ __forceinline__ const typename vec2<T>::type* tw_t(const Tables& tb);
template <> __device__ __forceinline__ const double2* tw_t<double>(const Tables& tb) { return tb.tw_t; }
template <> __device__ __forceinline__ const float2* tw_t<float>(const Tables& tb) { return tb.tw_t32; }
template <typename T> __device__ __forceinline__ const typename vec2<T>::type* tw_z(const Tables& tb);
template <> __device__ __forceinline__ const double2* tw_z<double>(const Tables& tb) { return tb.tw_z; }
template <> __device__ __forceinline__ const float2* tw_z<float>(const Tables& tb) { return tb.tw_z32; }

// Source field of a member: the state in the predictor phase, the iterate in corrector phases.
__device__ __forceinline__ const double2* member_source(const Tables& tb, const Bufs& bf, const Ctl* ctl, int mloc,
                                                        const double2* src_override, bool& skip) {
  skip = false;
  if (src_override) return src_override;
  int ph = ctl->phase[tb.mem0 + mloc];
  if (ph < 0) { skip = true; return nullptr; }
  int which = (ph == 0) ? ctl->parity : (ctl->parity ^ 1);
  return bf.U[which] + (size_t)mloc * 3 * tb.S;
}

// ---------------------------------------------------------------- theta inverse
template <typename T>
__global__ void __launch_bounds__(256) nl_theta_inv(Tables tb, Bufs bf, const Ctl* ctl, const double2* src_override,
                                                    int LC) {
  const int mloc = blockIdx.z, i = blockIdx.y, l0 = blockIdx.x * LC;
  bool skip;
  const double2* U = member_source(tb, bf, ctl, mloc, src_override, skip);
  if (skip) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  cpx<T>* buf = reinterpret_cast<cpx<T>*>(smraw);
  const int NR = tb.NR, NT = tb.NT, NZ = tb.NZ, NTP = tb.NTP, NTNZ = tb.NTNZ;
  const long long S = tb.S;
  const int lc_n = min(LC, NZ - l0);
  const int left = max(0, i - IW), right = min(i + IW, NR - 1);
  const int len = right + 1 - left, i0 = i + IW - right;
  const double rinv = tb.rinv[i];
  cpx<T>* G = reinterpret_cast<cpx<T>*>(bf.G) + (size_t)mloc * 9 * NR * NTP * NZ;
  for (int f = 0; f < 9; f++) {
    const int c = f % 3;
    const double2* Uc = U + c * S;
    for (int idx = threadIdx.x; idx < NTP * LC; idx += blockDim.x) {
      int p = idx / LC, lc = idx - p * LC;
      double2 v = make_double2(0.0, 0.0);
      int it = (p < NT / 2) ? p : (p >= NT ? p - NT / 2 : -1);
      if (lc < lc_n && it >= 0) {
        int l = l0 + lc;
        size_t col = (size_t)it * NZ + l;
        if (f < 3) {
          v = Uc[(size_t)i * NTNZ + col];
        } else if (f < 6) {  // derivr_k, mod_radialFD.cu:10-30 (flag 1 for u_r, u_theta; 0 for u_z)
          int m = it < NT / 2 ? it : it - NT;
          int flag = (c < 2) ? 1 : 0;
          int tab = abs((abs(m) % 2) - flag);
          const double* Dr = tb.D + tab * STEN * NR + STEN * i + i0;
          double sx = 0.0, sy = 0.0;
          for (int j = 0; j < len; j++) {
            double de = __ldg(Dr + j);
            double2 a = Uc[(size_t)(left + j) * NTNZ + col];
            sx += de * a.x;
            sy += de * a.y;
          }
          v = make_double2(sx, sy);
        } else {  // derivt_k, mod_deriv.cu:10-21
          int m = it < NT / 2 ? it : it - NT;
          double kt = tb.kts * (double)m;
          double2 a = Uc[(size_t)i * NTNZ + col];
          v = make_double2(-kt * a.y * rinv, kt * a.x * rinv);
        }
      }
      buf[idx] = mk<T>((T)v.x, (T)v.y);
    }
    __syncthreads();
    fft_batch<T, +1, MAXR, true>(buf, tb.pt, LC, LC, 1, tw_t<T>(tb));
    cpx<T>* Gf = G + ((size_t)f * NR + i) * NTP * NZ;
    for (int idx = threadIdx.x; idx < NTP * LC; idx += blockDim.x) {
      int p = idx / LC, lc = idx - p * LC;
      if (lc < lc_n) Gf[(size_t)p * NZ + l0 + lc] = buf[idx];
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- z stage
// Field order of the 12 physical arrays: u_r,u_t,u_z, dr u_r,dr u_t,dr u_z,
// dt u_r,dt u_t,dt u_z, dz u_r,dz u_t,dz u_z.  Pair t holds fields (2t, 2t+1).
template <typename T, int RPB>
__global__ void __launch_bounds__(512) nl_z(Tables tb, Bufs bf, const Ctl* ctl, int standalone) {
  const int mloc = blockIdx.z, i = blockIdx.y, j0 = blockIdx.x * RPB;
  if (!standalone && ctl->phase[tb.mem0 + mloc] < 0) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  cpx<T>* Z = reinterpret_cast<cpx<T>*>(smraw);  // [RPB*6][NZR]
  const int NR = tb.NR, NZ = tb.NZ, NTP = tb.NTP, NZR = tb.NZR;
  const cpx<T>* G = reinterpret_cast<const cpx<T>*>(bf.G) + (size_t)mloc * 9 * NR * NTP * NZ;
  cpx<T>* H = reinterpret_cast<cpx<T>*>(bf.H) + (size_t)mloc * 3 * NR * NTP * NZ;
  const T kzs = (T)tb.kzs;
  // Hermitian-extended spectra, two real fields per complex transform.
  for (int idx = threadIdx.x; idx < RPB * 6 * NZR; idx += blockDim.x) {
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
        cpx<T> g = G[(((size_t)src * NR + i) * NTP + j) * NZ + qq];
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
  fft_batch<T, +1, MAXR, false>(Z, tb.pz, RPB * 6, 1, NZR, tw_z<T>(tb));
  // -(u.grad)u (calcNonlinear_k), packed for the forward transforms:
  // RPB 2: slot0 = (Nr0, Nt0), slot1 = (Nr1, Nt1), slot2 = (Nz0, Nz1); RPB 1: slot0 = (Nr, Nt), slot1 = (Nz, 0).
  const T rinv = (T)tb.rinv[i];
  for (int n = threadIdx.x; n < NZR; n += blockDim.x) {
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
  const int nfwd = (RPB == 2) ? 3 : 2;
  fft_batch<T, -1, MAXR, false>(Z, tb.pz, nfwd, 1, NZR, tw_z<T>(tb));
  // Unpack: x = a + i b  ->  A_q = (X_q + conj X_{-q})/2,  B_q = (X_q - conj X_{-q})/(2i).
  const int NQ = NZ - 1;
  for (int idx = threadIdx.x; idx < RPB * 3 * NQ; idx += blockDim.x) {
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
    H[(((size_t)c * NR + i) * NTP + j) * NZ + q] = v;
  }
}

// ---------------------------------------------------------------- theta forward
template <typename T>
__global__ void __launch_bounds__(256) nl_theta_fwd(Tables tb, Bufs bf, const Ctl* ctl, const double2* src_override,
                                                    double2* dst_override, int LC) {
  const int mloc = blockIdx.z, i = blockIdx.y, l0 = blockIdx.x * LC;
  bool skip;
  const double2* U = member_source(tb, bf, ctl, mloc, src_override, skip);
  if (skip) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  cpx<T>* buf = reinterpret_cast<cpx<T>*>(smraw);
  const int NR = tb.NR, NT = tb.NT, NZ = tb.NZ, NTP = tb.NTP, NTNZ = tb.NTNZ;
  const long long S = tb.S;
  const int lc_n = min(LC, NZ - l0);
  const cpx<T>* H = reinterpret_cast<const cpx<T>*>(bf.H) + (size_t)mloc * 3 * NR * NTP * NZ;
  double2* Nout = dst_override ? dst_override : bf.N + (size_t)mloc * 3 * S;
  // Wall derivative of u_z(0,0) for the mean forcing (pressGrad_k).
  double dwall = 0.0;
  if (l0 == 0) {
    const double* Dw = tb.D + STEN * (NR - 1) + IW;
    for (int j = 0; j <= IW; j++) dwall += Dw[j] * U[2 * S + (size_t)(NR - 1 - IW + j) * NTNZ].x;
  }
  for (int c = 0; c < 3; c++) {
    const cpx<T>* Hc = H + ((size_t)c * NR + i) * NTP * NZ;
    for (int idx = threadIdx.x; idx < NTP * LC; idx += blockDim.x) {
      int p = idx / LC, lc = idx - p * LC;
      int l = l0 + lc;
      buf[idx] = (lc < lc_n && l < NZ - 1) ? Hc[(size_t)p * NZ + l] : mk<T>(0, 0);
    }
    __syncthreads();
    fft_batch<T, -1, MAXR, true>(buf, tb.pt, LC, LC, 1, tw_t<T>(tb));
    for (int idx = threadIdx.x; idx < NT * LC; idx += blockDim.x) {
      int it = idx / LC, lc = idx - it * LC;
      if (lc >= lc_n) continue;
      int l = l0 + lc;
      int p = it < NT / 2 ? it : NTP + it - NT;
      cpx<T> b = buf[p * LC + lc];
      double2 v = make_double2((double)b.x * tb.inv_norm, (double)b.y * tb.inv_norm);
      if (it == NT / 2 || l == NZ - 1) v = make_double2(0.0, 0.0);
      if (c == 2 && it == 0 && l == 0) v.x -= tb.two_re * dwall;
      Nout[c * S + (size_t)i * NTNZ + (size_t)it * NZ + l] = v;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- launcher
static int theta_chunk(int NZ) {
  int nchunk = (NZ + 15) / 16;
  return (NZ + nchunk - 1) / nchunk;
}

template <typename T>
static void launch_nl_t(const Tables& tb, const Bufs& bf, Ctl* dctl, const double2* src, double2* dst, cudaStream_t st,
                        int mask) {
  int LC = theta_chunk(tb.NZ);
  int nchunk = (tb.NZ + LC - 1) / LC;
  int nm = src ? 1 : tb.nmem;
  dim3 g1(nchunk, tb.NR, nm);
  size_t sm1 = sizeof(cpx<T>) * tb.NTP * LC;
  if (mask & 1) nl_theta_inv<T><<<g1, 256, sm1, st>>>(tb, bf, dctl, src, LC);
  // z stage: two theta rows per block when it fits, else one.
  int rpb = 2, thr = 256;
  auto fits = [&](int r, int t) { return max_butterflies(tb.pz, 6 * r) <= MAXR * t; };
  if (!fits(2, 256)) {
    if (fits(2, 512) && sizeof(cpx<T>) * 12 * tb.NZR <= 96 * 1024) thr = 512;
    else { rpb = 1; thr = fits(1, 256) ? 256 : 512; }
  }
  size_t sm2 = sizeof(cpx<T>) * 6 * rpb * tb.NZR;
  dim3 g2((tb.NTP + rpb - 1) / rpb, tb.NR, nm);
  if (mask & 2) {
    if (rpb == 2) nl_z<T, 2><<<g2, thr, sm2, st>>>(tb, bf, dctl, src ? 1 : 0);
    else nl_z<T, 1><<<g2, thr, sm2, st>>>(tb, bf, dctl, src ? 1 : 0);
  }
  if (mask & 4) nl_theta_fwd<T><<<g1, 256, sm1, st>>>(tb, bf, dctl, src, dst, LC);
}

int kernels_per_nonlinear() { return 3; }

void configure_transform_kernels() {
  cudaFuncSetAttribute(nl_z<double, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  cudaFuncSetAttribute(nl_z<double, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  cudaFuncSetAttribute(nl_z<float, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  cudaFuncSetAttribute(nl_z<float, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  cudaFuncSetAttribute(nl_theta_inv<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  cudaFuncSetAttribute(nl_theta_inv<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  cudaFuncSetAttribute(nl_theta_fwd<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  cudaFuncSetAttribute(nl_theta_fwd<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

void launch_nonlinear(const Tables& tb, const Bufs& bf, Ctl* dctl, bool mixed, const double2* src, double2* dst,
                      cudaStream_t st, int mask) {
  if (mixed) launch_nl_t<float>(tb, bf, dctl, src, dst, st, mask);
  else launch_nl_t<double>(tb, bf, dctl, src, dst, st, mask);
}

}  // namespace nsp
