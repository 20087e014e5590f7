// nsp_fft.cuh -- batched mixed-radix (4/2/3) complex FFTs in shared memory.
//
// In-place Stockham autosort: every stage loads each thread's butterfly inputs
// into registers, synchronises the block, and writes the outputs to their
// Stockham positions, so no ping-pong buffer is needed.  A stage of radix P
// with sub-transform size Ns reads x[j + q n/P], twiddles by w^(q (j mod Ns) n/(Ns P)),
// applies the P-point DFT and writes x[(j/Ns) Ns P + j mod Ns + q Ns]; the result
// is in natural order.  Twiddles come from a table tw[e] = exp(-2 pi i e / n)
// (conjugated for the inverse), computed on the host from long-double sin/cos.
#pragma once
#include <cuda_runtime.h>

#include "nsp_internal.h"

namespace nsp {

// Aligned to its full size so that loads and stores of a complex value are single vector accesses.
template <typename T> struct alignas(2 * sizeof(T)) cpx { T x, y; };
template <typename T> struct vec2;
template <> struct vec2<double> { using type = double2; };
template <> struct vec2<float> { using type = float2; };

template <typename T> __device__ __forceinline__ cpx<T> mk(T x, T y) { cpx<T> r; r.x = x; r.y = y; return r; }
template <typename T> __device__ __forceinline__ cpx<T> cadd(cpx<T> a, cpx<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ cpx<T> csub(cpx<T> a, cpx<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ cpx<T> cmulv(cpx<T> a, cpx<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// multiply by sign*i
template <typename T, int SIGN> __device__ __forceinline__ cpx<T> muli(cpx<T> a) {
  return SIGN > 0 ? mk<T>(-a.y, a.x) : mk<T>(a.y, -a.x);
}

template <typename T, int SIGN, int P> __device__ __forceinline__ void dft(cpx<T>* v) {
  if (P == 2) {
    cpx<T> a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if (P == 4) {
    cpx<T> t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
    cpx<T> t2 = cadd(v[1], v[3]), t3 = muli<T, SIGN>(csub(v[1], v[3]));
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
  } else {  // P == 3
    const T s3 = (T)0.8660254037844386;  // sin(pi/3)
    cpx<T> s = cadd(v[1], v[2]), d = csub(v[1], v[2]);
    cpx<T> a = v[0];
    v[0] = cadd(a, s);
    cpx<T> m = mk<T>(a.x - (T)0.5 * s.x, a.y - (T)0.5 * s.y);
    cpx<T> id = muli<T, SIGN>(d);
    v[1] = mk<T>(m.x + s3 * id.x, m.y + s3 * id.y);
    v[2] = mk<T>(m.x - s3 * id.x, m.y - s3 * id.y);
  }
}

// One Stockham stage over nb transforms of length n.  Element e of transform t
// lives at buf[t*bs + e*es].  TFAST: consecutive threads take consecutive
// transforms (for element-strided layouts), else consecutive butterflies.
template <typename T, int SIGN, int P, int MAXR, bool TFAST>
__device__ __forceinline__ void fft_stage(cpx<T>* buf, int n, int nb, int es, int bs, int Ns,
                                          const typename vec2<T>::type* __restrict__ tw) {
  const int nbf = n / P;
  const int total = nb * nbf;
  const int tstride = n / (Ns * P);
  cpx<T> v[MAXR][P];
#pragma unroll
  for (int rr = 0; rr < MAXR; rr++) {
    int b = threadIdx.x + rr * blockDim.x;
    if (b < total) {
      int t = TFAST ? b % nb : b / nbf;
      int j = TFAST ? b / nb : b - t * nbf;
      const cpx<T>* x = buf + (size_t)t * bs;
#pragma unroll
      for (int q = 0; q < P; q++) v[rr][q] = x[(j + q * nbf) * es];
    }
  }
  __syncthreads();
#pragma unroll
  for (int rr = 0; rr < MAXR; rr++) {
    int b = threadIdx.x + rr * blockDim.x;
    if (b < total) {
      int t = TFAST ? b % nb : b / nbf;
      int j = TFAST ? b / nb : b - t * nbf;
      int k = j % Ns;
      if (k) {
#pragma unroll
        for (int q = 1; q < P; q++) {
          typename vec2<T>::type w = __ldg(tw + (q * k * tstride) % n);
          cpx<T> wc = mk<T>(w.x, SIGN > 0 ? -w.y : w.y);
          v[rr][q] = cmulv(v[rr][q], wc);
        }
      }
      dft<T, SIGN, P>(v[rr]);
      cpx<T>* x = buf + (size_t)t * bs;
      int base = (j / Ns) * Ns * P + k;
#pragma unroll
      for (int q = 0; q < P; q++) x[(base + q * Ns) * es] = v[rr][q];
    }
  }
  __syncthreads();
}

// Full transform (SIGN -1 forward, +1 inverse, unnormalised).  The caller
// synchronises before the call (data written) and may read right after.
template <typename T, int SIGN, int MAXR, bool TFAST>
__device__ void fft_batch(cpx<T>* buf, const FftPlan& pl, int nb, int es, int bs,
                          const typename vec2<T>::type* __restrict__ tw) {
  int Ns = 1;
  for (int s = 0; s < pl.nst; s++) {
    int P = pl.rad[s];
    if (P == 4) fft_stage<T, SIGN, 4, MAXR, TFAST>(buf, pl.n, nb, es, bs, Ns, tw);
    else if (P == 2) fft_stage<T, SIGN, 2, MAXR, TFAST>(buf, pl.n, nb, es, bs, Ns, tw);
    else fft_stage<T, SIGN, 3, MAXR, TFAST>(buf, pl.n, nb, es, bs, Ns, tw);
    Ns *= P;
  }
}

// ---------------------------------------------------------------------------
// Compile-time variant: length N, batch NB, element stride ES, batch stride BS
// and block size NTH are template parameters, so every index division is by a
// constant (multiply-shift) and the register staging holds exactly the rounds
// each stage needs.
__host__ __device__ constexpr int ct_radix(int n, int s) {
  int k = 0;
  while (n % 4 == 0) { if (k == s) return 4; n /= 4; k++; }
  while (n % 2 == 0) { if (k == s) return 2; n /= 2; k++; }
  while (n % 3 == 0) { if (k == s) return 3; n /= 3; k++; }
  return 0;
}
__host__ __device__ constexpr int ct_nstages(int n) {
  int k = 0;
  while (ct_radix(n, k)) k++;
  return k;
}

template <typename T, int SIGN, int N, int NB, int ES, int BS, bool TFAST, int NTH, int P, int NS>
__device__ __forceinline__ void fft_stage_ct(cpx<T>* buf, const typename vec2<T>::type* __restrict__ tw) {
  constexpr int NBF = N / P;
  constexpr int TOTAL = NB * NBF;
  constexpr int R = (TOTAL + NTH - 1) / NTH;
  constexpr int TSTR = N / (NS * P);
  cpx<T> v[R][P];
#pragma unroll
  for (int rr = 0; rr < R; rr++) {
    int b = threadIdx.x + rr * NTH;
    if (TOTAL % NTH == 0 || b < TOTAL) {
      int t = TFAST ? b % NB : b / NBF;
      int j = TFAST ? b / NB : b - t * NBF;
      const cpx<T>* x = buf + t * BS;
#pragma unroll
      for (int q = 0; q < P; q++) v[rr][q] = x[(j + q * NBF) * ES];
    }
  }
  __syncthreads();
#pragma unroll
  for (int rr = 0; rr < R; rr++) {
    int b = threadIdx.x + rr * NTH;
    if (TOTAL % NTH == 0 || b < TOTAL) {
      int t = TFAST ? b % NB : b / NBF;
      int j = TFAST ? b / NB : b - t * NBF;
      int k = (NS == 1) ? 0 : j % NS;
      if (NS > 1) {
#pragma unroll
        for (int q = 1; q < P; q++) {
          typename vec2<T>::type w = __ldg(tw + q * k * TSTR);
          v[rr][q] = cmulv(v[rr][q], mk<T>(w.x, SIGN > 0 ? -w.y : w.y));
        }
      }
      dft<T, SIGN, P>(v[rr]);
      cpx<T>* x = buf + t * BS;
      int base = (NS == 1) ? j * P : (j / NS) * NS * P + k;
#pragma unroll
      for (int q = 0; q < P; q++) x[(base + q * NS) * ES] = v[rr][q];
    }
  }
  __syncthreads();
}

template <typename T, int SIGN, int N, int NB, int ES, int BS, bool TFAST, int NTH, int S = 0, int NS = 1>
__device__ __forceinline__ void fft_ct(cpx<T>* buf, const typename vec2<T>::type* __restrict__ tw) {
  if constexpr (S < ct_nstages(N)) {
    constexpr int P = ct_radix(N, S);
    fft_stage_ct<T, SIGN, N, NB, ES, BS, TFAST, NTH, P, NS>(buf, tw);
    fft_ct<T, SIGN, N, NB, ES, BS, TFAST, NTH, S + 1, NS * P>(buf, tw);
  }
}

// Largest butterfly count of any stage (for the MAXR bound check on the host).
inline int max_butterflies(const FftPlan& pl, int nb) {
  int mx = 0;
  for (int s = 0; s < pl.nst; s++) {
    int b = nb * (pl.n / pl.rad[s]);
    if (b > mx) mx = b;
  }
  return mx;
}

inline bool make_plan(int n, FftPlan& pl) {
  pl.n = n;
  pl.nst = 0;
  int m = n;
  while (m % 4 == 0 && pl.nst < MAXPLAN) { pl.rad[pl.nst++] = 4; m /= 4; }
  while (m % 2 == 0 && pl.nst < MAXPLAN) { pl.rad[pl.nst++] = 2; m /= 2; }
  while (m % 3 == 0 && pl.nst < MAXPLAN) { pl.rad[pl.nst++] = 3; m /= 3; }
  return m == 1;
}

}  // namespace nsp
