// nsp_linear.cu -- the linear part of the predictor and corrector, one CTA per
// block of LM (m, k_z) mode lines of one member, all in FP64.
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
// (r, mode), the banded solves one thread per (component, mode) sweeping r with
// the precomputed factors (read coalesced across modes).  u^n in +/- form (uw)
// is recomputed from the state instead of stored.
#include <cstdio>

#include "nsp_internal.h"

namespace nsp {


__device__ __forceinline__ double2 c2(double x, double y) { return make_double2(x, y); }

// One forward-substitution row: x -= L(i-3) x_{i-3} + L(i-2) x_{i-2} + L(i-1) x_{i-1},
// in the reference's column order.  Factors of columns outside the band are stored
// as 0 (and the carried x start at 0), so edge rows need no branches.
__device__ __forceinline__ void fwd_row(double2& x, const double* l, double2& xm1, double2& xm2, double2& xm3) {
  x.x -= l[0] * xm3.x; x.y -= l[0] * xm3.y;
  x.x -= l[1] * xm2.x; x.y -= l[1] * xm2.y;
  x.x -= l[2] * xm1.x; x.y -= l[2] * xm1.y;
  xm3 = xm2; xm2 = xm1; xm1 = x;
}
// One backward row, farther neighbours first so that only one multiply-add and the
// pivot multiply wait on the row just finished: x = (x - U3 x3 - U2 x2 - U1 x1) / U_ii.
__device__ __forceinline__ void bwd_row(double2& x, const double* u, double2& xp1, double2& xp2, double2& xp3) {
  x.x -= u[0] * xp3.x; x.y -= u[0] * xp3.y;
  x.x -= u[1] * xp2.x; x.y -= u[1] * xp2.y;
  x.x -= u[2] * xp1.x; x.y -= u[2] * xp1.y;
  x.x *= u[3]; x.y *= u[3];
  xp3 = xp2; xp2 = xp1; xp1 = x;
}

// Forward + backward substitution of one mode line held in X[i*ld] (i = 0..NR-1).
// Factor rows are fetched four at a time so that their L2 latencies overlap.
__device__ __forceinline__ void solve_line(double2* X, int ld, const double* __restrict__ f, int NTNZ, int NR) {
  const size_t rs = (size_t)NFAC * NTNZ;  // row stride of the factor table
  double2 xm1 = c2(0, 0), xm2 = c2(0, 0), xm3 = c2(0, 0);
  int i = 0;
  for (; i + 4 <= NR; i += 4) {
    double l[4][3];
    double2 b[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const double* fr = f + (i + r) * rs;
      l[r][0] = __ldg(fr); l[r][1] = __ldg(fr + NTNZ); l[r][2] = __ldg(fr + 2 * NTNZ);
      b[r] = X[(i + r) * ld];
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      fwd_row(b[r], l[r], xm1, xm2, xm3);
      X[(i + r) * ld] = b[r];
    }
  }
  for (; i < NR; i++) {
    const double* fr = f + i * rs;
    double l[3] = {__ldg(fr), __ldg(fr + NTNZ), __ldg(fr + 2 * NTNZ)};
    double2 x = X[i * ld];
    fwd_row(x, l, xm1, xm2, xm3);
    X[i * ld] = x;
  }
  double2 xp1 = c2(0, 0), xp2 = c2(0, 0), xp3 = c2(0, 0);
  i = NR - 1;
  for (; i >= 3; i -= 4) {
    double u[4][4];
    double2 b[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const double* fr = f + (i - r) * rs;
      u[r][0] = __ldg(fr + 6 * NTNZ); u[r][1] = __ldg(fr + 5 * NTNZ);
      u[r][2] = __ldg(fr + 4 * NTNZ); u[r][3] = __ldg(fr + 3 * NTNZ);
      b[r] = X[(i - r) * ld];
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      bwd_row(b[r], u[r], xp1, xp2, xp3);
      X[(i - r) * ld] = b[r];
    }
  }
  for (; i >= 0; i--) {
    const double* fr = f + i * rs;
    double u[4] = {__ldg(fr + 6 * NTNZ), __ldg(fr + 5 * NTNZ), __ldg(fr + 4 * NTNZ), __ldg(fr + 3 * NTNZ)};
    double2 x = X[i * ld];
    bwd_row(x, u, xp1, xp2, xp3);
    X[i * ld] = x;
  }
}

template <int LM, int NTH>
__global__ void __launch_bounds__(NTH) linear_k(Tables tb, Bufs bf, Ctl* ctl) {
  const int mloc = blockIdx.y, gm = tb.mem0 + mloc;
  const int ph = ctl->phase[gm];
  if (ph < 0) return;
  const bool pred = (ph == 0);
  const int par = ctl->parity;
  const int NR = tb.NR, NT = tb.NT, NZ = tb.NZ, NTNZ = tb.NTNZ;
  const long long S = tb.S;
  const int k0 = blockIdx.x * LM;
  const int LN = NR * LM;
  extern __shared__ double2 sm[];
  double2* W = sm;           // [3][NR][LM] u^n in +/- form
  double2* R = sm + 3 * LN;  // [3][NR][LM] right-hand side, then the new velocity
  double2* P = W;            // divergence / pressure (W is dead by then)
  __shared__ double2 dvs[LM];
  __shared__ double wnum[NTH / 32], wden[NTH / 32];
  __shared__ int bad;
  const double2* Un = bf.U[par] + (size_t)mloc * 3 * S;
  double2* Ui = bf.U[par ^ 1] + (size_t)mloc * 3 * S;
  float2* Ui32 = bf.U32[par ^ 1] ? bf.U32[par ^ 1] + (size_t)mloc * 3 * S : nullptr;  // mixed form
  const double2* Nn = bf.N + (size_t)mloc * 3 * S;
  double2* Rw = bf.RHSW + (size_t)mloc * 3 * S;
  const int tid = threadIdx.x, nth = blockDim.x;
  if (tid == 0) bad = 0;

  // The explicit part of the right-hand side, e = u^n/dt + (1-d_im)/Re L+- u^n
  // (addLaplacian, mod_linear.cu:12-51), is the same in the predictor and in every
  // corrector of a step.  The predictor computes it once and stores
  // rhsw' = (1-d_im) N(u^n)+- + e; a corrector's right-hand side is then
  // d_im N(u_i)+- + rhsw' (addRHS_k + addLaplacian), with no stencil and no read of u^n.
  if (pred) {
    // A. u^n -> +/- (uw) into W, N(u^n) -> +/- into R.
    for (int p = tid; p < LN; p += nth) {
      int i = p / LM, mm = p - i * LM, k = k0 + mm;
      if (k >= NTNZ) {
        for (int c = 0; c < 3; c++) { W[c * LN + p] = c2(0, 0); R[c * LN + p] = c2(0, 0); }
        continue;
      }
      size_t h = (size_t)i * NTNZ + k;
      double2 ur = Un[h], ut = Un[S + h], uz = Un[2 * S + h];
      W[p] = c2(ur.x - ut.y, ur.y + ut.x);
      W[LN + p] = c2(ur.x + ut.y, ur.y - ut.x);
      W[2 * LN + p] = uz;
      double2 nr = Nn[h], nt = Nn[S + h], nz = Nn[2 * S + h];
      R[p] = c2(nr.x - nt.y, nr.y + nt.x);
      R[LN + p] = c2(nr.x + nt.y, nr.y - nt.x);
      R[2 * LN + p] = nz;
    }
    __syncthreads();
    // B. e = u/dt + (1-d_im)/Re (L_r - k_z^2 - m^2/r^2 [-1/r^2 -+ 2m/r^2]) u; rhs = N + e;
    //    rhsw' = (1-d_im) N + e; rhs +/- -> r/theta.
    for (int p = tid; p < LN; p += nth) {
      int i = p / LM, mm = p - i * LM, k = k0 + mm;
      if (k >= NTNZ) continue;
      int it = k / NZ, l = k - it * NZ, m = it < NT / 2 ? it : it - NT;
      double kt = tb.kts * (double)m, kz = tb.kzs * (double)l;
      int left = max(0, i - IW), right = min(i + IW, NR - 1), len = right + 1 - left, i0 = i + IW - right;
      double ir2 = tb.rinv2[i];
      double base = -kz * kz - kt * kt * ir2;
      double pm = -ir2 - 2.0 * kt * ir2, mm2 = -ir2 + 2.0 * kt * ir2;
      size_t h = (size_t)i * NTNZ + k;
      double2 out[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        int tab = abs((abs(m) % 2) - (c < 2 ? 1 : 0));
        const double* Lr = tb.Luc + tab * STEN * NR + STEN * i + i0;  // (1-d_im)/Re * L_r
        const double2* Wc = W + c * LN + mm;
        double sx = 0.0, sy = 0.0;
        for (int j = 0; j < len; j++) {
          double de = __ldg(Lr + j);
          double2 a = Wc[(left + j) * LM];
          sx += de * a.x;
          sy += de * a.y;
        }
        double2 aux = Wc[i * LM];
        double de = base + (c == 0 ? pm : (c == 1 ? mm2 : 0.0));
        double dd = tb.c_ex * de + tb.inv_dt;  // diagonal: (1-d_im)/Re (-k_z^2 - m^2/r^2 ...) + 1/dt
        sx += dd * aux.x;
        sy += dd * aux.y;
        double2 n = R[c * LN + p];
        out[c] = c2(n.x + sx, n.y + sy);
        Rw[c * S + h] = c2(tb.one_m_dim * n.x + sx, tb.one_m_dim * n.y + sy);
      }
      R[p] = c2(0.5 * (out[0].x + out[1].x), 0.5 * (out[0].y + out[1].y));
      R[LN + p] = c2(0.5 * (out[0].y - out[1].y), -0.5 * (out[0].x - out[1].x));
      R[2 * LN + p] = out[2];
    }
  } else {
    // A+B. rhs = d_im N(u_i)+- + rhsw', then +/- -> r/theta.
    for (int p = tid; p < LN; p += nth) {
      int i = p / LM, mm = p - i * LM, k = k0 + mm;
      if (k >= NTNZ) {
        for (int c = 0; c < 3; c++) R[c * LN + p] = c2(0, 0);
        continue;
      }
      size_t h = (size_t)i * NTNZ + k;
      double2 nr = Nn[h], nt = Nn[S + h], nz = Nn[2 * S + h];
      double2 w0 = Rw[h], w1 = Rw[S + h], w2 = Rw[2 * S + h];
      double2 np = c2(nr.x - nt.y, nr.y + nt.x), nm = c2(nr.x + nt.y, nr.y - nt.x);
      np = c2(tb.d_im * np.x + w0.x, tb.d_im * np.y + w0.y);
      nm = c2(tb.d_im * nm.x + w1.x, tb.d_im * nm.y + w1.y);
      nz = c2(tb.d_im * nz.x + w2.x, tb.d_im * nz.y + w2.y);
      R[p] = c2(0.5 * (np.x + nm.x), 0.5 * (np.y + nm.y));
      R[LN + p] = c2(0.5 * (np.y - nm.y), -0.5 * (np.x - nm.x));
      R[2 * LN + p] = nz;
    }
  }
  __syncthreads();

  // C. divergence of rhs into P; wall row = 0 (write_bcon).
  for (int p = tid; p < LN; p += nth) {
    int i = p / LM, mm = p - i * LM, k = k0 + mm;
    double2 d = c2(0, 0);
    if (k < NTNZ && i < NR - 1) {
      int it = k / NZ, l = k - it * NZ, m = it < NT / 2 ? it : it - NT;
      double kt = tb.kts * (double)m, kz = tb.kzs * (double)l;
      int left = max(0, i - IW), right = min(i + IW, NR - 1), len = right + 1 - left, i0 = i + IW - right;
      int tab = abs((abs(m) % 2) - 1);
      const double* Dr = tb.D + tab * STEN * NR + STEN * i + i0;
      double sx = 0.0, sy = 0.0;
      for (int j = 0; j < len; j++) {
        double de = __ldg(Dr + j);
        double2 a = R[(left + j) * LM + mm];
        sx += de * a.x;
        sy += de * a.y;
      }
      double ri = tb.rinv[i], kti = kt * ri;
      double2 rr = R[p], rt = R[LN + p], rz = R[2 * LN + p];
      sx += rr.x * ri; sy += rr.y * ri;
      sx -= kti * rt.y; sy += kti * rt.x;
      sx -= kz * rz.y; sy += kz * rz.x;
      d = c2(sx, sy);
    }
    P[p] = d;
  }
  __syncthreads();

  // D. pressure Poisson solve, one thread per mode.
  if (tid < LM && k0 + tid < NTNZ) solve_line(P + tid, LM, tb.fac + 3 * (size_t)NR * NFAC * NTNZ + k0 + tid, NTNZ, NR);
  __syncthreads();

  // E. rhs -= grad p, r/theta -> +/-, wall rows = 0.
  for (int p = tid; p < LN; p += nth) {
    int i = p / LM, mm = p - i * LM, k = k0 + mm;
    if (k >= NTNZ) continue;
    double2 up = c2(0, 0), um = c2(0, 0), rz = c2(0, 0);
    if (i < NR - 1) {
      int it = k / NZ, l = k - it * NZ, m = it < NT / 2 ? it : it - NT;
      double kt = tb.kts * (double)m, kz = tb.kzs * (double)l;
      int left = max(0, i - IW), right = min(i + IW, NR - 1), len = right + 1 - left, i0 = i + IW - right;
      int tab = abs(m) % 2;
      const double* Dr = tb.D + tab * STEN * NR + STEN * i + i0;
      double sx = 0.0, sy = 0.0;
      for (int j = 0; j < len; j++) {
        double de = __ldg(Dr + j);
        double2 a = P[(left + j) * LM + mm];
        sx += de * a.x;
        sy += de * a.y;
      }
      double kti = kt * tb.rinv[i];
      double2 pp = P[p], rr = R[p], rt = R[LN + p];
      rz = R[2 * LN + p];
      rr.x -= sx; rr.y -= sy;
      rt.x += kti * pp.y; rt.y -= kti * pp.x;
      rz.x += kz * pp.y; rz.y -= kz * pp.x;
      up = c2(rr.x - rt.y, rr.y + rt.x);
      um = c2(rr.x + rt.y, rr.y - rt.x);
    }
    R[p] = up; R[LN + p] = um; R[2 * LN + p] = rz;
  }
  __syncthreads();

  // F. Helmholtz solves for u+, u-, u_z.
  if (tid < 3 * LM) {
    int c = tid / LM, mm = tid - c * LM;
    if (k0 + mm < NTNZ) solve_line(R + c * LN + mm, LM, tb.fac + (size_t)c * NR * NFAC * NTNZ + k0 + mm, NTNZ, NR);
  }
  __syncthreads();

  // G1. wall divergence of the solution (in r/theta form) per mode.
  if (tid < LM) {
    int mm = tid, k = k0 + mm;
    double2 dv = c2(0, 0);
    if (k < NTNZ) {
      int it = k / NZ, l = k - it * NZ, m = it < NT / 2 ? it : it - NT;
      double kt = tb.kts * (double)m, kz = tb.kzs * (double)l;
      int tab = abs((abs(m) % 2) - 1);
      const double* Dw = tb.D + tab * STEN * NR + STEN * (NR - 1) + IW;
      double sx = 0.0, sy = 0.0;
      double2 urw = c2(0, 0), utw = c2(0, 0);
      for (int j = 0; j <= IW; j++) {
        int row = NR - 1 - IW + j;
        double2 a = R[row * LM + mm], b = R[LN + row * LM + mm];
        double2 ur = c2(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
        double de = __ldg(Dw + j);
        sx += de * ur.x;
        sy += de * ur.y;
        if (j == IW) { urw = ur; utw = c2(0.5 * (a.y - b.y), -0.5 * (a.x - b.x)); }
      }
      double2 uzw = R[2 * LN + (NR - 1) * LM + mm];
      sx += urw.x; sy += urw.y;
      sx += -kt * utw.y; sy += kt * utw.x;
      sx += -kz * uzw.y; sy += kz * uzw.x;
      dv = c2(-sx, -sy);
    }
    dvs[mm] = dv;
  }
  __syncthreads();

  // G2. u += (-div_wall) V, back to r/theta, mode (0,0) constraints.
  for (int p = tid; p < LN; p += nth) {
    int i = p / LM, mm = p - i * LM, k = k0 + mm;
    if (k >= NTNZ) continue;
    double2 up = R[p], um = R[LN + p], uz = R[2 * LN + p];
    double2 dv = dvs[mm];
    size_t hv = (size_t)i * NTNZ + k;
    double2 v0 = tb.V[hv], v1 = tb.V[S + hv], v2 = tb.V[2 * S + hv];
    up.x += dv.x * v0.x - dv.y * v0.y; up.y += dv.x * v0.y + dv.y * v0.x;
    um.x += dv.x * v1.x - dv.y * v1.y; um.y += dv.x * v1.y + dv.y * v1.x;
    uz.x += dv.x * v2.x - dv.y * v2.y; uz.y += dv.x * v2.y + dv.y * v2.x;
    double2 ur = c2(0.5 * (up.x + um.x), 0.5 * (up.y + um.y));
    double2 ut = c2(0.5 * (up.y - um.y), -0.5 * (up.x - um.x));
    if (k == 0) { ur = c2(0, 0); ut.y = 0.0; uz.y = 0.0; }
    R[p] = ur; R[LN + p] = ut; R[2 * LN + p] = uz;
  }
  __syncthreads();

  // H. constant mass flux on mode (0,0).
  if (k0 == 0 && tid == 0) {
    double Q = 0.0;
    for (int i = 0; i < NR; i++) Q += tb.rdr[i] * R[2 * LN + i * LM].x;
    double corr = (tb.Qdes - Q) / tb.Qc;
    for (int i = 0; i < NR; i++) R[2 * LN + i * LM].x += corr * tb.uc[i];
  }
  __syncthreads();

  // I. store the new iterate; corrector: convergence measure against the previous one.
  double lnum = 0.0, lden = 0.0;
  bool nonfin = false;
  for (int p = tid; p < LN; p += nth) {
    int i = p / LM, mm = p - i * LM, k = k0 + mm;
    if (k >= NTNZ) continue;
    size_t h = (size_t)i * NTNZ + k;
    double n1 = 0.0, d1 = 0.0;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double2 v = R[c * LN + p];
      if (!pred) {
        double2 o = Ui[c * S + h];
        double ex = o.x - v.x, ey = o.y - v.y;
        n1 = fmax(n1, ex * ex + ey * ey);
        d1 = fmax(d1, o.x * o.x + o.y * o.y);
      }
      nonfin |= !(isfinite(v.x) && isfinite(v.y));
      Ui[c * S + h] = v;
      if (Ui32) Ui32[c * S + h] = make_float2((float)v.x, (float)v.y);
    }
    lnum = fmax(lnum, n1);
    lden = fmax(lden, d1);
  }
  if (nonfin) bad = 1;
  if (!pred) {
    for (int o = 16; o > 0; o >>= 1) {
      lnum = fmax(lnum, __shfl_xor_sync(0xffffffffu, lnum, o));
      lden = fmax(lden, __shfl_xor_sync(0xffffffffu, lden, o));
    }
    if ((tid & 31) == 0) { wnum[tid >> 5] = lnum; wden[tid >> 5] = lden; }
  }
  __syncthreads();
  if (tid == 0) {
    if (!pred) {
      double a = 0.0, b = 0.0;
      for (int w = 0; w < nth / 32; w++) { a = fmax(a, wnum[w]); b = fmax(b, wden[w]); }
      atomicMax(ctl->num + gm, (unsigned long long)__double_as_longlong(a));
      atomicMax(ctl->den + gm, (unsigned long long)__double_as_longlong(b));
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
    if (!any) {
      ctl->parity ^= 1;
      ctl->step += 1;
    }
    ctl->any = any;
    if (use_cond) cudaGraphSetConditional(h, any ? 1u : 0u);
  }
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

__global__ void lusolve_k(Tables tb, int kind, const double2* rhs, double2* sol) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= tb.NTNZ) return;
  for (int i = 0; i < tb.NR; i++) sol[(size_t)i * tb.NTNZ + k] = rhs[(size_t)i * tb.NTNZ + k];
  solve_line(sol + k, tb.NTNZ, tb.fac + (size_t)kind * tb.NR * NFAC * tb.NTNZ + k, tb.NTNZ, tb.NR);
}

// Block shapes of the linear pass (modes per block, threads): the candidates of the
// setup-time autotuner.  Shared memory per block is 6 radial lines per mode.
struct LinShape { int LM, NTH; };
static const LinShape kLinShapes[LIN_VARIANTS] = {{16, 256}, {8, 128}, {8, 256}, {4, 128},
                                                  {12, 192}, {12, 256}, {24, 384}, {32, 512}};

int linear_default_variant(int NR) { return NR <= 64 ? 0 : 2; }

bool linear_variant_fits(int v, int NR) {
  return v >= 0 && v < LIN_VARIANTS && sizeof(double2) * 6 * (size_t)NR * kLinShapes[v].LM <= 200 * 1024;
}

void configure_linear_kernels() {
  const int big = 200 * 1024;
  cudaFuncSetAttribute(linear_k<16, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(linear_k<8, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(linear_k<8, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(linear_k<4, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(linear_k<12, 192>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(linear_k<12, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(linear_k<24, 384>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
  cudaFuncSetAttribute(linear_k<32, 512>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
}

void launch_linear(const Tables& tb, const Bufs& bf, Ctl* dctl, cudaStream_t st) {
  int v = linear_variant_fits(tb.lin_variant, tb.NR) ? tb.lin_variant : linear_default_variant(tb.NR);
  const LinShape s = kLinShapes[v];
  dim3 grid((tb.NTNZ + s.LM - 1) / s.LM, tb.nmem);
  size_t smem = sizeof(double2) * 6 * (size_t)tb.NR * s.LM;
  switch (v) {
    case 0: linear_k<16, 256><<<grid, 256, smem, st>>>(tb, bf, dctl); break;
    case 1: linear_k<8, 128><<<grid, 128, smem, st>>>(tb, bf, dctl); break;
    case 2: linear_k<8, 256><<<grid, 256, smem, st>>>(tb, bf, dctl); break;
    case 3: linear_k<4, 128><<<grid, 128, smem, st>>>(tb, bf, dctl); break;
    case 4: linear_k<12, 192><<<grid, 192, smem, st>>>(tb, bf, dctl); break;
    case 5: linear_k<12, 256><<<grid, 256, smem, st>>>(tb, bf, dctl); break;
    case 6: linear_k<24, 384><<<grid, 384, smem, st>>>(tb, bf, dctl); break;
    default: linear_k<32, 512><<<grid, 512, smem, st>>>(tb, bf, dctl); break;
  }
}

void launch_converge(Ctl* dctl, int nmem, unsigned long long cond_handle, int use_cond, cudaStream_t st) {
  (void)nmem;
  converge_k<<<1, 256, 0, st>>>(dctl, (cudaGraphConditionalHandle)cond_handle, use_cond);
}

void launch_lusolve(const Tables& tb, int kind, const double2* rhs, double2* sol, cudaStream_t st) {
  lusolve_k<<<(tb.NTNZ + 127) / 128, 128, 0, st>>>(tb, kind, rhs, sol);
}

}  // namespace nsp
