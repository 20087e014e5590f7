// nsp_setup.cpp -- host construction of the radial operators of one member group.
//
// Everything here runs once per group at nsp_setup time, in FP64 on the host
// (built with -ffp-contract=off so x86_64 and aarch64 hosts give the same bits):
//   * the wall-clustered grid, Fornberg finite-difference weights with axis
//     parity folding, quadrature weights and Laplacian rows
//     (init_fd, mod_radialFD.cu:199-312; fd_weights :365-395; get_dr0 :316-350);
//   * the banded Doolittle factors of the three Helmholtz operators and the
//     pressure-Poisson operator for every (m, k_z) mode.  The reference
//     re-factorises inside every solve (LUsolve_*_k, mod_linear.cu:55-646); the
//     factors do not depend on the right-hand side, so they are computed once
//     here in the same operation order and stored (1/U_ii instead of U_ii);
//   * the influence-matrix correction (setBCon, mod_boundary.cu:205-255 and
//     calc_invM_k :66-196).  Only column 3 of the 4x4 inverse is ever used
//     (compcoef_k :50), so per mode the three correction profiles
//     V_c = invM[c][3] u_h,c + invM[3][3] u_hP,c are precomputed and the step
//     applies u_c += (-div_wall) V_c;
//   * the flux response uc and Qc (setCublasFlux, mod_cublasflux.cu:56-81).
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "nsp_internal.h"

namespace nsp {

namespace {

struct cd {
  double x, y;
};
inline cd cmul(cd a, cd b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }

// Fornberg's recursion for the weights of derivatives 0..m at z on the points
// x[0..n-1]; w[k*n + j] is the weight of point j for derivative k.
void fornberg(double z, const double* x, int n, int m, std::vector<double>& w) {
  w.assign((size_t)n * (m + 2), 0.0);
  double c1 = 1.0, c4 = x[0] - z;
  w[0] = 1.0;
  for (int i = 1; i < n; i++) {
    int mn = i < m ? i : m;
    double c2 = 1.0, c5 = c4;
    c4 = x[i] - z;
    for (int j = 0; j < i; j++) {
      double c3 = x[i] - x[j];
      c2 = c2 * c3;
      if (j == i - 1) {
        for (int k = mn; k > 0; k--) w[(size_t)k * n + i] = c1 * ((double)k * w[(size_t)(k - 1) * n + i - 1] - c5 * w[(size_t)k * n + i - 1]) / c2;
        w[i] = -c1 * c5 * w[i - 1] / c2;
      }
      for (int k = mn; k > 0; k--) w[(size_t)k * n + j] = (c4 * w[(size_t)k * n + j] - (double)k * w[(size_t)(k - 1) * n + j]) / c3;
      w[j] = c4 * w[j] / c3;
    }
    c1 = c2;
  }
}

}  // namespace

void radial_fd(int NR, HostOps& o) {
  const int hD = STEN * NR;
  o.NR = NR;
  o.r.assign(NR, 0.0);
  o.rdr.assign(NR, 0.0);
  o.D.assign(2 * hD, 0.0);
  o.D2.assign(2 * hD, 0.0);
  o.Lu.assign(2 * hD, 0.0);
  o.Lp.assign(2 * hD, 0.0);
  o.dr0.assign(IW + 1, 0.0);
  std::vector<double>& r = o.r;
  // Grid: Chebyshev-like points shifted ten times towards the axis.
  int N_p = NR + (int)std::sqrt((double)NR);
  for (int i = N_p - NR; i < N_p; i++) {
    int ir = N_p - i - 1;
    r[i - N_p + NR] = 0.5 * (1.0 + std::cos(0.5 * PI2 * ((double)ir / (double)N_p)));
  }
  for (int pass = 0; pass < 10; pass++) {
    double dr = 1.5 * r[0] - 0.5 * r[1];
    for (int j = 0; j < NR; j++) r[j] = r[j] * (1.0 + dr) - dr;
  }
  // Extended points: IW mirror images -r across the axis, then the grid.
  std::vector<double> ext(NR + IW), rin(NR + 1);
  for (int i = 0; i < NR + IW; i++) ext[i] = (i < IW) ? -r[IW - i - 1] : r[i - IW];
  rin[0] = 0.0;
  for (int i = 0; i < NR; i++) rin[i + 1] = r[i];
  std::vector<double> w;
  // First and second derivative rows.  Near the axis the weights of mirror
  // points fold onto their images: with + for the even table and - for the odd.
  for (int i = 0; i < NR; i++) {
    int right = (2 * IW + i < NR + IW - 1) ? 2 * IW + i : NR + IW - 1;
    int len = 1 + right - i;
    fornberg(ext[i + IW], &ext[i], len, 2, w);
    int ghosts = (i < IW) ? IW - i : 0;
    int i0 = (i < IW) ? 0 : STEN - len;
    for (int j = 0; j < len; j++) {
      double w1 = w[(size_t)len + j], w2 = w[(size_t)2 * len + j];
      int e;
      double sgn;
      if (j < ghosts) { e = ghosts - j - 1; sgn = -1.0; }
      else { e = (i < IW) ? j - ghosts : i0 + j; sgn = 1.0; }
      o.D[e + STEN * i] += w1;
      o.D2[e + STEN * i] += w2;
      if (sgn > 0) { o.D[hD + e + STEN * i] += w1; o.D2[hD + e + STEN * i] += w2; }
      else { o.D[hD + e + STEN * i] -= w1; o.D2[hD + e + STEN * i] -= w2; }
    }
  }
  // Quadrature weights of (1/pi) int int f r dr dtheta: each row integrates its
  // Taylor expansion at r_i over [r_{i-1}, r_{i+1}] times r_i; mirror points fold
  // evenly.  The k = len term (beyond the computed derivatives) is zero.
  for (int i = 0; i < NR; i++) {
    int right = (2 * IW + i < NR + IW - 1) ? 2 * IW + i : NR + IW - 1;
    int len = 1 + right - i, left2 = (i - IW > 0) ? i - IW : 0;
    fornberg(ext[i + IW], &ext[i], len, len - 1, w);
    int ghosts = (i < IW) ? IW - i : 0;
    for (int j = 0; j < ghosts; j++) {
      int img = 2 * ghosts - 1 - j;
      for (int k = 0; k < len; k++) w[(size_t)k * len + img] += w[(size_t)k * len + j];
    }
    double e1 = 1.0, e2 = 1.0;
    int ip2 = (i + 2 < NR) ? i + 2 : NR;
    for (int k = 0; k < len + 1; k++) {
      e1 = e1 * (rin[ip2] - rin[i + 1]) / ((double)(k + 1));
      e2 = e2 * (rin[i] - rin[i + 1]) / ((double)(k + 1));
      if (k == len) continue;
      for (int j = 0; j < len - ghosts; j++) o.rdr[left2 + j] += (e1 - e2) * r[i] * w[(size_t)k * len + ghosts + j];
    }
  }
  // Laplacian rows D2 + D/r; wall row: identity for velocity, D (Neumann) for pressure.
  for (int i = 0; i < NR; i++)
    for (int j = 0; j < STEN; j++) {
      int e = j + STEN * i;
      for (int t = 0; t < 2; t++) {
        if (i < NR - 1) {
          o.Lu[t * hD + e] = o.D2[t * hD + e] + o.D[t * hD + e] / r[i];
          o.Lp[t * hD + e] = o.D2[t * hD + e] + o.D[t * hD + e] / r[i];
        } else {
          o.Lu[t * hD + e] = (j < STEN - 1) ? 0.0 : 1.0;
          o.Lp[t * hD + e] = o.D[t * hD + e];
        }
      }
    }
  // Interpolation weights to r = 0 from r_0..r_IW (centreline velocity).
  fornberg(0.0, r.data(), IW + 1, 0, w);
  for (int i = 0; i <= IW; i++) o.dr0[i] = w[i];
}

namespace {

struct ModeOps {
  int NR;
  const HostOps* o;
  double c_im, inv_dt;
};

// Doolittle factors of one banded operator row by row, in the operation order of
// LUsolve_*_k.  kind 0: u+, 1: u-, 2: u_z, 3: p.  Writes f[i*NFAC + e].
void factor_mode(const ModeOps& M, int kind, int m, double kt, double kz, bool mode00, double* f) {
  const int NR = M.NR;
  const int hD = STEN * NR;
  int odd = kind <= 1 ? 1 : 0;
  int tab = std::abs((std::abs(m) % 2) - odd);
  const double* LHS = (kind == 3 ? M.o->Lp.data() : M.o->Lu.data()) + tab * hD;
  const double* r = M.o->r.data();
  std::vector<double> U((size_t)NR * (IW + 1), 0.0);
  double L[IW + 1];
  bool zz = (kind == 3) && mode00;
  for (int i = 0; i < NR; i++) {
    int left = i - IW > 0 ? i - IW : 0, right = i + IW < NR - 1 ? i + IW : NR - 1;
    int i0 = i + IW - right, coun = 0;
    bool wall = (i == NR - 1);
    double r2 = r[i] * r[i];
    for (int j = 0; j < i - left; j++) {
      double XM = LHS[j + i0 + STEN * i];
      if (!wall && kind != 3) XM = -(M.c_im) * XM;
      if (wall && zz) XM = 0.0;
      L[j] = XM;
      coun += 1;
      for (int h = 0; h < j; h++) L[j] -= L[h] * U[(size_t)(IW + 1) * (h + left) + j - h];
      L[j] = L[j] / U[(size_t)(j + left) * (IW + 1)];
    }
    int coun2 = coun;
    for (int j = 0; j < right - i + 1; j++) {
      double XM = LHS[STEN * i + i0 + coun];
      if (!wall) {
        if (j == 0) {
          if (kind == 0) XM += -(1.0 / r2) - (2.0 * kt / r2) - kz * kz - kt * kt / r2;
          else if (kind == 1) XM += -(1.0 / r2) + (2.0 * kt / r2) - kz * kz - kt * kt / r2;
          else XM += -kz * kz - kt * kt / r2;
          if (kind != 3) XM = M.inv_dt - M.c_im * XM;
        } else if (kind != 3) {
          XM = -(M.c_im) * XM;
        }
      } else if (zz) {
        XM = (j == 0) ? 1.0 : 0.0;
      }
      double& Uij = U[j + (size_t)(IW + 1) * i];
      Uij = XM;
      int hleft = coun - IW > 0 ? coun - IW : 0;
      coun += 1;
      for (int h = hleft; h < i - left; h++) Uij -= L[h] * U[(size_t)(IW + 1) * (h + left) + j + coun2 - h];
    }
    double* fr = f + (size_t)i * NFAC;
    for (int d = 1; d <= IW; d++) {  // column i-d sits at L[i-d-left]
      int j = i - d - left;
      fr[IW - d] = (j >= 0) ? L[j] : 0.0;
    }
    fr[IW] = 1.0 / U[(size_t)i * (IW + 1)];
    for (int d = 1; d <= IW; d++) fr[IW + d] = (i + d <= right) ? U[d + (size_t)(IW + 1) * i] : 0.0;
  }
}

// Forward and backward substitution with stored factors (the device algorithm).
void solve_mode(int NR, const double* f, cd* x) {
  for (int i = 0; i < NR; i++) {
    const double* fr = f + (size_t)i * NFAC;
    for (int d = (i < IW ? i : IW); d >= 1; d--) {
      x[i].x -= fr[IW - d] * x[i - d].x;
      x[i].y -= fr[IW - d] * x[i - d].y;
    }
  }
  for (int i = NR - 1; i >= 0; i--) {
    const double* fr = f + (size_t)i * NFAC;
    for (int d = 1; d <= IW && i + d < NR; d++) {
      x[i].x -= fr[IW + d] * x[i + d].x;
      x[i].y -= fr[IW + d] * x[i + d].y;
    }
    x[i].x = x[i].x * fr[IW];
    x[i].y = x[i].y * fr[IW];
  }
}

// Wall divergence of a (u_r, u_theta, u_z) mode line (divWall_k, mod_radialFD.cu:34-63).
cd div_wall(const HostOps& o, int NR, int m, double kt, double kz, const cd* ur, const cd* ut, const cd* uz) {
  int tab = std::abs((std::abs(m) % 2) - 1);
  const double* D = o.D.data() + tab * STEN * NR + STEN * (NR - 1);
  cd p = {0.0, 0.0};
  for (int j = 0; j <= IW; j++) {
    p.x += D[j + IW] * ur[NR - 1 - IW + j].x;
    p.y += D[j + IW] * ur[NR - 1 - IW + j].y;
  }
  int w = NR - 1;
  p.x += ur[w].x;
  p.y += ur[w].y;
  p.x += -kt * ut[w].y;
  p.y += kt * ut[w].x;
  p.x += -kz * uz[w].y;
  p.y += kz * uz[w].x;
  return p;
}

}  // namespace

void build_operators(const nsp_params& p, HostOps& o) {
  const int NR = p.NR, NT = p.NT, NZ = p.NZ, NTNZ = NT * NZ;
  radial_fd(NR, o);
  ModeOps M{NR, &o, p.d_im / p.Re, 1.0 / p.dt};
  const double kts = PI2 / p.LT, kzs = PI2 / p.LZ;
  o.fac.assign((size_t)4 * NR * NFAC * NTNZ, 0.0);
  o.V.assign((size_t)3 * NR * NTNZ, double2{0.0, 0.0});
  std::vector<double> f((size_t)NR * NFAC);
  std::vector<double> fk[4];
  for (auto& v : fk) v.resize((size_t)NR * NFAC);
  std::vector<cd> uh[3], ph(NR), uP[3], zero(NR, cd{0.0, 0.0}), tr(NR), tt(NR);
  for (int c = 0; c < 3; c++) { uh[c].resize(NR); uP[c].resize(NR); }
  const int hD = STEN * NR;
  for (int k = 0; k < NTNZ; k++) {
    int it = k / NZ, l = k % NZ;
    int m = it < NT / 2 ? it : it - NT;
    double kt = kts * (double)m, kz = kzs * (double)l;
    bool m00 = (m == 0 && l == 0);
    for (int op = 0; op < 4; op++) {
      factor_mode(M, op, m, kt, kz, m00, fk[op].data());
      for (int i = 0; i < NR; i++)
        for (int e = 0; e < NFAC; e++)
          o.fac[(((size_t)op * NR + i) * NFAC + e) * NTNZ + k] = fk[op][(size_t)i * NFAC + e];
    }
    // Homogeneous solutions: unit wall values (1, 1, i) and pressure with p_wall = -1.
    for (int c = 0; c < 3; c++) {
      for (int i = 0; i < NR; i++) uh[c][i] = cd{0.0, 0.0};
      uh[c][NR - 1] = (c == 2) ? cd{0.0, 1.0} : cd{1.0, 0.0};
      solve_mode(NR, fk[c].data(), uh[c].data());
    }
    for (int i = 0; i < NR; i++) ph[i] = cd{0.0, 0.0};
    ph[NR - 1] = cd{-1.0, 0.0};
    solve_mode(NR, fk[3].data(), ph.data());
    // Wall divergences of the velocity solutions in r/theta form.
    cd a41, a42, a43, a44;
    for (int i = 0; i < NR; i++) {  // (u+, 0) -> r/theta
      cd u = uh[0][i];
      tr[i] = cd{0.5 * (u.x + 0.0), 0.5 * (u.y + 0.0)};
      tt[i] = cd{0.5 * (u.y - 0.0), -0.5 * (u.x - 0.0)};
    }
    a41 = div_wall(o, NR, m, kt, kz, tr.data(), tt.data(), zero.data());
    for (int i = 0; i < NR; i++) {  // (0, u-) -> r/theta
      cd u = uh[1][i];
      tr[i] = cd{0.5 * (0.0 + u.x), 0.5 * (0.0 + u.y)};
      tt[i] = cd{0.5 * (0.0 - u.y), -0.5 * (0.0 - u.x)};
    }
    a42 = div_wall(o, NR, m, kt, kz, tr.data(), tt.data(), zero.data());
    a43 = div_wall(o, NR, m, kt, kz, zero.data(), zero.data(), uh[2].data());
    // Pressure-driven velocity grad p_h (derivr flag 0, derivt, derivz), then +/- form.
    {
      int tab = std::abs(m) % 2;
      const double* D = o.D.data() + tab * hD;
      for (int i = 0; i < NR; i++) {
        int left = i - IW > 0 ? i - IW : 0, right = i + IW < NR - 1 ? i + IW : NR - 1;
        int len = right + 1 - left, i0 = i + IW - right;
        cd s = {0.0, 0.0};
        for (int j = 0; j < len; j++) {
          s.x += D[STEN * i + j + i0] * ph[left + j].x;
          s.y += D[STEN * i + j + i0] * ph[left + j].y;
        }
        uP[0][i] = s;
        uP[1][i] = cd{-kt * ph[i].y / o.r[i], kt * ph[i].x / o.r[i]};
        uP[2][i] = cd{-kz * ph[i].y, kz * ph[i].x};
      }
    }
    a44 = div_wall(o, NR, m, kt, kz, uP[0].data(), uP[1].data(), uP[2].data());
    for (int i = 0; i < NR; i++) {
      cd a = uP[0][i], b = uP[1][i];
      uP[0][i] = cd{a.x - b.y, a.y + b.x};
      uP[1][i] = cd{a.x + b.y, a.y - b.x};
    }
    int w = NR - 1;
    cd a14 = uP[0][w], a24 = uP[1][w], a34 = uP[2][w], ax, Det;
    ax.x = a44.x - a24.x * a42.x + a24.y * a42.y - a14.x * a41.x + a14.y * a41.y;
    ax.y = a44.y - a24.x * a42.y - a24.y * a42.x - a14.x * a41.y - a14.y * a41.x;
    Det.x = -ax.y - a34.x * a43.x + a34.y * a43.y;
    Det.y = ax.x - a34.x * a43.y - a34.y * a43.x;
    double D1 = Det.x * Det.x + Det.y * Det.y;
    cd iDet = {Det.x / D1, -Det.y / D1};
    cd col3[4] = {cd{a14.y, -a14.x}, cd{a24.y, -a24.x}, cd{-a34.x, -a34.y}, cd{0.0, 1.0}};
    for (int j = 0; j < 4; j++) col3[j] = cmul(col3[j], iDet);
    // Mode (0,0): p_h is constant, so grad p_h and the determinant vanish in exact
    // arithmetic and the reference inverts rounding noise (0/0 = NaN when the noise
    // is exactly zero).  The exact correction only changes u_r(0,0), which modeZZ
    // sets to zero, so no correction is applied to this mode.
    if (m00)
      for (int j = 0; j < 4; j++) col3[j] = cd{0.0, 0.0};
    for (int c = 0; c < 3; c++)
      for (int i = 0; i < NR; i++) {
        cd v1 = cmul(col3[c], uh[c][i]), v2 = cmul(col3[3], uP[c][i]);
        o.V[((size_t)c * NR + i) * NTNZ + k] = double2{v1.x + v2.x, v1.y + v2.y};
      }
  }
  // Flux response: u_z-Helmholtz with unit right-hand side, zero wall value, mode (0,0).
  {
    std::vector<cd> x(NR, cd{1.0, 0.0});
    x[NR - 1] = cd{0.0, 0.0};
    factor_mode(M, 2, 0, 0.0, 0.0, true, f.data());
    solve_mode(NR, f.data(), x.data());
    o.uc.resize(NR);
    double Q = 0.0;
    for (int i = 0; i < NR; i++) {
      o.uc[i] = x[i].x;
      Q += o.rdr[i] * o.uc[i];
    }
    o.Qc = Q;
  }
}

}  // namespace nsp
