// nsp_setup_mode.h -- per-mode operator construction, shared by the host build
// (nsp_setup.cpp, -ffp-contract=off) and the device build (nsp_setup_dev.cu,
// --fmad=false): one source, the same IEEE operations in the same order, so both
// produce the same bits.
//
// For one (m, k_z) mode of one parameter set (Re, dt):
//   * the banded Doolittle factors of the u+, u-, u_z Helmholtz operators and the
//     pressure-Poisson operator, in the operation order of LUsolve_*_k
//     (mod_linear.cu:55-646), stored as L(i-3..i-1), 1/U_ii, U(i+1..i+3) per row;
//   * the influence-matrix correction profiles V_c = invM[c][3] u_h,c + invM[3][3]
//     u_hP,c (setBCon, mod_boundary.cu:205-255; calc_invM_k :66-196; only column 3
//     of the inverse is used, compcoef_k :50).
// Arrays are reached through strided accessors: element e of a mode's array sits at
// base[e * stride], so the device keeps one mode per thread with coalesced columns.
#pragma once

#ifdef __CUDACC__
#define NSP_HD __host__ __device__
#else
#define NSP_HD
#endif

namespace nsp {
namespace setup {

constexpr int IW_ = 3;
constexpr int STEN_ = 7;
constexpr int NFAC_ = 7;

struct cd {
  double x, y;
};
NSP_HD inline cd cmul(cd a, cd b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }

template <typename T>
struct Strided {
  T* p;
  long long s;
  NSP_HD T& operator[](long long i) const { return p[i * s]; }
};

// Radial tables of one shape (init_fd): grid, first-derivative rows and Laplacian
// rows [2][NR][STEN] (0: even extension, 1: odd).
struct Radial {
  int NR;
  const double* r;
  const double* D;
  const double* Lu;
  const double* Lp;
};

// Doolittle factors of one banded operator (kind 0: u+, 1: u-, 2: u_z, 3: p) row by
// row; the last IW_+1 rows of U live in a ring buffer.  f[i*NFAC_ + e].
template <typename F>
NSP_HD void factor_mode(const Radial& R, double c_im, double inv_dt, int kind, int m, double kt, double kz,
                        bool mode00, F f) {
  const int NR = R.NR;
  const int hD = STEN_ * NR;
  const int odd = kind <= 1 ? 1 : 0;
  const int am = m < 0 ? -m : m;
  const int dt_ = (am % 2) - odd;
  const int tab = dt_ < 0 ? -dt_ : dt_;
  const double* LHS = (kind == 3 ? R.Lp : R.Lu) + tab * hD;
  const double* r = R.r;
  double U[(IW_ + 1) * (IW_ + 1)];  // row q at U[(q % (IW_+1)) * (IW_+1) + j]
  double L[IW_ + 1];
  const bool zz = (kind == 3) && mode00;
  for (int i = 0; i < NR; i++) {
    const int left = i - IW_ > 0 ? i - IW_ : 0, right = i + IW_ < NR - 1 ? i + IW_ : NR - 1;
    const int i0 = i + IW_ - right;
    int coun = 0;
    const bool wall = (i == NR - 1);
    const double r2 = r[i] * r[i];
    for (int j = 0; j < i - left; j++) {
      double XM = LHS[j + i0 + STEN_ * i];
      if (!wall && kind != 3) XM = -(c_im)*XM;
      if (wall && zz) XM = 0.0;
      L[j] = XM;
      coun += 1;
      for (int h = 0; h < j; h++) L[j] -= L[h] * U[((h + left) % (IW_ + 1)) * (IW_ + 1) + j - h];
      L[j] = L[j] / U[((j + left) % (IW_ + 1)) * (IW_ + 1)];
    }
    const int coun2 = coun;
    double* Ui = U + (i % (IW_ + 1)) * (IW_ + 1);
    for (int j = 0; j < right - i + 1; j++) {
      double XM = LHS[STEN_ * i + i0 + coun];
      if (!wall) {
        if (j == 0) {
          if (kind == 0) XM += -(1.0 / r2) - (2.0 * kt / r2) - kz * kz - kt * kt / r2;
          else if (kind == 1) XM += -(1.0 / r2) + (2.0 * kt / r2) - kz * kz - kt * kt / r2;
          else XM += -kz * kz - kt * kt / r2;
          if (kind != 3) XM = inv_dt - c_im * XM;
        } else if (kind != 3) {
          XM = -(c_im)*XM;
        }
      } else if (zz) {
        XM = (j == 0) ? 1.0 : 0.0;
      }
      double Uij = XM;
      const int hleft = coun - IW_ > 0 ? coun - IW_ : 0;
      coun += 1;
      for (int h = hleft; h < i - left; h++) Uij -= L[h] * U[((h + left) % (IW_ + 1)) * (IW_ + 1) + j + coun2 - h];
      Ui[j] = Uij;
    }
    for (int d = 1; d <= IW_; d++) {  // column i-d sits at L[i-d-left]
      const int j = i - d - left;
      f[(long long)i * NFAC_ + IW_ - d] = (j >= 0) ? L[j] : 0.0;
    }
    f[(long long)i * NFAC_ + IW_] = 1.0 / Ui[0];
    for (int d = 1; d <= IW_; d++) f[(long long)i * NFAC_ + IW_ + d] = (i + d <= right) ? Ui[d] : 0.0;
  }
}

// Forward and backward substitution with stored factors (the per-step algorithm).
template <typename F, typename X>
NSP_HD void solve_mode(int NR, F f, X x) {
  for (int i = 0; i < NR; i++) {
    for (int d = (i < IW_ ? i : IW_); d >= 1; d--) {
      const double w = f[(long long)i * NFAC_ + IW_ - d];
      cd xi = x[i];
      const cd xd = x[i - d];
      xi.x -= w * xd.x;
      xi.y -= w * xd.y;
      x[i] = xi;
    }
  }
  for (int i = NR - 1; i >= 0; i--) {
    cd xi = x[i];
    for (int d = 1; d <= IW_ && i + d < NR; d++) {
      const double w = f[(long long)i * NFAC_ + IW_ + d];
      const cd xd = x[i + d];
      xi.x -= w * xd.x;
      xi.y -= w * xd.y;
    }
    const double u = f[(long long)i * NFAC_ + IW_];
    xi.x = xi.x * u;
    xi.y = xi.y * u;
    x[i] = xi;
  }
}

// Wall divergence of a (u_r, u_theta, u_z) mode line (divWall_k, mod_radialFD.cu:34-63);
// the three lines are functors i -> cd.
template <typename A, typename B, typename C>
NSP_HD cd div_wall(const Radial& R, int m, double kt, double kz, A ur, B ut, C uz) {
  const int NR = R.NR;
  const int am = m < 0 ? -m : m;
  const int dt_ = (am % 2) - 1;
  const int tab = dt_ < 0 ? -dt_ : dt_;
  const double* D = R.D + tab * STEN_ * NR + STEN_ * (NR - 1);
  cd p = {0.0, 0.0};
  for (int j = 0; j <= IW_; j++) {
    const cd u = ur(NR - 1 - IW_ + j);
    p.x += D[j + IW_] * u.x;
    p.y += D[j + IW_] * u.y;
  }
  const int w = NR - 1;
  const cd a = ur(w), b = ut(w), c = uz(w);
  p.x += a.x;
  p.y += a.y;
  p.x += -kt * b.y;
  p.y += kt * b.x;
  p.x += -kz * c.y;
  p.y += kz * c.x;
  return p;
}

// Pressure-driven velocity at radius i: grad p_h (derivr flag 0, derivt, derivz).
template <typename P>
NSP_HD void grad_p(const Radial& R, int m, double kt, double kz, P ph, int i, cd* g) {
  const int NR = R.NR;
  const int tab = (m < 0 ? -m : m) % 2;
  const double* D = R.D + tab * STEN_ * NR;
  const int left = i - IW_ > 0 ? i - IW_ : 0, right = i + IW_ < NR - 1 ? i + IW_ : NR - 1;
  const int len = right + 1 - left, i0 = i + IW_ - right;
  cd s = {0.0, 0.0};
  for (int j = 0; j < len; j++) {
    const cd p = ph[left + j];
    s.x += D[STEN_ * i + j + i0] * p.x;
    s.y += D[STEN_ * i + j + i0] * p.y;
  }
  const cd p = ph[i];
  g[0] = s;
  g[1] = cd{-kt * p.y / R.r[i], kt * p.x / R.r[i]};
  g[2] = cd{-kz * p.y, kz * p.x};
}

// Everything of one mode.  fac[op]: factors of operator op; V[c]: correction profile
// of component c (also holds the homogeneous solution u_h,c on the way); ph: scratch
// line for the pressure solution.
template <typename F, typename VA, typename PA>
NSP_HD void setup_mode(const Radial& R, double c_im, double inv_dt, int m, double kt, double kz, bool m00, F fac0,
                       F fac1, F fac2, F fac3, VA V0, VA V1, VA V2, PA ph) {
  const int NR = R.NR;
  F fk[4] = {fac0, fac1, fac2, fac3};
  VA uh[3] = {V0, V1, V2};
  for (int op = 0; op < 4; op++) factor_mode(R, c_im, inv_dt, op, m, kt, kz, m00, fk[op]);
  // Homogeneous solutions: unit wall values (1, 1, i) and pressure with p_wall = -1.
  for (int c = 0; c < 3; c++) {
    for (int i = 0; i < NR; i++) uh[c][i] = cd{0.0, 0.0};
    uh[c][NR - 1] = (c == 2) ? cd{0.0, 1.0} : cd{1.0, 0.0};
    solve_mode(NR, fk[c], uh[c]);
  }
  for (int i = 0; i < NR; i++) ph[i] = cd{0.0, 0.0};
  ph[NR - 1] = cd{-1.0, 0.0};
  solve_mode(NR, fk[3], ph);
  // Wall divergences of the velocity solutions in r/theta form.
  const auto zero = [](int) { return cd{0.0, 0.0}; };
  const VA up = uh[0], um = uh[1], uz = uh[2];
  const cd a41 = div_wall(
      R, m, kt, kz, [&](int i) { const cd u = up[i]; return cd{0.5 * (u.x + 0.0), 0.5 * (u.y + 0.0)}; },
      [&](int i) { const cd u = up[i]; return cd{0.5 * (u.y - 0.0), -0.5 * (u.x - 0.0)}; }, zero);
  const cd a42 = div_wall(
      R, m, kt, kz, [&](int i) { const cd u = um[i]; return cd{0.5 * (0.0 + u.x), 0.5 * (0.0 + u.y)}; },
      [&](int i) { const cd u = um[i]; return cd{0.5 * (0.0 - u.y), -0.5 * (0.0 - u.x)}; }, zero);
  const cd a43 = div_wall(R, m, kt, kz, zero, zero, [&](int i) { return uz[i]; });
  // Pressure-driven velocity and its wall divergence.
  const cd a44 = div_wall(
      R, m, kt, kz, [&](int i) { cd g[3]; grad_p(R, m, kt, kz, ph, i, g); return g[0]; },
      [&](int i) { cd g[3]; grad_p(R, m, kt, kz, ph, i, g); return g[1]; },
      [&](int i) { cd g[3]; grad_p(R, m, kt, kz, ph, i, g); return g[2]; });
  // Wall values of the pressure-driven velocity in +/- form.
  cd gw[3];
  grad_p(R, m, kt, kz, ph, NR - 1, gw);
  const cd a14 = cd{gw[0].x - gw[1].y, gw[0].y + gw[1].x}, a24 = cd{gw[0].x + gw[1].y, gw[0].y - gw[1].x};
  const cd a34 = gw[2];
  cd ax, Det;
  ax.x = a44.x - a24.x * a42.x + a24.y * a42.y - a14.x * a41.x + a14.y * a41.y;
  ax.y = a44.y - a24.x * a42.y - a24.y * a42.x - a14.x * a41.y - a14.y * a41.x;
  Det.x = -ax.y - a34.x * a43.x + a34.y * a43.y;
  Det.y = ax.x - a34.x * a43.y - a34.y * a43.x;
  const double D1 = Det.x * Det.x + Det.y * Det.y;
  const cd iDet = {Det.x / D1, -Det.y / D1};
  cd col3[4] = {cd{a14.y, -a14.x}, cd{a24.y, -a24.x}, cd{-a34.x, -a34.y}, cd{0.0, 1.0}};
  for (int j = 0; j < 4; j++) col3[j] = cmul(col3[j], iDet);
  // Mode (0,0): p_h is constant, so grad p_h and the determinant vanish in exact
  // arithmetic and the reference inverts rounding noise (0/0 = NaN when the noise is
  // exactly zero).  The exact correction only changes u_r(0,0), which modeZZ sets to
  // zero, so no correction is applied to this mode.
  if (m00)
    for (int j = 0; j < 4; j++) col3[j] = cd{0.0, 0.0};
  for (int i = 0; i < NR; i++) {
    cd g[3];
    grad_p(R, m, kt, kz, ph, i, g);
    const cd uP[3] = {cd{g[0].x - g[1].y, g[0].y + g[1].x}, cd{g[0].x + g[1].y, g[0].y - g[1].x}, g[2]};
    for (int c = 0; c < 3; c++) {
      const cd v1 = cmul(col3[c], uh[c][i]), v2 = cmul(col3[3], uP[c]);
      uh[c][i] = cd{v1.x + v2.x, v1.y + v2.y};
    }
  }
}

}  // namespace setup
}  // namespace nsp
