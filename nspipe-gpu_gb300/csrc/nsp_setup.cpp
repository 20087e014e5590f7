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
#include "nsp_setup_mode.h"

namespace nsp {

namespace {

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

setup::Radial radial_view(const HostOps& o) { return setup::Radial{o.NR, o.r.data(), o.D.data(), o.Lu.data(), o.Lp.data()}; }

}  // namespace

// Factors and correction profiles of every mode of one parameter set, on the host:
// fac [4][NR][NFAC][NTNZ], V [3][NR][NTNZ].  Each mode is built in contiguous
// temporaries by the shared per-mode code, then scattered into the tables.
void mode_tables(const nsp_params& p, const HostOps& o, double* fac, double2* V) {
  using setup::cd;
  using setup::Strided;
  const int NR = p.NR, NT = p.NT, NZ = p.NZ;
  const long long NTNZ = (long long)NT * NZ;
  const setup::Radial R = radial_view(o);
  const double c_im = p.d_im / p.Re, inv_dt = 1.0 / p.dt;
  const double kts = PI2 / p.LT, kzs = PI2 / p.LZ;
  std::vector<double> fk((size_t)4 * NR * NFAC);
  std::vector<cd> vk((size_t)3 * NR), ph(NR);
  for (long long k = 0; k < NTNZ; k++) {
    const int it = (int)(k / NZ), l = (int)(k % NZ);
    const int m = it < NT / 2 ? it : it - NT;
    const double kt = kts * (double)m, kz = kzs * (double)l;
    Strided<double> f[4];
    Strided<cd> v[3];
    for (int op = 0; op < 4; op++) f[op] = Strided<double>{fk.data() + (size_t)op * NR * NFAC, 1};
    for (int c = 0; c < 3; c++) v[c] = Strided<cd>{vk.data() + (size_t)c * NR, 1};
    setup::setup_mode(R, c_im, inv_dt, m, kt, kz, m == 0 && l == 0, f[0], f[1], f[2], f[3], v[0], v[1], v[2],
                      Strided<cd>{ph.data(), 1});
    for (size_t e = 0; e < fk.size(); e++) fac[e * NTNZ + k] = fk[e];
    for (size_t e = 0; e < vk.size(); e++) V[e * NTNZ + k] = double2{vk[e].x, vk[e].y};
  }
}

// Flux response: u_z-Helmholtz with unit right-hand side, zero wall value, mode (0,0)
// (setCublasFlux, mod_cublasflux.cu:56-81).
void flux_response(const nsp_params& p, const HostOps& o, std::vector<double>& uc, double& Qc) {
  using setup::cd;
  using setup::Strided;
  const int NR = p.NR;
  std::vector<double> f((size_t)NR * NFAC);
  std::vector<cd> x(NR, cd{1.0, 0.0});
  x[NR - 1] = cd{0.0, 0.0};
  setup::factor_mode(radial_view(o), p.d_im / p.Re, 1.0 / p.dt, 2, 0, 0.0, 0.0, true, Strided<double>{f.data(), 1});
  setup::solve_mode(NR, Strided<double>{f.data(), 1}, Strided<cd>{x.data(), 1});
  uc.resize(NR);
  double Q = 0.0;
  for (int i = 0; i < NR; i++) {
    uc[i] = x[i].x;
    Q += o.rdr[i] * uc[i];
  }
  Qc = Q;
}

}  // namespace nsp
