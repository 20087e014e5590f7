/* nsp_oracle.c -- CPU FP64 restatement of the nsPipe-CUDA per-step path.
 *
 * TEST INFRASTRUCTURE (the parity oracle and the timed host baseline).  It is
 * loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU legs; the
 * product library never links it.  Built with -ffp-contract=off so the host
 * result does not depend on whether the compiler fuses multiply-adds (x86 and
 * aarch64 give identical bits).
 *
 * Each routine restates one function of the reference (Mordered/nsPipe-GPU,
 * Main_Code/src), keeping its operation order so that results agree with the
 * reference build to rounding.  The reference's 2-D cuFFT transforms
 * (mod_fft.cu:21-48) are replaced by a mixed-radix (2/3/4) FFT written here,
 * with twiddles from long-double cos/sin.
 *
 * One deliberate difference: the quadrature loop of init_fd
 * (mod_radialFD.cu:272-279) reads c[ir+k*len] for k == len, which for len == 7
 * is past the end of the 49-entry weight buffer (heap contents).  The value
 * multiplies h^8/8! (< 1e-14) and is taken as 0 here.
 */
#include "nsp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI2 6.283185307179586 /* head.h:12 */
#define PI_L 3.141592653589793238462643383279502884L

typedef struct { double x, y; } c2;

/* ---------------------------------------------------------------- FFT ---- */
typedef struct { int n; c2* w; } cplan; /* w[e] = exp(-2*pi*i*e/n) */

static void plan_init(cplan* P, int n) {
  P->n = n;
  P->w = (c2*)malloc(sizeof(c2) * (size_t)n);
  for (int e = 0; e < n; e++) {
    long long e4 = 4LL * e;
    if (e4 % n == 0) {             /* quarter turns: exact */
      int q = (int)(e4 / n) & 3;
      static const double cx[4] = {1.0, 0.0, -1.0, 0.0};
      static const double sy[4] = {0.0, -1.0, 0.0, 1.0};
      P->w[e].x = cx[q];
      P->w[e].y = sy[q];
    } else {
      long double a = -2.0L * PI_L * (long double)e / (long double)n;
      P->w[e].x = (double)cosl(a);
      P->w[e].y = (double)sinl(a);
    }
  }
}

static inline c2 tw(const cplan* P, long long e, int sign) {
  c2 w = P->w[e % P->n];
  if (sign > 0) w.y = -w.y;
  return w;
}

static inline c2 cmul(c2 a, c2 b) {
  c2 r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}

/* out[k] = sum_j in[j*is] * exp(sign*2*pi*i*j*k/n); n = P->n / tws. */
static void fft_rec(const c2* in, size_t is, c2* out, int n, int tws, const cplan* P, int sign) {
  if (n == 1) { out[0] = in[0]; return; }
  int p = (n % 4 == 0) ? 4 : (n % 2 == 0) ? 2 : 3;
  int m = n / p;
  for (int q = 0; q < p; q++) fft_rec(in + q * is, is * (size_t)p, out + q * m, m, tws * p, P, sign);
  int wp = P->n / p; /* table stride of the p-point roots */
  for (int k = 0; k < m; k++) {
    c2 t[4], y[4];
    for (int q = 0; q < p; q++) {
      t[q] = out[q * m + k];
      if (q && k) t[q] = cmul(t[q], tw(P, (long long)q * k * tws, sign));
    }
    for (int s = 0; s < p; s++) {
      c2 acc = t[0];
      for (int q = 1; q < p; q++) {
        c2 v = cmul(t[q], tw(P, (long long)((q * s) % p) * wp, sign));
        acc.x += v.x;
        acc.y += v.y;
      }
      y[s] = acc;
    }
    for (int s = 0; s < p; s++) out[s * m + k] = y[s];
  }
}

/* --------------------------------------------------------------- context -- */
struct orc_ctx {
  orc_params p;
  int NR, NT, NZ, sten, iw, NTP, NZP, NZR;
  size_t S, NTNZ;
  double c_im, c_ex, inv_dt, two_re; /* d_im/Re, (1-d_im)/Re, 1/dt, 2/Re */
  double *r, *rdr, *D, *Lu, *Lp, *dr0;
  c2 *uh_r, *uh_t, *uh_z, *uhP_r, *uhP_t, *uhP_z, *invM, *div1, *coef;
  double* uc;
  double Qc;
  cplan pt, pz;
  c2 *rhs[3], *uw[3], *rhsw[3], *ui[3], *dur[3];
  double *d1, *d2;
};

static inline double dmax(double a, double b) { return fmax(a, b); } /* CUDA max() on doubles */

static inline int signed_mode(const orc_ctx* c, int it) { return it < c->NT / 2 ? it : it - c->NT; }
static inline double kt_of(const orc_ctx* c, int m) { return (PI2 / c->p.LT) * (double)m; }
static inline double kz_of(const orc_ctx* c, int l) { return (PI2 / c->p.LZ) * (double)l; }

/* Each call sets its context's thread count (0: every processor), so that a context
 * with an explicit count leaves no lasting setting for the others. */
static void set_threads(const orc_ctx* c) {
#ifdef _OPENMP
  omp_set_num_threads(c->p.nthreads > 0 ? c->p.nthreads : omp_get_num_procs());
#else
  (void)c;
#endif
}

/* ------------------------------------------------- radial FD (setup) ----- */
/* fd_weights: mod_radialFD.cu:365-395 (Fornberg's recursion). c has csz
 * entries laid out c[j + n*k] (point j, derivative k). */
static void fd_weights(double* c, int csz, const double* rau, int row, int left, int right, int m, int iw) {
  int n = 1 + right - left;
  double x[64];
  double x0 = rau[row + iw];
  for (int i = 0; i < csz; i++) c[i] = 0.0;
  c[0] = 1.0;
  double c1 = 1.0, c2v, c3, c4, c5;
  for (int i = 0; i < n; i++) x[i] = rau[i + row];
  c4 = x[0] - x0;
  for (int i = 1; i < n; i++) {
    int mn = i < m ? i : m;
    c2v = 1.0;
    c5 = c4;
    c4 = x[i] - x0;
    for (int j = 0; j < i; j++) {
      c3 = x[i] - x[j];
      c2v = c2v * c3;
      if (j == i - 1) {
        for (int k = mn; k > 0; k--) c[i + n * k] = c1 * ((double)k * c[i - 1 + n * (k - 1)] - c5 * c[i - 1 + n * k]) / c2v;
        c[i] = -c1 * c5 * c[i - 1] / c2v;
      }
      for (int k = mn; k > 0; k--) c[j + n * k] = (c4 * c[j + n * k] - (double)k * c[j + (k - 1) * n]) / c3;
      c[j] = c4 * c[j] / c3;
    }
    c1 = c2v;
  }
}

/* init_fd: mod_radialFD.cu:199-312. */
static void init_fd(orc_ctx* c) {
  int NR = c->NR, sten = c->sten, iw = c->iw, hD = sten * NR;
  double* r = c->r;
  double* rau = (double*)calloc((size_t)(NR + iw), sizeof(double));
  double* r_i = (double*)calloc((size_t)(NR + 1), sizeof(double));
  double* D2 = (double*)calloc((size_t)(2 * hD), sizeof(double));
  int csz = sten * sten;
  double* cw = (double*)calloc((size_t)csz + 64, sizeof(double)); /* tail reads as 0 */
  double* D = c->D;
  for (int i = 0; i < 2 * hD; i++) { D[i] = 0.0; D2[i] = 0.0; }
  for (int i = 0; i < NR; i++) c->rdr[i] = 0.0;
  /* 0.0 grid (:211-216) */
  int N_p = NR + (int)sqrt((double)NR);
  for (int i = N_p - NR; i < N_p; i++) {
    int ir = N_p - i - 1;
    r[i - N_p + NR] = 0.5 * (1.0 + cos(0.5 * PI2 * ((double)ir / (double)N_p)));
  }
  for (int it = 0; it < 10; it++) {
    double dr = 1.5 * r[0] - 0.5 * r[1];
    for (int j = 0; j < NR; j++) r[j] = r[j] * (1.0 + dr) - dr;
  }
  /* 0.1 auxiliary grids (:218-219) */
  for (int i = 0; i < NR; i++) r_i[i + 1] = r[i];
  r_i[0] = 0.0;
  for (int i = 0; i < NR + iw; i++) rau[i] = (i < iw) ? -r[iw - i - 1] : r[i - iw];
  /* 1 derivative weights (:221-252) */
  int coun = iw;
  for (int i = 0; i < NR; i++) {
    int left = i, right = (iw + iw + i < NR + iw - 1) ? iw + iw + i : NR + iw - 1;
    int len = 1 + right - left;
    fd_weights(cw, csz, rau, i, left, right, 2, iw);
    if (i < iw) {
      for (int j = 0; j < len; j++) {
        int ir;
        if (j < coun) {
          ir = coun - j - 1;
          D[ir + sten * i] += cw[len + j];
          D[hD + ir + sten * i] -= cw[len + j];
          D2[ir + sten * i] += cw[2 * len + j];
          D2[hD + ir + sten * i] -= cw[2 * len + j];
        } else {
          ir = j - coun;
          D[ir + sten * i] += cw[len + j];
          D[hD + ir + sten * i] += cw[len + j];
          D2[ir + sten * i] += cw[2 * len + j];
          D2[hD + ir + sten * i] += cw[2 * len + j];
        }
      }
      coun -= 1;
    } else {
      int i0 = sten - len;
      for (int j = 0; j < len; j++) {
        int ir = i0 + j;
        D[ir + sten * i] += cw[len + j];
        D[hD + ir + sten * i] += cw[len + j];
        D2[ir + sten * i] += cw[2 * len + j];
        D2[hD + ir + sten * i] += cw[2 * len + j];
      }
    }
  }
  /* 2 integration weights rdr (:255-280) */
  coun = iw;
  for (int i = 0; i < NR; i++) {
    int left = i, right = (iw + iw + i < NR + iw - 1) ? iw + iw + i : NR + iw - 1;
    int len = 1 + right - left, left2 = (i - iw > 0) ? i - iw : 0;
    fd_weights(cw, csz, rau, i, left, right, len - 1, iw);
    for (int t = csz; t < csz + 64; t++) cw[t] = 0.0;
    int i0 = 0;
    double e1 = 1.0, e2 = 1.0;
    if (i < iw) {
      i0 = coun;
      for (int j = 0; j < coun; j++) {
        int ir = coun + coun - 1 - j;
        for (int k = 0; k < len; k++) cw[ir + k * len] += cw[j + k * len];
      }
      coun -= 1;
    }
    for (int k = 0; k < len + 1; k++) {
      int ip2 = (i + 2 < NR) ? i + 2 : NR;
      e1 = e1 * (r_i[ip2] - r_i[i + 1]) / ((double)(k + 1));
      e2 = e2 * (r_i[i] - r_i[i + 1]) / ((double)(k + 1));
      for (int j = 0; j < len - i0; j++) {
        int ir = i0 + j;
        c->rdr[left2 + j] += (e1 - e2) * r[i] * cw[ir + k * len];
      }
    }
  }
  /* 3 radial Laplacian rows (:282-302) */
  for (int i = 0; i < NR; i++) {
    if (i < NR - 1) {
      for (int j = 0; j < sten; j++) {
        int ir = j + sten * i;
        c->Lu[ir] = D2[ir] + D[ir] / r[i];
        c->Lu[hD + ir] = D2[hD + ir] + D[hD + ir] / r[i];
        c->Lp[ir] = D2[ir] + D[ir] / r[i];
        c->Lp[hD + ir] = D2[hD + ir] + D[hD + ir] / r[i];
      }
    } else {
      for (int j = 0; j < sten; j++) {
        int ir = j + sten * i;
        if (j < sten - 1) { c->Lu[ir] = 0.0; c->Lu[hD + ir] = 0.0; }
        else { c->Lu[ir] = 1.0; c->Lu[hD + ir] = 1.0; }
        c->Lp[ir] = D[ir];
        c->Lp[hD + ir] = D[hD + ir];
      }
    }
  }
  /* get_dr0: mod_radialFD.cu:316-350 (Lagrange weights to r = 0, m = 0). */
  {
    int n = iw + 1;
    double x[64], cc[64];
    for (int i = 0; i < n; i++) cc[i] = 0.0;
    cc[0] = 1.0;
    double c1 = 1.0, c2v, c3, c4, c5, x0 = 0.0;
    for (int i = 0; i < n; i++) x[i] = r[i];
    c4 = x[0] - x0;
    for (int i = 1; i < n; i++) {
      c2v = 1.0;
      c5 = c4;
      c4 = x[i] - x0;
      for (int j = 0; j < i; j++) {
        c3 = x[i] - x[j];
        c2v = c2v * c3;
        if (j == i - 1) cc[i] = -c1 * c5 * cc[i - 1] / c2v;
        cc[j] = c4 * cc[j] / c3;
      }
      c1 = c2v;
    }
    for (int i = 0; i < n; i++) c->dr0[i] = cc[i];
  }
  free(rau); free(r_i); free(D2); free(cw);
}

/* ------------------------------------------------------ spectral ops ----- */
/* derivr_k: mod_radialFD.cu:10-30. */
static void derivr(orc_ctx* c, c2* dur, const c2* u, int flag) {
  int NR = c->NR, NT = c->NT, NZ = c->NZ, sten = c->sten, iw = c->iw;
  size_t NTNZ = c->NTNZ;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < NR; i++) {
    for (size_t k = 0; k < NTNZ; k++) {
      int it = signed_mode(c, (int)(k / NZ));
      int left = i - iw > 0 ? i - iw : 0, right = i + iw < NR - 1 ? i + iw : NR - 1;
      int ip0 = abs((abs(it) % 2) - flag) * sten * NR;
      int len = right + 1 - left, i0 = i + iw - right;
      c2 prod = {0.0, 0.0};
      for (int j = 0; j < len; j++) {
        double de = c->D[ip0 + sten * i + j + i0];
        c2 a = u[(size_t)(left + j) * NTNZ + k];
        prod.x += de * a.x;
        prod.y += de * a.y;
      }
      dur[(size_t)i * NTNZ + k] = prod;
    }
  }
  (void)NT;
}

/* derivt_k / derivz_k: mod_deriv.cu:10-35. */
static void derivt(orc_ctx* c, c2* g, const c2* u) {
  size_t NTNZ = c->NTNZ;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->NR; i++)
    for (size_t k = 0; k < NTNZ; k++) {
      double kt = kt_of(c, signed_mode(c, (int)(k / c->NZ)));
      size_t h = (size_t)i * NTNZ + k;
      c2 a = u[h];
      g[h].x = -kt * a.y / c->r[i];
      g[h].y = kt * a.x / c->r[i];
    }
}
static void derivz(orc_ctx* c, c2* g, const c2* u) {
  size_t NTNZ = c->NTNZ;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->NR; i++)
    for (size_t k = 0; k < NTNZ; k++) {
      double kz = kz_of(c, (int)(k % c->NZ));
      size_t h = (size_t)i * NTNZ + k;
      c2 a = u[h];
      g[h].x = -kz * a.y;
      g[h].y = kz * a.x;
    }
}

/* div_k: mod_radialFD.cu:67-96. */
static void divergence(orc_ctx* c, c2* div, const c2* ur, const c2* ut, const c2* uz) {
  int NR = c->NR, NZ = c->NZ, sten = c->sten, iw = c->iw;
  size_t NTNZ = c->NTNZ;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < NR; i++)
    for (size_t k = 0; k < NTNZ; k++) {
      size_t h = (size_t)i * NTNZ + k;
      int l = (int)(k % NZ), it = signed_mode(c, (int)(k / NZ));
      int left = i - iw > 0 ? i - iw : 0, right = i + iw < NR - 1 ? i + iw : NR - 1;
      double kt = kt_of(c, it), kz = kz_of(c, l);
      int ip0 = abs((abs(it) % 2) - 1) * sten * NR;
      double rK = c->r[i];
      int len = right + 1 - left, i0 = i + iw - right;
      c2 prod = {0.0, 0.0};
      for (int j = 0; j < len; j++) {
        double de = c->D[ip0 + sten * i + j + i0];
        c2 a = ur[(size_t)(left + j) * NTNZ + k];
        prod.x += de * a.x;
        prod.y += de * a.y;
      }
      prod.x += ur[h].x / rK;
      prod.y += ur[h].y / rK;
      prod.x += -kt * ut[h].y / rK;
      prod.y += kt * ut[h].x / rK;
      prod.x += -kz * uz[h].y;
      prod.y += kz * uz[h].x;
      div[h] = prod;
    }
}

/* divWall_k: mod_radialFD.cu:34-63 (wall row i = NR-1, r = 1). */
static void div_wall(orc_ctx* c, c2* div1, const c2* ur, const c2* ut, const c2* uz) {
  int NR = c->NR, NZ = c->NZ, sten = c->sten, iw = c->iw;
  size_t NTNZ = c->NTNZ;
  int i = NR - 1;
#pragma omp parallel for schedule(static)
  for (size_t k = 0; k < NTNZ; k++) {
    size_t h = (size_t)i * NTNZ + k;
    int l = (int)(k % NZ), it = signed_mode(c, (int)(k / NZ));
    int left = i - iw, right = NR - 1;
    double kt = kt_of(c, it), kz = kz_of(c, l);
    int ip0 = abs((abs(it) % 2) - 1) * sten * NR;
    int len = right + 1 - left, i0 = i + iw - right;
    c2 prod = {0.0, 0.0};
    for (int j = 0; j < len; j++) {
      double de = c->D[ip0 + sten * i + j + i0];
      c2 a = ur[(size_t)(left + j) * NTNZ + k];
      prod.x += de * a.x;
      prod.y += de * a.y;
    }
    prod.x += ur[h].x;
    prod.y += ur[h].y;
    prod.x += -kt * ut[h].y;
    prod.y += kt * ut[h].x;
    prod.x += -kz * uz[h].y;
    prod.y += kz * uz[h].x;
    div1[k] = prod;
  }
}

/* pressGrad_k: mod_radialFD.cu:100-111. */
static void press_grad(orc_ctx* c, c2* duz, const c2* uz) {
  int NR = c->NR, sten = c->sten, iw = c->iw;
  int iE = NR - 1, left = iE - iw, right = NR - 1, i0 = iE + iw - right, len = right + 1 - left;
  double du = 0.0;
  for (int j = 0; j < len; j++) du += c->D[sten * iE + j + i0] * uz[(size_t)(left + j) * c->NTNZ].x;
  for (int i = 0; i < NR; i++) duz[(size_t)i * c->NTNZ].x -= c->two_re * du;
}

/* addGrad_k: mod_radialFD.cu:115-143. */
static void add_grad(orc_ctx* c, c2* rr, c2* rt, c2* rz, const c2* p) {
  int NR = c->NR, NZ = c->NZ, sten = c->sten, iw = c->iw;
  size_t NTNZ = c->NTNZ;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < NR; i++)
    for (size_t k = 0; k < NTNZ; k++) {
      size_t h = (size_t)i * NTNZ + k;
      int l = (int)(k % NZ), it = signed_mode(c, (int)(k / NZ));
      int left = i - iw > 0 ? i - iw : 0, right = i + iw < NR - 1 ? i + iw : NR - 1;
      double kt = kt_of(c, it), kz = kz_of(c, l);
      int ip0 = abs((abs(it) % 2) - 0) * sten * NR;
      double rK = c->r[i];
      int len = right + 1 - left, i0 = i + iw - right;
      c2 prod = {0.0, 0.0};
      for (int j = 0; j < len; j++) {
        double de = c->D[ip0 + sten * i + j + i0];
        c2 a = p[(size_t)(left + j) * NTNZ + k];
        prod.x += de * a.x;
        prod.y += de * a.y;
      }
      rr[h].x -= prod.x;
      rr[h].y -= prod.y;
      rt[h].x -= -kt * p[h].y / rK;
      rt[h].y -= kt * p[h].x / rK;
      rz[h].x -= -kz * p[h].y;
      rz[h].y -= kz * p[h].x;
    }
}

/* addLap_k: mod_linear.cu:12-51. flag 0: u+, 1: u-, 2: uz. */
static void add_lap(orc_ctx* c, c2* rhs, const c2* u, int flag) {
  int NR = c->NR, NZ = c->NZ, sten = c->sten, iw = c->iw;
  size_t NTNZ = c->NTNZ;
  int fp = abs(flag - 3) / 2;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < NR; i++)
    for (size_t k = 0; k < NTNZ; k++) {
      size_t h = (size_t)i * NTNZ + k;
      int l = (int)(k % NZ), it = signed_mode(c, (int)(k / NZ));
      int ip0 = abs((abs(it) % 2) - fp) * sten * NR;
      double kz = kz_of(c, l), kt = kt_of(c, it);
      int left = i - iw > 0 ? i - iw : 0, right = i + iw < NR - 1 ? i + iw : NR - 1;
      int len = right + 1 - left, i0 = i + iw - right;
      c2 prod = {0.0, 0.0};
      for (int j = 0; j < len; j++) {
        double de = c->Lu[ip0 + sten * i + j + i0];
        c2 a = u[(size_t)(left + j) * NTNZ + k];
        prod.x += de * a.x;
        prod.y += de * a.y;
      }
      c2 aux = u[h];
      double r2 = c->r[i] * c->r[i];
      double de = -kz * kz - kt * kt / r2;
      if (flag == 0) de += -(1.0 / r2) - (2.0 * kt / r2);
      else if (flag == 1) de += -(1.0 / r2) + (2.0 * kt / r2);
      prod.x += de * aux.x;
      prod.y += de * aux.y;
      prod.x *= c->c_ex;
      prod.y *= c->c_ex;
      prod.x += c->inv_dt * aux.x;
      prod.y += c->inv_dt * aux.y;
      rhs[h].x += prod.x;
      rhs[h].y += prod.y;
    }
}

/* Banded LU (Doolittle, no pivoting) factorised and solved per mode line:
 * LUsolve_up_k / um_k / uz_k / p_k, mod_linear.cu:55-646.  kind 0: u+,
 * 1: u-, 2: uz, 3: p.  Row i's packed entry e is column left + e - i0. */
static void lu_line(orc_ctx* c, c2* sol, const c2* rhs, size_t k, int kind) {
  int NR = c->NR, NZ = c->NZ, sten = c->sten, iw = c->iw;
  size_t NTNZ = c->NTNZ;
  int l = (int)(k % NZ), it = signed_mode(c, (int)(k / NZ));
  double kz = kz_of(c, l), kt = kt_of(c, it);
  int odd = (kind <= 1) ? 1 : 0;
  int ip0 = abs((abs(it) % 2) - odd) * sten * NR;
  const double* LHS = (kind == 3) ? c->Lp : c->Lu;
  int zz = (kind == 3) && abs(l) < 1 && abs(it) < 1;
  double L[16], U[16 * 256];
  c2 x[1024];
  int W = 1 + iw;
  for (int i = 0; i < NR; i++) {
    int left = i - iw > 0 ? i - iw : 0, right = i + iw < NR - 1 ? i + iw : NR - 1;
    int i0 = i + iw - right, coun = 0;
    int wall = (i == NR - 1);
    double r2 = c->r[i] * c->r[i];
    L[i - left] = 1.0;
    x[i] = rhs[(size_t)i * NTNZ + k];
    /* 1.1 columns in L */
    for (int j = 0; j < i - left; j++) {
      double XM = LHS[ip0 + j + i0 + sten * i];
      if (!wall && kind != 3) XM = -(c->c_im) * XM;
      if (wall && zz) XM = 0.0;
      L[j] = XM;
      coun += 1;
      if (j > 0)
        for (int hh = 0; hh < j; hh++) L[j] -= L[hh] * U[W * (hh + left) + j - hh];
      L[j] = L[j] / U[(j + left) * W];
      x[i].x -= L[j] * x[j + left].x;
      x[i].y -= L[j] * x[j + left].y;
    }
    int coun2 = coun;
    /* 1.2 columns in U */
    for (int j = 0; j < right - i + 1; j++) {
      double XM = LHS[ip0 + sten * i + i0 + coun];
      if (!wall) {
        if (j == 0) {
          if (kind == 0) XM += -(1.0 / r2) - (2.0 * kt / r2) - kz * kz - kt * kt / r2;
          else if (kind == 1) XM += -(1.0 / r2) + (2.0 * kt / r2) - kz * kz - kt * kt / r2;
          else XM += -kz * kz - kt * kt / r2;
          if (kind != 3) XM = c->inv_dt - c->c_im * XM;
        } else if (kind != 3) {
          XM = -(c->c_im) * XM;
        }
      } else if (zz) {
        XM = 0.0;
        if (j == 0) XM = 1.0;
      }
      U[j + W * i] = XM;
      int hleft = coun - iw > 0 ? coun - iw : 0;
      coun += 1;
      if (hleft < i - left)
        for (int hh = hleft; hh < i - left; hh++) U[j + W * i] -= L[hh] * U[W * (hh + left) + j + coun2 - hh];
    }
  }
  /* 3 backward substitution */
  int i = NR - 1;
  x[i].x = x[i].x / U[i * W];
  x[i].y = x[i].y / U[i * W];
  sol[(size_t)i * NTNZ + k] = x[i];
  for (i = NR - 2; i > -1; i--) {
    int right = i + iw < NR - 1 ? i + iw : NR - 1;
    for (int j = 1; j < right - i + 1; j++) {
      x[i].x -= U[i * W + j] * x[i + j].x;
      x[i].y -= U[i * W + j] * x[i + j].y;
    }
    x[i].x = x[i].x / U[i * W];
    x[i].y = x[i].y / U[i * W];
    sol[(size_t)i * NTNZ + k] = x[i];
  }
}

static void lusolve(orc_ctx* c, c2* sol, const c2* rhs, int kind) {
#pragma omp parallel for schedule(static)
  for (size_t k = 0; k < c->NTNZ; k++) lu_line(c, sol, rhs, k, kind);
}

/* mod_utils.cu:20-59 */
static void write_bcon(orc_ctx* c, c2* rhs, c2 b) {
  for (size_t k = 0; k < c->NTNZ; k++) rhs[(size_t)(c->NR - 1) * c->NTNZ + k] = b;
}
static void decouple_fwd(orc_ctx* c, c2* ur, c2* ut) {
#pragma omp parallel for schedule(static)
  for (size_t h = 0; h < c->S; h++) {
    c2 a = ur[h], b = ut[h], up, um;
    up.x = a.x - b.y; up.y = a.y + b.x;
    um.x = a.x + b.y; um.y = a.y - b.x;
    ur[h] = up; ut[h] = um;
  }
}
static void decouple_bwd(orc_ctx* c, c2* up, c2* um) {
#pragma omp parallel for schedule(static)
  for (size_t h = 0; h < c->S; h++) {
    c2 p = up[h], m = um[h], ur, ut;
    ur.x = 0.5 * (p.x + m.x); ur.y = 0.5 * (p.y + m.y);
    ut.x = 0.5 * (p.y - m.y); ut.y = -0.5 * (p.x - m.x);
    up[h] = ur; um[h] = ut;
  }
}
static void fill(orc_ctx* c, c2* u, c2 v) { for (size_t h = 0; h < c->S; h++) u[h] = v; }
static void copyf(orc_ctx* c, c2* dst, const c2* src) { memcpy(dst, src, sizeof(c2) * c->S); }

/* ------------------------------------------------- 2-D transforms -------- */
/* One radial level, inverse: padForward (mod_io_nonlinear.cu:173-192) +
 * Z2D 2-D transform dims {NTP, 2NZP-2} (mod_fft.cu:25-26,45-48).
 * spec: c2[NT][NZ]; phys: double[NTP][NZR]; g: scratch c2[NTP][NZP]. */
static void level_backward(orc_ctx* c, const c2* spec, double* phys, c2* g, c2* col, c2* tmp) {
  int NT = c->NT, NZ = c->NZ, NTP = c->NTP, NZP = c->NZP, NZR = c->NZR;
  for (int q = 0; q < NZ; q++) {
    for (int pp = 0; pp < NTP; pp++) {
      c2 a = {0.0, 0.0};
      if (pp < NT / 2) a = spec[pp * NZ + q];
      else if (pp > NT - 1) a = spec[(pp - NT / 2) * NZ + q];
      col[pp] = a;
    }
    fft_rec(col, 1, tmp, NTP, 1, &c->pt, +1);
    for (int pp = 0; pp < NTP; pp++) g[pp * NZP + q] = tmp[pp];
  }
  for (int pp = 0; pp < NTP; pp++) {
    /* C2R of length NZR: Hermitian extension, complex inverse, real part. */
    for (int q = 0; q < NZR; q++) col[q].x = col[q].y = 0.0;
    for (int q = 0; q < NZ && q <= NZR / 2; q++) col[q] = g[pp * NZP + q];
    for (int q = 1; q < NZ && q < NZR / 2; q++) { col[NZR - q].x = g[pp * NZP + q].x; col[NZR - q].y = -g[pp * NZP + q].y; }
    fft_rec(col, 1, tmp, NZR, 1, &c->pz, +1);
    for (int n = 0; n < NZR; n++) phys[(size_t)pp * NZR + n] = tmp[n].x;
  }
}

/* One radial level, forward: D2Z + normalize (mod_fft.cu:37-42,
 * mod_utils.cu:10-17) + padBackward (mod_io_nonlinear.cu:195-214). */
static void level_forward(orc_ctx* c, const double* phys, c2* spec, c2* g, c2* col, c2* tmp) {
  int NT = c->NT, NZ = c->NZ, NTP = c->NTP, NZP = c->NZP, NZR = c->NZR;
  double norm = (double)NTP * (double)NZR;
  for (int pp = 0; pp < NTP; pp++) {
    for (int n = 0; n < NZR; n++) { col[n].x = phys[(size_t)pp * NZR + n]; col[n].y = 0.0; }
    fft_rec(col, 1, tmp, NZR, 1, &c->pz, -1);
    for (int q = 0; q < NZ; q++) g[pp * NZP + q] = tmp[q];
  }
  for (int q = 0; q < NZ; q++) {
    for (int pp = 0; pp < NTP; pp++) col[pp] = g[pp * NZP + q];
    fft_rec(col, 1, tmp, NTP, 1, &c->pt, -1);
    for (int it = 0; it < NT; it++) {
      int ip = it < NT / 2 ? it : NTP + (it - NT);
      c2 a = tmp[ip];
      a.x = a.x / norm;
      a.y = a.y / norm;
      if (it == NT / 2 || q == NZ - 1) { a.x = 0.0; a.y = 0.0; }
      spec[it * NZ + q] = a;
    }
  }
}

/* nonlinear: mod_io_nonlinear.cu:380-409 with calcNonlinear_k :142-170,
 * evaluated one radial level at a time. */
static void nonlinear(orc_ctx* c, const c2* ur, const c2* ut, const c2* uz, c2* nr, c2* nt, c2* nz) {
  const c2* u[3] = {ur, ut, uz};
  derivr(c, c->dur[0], ur, 1);
  derivr(c, c->dur[1], ut, 1);
  derivr(c, c->dur[2], uz, 0);
  int NR = c->NR, NT = c->NT, NZ = c->NZ, NTP = c->NTP, NZP = c->NZP, NZR = c->NZR;
  size_t NTNZ = c->NTNZ, PL = (size_t)NTP * NZR;
  c2* out[3] = {nr, nt, nz};
#pragma omp parallel
  {
    double* ph = (double*)malloc(sizeof(double) * PL * 12);
    c2* spec = (c2*)malloc(sizeof(c2) * NTNZ);
    c2* g = (c2*)malloc(sizeof(c2) * (size_t)NTP * NZP);
    int nmax = NTP > NZR ? NTP : NZR;
    c2* col = (c2*)malloc(sizeof(c2) * nmax);
    c2* tmp = (c2*)malloc(sizeof(c2) * nmax);
#pragma omp for schedule(dynamic, 1)
    for (int i = 0; i < NR; i++) {
      const c2* ul[3];
      for (int f = 0; f < 3; f++) ul[f] = u[f] + (size_t)i * NTNZ;
      double rK = c->r[i];
      for (int f = 0; f < 3; f++) {
        level_backward(c, ul[f], ph + PL * f, g, col, tmp);
        level_backward(c, c->dur[f] + (size_t)i * NTNZ, ph + PL * (3 + f), g, col, tmp);
        for (size_t k = 0; k < NTNZ; k++) { /* derivt_k */
          double kt = kt_of(c, signed_mode(c, (int)(k / NZ)));
          c2 a = ul[f][k];
          spec[k].x = -kt * a.y / rK;
          spec[k].y = kt * a.x / rK;
        }
        level_backward(c, spec, ph + PL * (6 + f), g, col, tmp);
        for (size_t k = 0; k < NTNZ; k++) { /* derivz_k */
          double kz = kz_of(c, (int)(k % NZ));
          c2 a = ul[f][k];
          spec[k].x = -kz * a.y;
          spec[k].y = kz * a.x;
        }
        level_backward(c, spec, ph + PL * (9 + f), g, col, tmp);
      }
      double* Ur = ph; double* Ut = ph + PL; double* Uz = ph + 2 * PL;
      double* dr[3] = {ph + 3 * PL, ph + 4 * PL, ph + 5 * PL};
      double* dt[3] = {ph + 6 * PL, ph + 7 * PL, ph + 8 * PL};
      double* dz[3] = {ph + 9 * PL, ph + 10 * PL, ph + 11 * PL};
      for (size_t h = 0; h < PL; h++) { /* calcNonlinear_k */
        double vr = Ur[h], vt = Ut[h], vz = Uz[h];
        double udu_r = vr * dr[0][h] + vt * dt[0][h] + vz * dz[0][h] - vt * (vt / rK);
        double udu_t = vr * dr[1][h] + vt * dt[1][h] + vz * dz[1][h] + vr * (vt / rK);
        double udu_z = vr * dr[2][h] + vt * dt[2][h] + vz * dz[2][h];
        dr[0][h] = -udu_r; dr[1][h] = -udu_t; dr[2][h] = -udu_z;
      }
      for (int f = 0; f < 3; f++) level_forward(c, dr[f], out[f] + (size_t)i * NTNZ, g, col, tmp);
    }
    free(ph); free(spec); free(g); free(col); free(tmp);
  }
  press_grad(c, nz, uz);
  (void)NT;
}

/* ------------------------------------------------------- setup ----------- */
/* setBCon: mod_boundary.cu:205-255 with calc_invM_k :66-196. */
static void set_bcon(orc_ctx* c) {
  size_t S = c->S, NTNZ = c->NTNZ;
  c2* rhs = (c2*)malloc(sizeof(c2) * S);
  c2* aux = (c2*)malloc(sizeof(c2) * S);
  c2 *div2 = (c2*)malloc(sizeof(c2) * NTNZ), *div3 = (c2*)malloc(sizeof(c2) * NTNZ), *div4 = (c2*)malloc(sizeof(c2) * NTNZ);
  c2 uni = {0.0, 0.0}, bcon = {1.0, 0.0};
  fill(c, rhs, uni); write_bcon(c, rhs, bcon); lusolve(c, c->uh_r, rhs, 0);
  lusolve(c, c->uh_t, rhs, 1); bcon.x = 0.0; bcon.y = 1.0; fill(c, rhs, uni);
  write_bcon(c, rhs, bcon); lusolve(c, c->uh_z, rhs, 2); fill(c, rhs, uni);
  bcon.x = -1.0; bcon.y = 0.0; write_bcon(c, rhs, bcon); lusolve(c, aux, rhs, 3);
  /* div1 */
  copyf(c, c->uhP_r, c->uh_r); copyf(c, c->uhP_t, c->uh_t); copyf(c, c->uhP_z, c->uh_z);
  fill(c, c->uhP_t, uni); fill(c, c->uhP_z, uni);
  decouple_bwd(c, c->uhP_r, c->uhP_t);
  div_wall(c, c->div1, c->uhP_r, c->uhP_t, c->uhP_z);
  /* div2 */
  copyf(c, c->uhP_r, c->uh_r); copyf(c, c->uhP_t, c->uh_t); copyf(c, c->uhP_z, c->uh_z);
  fill(c, c->uhP_r, uni); fill(c, c->uhP_z, uni);
  decouple_bwd(c, c->uhP_r, c->uhP_t);
  div_wall(c, div2, c->uhP_r, c->uhP_t, c->uhP_z);
  /* div3 */
  copyf(c, c->uhP_r, c->uh_r); copyf(c, c->uhP_t, c->uh_t); copyf(c, c->uhP_z, c->uh_z);
  fill(c, c->uhP_r, uni); fill(c, c->uhP_t, uni);
  div_wall(c, div3, c->uhP_r, c->uhP_t, c->uhP_z); fill(c, c->uhP_z, uni);
  /* div4 and u_hP */
  derivr(c, c->uhP_r, aux, 0); derivt(c, c->uhP_t, aux); derivz(c, c->uhP_z, aux);
  div_wall(c, div4, c->uhP_r, c->uhP_t, c->uhP_z); decouple_fwd(c, c->uhP_r, c->uhP_t);
  /* calc_invM_k */
  for (size_t k = 0; k < NTNZ; k++) {
    size_t h = (size_t)(c->NR - 1) * NTNZ + k;
    c2 a14 = c->uhP_r[h], a24 = c->uhP_t[h], a34 = c->uhP_z[h], a44 = div4[k];
    c2 a41 = c->div1[k], a42 = div2[k], a43 = div3[k], Det, ax;
    c2 IA[16];
    ax.x = a44.x - a24.x * a42.x + a24.y * a42.y - a14.x * a41.x + a14.y * a41.y;
    ax.y = a44.y - a24.x * a42.y - a24.y * a42.x - a14.x * a41.y - a14.y * a41.x;
    Det.x = -ax.y - a34.x * a43.x + a34.y * a43.y;
    Det.y = ax.x - a34.x * a43.y - a34.y * a43.x;
    ax.x = a44.x - a24.x * a42.x + a24.y * a42.y;
    ax.y = a44.y - a24.x * a42.y - a24.y * a42.x;
    IA[0].x = -ax.y - a34.x * a43.x + a34.y * a43.y;
    IA[0].y = ax.x - a34.x * a43.y - a34.y * a43.x;
    IA[1].y = a14.x * a42.x - a14.y * a42.y;
    IA[1].x = -a14.x * a42.y - a14.y * a42.x;
    IA[2].x = a14.x * a43.x - a14.y * a43.y;
    IA[2].y = a14.x * a43.y + a14.y * a43.x;
    IA[3].x = a14.y; IA[3].y = -a14.x;
    IA[4].y = a24.x * a41.x - a24.y * a41.y;
    IA[4].x = -a24.x * a41.y - a24.y * a41.x;
    ax.x = a44.x - a14.x * a41.x + a14.y * a41.y;
    ax.y = a44.y - a14.x * a41.y - a14.y * a41.x;
    IA[5].x = -ax.y - a34.x * a43.x + a34.y * a43.y;
    IA[5].y = ax.x - a34.x * a43.y - a34.y * a43.x;
    IA[6].x = a24.x * a43.x - a24.y * a43.y;
    IA[6].y = a24.x * a43.y + a24.y * a43.x;
    IA[7].x = a24.y; IA[7].y = -a24.x;
    IA[8].x = a34.x * a41.x - a34.y * a41.y;
    IA[8].y = a34.x * a41.y + a34.y * a41.x;
    IA[9].x = a34.x * a42.x - a34.y * a42.y;
    IA[9].y = a34.x * a42.y + a34.y * a42.x;
    IA[10].x = a44.x - a14.x * a41.x + a14.y * a41.y - a24.x * a42.x + a24.y * a42.y;
    IA[10].y = a44.y - a14.x * a41.y - a14.y * a41.x - a24.x * a42.y - a24.y * a42.x;
    IA[11].x = -a34.x; IA[11].y = -a34.y;
    IA[12].x = a41.y; IA[12].y = -a41.x;
    IA[13].x = a42.y; IA[13].y = -a42.x;
    IA[14].x = -a43.x; IA[14].y = -a43.y;
    IA[15].x = 0.0; IA[15].y = 1.0;
    double D1 = Det.x * Det.x + Det.y * Det.y;
    Det.x = Det.x / D1;
    Det.y = -Det.y / D1;
    for (int e = 0; e < 16; e++) {
      c2 v;
      v.x = IA[e].x * Det.x - IA[e].y * Det.y;
      v.y = IA[e].x * Det.y + IA[e].y * Det.x;
      c->invM[e + k * 16] = v;
    }
  }
  free(rhs); free(aux); free(div2); free(div3); free(div4);
}

/* setCublasFlux: mod_cublasflux.cu:56-81. */
static void set_flux(orc_ctx* c) {
  c2* aux = (c2*)malloc(sizeof(c2) * c->S);
  c2* uaux = (c2*)malloc(sizeof(c2) * c->S);
  c2 uni = {1.0, 0.0}, bcon = {0.0, 0.0};
  fill(c, aux, uni); write_bcon(c, aux, bcon);
  lusolve(c, uaux, aux, 2);
  for (int i = 0; i < c->NR; i++) c->uc[i] = uaux[(size_t)i * c->NTNZ].x;
  double Q = 0.0;
  for (int i = 0; i < c->NR; i++) Q += c->rdr[i] * c->uc[i];
  c->Qc = Q;
  free(aux); free(uaux);
}

orc_ctx* orc_create(const orc_params* p) {
  orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
  c->p = *p;
  c->NR = p->NR; c->NT = p->NT; c->NZ = p->NZ;
  c->sten = p->sten > 0 ? p->sten : 7;
  c->iw = c->sten / 2;
  c->NTP = 3 * p->NT / 2;
  c->NZP = 3 * (p->NZ - 1) / 2 + 1;
  c->NZR = 2 * c->NZP - 2;
  c->NTNZ = (size_t)p->NT * p->NZ;
  c->S = (size_t)p->NR * c->NTNZ;
  c->c_im = p->d_im / p->Re;
  c->c_ex = (1.0 - p->d_im) / p->Re;
  c->inv_dt = 1.0 / p->dt;
  c->two_re = 2.0 / p->Re;
  set_threads(c);
  int NR = c->NR, sten = c->sten;
  c->r = (double*)calloc(NR, sizeof(double));
  c->rdr = (double*)calloc(NR, sizeof(double));
  c->dr0 = (double*)calloc(c->iw + 1, sizeof(double));
  c->D = (double*)calloc((size_t)2 * sten * NR, sizeof(double));
  c->Lu = (double*)calloc((size_t)2 * sten * NR, sizeof(double));
  c->Lp = (double*)calloc((size_t)2 * sten * NR, sizeof(double));
  c->uc = (double*)calloc(NR, sizeof(double));
  size_t S = c->S;
  c2** fields[] = {&c->uh_r, &c->uh_t, &c->uh_z, &c->uhP_r, &c->uhP_t, &c->uhP_z,
                   &c->rhs[0], &c->rhs[1], &c->rhs[2], &c->uw[0], &c->uw[1], &c->uw[2],
                   &c->rhsw[0], &c->rhsw[1], &c->rhsw[2], &c->ui[0], &c->ui[1], &c->ui[2],
                   &c->dur[0], &c->dur[1], &c->dur[2]};
  for (size_t f = 0; f < sizeof(fields) / sizeof(fields[0]); f++) *fields[f] = (c2*)calloc(S, sizeof(c2));
  c->invM = (c2*)calloc(16 * c->NTNZ, sizeof(c2));
  c->div1 = (c2*)calloc(c->NTNZ, sizeof(c2));
  c->coef = (c2*)calloc(4 * c->NTNZ, sizeof(c2));
  c->d1 = (double*)calloc(S, sizeof(double));
  c->d2 = (double*)calloc(S, sizeof(double));
  plan_init(&c->pt, c->NTP);
  plan_init(&c->pz, c->NZR);
  init_fd(c);
  set_flux(c);
  set_bcon(c);
  return c;
}

void orc_destroy(orc_ctx* c) {
  if (!c) return;
  free(c->r); free(c->rdr); free(c->dr0); free(c->D); free(c->Lu); free(c->Lp); free(c->uc);
  c2* fields[] = {c->uh_r, c->uh_t, c->uh_z, c->uhP_r, c->uhP_t, c->uhP_z, c->rhs[0], c->rhs[1], c->rhs[2],
                  c->uw[0], c->uw[1], c->uw[2], c->rhsw[0], c->rhsw[1], c->rhsw[2], c->ui[0], c->ui[1],
                  c->ui[2], c->dur[0], c->dur[1], c->dur[2], c->invM, c->div1, c->coef};
  for (size_t f = 0; f < sizeof(fields) / sizeof(fields[0]); f++) free(fields[f]);
  free(c->d1); free(c->d2); free(c->pt.w); free(c->pz.w);
  free(c);
}

/* ------------------------------------------------------ integrator ------- */
/* corBCon: mod_boundary.cu:269-278 with compcoef_k :42-62, addBCon_k :11-37. */
static void cor_bcon(orc_ctx* c, c2* ur, c2* ut, c2* uz) {
  size_t NTNZ = c->NTNZ;
  decouple_bwd(c, ur, ut);
  div_wall(c, c->div1, ur, ut, uz);
  decouple_fwd(c, ur, ut);
  for (size_t k = 0; k < NTNZ; k++) {
    c2 dv = {-c->div1[k].x, -c->div1[k].y};
    for (int j = 0; j < 4; j++) {
      c2 IM = c->invM[3 + 4 * j + 16 * k], a;
      a.x = dv.x * IM.x - dv.y * IM.y;
      a.y = dv.x * IM.y + dv.y * IM.x;
      c->coef[j + 4 * k] = a;
    }
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->NR; i++)
    for (size_t k = 0; k < NTNZ; k++) {
      size_t h = (size_t)i * NTNZ + k;
      c2 a0 = c->coef[4 * k], a1 = c->coef[1 + 4 * k], a2 = c->coef[2 + 4 * k], a3 = c->coef[3 + 4 * k];
      c2 uhr = c->uh_r[h], uht = c->uh_t[h], uhz = c->uh_z[h];
      c2 pr = c->uhP_r[h], pt = c->uhP_t[h], pz = c->uhP_z[h], ax;
      ax.x = a0.x * uhr.x - a0.y * uhr.y + a3.x * pr.x - a3.y * pr.y;
      ax.y = a0.x * uhr.y + a0.y * uhr.x + a3.x * pr.y + a3.y * pr.x;
      ur[h].x += ax.x; ur[h].y += ax.y;
      ax.x = a1.x * uht.x - a1.y * uht.y + a3.x * pt.x - a3.y * pt.y;
      ax.y = a1.x * uht.y + a1.y * uht.x + a3.x * pt.y + a3.y * pt.x;
      ut[h].x += ax.x; ut[h].y += ax.y;
      ax.x = a2.x * uhz.x - a2.y * uhz.y + a3.x * pz.x - a3.y * pz.y;
      ax.y = a2.x * uhz.y + a2.y * uhz.x + a3.x * pz.y + a3.y * pz.x;
      uz[h].x += ax.x; uz[h].y += ax.y;
    }
}

/* modeZZ_k: mod_integrate.cu:63-68. */
static void mode_zz(orc_ctx* c, c2* ur, c2* ut, c2* uz) {
  for (int i = 0; i < c->NR; i++) {
    size_t h = (size_t)i * c->NTNZ;
    ur[h].x = 0.0; ur[h].y = 0.0; ut[h].y = 0.0; uz[h].y = 0.0;
  }
}

/* adj_flux: mod_cublasflux.cu:90-103 (cublasDdot summed in index order). */
static void adj_flux(orc_ctx* c, c2* uz) {
  double Q = 0.0;
  for (int i = 0; i < c->NR; i++) Q += c->rdr[i] * uz[(size_t)i * c->NTNZ].x;
  double corr = (0.5 - Q) / c->Qc;
  for (int i = 0; i < c->NR; i++) uz[(size_t)i * c->NTNZ].x += corr * c->uc[i];
}

/* Common tail of predictor/corrector (mod_integrate.cu:174-192, :209-227):
 * rhs (+/- form, after the explicit part) -> new velocity in out (r/theta). */
static void linear_tail(orc_ctx* c, c2** rhs, const c2* const* uw, c2* scr_t, c2* scr_z, c2** out) {
  c2 zero = {0.0, 0.0};
  add_lap(c, rhs[0], uw[0], 0);
  add_lap(c, rhs[1], uw[1], 1);
  add_lap(c, rhs[2], uw[2], 2);
  decouple_bwd(c, rhs[0], rhs[1]);
  divergence(c, scr_t, rhs[0], rhs[1], rhs[2]);
  write_bcon(c, scr_t, zero);
  lusolve(c, scr_z, scr_t, 3);
  add_grad(c, rhs[0], rhs[1], rhs[2], scr_z);
  decouple_fwd(c, rhs[0], rhs[1]);
  write_bcon(c, rhs[0], zero); lusolve(c, out[0], rhs[0], 0);
  write_bcon(c, rhs[1], zero); lusolve(c, out[1], rhs[1], 1);
  write_bcon(c, rhs[2], zero); lusolve(c, out[2], rhs[2], 2);
  cor_bcon(c, out[0], out[1], out[2]);
  decouple_bwd(c, out[0], out[1]);
  mode_zz(c, out[0], out[1], out[2]);
  adj_flux(c, out[2]);
}

/* integrate: mod_integrate.cu:98-160 (nsteps steps, no file output). */
int orc_step(orc_ctx* c, double* urd, double* utd, double* uzd, int nsteps, int* iters, double* errs) {
  set_threads(c);
  c2* u[3] = {(c2*)urd, (c2*)utd, (c2*)uzd};
  size_t S = c->S;
  for (int s = 0; s < nsteps; s++) {
    nonlinear(c, u[0], u[1], u[2], c->rhs[0], c->rhs[1], c->rhs[2]);
    /* predictor :164-193 */
    decouple_fwd(c, u[0], u[1]);
    decouple_fwd(c, c->rhs[0], c->rhs[1]);
    for (int f = 0; f < 3; f++) { copyf(c, c->uw[f], u[f]); copyf(c, c->rhsw[f], c->rhs[f]); }
    linear_tail(c, c->rhs, (const c2* const*)c->uw, u[1], u[2], c->ui);
    double err = 1e98;
    int ite = 0;
    while (ite < c->p.maxit && err > c->p.tol) {
      ite += 1;
      nonlinear(c, c->ui[0], c->ui[1], c->ui[2], c->rhs[0], c->rhs[1], c->rhs[2]);
      /* corrector :197-228 */
      decouple_fwd(c, c->rhs[0], c->rhs[1]);
      for (int f = 0; f < 3; f++) /* addRHS_k :43-59 */
        for (size_t h = 0; h < S; h++) {
          c->rhs[f][h].x = c->p.d_im * c->rhs[f][h].x + (1.0 - c->p.d_im) * c->rhsw[f][h].x;
          c->rhs[f][h].y = c->p.d_im * c->rhs[f][h].y + (1.0 - c->p.d_im) * c->rhsw[f][h].y;
        }
      linear_tail(c, c->rhs, (const c2* const*)c->uw, u[1], u[2], u);
      /* measucorr :232-241 with mcor_k :9-40 and iden_max (mod_cublasflux.cu:106-116) */
      double num = 0.0, den = 0.0;
      for (size_t h = 0; h < S; h++) {
        double n1 = 0.0, d1 = 0.0;
        for (int f = 0; f < 3; f++) {
          c2 a = c->ui[f][h], b = u[f][h], ax;
          ax.x = a.x - b.x; ax.y = a.y - b.y;
          n1 = dmax(n1, ax.x * ax.x + ax.y * ax.y);
        }
        for (int f = 0; f < 3; f++) {
          c2 a = c->ui[f][h];
          d1 = dmax(d1, a.x * a.x + a.y * a.y);
        }
        num = dmax(num, n1);
        den = dmax(den, d1);
      }
      err = num / den;
      for (int f = 0; f < 3; f++) copyf(c, c->ui[f], u[f]);
    }
    if (iters) iters[s] = ite;
    if (errs) errs[s] = err;
  }
  return 0;
}

/* ------------------------------------------------------ exports ---------- */
void orc_get_grid(const orc_ctx* c, double* r, double* rdr, double* D, double* Lu, double* Lp, double* dr0) {
  size_t n = (size_t)2 * c->sten * c->NR;
  if (r) memcpy(r, c->r, sizeof(double) * c->NR);
  if (rdr) memcpy(rdr, c->rdr, sizeof(double) * c->NR);
  if (D) memcpy(D, c->D, sizeof(double) * n);
  if (Lu) memcpy(Lu, c->Lu, sizeof(double) * n);
  if (Lp) memcpy(Lp, c->Lp, sizeof(double) * n);
  if (dr0) memcpy(dr0, c->dr0, sizeof(double) * (c->iw + 1));
}

void orc_get_setup(const orc_ctx* c, double* uc, double* Qc, double* invM, double* uh_r, double* uh_t,
                   double* uh_z, double* uhP_r, double* uhP_t, double* uhP_z) {
  size_t S = c->S;
  if (uc) memcpy(uc, c->uc, sizeof(double) * c->NR);
  if (Qc) *Qc = c->Qc;
  if (invM) memcpy(invM, c->invM, sizeof(c2) * 16 * c->NTNZ);
  if (uh_r) memcpy(uh_r, c->uh_r, sizeof(c2) * S);
  if (uh_t) memcpy(uh_t, c->uh_t, sizeof(c2) * S);
  if (uh_z) memcpy(uh_z, c->uh_z, sizeof(c2) * S);
  if (uhP_r) memcpy(uhP_r, c->uhP_r, sizeof(c2) * S);
  if (uhP_t) memcpy(uhP_t, c->uhP_t, sizeof(c2) * S);
  if (uhP_z) memcpy(uhP_z, c->uhP_z, sizeof(c2) * S);
}

void orc_derivr(orc_ctx* c, double* dur, const double* u, int flag) { set_threads(c); derivr(c, (c2*)dur, (const c2*)u, flag); }
void orc_lusolve_u(orc_ctx* c, double* sol, const double* rhs, int flag) { set_threads(c); lusolve(c, (c2*)sol, (const c2*)rhs, flag); }
void orc_lusolve_p(orc_ctx* c, double* sol, const double* rhs) { set_threads(c); lusolve(c, (c2*)sol, (const c2*)rhs, 3); }
void orc_add_laplacian(orc_ctx* c, double* rhs, const double* u, int flag) { set_threads(c); add_lap(c, (c2*)rhs, (const c2*)u, flag); }
void orc_divergence(orc_ctx* c, double* div, const double* ur, const double* ut, const double* uz) {
  set_threads(c);
  divergence(c, (c2*)div, (const c2*)ur, (const c2*)ut, (const c2*)uz);
}
void orc_div_wall(orc_ctx* c, double* div1, const double* ur, const double* ut, const double* uz) {
  set_threads(c);
  div_wall(c, (c2*)div1, (const c2*)ur, (const c2*)ut, (const c2*)uz);
}
void orc_nonlinear(orc_ctx* c, const double* ur, const double* ut, const double* uz, double* nr, double* nt, double* nz) {
  set_threads(c);
  nonlinear(c, (const c2*)ur, (const c2*)ut, (const c2*)uz, (c2*)nr, (c2*)nt, (c2*)nz);
}
void orc_level_backward(orc_ctx* c, const double* spec_level, double* phys_level) {
  int nmax = c->NTP > c->NZR ? c->NTP : c->NZR;
  c2* g = (c2*)malloc(sizeof(c2) * (size_t)c->NTP * c->NZP);
  c2* col = (c2*)malloc(sizeof(c2) * nmax);
  c2* tmp = (c2*)malloc(sizeof(c2) * nmax);
  level_backward(c, (const c2*)spec_level, phys_level, g, col, tmp);
  free(g); free(col); free(tmp);
}
void orc_level_forward(orc_ctx* c, const double* phys_level, double* spec_level) {
  int nmax = c->NTP > c->NZR ? c->NTP : c->NZR;
  c2* g = (c2*)malloc(sizeof(c2) * (size_t)c->NTP * c->NZP);
  c2* col = (c2*)malloc(sizeof(c2) * nmax);
  c2* tmp = (c2*)malloc(sizeof(c2) * nmax);
  level_forward(c, phys_level, (c2*)spec_level, g, col, tmp);
  free(g); free(col); free(tmp);
}

/* wrt_frc_k: mod_io_nonlinear.cu:40-52 (centreline velocity and u_tau). */
void orc_friction(orc_ctx* c, const double* uzd, double* u_centre, double* u_tau) {
  const c2* uz = (const c2*)uzd;
  double uc = 0.0, du = 0.0;
  for (int i = 0; i < c->iw + 1; i++) uc += uz[(size_t)i * c->NTNZ].x * c->dr0[i];
  for (int i = 0; i < c->sten; i++) du += uz[(size_t)(c->NR - c->sten + i) * c->NTNZ].x * c->D[(c->NR - 1) * c->sten + i];
  *u_centre = uc;
  *u_tau = sqrt(fabs(du) / c->p.Re);
}
