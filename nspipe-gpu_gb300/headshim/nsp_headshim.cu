// nsp_headshim.cu -- the reference's own C++ entry points (Main_Code/src/head.h:77-152)
// implemented on the GB300 stepper, so that the reference's main.cu links against it
// unchanged.  Compiled per configuration, like the reference itself: -I <the directory
// of the configuration's head.h> -I <this repo>/include, linked with libnspipe_gb300.so.
//
// The call sequence of main.cu:16-50 maps as follows:
//   init_fd          -> nsp_create + nsp_setup (parameters from the head.h macros),
//                       r and rdr from nsp_grid (mod_radialFD.cu:199-312)
//   setFft, setLinear, setCublasFlux, setDeriv, setNonlinear, setInt, setBCon
//                    -> nothing left to do (nsp_setup built every table)
//   setIO            -> nsp_run_open: the four io_*.txt files in the working directory
//                       with the head.h schedule dt_frc/dc_frc, dt_qcr/dc_qcr, dt_mnp/dc_mnp
//   initField        -> the restart branch: u?_s.bin (mod_io_nonlinear.cu:424-429)
//   integrate        -> nsp_run_advance over nsteps steps (mod_integrate.cu:98-160),
//                       progress lines as the reference prints them
//   wBufferBinary, rBufferBinary -> the same raw files (mod_io_nonlinear.cu:528-565)
//   *Destroy         -> nsp_run_close (IODestroy) and nsp_destroy (IntDestroy)
// and nonlinear, LUsolve_u, LUsolve_p are the operator entry points of the C ABI.
// The reference's built-in initial perturbation (initField with restart == 0,
// mod_io_nonlinear.cu:430-447) is not provided: such a build stops with a message.
//
// head.h defines NR, NT, Re, dt, tol, dt_frc, ... as object-like macros, so every use of
// the C ABI's structure fields sits above the #include "head.h" line.
#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>

#include "nspipe_gb300.h"

namespace {

nsp_ctx* g_ctx = nullptr;
nsp_run* g_run = nullptr;

void shim_check(int rc, const char* what) {
  if (rc != NSP_OK) {
    fprintf(stderr, "nspipe-gb300: %s failed (%d): %s\n", what, rc, nsp_last_error(g_ctx));
    exit(1);
  }
}

void shim_create(int nr, int nt, int nz, double lt, double lz, double re, double dt_, double dim, int it, double tl,
                 int st) {
  nsp_params p;
  nsp_default_params(&p);
  p.NR = nr; p.NT = nt; p.NZ = nz; p.LT = lt; p.LZ = lz; p.Re = re;
  p.dt = dt_; p.d_im = dim; p.maxit = it; p.tol = tl; p.sten = st;
  int dev = 0;
  cudaGetDevice(&dev);
#ifdef NSP_SHIM_MIXED
  const int precision = NSP_MIXED;
#else
  const int precision = NSP_FP64;  // the drop-in form
#endif
  shim_check(nsp_create(&p, 1, precision, dev, &g_ctx), "nsp_create");
  shim_check(nsp_setup(g_ctx), "nsp_setup");
}

void shim_open_run(double frc, double qcr, double mnp, int rows) {
  nsp_run_opts o;
  nsp_run_default_opts(&o);
  o.out_dir = ".";
  o.dt_frc = frc; o.dt_qcr = qcr; o.dt_mnp = mnp;
  o.rows_per_write = rows;
  o.final_state = 0;  // main.cu writes ur.bin, ut.bin, uz.bin itself
  o.verbose = 1;
  shim_check(nsp_run_open(g_ctx, &o, &g_run), "nsp_run_open");
}

}  // namespace

#include "head.h"

// RADIAL OPERATIONS ..........................................................
void init_fd(double* r_h, double* Lu_h, double* Lp_h, double* rdr_h) {
  if (!g_ctx) shim_create(NR, NT, NZ, LT, LZ, Re, dt, d_im, maxit, tol, sten);
  shim_check(nsp_grid(g_ctx, 0, r_h, rdr_h), "nsp_grid");
  // The operator tables live in the context; the caller's copies are only passed on
  // to setLinear, which has nothing left to do.
  for (int i = 0; i < 2 * sten * NR; i++) Lu_h[i] = Lp_h[i] = 0.0;
}

// SETTERS (every table was built by nsp_setup) ..............................
void setFft(size_p) {}
void setLinear(double*, double*, double*) {}
void setCublasFlux(double*) {}
void setDeriv(double*) {}
void setNonlinear(void) {}
void setInt(void) {}
void setBCon(void) {}

// INOUT ........................................................................
void setIO(double*) { shim_open_run(dt_frc, dt_qcr, dt_mnp, dc_frc); }

void wBufferBinary(double* w, const char* file, size_t elsize, size_t elements) {
  double* h = (double*)malloc(elsize * elements);
  CHECK_CUDART(cudaMemcpy(h, w, elsize * elements, cudaMemcpyDeviceToHost));
  FILE* fp = fopen(file, "wb");
  if (fp == NULL) { printf("\nwriting error: %s", file); exit(1); }
  if (fwrite(h, elsize, elements, fp) != elements) { printf("\nwriting error: %s", file); exit(1); }
  fclose(fp);
  free(h);
}

void rBufferBinary(double* w, const char* file, size_t elsize, size_t elements) {
  double* h = (double*)malloc(elsize * elements);
  FILE* fp = fopen(file, "rb");
  if (fp == NULL) { printf("\nreading error: %s", file); exit(1); }
  if (fread(h, elsize, elements, fp) != elements) { printf("\nreading error: %s", file); exit(1); }
  fclose(fp);
  CHECK_CUDART(cudaMemcpy(w, h, elsize * elements, cudaMemcpyHostToDevice));
  free(h);
}

void initField(vfield u) {
  if (restart > 0) {
    printf("Reading initial condition\n");
    rBufferBinary((double*)u.r, "ur_s.bin", sizeof(double2), (size_t)NR * NT * NZ);
    rBufferBinary((double*)u.t, "ut_s.bin", sizeof(double2), (size_t)NR * NT * NZ);
    rBufferBinary((double*)u.z, "uz_s.bin", sizeof(double2), (size_t)NR * NT * NZ);
  } else {
    fprintf(stderr, "nspipe-gb300: the built-in initial perturbation (restart 0) is not provided; "
                    "set restart to 1 and supply ur_s.bin, ut_s.bin, uz_s.bin\n");
    exit(1);
  }
}

void IODestroy(void) {
  shim_check(nsp_run_close(g_run), "nsp_run_close");
  g_run = nullptr;
}

// INTEGRATE .....................................................................
void integrate(vfield u, vfield) {
  shim_check(nsp_set_state_device(g_ctx, 0, u.r, u.t, u.z), "nsp_set_state_device");
  shim_check(nsp_run_advance(g_run, nsteps, NULL), "nsp_run_advance");
  shim_check(nsp_get_state_device(g_ctx, 0, u.r, u.t, u.z), "nsp_get_state_device");
}

void IntDestroy(void) {
  nsp_destroy(g_ctx);
  g_ctx = nullptr;
}

// OPERATORS ......................................................................
void nonlinear(vfield u, vfield du) {
  shim_check(nsp_nonlinear(g_ctx, 0, u.r, u.t, u.z, du.r, du.t, du.z), "nsp_nonlinear");
}
void LUsolve_u(double2* sol, double2* RHS, int flag) { shim_check(nsp_lusolve(g_ctx, 0, flag, RHS, sol), "nsp_lusolve"); }
void LUsolve_p(double2* sol, double2* RHS) { shim_check(nsp_lusolve(g_ctx, 0, 3, RHS, sol), "nsp_lusolve"); }

// DESTROYERS with nothing to free ................................................
void fftDestroy(void) {}
void LinearDestroy(void) {}
void FluxDestroy(void) {}
void DerivDestroy(void) {}
void BConDestroy(void) {}
void NonDestroy(void) {}
