/* nsp_oracle.h -- CPU FP64 restatement of the nsPipe-CUDA per-step path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity oracle for the GPU
 * stepper and the timed host baseline.  Only tests/, __graft_entry__.smoke()
 * and bench.py (cpu_baseline / --impl reference legs) may load it.  The
 * product library never links or calls it.
 *
 * Every array argument of type double* holding a spectral field is an
 * interleaved complex array double2[NR][NT][NZ] (the reference layout of
 * head.h:73 / mod_deriv.cu:15-17): index h = i*NT*NZ + it*NZ + l.
 */
#ifndef NSP_ORACLE_H
#define NSP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int    NR, NT, NZ;      /* radial points, theta slots (even), axial modes (odd) */
  double LT, LZ;          /* domain lengths: reference head.h:21-22                */
  double Re;              /* Reynolds number (head.h:25)                           */
  double dt, d_im;        /* time step, implicit factor (head.h:48-49)             */
  int    maxit;           /* corrector iterations cap (head.h:51)                  */
  double tol;             /* convergence tolerance on the squared ratio (head.h:52)*/
  int    sten;            /* radial stencil width, 7 in the reference (head.h:44)  */
  int    nthreads;        /* OpenMP threads used by the oracle (<=0: runtime default) */
} orc_params;

typedef struct orc_ctx orc_ctx;

orc_ctx* orc_create(const orc_params* p);          /* init_fd + setBCon + setCublasFlux */
void     orc_destroy(orc_ctx* c);

/* Tables built by init_fd (mod_radialFD.cu:199-312) and get_dr0 (:316-350). */
void orc_get_grid(const orc_ctx* c, double* r, double* rdr, double* D, double* Lu, double* Lp, double* dr0);
/* Setup products (mod_boundary.cu:205-255, mod_cublasflux.cu:56-81). */
void orc_get_setup(const orc_ctx* c, double* uc, double* Qc, double* invM, double* uh_r, double* uh_t,
                   double* uh_z, double* uhP_r, double* uhP_t, double* uhP_z);

/* Single operators on full fields. */
void orc_derivr(orc_ctx* c, double* dur, const double* u, int flag);
void orc_lusolve_u(orc_ctx* c, double* sol, const double* rhs, int flag);
void orc_lusolve_p(orc_ctx* c, double* sol, const double* rhs);
void orc_add_laplacian(orc_ctx* c, double* rhs, const double* u, int flag);
void orc_divergence(orc_ctx* c, double* div, const double* ur, const double* ut, const double* uz);
void orc_div_wall(orc_ctx* c, double* div1, const double* ur, const double* ut, const double* uz);
void orc_nonlinear(orc_ctx* c, const double* ur, const double* ut, const double* uz,
                   double* nr, double* nt, double* nz);
/* Physical-space 2-D transforms of one radial level: spectral double2[NT][NZ] <-> real
 * double[NTP][NZR] (the physical theta x z points of the in-place cuFFT layout of
 * mod_fft.cu:23-26, without its two padding entries per theta row). */
void orc_level_backward(orc_ctx* c, const double* spec_level, double* phys_level);
void orc_level_forward(orc_ctx* c, const double* phys_level, double* spec_level);

/* nsteps full time steps (mod_integrate.cu:98-160) in place on u (r/theta form).
 * iters[s] receives the corrector iteration count of step s, errs[s] the final err.
 * Returns 0. */
int orc_step(orc_ctx* c, double* ur, double* ut, double* uz, int nsteps, int* iters, double* errs);

/* Diagnostics reused as accuracy metrics (mod_io_nonlinear.cu:40-52). */
void orc_friction(orc_ctx* c, const double* uz, double* u_centre, double* u_tau);

#ifdef __cplusplus
}
#endif
#endif
