// nsp_internal.h -- device-side data structures shared by the kernels and the host API.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <string>
#include <vector>

#include "../../include/nspipe_gb300.h"

namespace nsp {

constexpr double PI2 = 6.283185307179586;  // the reference's 2*pi literal (head.h:12)
constexpr int STEN = 7;                     // radial stencil width (head.h:44)
constexpr int IW = 3;                       // half stencil (head.h:45)
constexpr int NFAC = 7;                     // stored factor entries per row: L(i-3..i-1), 1/U_ii, U(i+1..i+3)
constexpr int MAXPLAN = 12;                 // radix stages of one transform length

// FFT plan for one length: radices applied in order (Stockham, natural order out).
struct FftPlan {
  int n;
  int nst;
  int rad[MAXPLAN];
};

// Operator tables of one group of members sharing (NR, NT, NZ, LT, LZ, dt, d_im):
// one launch per stage covers the whole group.  Members may differ in Re; each
// distinct Re is an operator parameter set, and the Re-dependent tables (fac, V,
// Luc, uc, sscal) hold nsets consecutive sets.  All pointers are device memory;
// the struct is passed to kernels by value.
struct Tables {
  int NR, NT, NZ, NTP, NZP, NZR, NTNZ;
  long long S;         // NR*NT*NZ
  int nmem;            // members in this group
  int mem0;            // global index of the group's first member
  double kts, kzs;     // 2pi/LT, 2pi/LZ (wavenumber scales, mod_deriv.cu:17,31)
  double inv_dt, c_ex, d_im, one_m_dim, two_re, Qdes, Qc, inv_norm;
  // FP32 copies for the FP32 transform kernels (a conversion from FP64 issues on the slow
  // FP64 pipe, so the kernels read these instead of converting per thread)
  float kts32, kzs32, inv_norm32;
  const double* r;
  const double* rinv;
  const float* rinv32;
  const double* rinv2;  // 1/(r*r)
  const double* rdr;
  const double* uc;
  const double* D;     // [2][NR][7]: first derivative, parity tables (0 even-extended, 1 odd)
  const double* Ddiv;  // D with 1/r_i added to row i's centre weight: d_r u + u / r in one stencil
  const float* Ddiv32; // the same in FP32 (mixed form, corrector increment passes)
  const float* D32;    // the same in FP32 (mixed-form transforms)
  const double* Lu;    // [2][NR][7]: radial Laplacian rows with identity wall row
  const double* Luc;   // (1-d_im)/(2 Re) * Lu (explicit part of the Laplacian, pre-scaled)
  const float* Luc32;  // the same in FP32 (mixed form: the explicit stencil runs on the FP32 mirror)
  const double* fac;   // [4][NR][7][NTNZ]: banded LU factors of u+, u-, u_z, p
  const double2* V;    // [3][NR][NTNZ]: influence-matrix correction profiles (+, -, z)
  const float2* V32;   // mixed form: the same in FP32 (the corrector increments' correction)
  const float2* facdf;  // mixed form: fac as double-float pairs (hi, lo), backward entries divided by U_ii
  const float* fac32;   // mixed form: the same in FP32 (the increment passes' Helmholtz solves)
  const float2* Vdf;    // mixed form: V as double-float pairs, real and imaginary part of each entry
  const float2* Ddf;    // mixed form: D, Ddiv and 1/r as double-float pairs (the predictor's stencils)
  const float2* Ddivdf;
  const float2* rinvdf;
  const double2* tw_t; // [NTP] exp(-2 pi i e/NTP), FP64
  const double2* tw_z; // [NZR]
  const float2* tw_t32;
  const float2* tw_z32;
  FftPlan pt, pz;
  int lin_variant;     // block shape of the linear pass (autotuned at setup)
  int lin_variant_inc; // mixed form: block shape of the increment (corrector) pass
  int z_variant;       // z-stage kernel (autotuned at setup): 0 radix-stage, k >= 1 the k-th
                       // two-pass N1 x N2 split compiled for the length and precision
  int nsets;           // operator parameter sets (distinct Re) of the group
  const int* mset;     // [nmem] parameter set of each member
  const double* sscal; // [nsets][4]: (1-d_im)/Re, 2/Re, Qc, Re
  const float* dft_inv; // mixed form, tensor-core theta transforms: DFT-matrix operand images
  const float* dft_fwd; //   ([hi | lo] x N x K core matrices, nsp_theta_tc.cu)
  int tc_theta;        // 1: the mixed form's theta transforms run as tcgen05 GEMMs
  int nsm;             // SM count (persistent grids)
  unsigned long long* bc;  // bounds record of the bounds-checked build (nsp_bounds.cuh); unused otherwise
};

#ifdef __CUDACC__
// Operator parameter set of a member (0 when the group has a single Re).
__device__ __forceinline__ int member_set(const Tables& tb, int mloc) { return tb.nsets > 1 ? tb.mset[mloc] : 0; }
#endif

constexpr int LIN_VARIANTS = 12;
int linear_default_variant(int NR);
bool linear_variant_fits(int v, int NR);
void linear_shape(int v, int* LM, int* NTH);  // modes per block, threads of a variant

// Batched per-group member buffers.
struct Bufs {
  double2* U[2];       // [nmem][3][S]: state / corrector iterate, roles swap each step (parity)
  float2* U32[2];      // mixed form only: FP32 copies of U[0], U[1] read by the transforms
  float2* DR32[2];     // mixed form only: d_r of U32[k] (7-point parity stencil, FP32), written
                       // with U32 so that the theta-inverse reads it instead of re-gathering levels
  double2* RHSW;       // [nmem][3][S]: [(1-d_im) N(u^n) + u^n/dt + (1-d_im)/Re L u^n] / 2, r/theta form
  double2* N;          // [nmem][3][S]: nonlinear term output
  // Mixed form (N and RHSW are null there): N and the increment passes' N_{i-1} hold FP32
  // numbers -- the transforms' values plus FP32 mean-flow terms -- except on the line
  // Re N_z(0,0), which carries the FP64 wall forcing.
  float2* N32;         // [nmem][3][S]: N in FP32, without the forcing
  double* NF;          // [nmem]: the forcing -(2/Re) d_r u_z(0,0)|wall, added to Re N_z(0,0) at every level
  float2* RHSW32;      // [nmem][3][S]: N_{i-1} in FP32 (its Re N_z(0,0) line unused)
  double* RW00;        // [nmem][NR]: Re N_z(0,0) of N_{i-1} in FP64, forcing included
  void* G;             // [nmem][9][NR][NTP][NZ] complex T: theta-inverse of u, dr u, i m u / r
  void* H;             // [nmem][3][NR][NTP][NZ] complex T: z-forward of the nonlinear product
  float* MEAN;         // mixed form only: [nmem][NR][MEAN_N] mean flow of the transform input
                       // (V = Re u_r, W = Re u_theta, U = Re u_z at mode (0,0), W', U'),
                       // written by the theta-inverse, read by the linear pass
};
enum { MEAN_V = 0, MEAN_W, MEAN_U, MEAN_WP, MEAN_UP, MEAN_N };

// Device control block of one context.  phase[m]: 0 = predictor pending,
// p > 0 = corrector iteration p pending, -1 = converged for this step.
struct Ctl {
  int parity;          // U[parity] holds the state u^n, U[parity^1] the iterate
  int step;            // steps completed in the current nsp_step call
  int any;             // host-visible copy of the loop condition
  int nmem;
  int maxit;
  double tol;
  int* phase;
  int* ite;
  int* status;
  unsigned long long* num;  // max |u_i - u|^2 as ordered bits (>= 0)
  unsigned long long* den;  // max |u_i|^2
  double* err;
  int* hist;           // [cap][nmem]: iterations of each step of the call
  int* unconv;         // [nmem]: steps of the current call whose corrector loop stopped at
                       // maxit with err > tol (the reference moves on silently)
  int hist_cap;
  int fault;           // nonzero: a device-side wait ran out and a kernel abandoned its work
  int hold;            // nonzero: a completed step keeps parity and step count (chunked
                       // steps: members advance chunk by chunk, then finish_step flips once)
  int inject;          // test hook (nsp_debug_inject): bit 0 -- the tensor-core transforms'
                       // operand-image barrier is never arrived on, so their bounded wait runs out
};

// Kernel launchers (nsp_transform.cu, nsp_linear.cu).
// Nonlinear term of every active member of a group (or of one explicit field).
// mask selects the kernels: bit 0 theta-inverse, bit 1 z stage, bit 2 theta-forward.
// src32_override: FP32 copy of src_override (mixed form, explicit-field calls only).
void launch_nonlinear(const Tables& tb, const Bufs& bf, Ctl* dctl, bool mixed, const double2* src_override,
                      double2* dst_override, cudaStream_t st, int mask = 7, const float2* src32_override = nullptr);
// Which linear-pass kernels a launch issues: the predictor's (the full pass), the
// correctors' (the mixed form's increment pass; the full pass again in the FP64 form)
// or both (each returns at once in the other's passes; the FP64 form launches its one
// kernel once).
enum { LIN_PRED = 1, LIN_CORR = 2, LIN_BOTH = 3 };
void launch_linear(const Tables& tb, const Bufs& bf, Ctl* dctl, cudaStream_t st, int which = LIN_BOTH);
void launch_converge(Ctl* dctl, int nmem, unsigned long long cond_handle, int use_cond, cudaStream_t st);
// Completes a step taken in member chunks: parity flip and step count (converge_k's
// completion work, held back while the chunks ran).
void launch_finish_step(Ctl* dctl, cudaStream_t st);
void launch_lusolve(const Tables& tb, int kind, const double2* rhs, double2* sol, cudaStream_t st);
void launch_fp64_peak(double* out, int blocks, int threads, int iters, cudaStream_t st);
// max |div u| over the interior rows -> out[0], over the wall row -> out[1] (ordered bits);
// nmem consecutive members from U: out[2 * member + 0/1].
void launch_diag_div(const Tables& tb, const double2* U, unsigned long long* out, cudaStream_t st, int nmem = 1);
// Per-level partials of the q / u cross-section diagnostics: part[member][2][NR][NZR].
void launch_diag_cross(const Tables& tb, const double2* U, double* part, cudaStream_t st, int nmem = 1);
// Re u_z(0,0)(r_i) of nmem consecutive members: out[member][NR].
void launch_gather_mean(const Tables& tb, const double2* U, double* out, int nmem, cudaStream_t st);
// Fixed device scratch of the allocation-free entry point (nsp_noalloc.cu).
size_t noalloc_scratch_bytes();
cudaError_t noalloc_scratch(int device, void** ptr);
// FP32 copy of nmem x 3 x S complex values (the mixed form's transform input).
void launch_to_f32(const double2* src, float2* dst, long long n, cudaStream_t st);
void launch_split_df(const double* src, float2* dst, long long n, cudaStream_t st);
void launch_split_fac(const double* fac, float2* dfo, float* f32o, long long n, int NTNZ, cudaStream_t st);
// The FP32 mirror and its radial derivative (DR32) of a group's state U (mixed form).
void launch_mirror(const Tables& tb, const double2* U, float2* U32, float2* DR32, cudaStream_t st);
int kernels_per_nonlinear();
// z-stage kernels of a length (nsp_transform.cu): the number of two-pass splits compiled
// for NZR (rows per block dividing NTP) in the precision, and a description of variant v.
int z_variants(int NZR, int NTP, bool fp32);
int z_default_variant(int NZR, int NTP, bool fp32);
std::string z_variant_name(int NZR, int NTP, bool fp32, int v);
// Tensor-core theta transforms (nsp_theta_tc.cu).
bool theta_tc_supported(int NT, int NTP);
std::vector<float> theta_dft_image(int NT, int NTP, bool inverse, double scale);
void configure_theta_tc_kernels();
// dir 0: inverse (u, d_r u, i m u / r -> G); dir 1: forward (H -> N).
void launch_theta_tc(const Tables& tb, const Bufs& bf, Ctl* dctl, int dir, const double2* src, const float2* src32,
                     double2* dst, cudaStream_t st);

// Records msg as the context's last error (nsp_last_error) and returns code.
int ctx_fail(nsp_ctx* c, int code, const std::string& msg);
// Records the failure of a context-free call (nsp_last_error(NULL)), per thread.
void set_host_error(const std::string& msg);
// Re_Mesh plans (nsp_remesh.cu): launch over `count` members (host arrays of device
// pointers to each member's three components), shapes and device of a plan.
int remesh_launch(nsp_remesh* p, int count, const void* const* src, void* const* dst, cudaStream_t st);
void remesh_shape(const nsp_remesh* p, int* old3, int* new3);
int remesh_device(const nsp_remesh* p);

// Host-side operator construction (nsp_setup.cpp).
// Radial tables of one shape (radial_fd) and, in a group, its first parameter set's
// flux response (flux_response).
struct HostOps {
  int NR;
  std::vector<double> r, rdr, D, D2, Lu, Lp, dr0;
  std::vector<double> uc;
  double Qc;
};
void radial_fd(int NR, HostOps& out);
// One parameter set's mode tables on the host: fac [4][NR][NFAC][NT*NZ], V [3][NR][NT*NZ].
void mode_tables(const nsp_params& p, const HostOps& o, double* fac, double2* V);
// Flux response of one parameter set (mode (0,0) u_z solve with unit forcing) and its flux.
void flux_response(const nsp_params& p, const HostOps& o, std::vector<double>& uc, double& Qc);
// The same mode tables on the device (nsp_setup_dev.cu), bit-identical to mode_tables:
// nsets parameter sets of one shape (set k: c_im[k] = d_im / Re_k), written set-major
// into fac and V (device memory).  r, D, Lu, Lp: device copies of o's radial tables.
int launch_mode_tables(const nsp_params& p, int nsets, const double* c_im_host, const double* r, const double* D,
                       const double* Lu, const double* Lp, double* fac, double2* V, cudaStream_t st, std::string* err);

}  // namespace nsp
