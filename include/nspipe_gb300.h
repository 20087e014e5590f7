/* nspipe_gb300.h -- C ABI of the GB300 pipe-flow time stepper.
 *
 * Drop-in replacement for the per-step entry points of nsPipe-CUDA
 * (Mordered/nsPipe-GPU, Main_Code/src).  The reference exposes C++-linkage
 * functions declared in head.h:77-152 and configured by compile-time #defines
 * (head.h:16-61); this library takes the same parameters at run time, keeps the
 * same spectral state layout and restart/checkpoint file format, and returns
 * status codes instead of calling exit() (head.h:64-70, mod_fft.cu:12-18,
 * mod_cublasflux.cu:33-38).
 *
 * State layout (head.h:73, mod_deriv.cu:15-17): each velocity component is an
 * interleaved complex double array double2[NR][NT][NZ], index
 * h = i*NT*NZ + it*NZ + l, radial point i, azimuthal slot it (signed mode
 * m = it < NT/2 ? it : it-NT), axial mode l = 0..NZ-1 (k_z >= 0 only).  At step
 * boundaries the state is in (u_r, u_theta, u_z) form.
 *
 * A context holds an ensemble of independent pipes ("members").  Members with
 * equal (NR, NT, NZ, LT, LZ, Re, dt, d_im, sten) share one set of operator
 * tables; members of different shapes (uneven batches) are allowed.  Each
 * context owns one CUDA stream on one device; one host thread per context.
 * All functions return NSP_OK (0) or an NSP_ERR_* code; nsp_last_error()
 * describes the last failure.
 */
#ifndef NSPIPE_GB300_H
#define NSPIPE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NSP_OK 0
#define NSP_ERR_ARG 1        /* invalid argument or parameter combination         */
#define NSP_ERR_CUDA 2       /* CUDA runtime failure (message in nsp_last_error)   */
#define NSP_ERR_IO 3         /* restart/checkpoint file missing, short or unwritable */
#define NSP_ERR_NONFINITE 4  /* a member's field became NaN/Inf during nsp_step    */
#define NSP_ERR_STATE 5      /* call out of order (e.g. nsp_step before nsp_setup) */
#define NSP_ERR_NOMEM 6      /* device allocation failed                           */
#define NSP_ERR_DEVICE 7     /* a bounded device-side wait ran out (a tensor-core
                                tile pipeline did not complete); results invalid   */
#define NSP_ERR_MAXIT 8      /* strict mode only (nsp_set_strict): a member's corrector
                                loop stopped at maxit with err > tol; the steps were
                                taken as the reference takes them                   */

#define NSP_FP64 0  /* plain form: every operation in FP64 (matches the reference)         */
#define NSP_MIXED 1 /* transforms + nonlinear product in FP32 (theta DFT 3xTF32); solves and corrections
                             in double-float (FP32 pairs) or FP32 on corrector increments; state in FP64 */

/* Run-time copy of the reference's compile-time parameters (head.h:16-61). */
typedef struct nsp_params {
  int NR, NT, NZ;  /* radial points; 2*m_theta theta slots (even); m_z+1 axial modes (odd)  head.h:16-18 */
  double LT, LZ;   /* azimuthal and axial domain lengths                                    head.h:21-22 */
  double Re;       /* Reynolds number                                                        head.h:25    */
  double dt;       /* time step (code units)                                                 head.h:48    */
  double d_im;     /* implicitness factor                                                    head.h:49    */
  int maxit;       /* corrector iteration cap                                                head.h:51    */
  double tol;      /* convergence tolerance on max|du|^2/max|u|^2                            head.h:52    */
  int sten;        /* radial stencil width; 7 (the reference's value) is supported           head.h:44    */
  double Qdes;     /* prescribed mass flux, 0.5 in the reference                  mod_cublasflux.cu:92    */
} nsp_params;

/* Diagnostics of one member (the quantities of wrt_frc_k, mod_io_nonlinear.cu:40-52,
 * plus the last step's corrector record). */
typedef struct nsp_diag_out {
  double u_centre;    /* centreline u_z(0,0) interpolated to r = 0 (dr0 weights)         */
  double u_tau;       /* sqrt(|d u_z(0,0)/dr|_wall / Re)                                 */
  double flux;        /* sum_i rdr_i Re u_z(0,0)(r_i)                                    */
  double last_err;    /* convergence measure of the last corrector iteration             */
  int last_iters;     /* corrector iterations of the last step                           */
  int status;         /* NSP_OK or NSP_ERR_NONFINITE                                     */
  double re_tau;      /* friction Reynolds number Re * u_tau                             */
  double div_max;     /* max |div u| over the interior rows (div_k, mod_radialFD.cu:67-96) */
  double div_wall;    /* max |div u| on the wall row, the quantity the influence-matrix
                         correction drives to zero (divWall_k, mod_radialFD.cu:34-63)     */
  int unconverged_steps; /* steps of the last nsp_step / nsp_step_host call whose corrector
                            loop stopped at maxit with err > tol (the reference moves on
                            silently, mod_integrate.cu:120)                               */
} nsp_diag_out;

typedef struct nsp_ctx nsp_ctx;

/* Fills *p with the reference defaults (head.h:16-61: NR=48, NT=64, NZ=257, LT=2pi,
 * LZ=100, Re=1850, dt=0.01, d_im=0.51, maxit=10, tol=5e-8, sten=7) and Qdes=0.5. */
int nsp_default_params(nsp_params* p);

/* Creates a context for n_members pipes with parameters members[0..n_members-1] on
 * CUDA device `device`, in precision NSP_FP64 or NSP_MIXED, and allocates every
 * device buffer.  Replaces main.cu:16-33 (cudaSetDevice + the cudaMalloc of u, rhs). */
int nsp_create(const nsp_params* members, int n_members, int precision, int device, nsp_ctx** out);

/* Builds the radial grid, finite-difference weights, quadrature weights, the banded
 * LU factors of the Helmholtz/Poisson operators, the influence-matrix correction
 * vectors and the flux response.  Replaces init_fd (mod_radialFD.cu:199-312),
 * setLinear (mod_linear.cu:685-695), setCublasFlux (mod_cublasflux.cu:56-81) and
 * setBCon (mod_boundary.cu:205-255). */
int nsp_setup(nsp_ctx* ctx);

/* Restart files: three raw little-endian double2[NR][NT][NZ] files, byte-identical to
 * rBufferBinary / wBufferBinary (mod_io_nonlinear.cu:528-565; initField's restart
 * branch :426-429; the final dump main.cu:42-44). */
int nsp_load_state(nsp_ctx* ctx, int member, const char* file_r, const char* file_t, const char* file_z);
int nsp_save_state(nsp_ctx* ctx, int member, const char* file_r, const char* file_t, const char* file_z);

/* State transfer.  Host pointers: interleaved complex double arrays of NR*NT*NZ
 * values.  Device pointers: same layout in device memory on the context's device
 * (the caller-owned vfield of main.cu:30-33).  The host variants also accept
 * member = NSP_ALL_MEMBERS: each pointer then holds that component of every member,
 * back to back in member order (one synchronisation for the whole ensemble). */
#define NSP_ALL_MEMBERS (-1)
/* Setting a member's state clears its status (NSP_ERR_NONFINITE of an earlier state). */
int nsp_set_state_host(nsp_ctx* ctx, int member, const double* ur, const double* ut, const double* uz);
int nsp_get_state_host(nsp_ctx* ctx, int member, double* ur, double* ut, double* uz);
int nsp_set_state_device(nsp_ctx* ctx, int member, const void* ur, const void* ut, const void* uz);
int nsp_get_state_device(nsp_ctx* ctx, int member, void* ur, void* ut, void* uz);

/* Advances every member by nsteps time steps: nonlinear term, predictor, and
 * corrector iterations until err <= tol or maxit (integrate, mod_integrate.cu:98-160;
 * predictor :164-193; corrector :197-228; measucorr :232-241), each member with its
 * own iteration count.  One CUDA graph per step; the corrector loop is a device-side
 * conditional node.  iters_out (optional) receives nsteps*n_members counts,
 * step-major.  Returns NSP_ERR_NONFINITE if any member's convergence measure became
 * NaN/Inf (the other members are still advanced).  A step whose corrector loop stops
 * at maxit with err > tol is taken as in the reference, which continues silently
 * (mod_integrate.cu:120); it is counted per member (nsp_diag_out.unconverged_steps)
 * and, in strict mode (nsp_set_strict), makes the call return NSP_ERR_MAXIT after all
 * nsteps steps. */
int nsp_step(nsp_ctx* ctx, int nsteps, int* iters_out);

/* Host-resident form of integrate() over the whole ensemble: the states in `in` are
 * advanced by nsteps steps and written to `out`.  Both hold every member's field
 * member-major -- member 0's u_r, u_theta, u_z, then member 1's, ... (3*NR*NT*NZ
 * complex doubles per member); in and out may alias.  The result equals
 * nsp_set_state_host + nsp_step + nsp_get_state_host bit for bit.  The members are
 * stepped in chunks, each with its own step graph, so that the first step's copies in
 * and the last step's copies out overlap the other chunks' compute; the host arrays
 * should be pinned (cudaHostAlloc / cudaHostRegister) for the copies to overlap.
 * iters_out and the status codes as nsp_step. */
int nsp_step_host(nsp_ctx* ctx, int nsteps, const double* in, double* out, int* iters_out);

/* The nonlinear term -(u.grad)u of one member's field (r/theta form), 3/2-dealiased,
 * with the mean pressure-gradient forcing on mode (0,0) (nonlinear,
 * mod_io_nonlinear.cu:380-409).  All six pointers are device arrays of NR*NT*NZ
 * complex doubles; the evaluation uses the context's precision. */
int nsp_nonlinear(nsp_ctx* ctx, int member, const void* ur, const void* ut, const void* uz,
                  void* nr, void* nt, void* nz);

/* The nonlinear term of one member's field, computed without allocating any device
 * memory (no counterpart in the reference).  For callers that cannot allocate while
 * they run: hosts whose device-memory budget is fixed after start-up, applications
 * whose own pool allocator owns the device memory, and loops that cannot afford
 * cudaMalloc/cudaFree, which may synchronise the device.  u3 and n3 are device
 * arrays of 3*NR*NT*NZ complex doubles, the components (r, theta, z) back to back.
 * The transform intermediates live in a fixed 32 MiB __device__ array that every
 * process loading this library holds on each GPU it uses; a member whose
 * intermediates need more (9+3 complex arrays of NR*(3NT/2)*NZ in the working
 * precision, plus an FP32 copy of the input in the mixed form) is rejected with
 * NSP_ERR_ARG.  The first call on a device looks up the array's device address, so
 * make that first call before any stream capture.  The array is shared by every
 * call: calls that overlap on the GPU (other threads, other contexts on the same
 * device) race on it.  Nothing in it needs to start at zero.  u3 and n3 must not
 * overlap (NSP_ERR_ARG).  The cached address belongs to the device's primary context:
 * do not call this on a device after cudaDeviceReset of that device.  Synchronises the
 * context's stream; NSP_ERR_DEVICE as nsp_nonlinear if a tensor-core wait ran out. */
int nsp_nonlinear_static(nsp_ctx* ctx, int member, const void* u3, void* n3);

/* One banded solve on one member's operators (LUsolve_u flag 0/1/2 and LUsolve_p,
 * mod_linear.cu:664-679): kind 0 = u+, 1 = u-, 2 = u_z, 3 = pressure.  rhs and sol
 * are device arrays of NR*NT*NZ complex doubles (rhs is not modified).  Kinds 4..7:
 * the solve of kind - 4 in double-float (FP32 pairs, about 48 bits), the form the
 * mixed form's predictor (all kinds) and corrector passes (kind 3) use; mixed-form
 * contexts only (NSP_ERR_ARG otherwise). */
int nsp_lusolve(nsp_ctx* ctx, int member, int kind, const void* rhs, void* sol);

/* Diagnostics of one member (synchronises the context's stream). */
int nsp_diag(nsp_ctx* ctx, int member, nsp_diag_out* out);

/* Radial grid r[NR] and quadrature weights rdr[NR] of a member (after nsp_setup). */
int nsp_grid(nsp_ctx* ctx, int member, double* r, double* rdr);

/* Mean axial velocity profile Re u_z(m=0, k_z=0)(r_i), i = 0..NR-1, of one member:
 * the data row of wrt_mpr / wrt_mnp_k (mod_io_nonlinear.cu:119-129, 663-687)
 * without the time stamp.  out holds NR doubles (host memory). */
int nsp_mean_profile(nsp_ctx* ctx, int member, double* out);

/* Cross-section integrals of one member at the NZR = 3(NZ-1) physical axial points
 * z_n: q[n] = sum_i rdr_i <u_r^2 + u_theta^2>_theta and u[n] = sum_i rdr_i <u_z^2>_theta,
 * the data rows of wrt_qcr / wrt_ucr (mod_io_nonlinear.cu:572-660; theta rule of
 * q1kernel_k, radial rule of intq, mod_cublasflux.cu:119-130) without the time stamp.
 * Computed in FP64 on the device; q and u are host arrays of NZR doubles. */
int nsp_cross_sections(nsp_ctx* ctx, int member, double* q, double* u);

/* The same three diagnostics for every member at once (one launch per member group and
 * kernel, one synchronisation): out[n_members]; mean profiles and cross sections of all
 * members back to back in member order (sum of NR_m, resp. NZR_m values).  Values equal
 * the per-member calls' bit for bit. */
int nsp_diag_all(nsp_ctx* ctx, nsp_diag_out* out);
int nsp_mean_profile_all(nsp_ctx* ctx, double* out);
int nsp_cross_sections_all(nsp_ctx* ctx, double* q, double* u);

/* Number of kernel launches issued by the last nsp_step call (all graph nodes run). */
long long nsp_kernel_launches(nsp_ctx* ctx);

/* Introspection (no reference counterpart): writes a JSON object describing the
 * context's execution choices -- precision, whether the step is a CUDA graph, and
 * per member group its shape, member count, the autotuned linear-pass block
 * (modes, threads; in the mixed form also the corrector's increment pass, as
 * "linear_block_corrector") and the theta-transform path ("fft-fp64", "fft-fp32"
 * or "tcgen05-3xtf32") -- into buf (NUL-terminated).  NSP_ERR_ARG if cap is too small. */
int nsp_describe(nsp_ctx* ctx, char* buf, int cap);

/* Makes the context launch its work on `stream` (a cudaStream_t of the context's
 * device); NULL restores the context's own stream.  The reference runs on the
 * legacy default stream (no equivalent entry point). */
int nsp_set_stream(nsp_ctx* ctx, void* stream);

/* Strict convergence (no reference counterpart; the reference's integrate() moves on
 * silently at maxit, mod_integrate.cu:120): with strict != 0, nsp_step, nsp_step_host
 * and nsp_run_advance return NSP_ERR_MAXIT when a member's corrector loop stopped at
 * maxit with err > tol in one of the call's steps (NSP_ERR_NONFINITE takes precedence).
 * The states are those of the non-strict call.  Default 0. */
int nsp_set_strict(nsp_ctx* ctx, int strict);

/* Bounds record (no reference counterpart; the reference's kernels are unchecked).  The
 * library built with -DNSP_BOUNDS_CHECK (libnspipe_gb300_bc.so) checks every global
 * index that its step kernels compute -- state, nonlinear term, right-hand side and
 * correction slabs, transform intermediates, factor rows, stencil taps -- against the
 * extent it addresses, skips an access outside it and records it.  out[0] the number
 * of violations since the context was created, out[1] the first one's check site,
 * out[2] its index, out[3] the extent, out[4] 1 in the bounds-checked build (0: the
 * normal build, whose record stays 0).  Synchronises the context's stream. */
int nsp_bounds_report(nsp_ctx* ctx, long long* out);

/* Measurement hook (no reference counterpart): average device time in ms of one
 * launch of each kernel of the step, over `reps` back-to-back launches timed with
 * CUDA events on the context's stream, every member in corrector mode:
 * ms_out[0] theta-inverse transforms, [1] z transforms + nonlinear product,
 * [2] theta-forward transforms, [3] linear predictor/corrector pass, [4] convergence
 * bookkeeping.  The state is preserved; the corrector iterate buffers are overwritten. */
int nsp_profile_stages(nsp_ctx* ctx, int reps, double* ms_out);

/* Measurement hook (no reference counterpart): average device time in ms of one launch
 * of the linear pass with every member in its predictor pass (ms_out[0]) and in a
 * corrector pass (ms_out[1]; the mixed form's increment pass), over `reps` launches
 * timed with CUDA events on the context's stream.  The state is preserved; the
 * corrector iterate buffers are overwritten. */
int nsp_profile_linear(nsp_ctx* ctx, int reps, double* ms_out);

/* Measurement hook (no reference counterpart): FP64 multiply-add throughput of the
 * context's device in TFLOP/s (8 independent chains per thread, no memory traffic,
 * best of 3 timed launches), the denominator of the FP64 roofline. */
int nsp_measure_fp64_peak(nsp_ctx* ctx, double* tflops);

/* Parameters of one member; the context's member count and precision (either
 * output pointer may be NULL). */
int nsp_get_params(nsp_ctx* ctx, int member, nsp_params* out);
int nsp_info(nsp_ctx* ctx, int* n_members, int* precision);

/* ---- Time-integration driver ------------------------------------------------------
 * The reference's integrate() (mod_integrate.cu:98-160) around nsp_step: the time
 * accumulators and output cadence of mod_integrate.cu:109,131-152, the diagnostic
 * files of setIO / wrt_frc / wrt_qcr / wrt_ucr / wrt_mpr (mod_io_nonlinear.cu:260-318,
 * 460-687) in the reference's text formats, the final state dump of main.cu:42-44, and
 * (no reference counterpart) periodic checkpoints with a metadata sidecar from which
 * an interrupted run resumes with the same output files it would have written.
 *
 * Output cadence, per member and per file: after each step the member's dt is added
 * to its time t and to the file's accumulator (double additions, in the reference's
 * order); when the accumulator is >= the file's interval a row is sampled and the
 * accumulator reset to 0.  An interval < 0 switches the file off.
 *
 * Files, one member: io_friction.txt, io_qcross.txt, io_ucross.txt and io_meanpr.txt
 * in out_dir; several members: the same names in out_dir/member_NNNN/ (NNNN the
 * member index, 4 digits).  Formats (each value "%.8e", as the reference prints):
 *   io_friction.txt  rows "t  u_centre  u_tau"                            (no header)
 *   io_qcross.txt    header 0, z_0 .. z_{NZR-1}; rows t, q[NZR]    (z_n = LZ n / NZR)
 *   io_ucross.txt    header 0, z_0 .. z_{NZR-1}; rows t, u[NZR]
 *   io_meanpr.txt    header 0, r_0 .. r_{NR-1};  rows t, Re u_z(0,0)(r_i)
 * The reference writes rows in blocks of dc rows and drops a final partial block;
 * here rows are written in blocks of rows_per_write, and every pending row is written
 * at each checkpoint and by nsp_run_close.
 *
 * Checkpoints: ckpt_dir/step_SSSSSSSSSS/ (S the steps since the run opened, 10
 * digits) holds each member's ur_s.bin, ut_s.bin, uz_s.bin (one member: in the
 * directory itself, so that it is a restart directory of the reference, initField
 * mod_io_nonlinear.cu:426-429; several: in member_NNNN/) and checkpoint.json, written
 * last: the parameters, time, step and output accumulators of every member, the
 * FNV-1a 64 checksum of each state file and the size each output file had.  Writing
 * a checkpoint removes the directory's checkpoints of later steps (left by a run that
 * was resumed from an earlier checkpoint). */
typedef struct nsp_run_opts {
  const char* out_dir;  /* directory of the diagnostic files (created); NULL: no files   */
  double dt_frc;        /* interval of io_friction.txt rows              head.h:33     */
  double dt_qcr;        /* of io_qcross.txt and io_ucross.txt rows      head.h:36     */
  double dt_mnp;        /* of io_meanpr.txt rows                        head.h:39     */
  int rows_per_write;   /* rows buffered per file write (dc_frc/dc_qcr/dc_mnp) head.h:34-40 */
  const char* ckpt_dir; /* checkpoint directory (created); NULL: no checkpoints          */
  int ckpt_every;       /* steps between periodic checkpoints; 0: only nsp_run_checkpoint */
  int ckpt_keep;        /* complete checkpoints kept, older ones removed; 0: keep all    */
  int final_state;      /* nsp_run_close writes ur.bin, ut.bin, uz.bin of each member to
                           its output directory (main.cu:42-44)                         */
  int verbose;          /* print the reference's progress lines at each friction row
                           (mod_integrate.cu:136)                                       */
} nsp_run_opts;

typedef struct nsp_run nsp_run;

/* The reference's schedule: out_dir ".", every interval 0.5, 100 rows per write, no
 * checkpoints (ckpt_every 0, ckpt_keep 2), final_state 1, verbose 0. */
int nsp_run_default_opts(nsp_run_opts* o);

/* Starts a run at t = 0 on the context's current state (after nsp_setup and the
 * initial field): creates the output files and writes their header rows (setIO). */
int nsp_run_open(nsp_ctx* ctx, const nsp_run_opts* o, nsp_run** out);

/* Resumes a run from a checkpoint: ckpt is a step_* directory, or a checkpoint
 * directory (its newest complete checkpoint is taken).  Checks that the context has
 * the checkpoint's members and parameters and that every state file has its recorded
 * size and checksum (NSP_ERR_ARG / NSP_ERR_IO otherwise), loads the states, restores
 * the times and accumulators, and cuts each output file back to its recorded size so
 * that the rows written after the checkpoint are written again exactly once. */
int nsp_run_resume(nsp_ctx* ctx, const nsp_run_opts* o, const char* ckpt, nsp_run** out);

/* Advances every member by nsteps steps (nsp_step in chunks that end where a row or a
 * periodic checkpoint is due), writing rows and checkpoints on the way.  iters_out
 * (optional): nsteps * n_members corrector iteration counts, step-major.  A member
 * whose field becomes non-finite ends the call with NSP_ERR_NONFINITE after the rows
 * of that chunk are written, and no checkpoint is written for that state; in strict
 * mode (nsp_set_strict) a step that stopped at maxit without convergence ends the call
 * the same way with NSP_ERR_MAXIT. */
int nsp_run_advance(nsp_run* run, int nsteps, int* iters_out);

/* Writes a checkpoint of the current state now (pending rows are written first). */
int nsp_run_checkpoint(nsp_run* run);

/* Time and steps of one member since the run's t = 0. */
int nsp_run_time(nsp_run* run, int member, double* t, long long* steps);

/* Writes pending rows, the final states when final_state is set, closes the files and
 * frees the run (not the context).  A NULL run is a no-op. */
int nsp_run_close(nsp_run* run);

/* Host only (no context, no GPU): finds the checkpoint as nsp_run_resume does, checks
 * its state files against the sidecar, and copies the sidecar (JSON) and the resolved
 * checkpoint directory into json / path (either may be NULL; NUL-terminated).
 * NSP_ERR_IO for a missing, incomplete or corrupt checkpoint, NSP_ERR_ARG if a buffer
 * is too small. */
int nsp_checkpoint_info(const char* ckpt, char* json, int json_cap, char* path, int path_cap);

/* Host only: the output cadence.  For nsteps steps of length dt from accumulator *acc,
 * due[j] = 1 if a row is sampled after step j+1, else 0; *acc is updated.  An
 * interval < 0 gives no rows. */
int nsp_output_schedule(double dt, double interval, int nsteps, double* acc, unsigned char* due);

/* ---- Re_Mesh: change of resolution ------------------------------------------------
 * The reference's Re_Mesh tool (tools/Re_Mesh/src/mod_remesh.cu:50-124; its main
 * main.cu:14-33) as a batched device kernel.  A plan maps fields of shape (NR, NT, NZ)
 * to (Nrd, Ntd, Nzd): radial Lagrange interpolation on 2*iw points of the old grid
 * extended by iw points mirrored across the axis, with even / odd folding by the
 * parity of m and component (rmsh_k :8-29; weights fd_weights_rmsh :152-178; table
 * :70-115, the mirrored points' columns as the tool assigns them); theta and z modes
 * kept where both grids have them (-Ntd/2 <= m < Ntd/2, l < Nzd), zero elsewhere;
 * mode (0,0) with u_r = 0 and zero imaginary parts (modeZZ_k :34-40).  Grids of both
 * resolutions are init_fd's.  A member's field is its three components (u_r, u_theta,
 * u_z) back to back, each in the state layout above. */
typedef struct nsp_remesh nsp_remesh;

/* Builds the plan's tables on the host (no device work until the first launch);
 * iw in [1, 8] (the tool's default is 3). */
int nsp_remesh_create(int NR, int NT, int NZ, int Nrd, int Ntd, int Nzd, int iw, int device, nsp_remesh** out);
/* The interpolation tables RM[2][Nrd][NR] (0: even folding, 1: odd) into out (host). */
int nsp_remesh_matrix(const nsp_remesh* rm, double* out);
/* Remeshes `count` fields in one launch on `stream` (NULL: the legacy stream) and
 * waits for it: src[k] / dst[k] are device pointers (host arrays of them) to member
 * k's old / new field.  Every value of each dst field is written. */
int nsp_remesh_device(nsp_remesh* rm, int count, const void* const* src, void* const* dst, void* stream);
/* Remeshes context members in one launch: the state of src member src_members[k]
 * becomes the state of dst member dst_members[k] (src and dst may be the same context,
 * e.g. two groups of an uneven ensemble).  Shapes must be the plan's. */
int nsp_remesh_members(nsp_remesh* rm, nsp_ctx* src, const int* src_members, nsp_ctx* dst, const int* dst_members,
                       int count);
/* The tool itself: reads ur_o.bin, ut_o.bin, uz_o.bin from dir_in, writes ur_s.bin,
 * ut_s.bin, uz_s.bin to dir_out (mod_remesh.cu:56-58, main.cu:28-30). */
int nsp_remesh_files(nsp_remesh* rm, const char* dir_in, const char* dir_out);
int nsp_remesh_destroy(nsp_remesh* rm);

/* Test hook for the device-side failure path (no reference counterpart).  flags bit 0:
 * the mixed form's tensor-core transforms do not load their DFT-matrix operand, so the
 * bounded wait for it runs out (after 4096 polls instead of the normal limit); they
 * record a device fault, skip their tiles and return, and the next nsp_step reports
 * NSP_ERR_DEVICE.  No fault, trap or unbounded wait is involved; the context stays
 * usable.  0 clears. */
int nsp_debug_inject(nsp_ctx* ctx, int flags);

/* Waits for all work of the context. */
int nsp_sync(nsp_ctx* ctx);

/* The last failure of the context; with ctx NULL, the last failure of a context-free
 * call (nsp_remesh_*, nsp_checkpoint_info) in the calling thread. */
const char* nsp_last_error(nsp_ctx* ctx);
int nsp_destroy(nsp_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif
