// nsp_setup_dev.cu -- the mode tables of nsp_setup built on the device: one thread per
// (parameter set, mode), running the per-mode construction of nsp_setup_mode.h that
// the host build runs (this unit is compiled with --fmad=false, so every operation is
// the same IEEE multiply, add or divide as in the host build and the tables are
// bit-identical).  Factors and profiles are written straight into the group's tables
// in their [..][NT*NZ] layout, consecutive threads on consecutive modes (coalesced);
// the pressure solution of each mode goes to a scratch line with the same layout.
// Replaces the host construction whose cost grows with the number of distinct Re in
// an ensemble (setBCon / setLinear per member in the reference: mod_boundary.cu:205-255,
// mod_linear.cu:685-695).
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "nsp_internal.h"
#include "nsp_setup_mode.h"

namespace nsp {

namespace {

constexpr int SETUP_THREADS = 128;

struct SetupArgs {
  setup::Radial R;
  int NT, NZ;
  long long NTNZ;
  double kts, kzs, inv_dt;
  int set0;                 // first set of this launch
  const double* c_im;       // [nsets]
  double* fac;              // [nsets][4][NR][NFAC][NTNZ]
  double2* V;               // [nsets][3][NR][NTNZ]
  double2* ph;              // [sets of this launch][NR][NTNZ]
};

__global__ void __launch_bounds__(SETUP_THREADS) mode_tables_k(SetupArgs a) {
  using setup::cd;
  using setup::Strided;
  const long long k = (long long)blockIdx.x * SETUP_THREADS + threadIdx.x;
  if (k >= a.NTNZ) return;
  const int sl = blockIdx.y, set = a.set0 + sl;
  const int NR = a.R.NR;
  const int it = (int)(k / a.NZ), l = (int)(k % a.NZ);
  const int m = it < a.NT / 2 ? it : it - a.NT;
  const double kt = a.kts * (double)m, kz = a.kzs * (double)l;
  const long long fset = (long long)4 * NR * NFAC * a.NTNZ, vset = (long long)3 * NR * a.NTNZ;
  double* fac = a.fac + set * fset + k;
  cd* V = reinterpret_cast<cd*>(a.V + set * vset) + k;
  Strided<double> f[4];
  Strided<cd> v[3];
  for (int op = 0; op < 4; op++) f[op] = Strided<double>{fac + (long long)op * NR * NFAC * a.NTNZ, a.NTNZ};
  for (int c = 0; c < 3; c++) v[c] = Strided<cd>{V + (long long)c * NR * a.NTNZ, a.NTNZ};
  Strided<cd> ph{reinterpret_cast<cd*>(a.ph) + (long long)sl * NR * a.NTNZ + k, a.NTNZ};
  setup::setup_mode(a.R, a.c_im[set], a.inv_dt, m, kt, kz, m == 0 && l == 0, f[0], f[1], f[2], f[3], v[0], v[1],
                    v[2], ph);
}

}  // namespace

int launch_mode_tables(const nsp_params& p, int nsets, const double* c_im_host, const double* r, const double* D,
                       const double* Lu, const double* Lp, double* fac, double2* V, cudaStream_t st, std::string* err) {
  const long long NTNZ = (long long)p.NT * p.NZ;
  const size_t ph_set = sizeof(double2) * (size_t)p.NR * NTNZ;
  // scratch for at most ~256 MB of pressure lines per launch
  const int chunk = std::max(1, std::min(nsets, (int)((256u << 20) / std::max<size_t>(ph_set, 1))));
  double* d_cim = nullptr;
  double2* d_ph = nullptr;
  cudaError_t e = cudaMalloc(&d_cim, sizeof(double) * nsets);
  if (e == cudaSuccess) e = cudaMalloc(&d_ph, ph_set * chunk);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_cim, c_im_host, sizeof(double) * nsets, cudaMemcpyHostToDevice, st);
  SetupArgs a{setup::Radial{p.NR, r, D, Lu, Lp}, p.NT, p.NZ, NTNZ, PI2 / p.LT, PI2 / p.LZ, 1.0 / p.dt, 0, d_cim,
              fac, V, d_ph};
  for (int s0 = 0; e == cudaSuccess && s0 < nsets; s0 += chunk) {
    a.set0 = s0;
    dim3 grid((unsigned)((NTNZ + SETUP_THREADS - 1) / SETUP_THREADS), (unsigned)std::min(chunk, nsets - s0));
    mode_tables_k<<<grid, SETUP_THREADS, 0, st>>>(a);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess && err) *err = std::string("device operator setup: ") + cudaGetErrorString(e);
  cudaFree(d_cim);
  cudaFree(d_ph);
  return e == cudaSuccess ? NSP_OK : (e == cudaErrorMemoryAllocation ? NSP_ERR_NOMEM : NSP_ERR_CUDA);
}

}  // namespace nsp
