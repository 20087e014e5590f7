// nsp_remesh.cu -- change of resolution of saved fields, batched on the device: the
// reference Re_Mesh tool (tools/Re_Mesh/src/mod_remesh.cu:50-124, rmsh_k :8-29,
// modeZZ_k :34-40, fd_weights_rmsh :152-178; driver main.cu:14-33).
//
// Host: the radial interpolation tables RM[2][Nrd][NR] (even / odd axis folding) are
// built exactly as the tool builds them, then stored as compressed rows (the nonzero
// columns of each row in increasing order, at most 2 iw of them).
//
// Device: one launch for any number of members.  A block owns one destination theta
// slot and a tile of TL axial modes of one component of one member: it stages the
// source radial lines of that tile (NR x TL complex values, one coalesced read of the
// source) in shared memory, then writes every destination radius of the tile (one
// coalesced write).  Destination modes the source does not have are written as zeros,
// so the destination needs no prior clearing.  Each output is the FMA chain of the
// row's nonzero weights in column order -- the tool's own chain over all NR columns
// with the zero terms, which leave the sum unchanged, skipped.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "nsp_internal.h"

struct nsp_remesh {
  int NR, NT, NZ, Nrd, Ntd, Nzd, iw, K;
  int device;
  std::vector<double> RM;   // [2][Nrd][NR]
  std::vector<int> col, cnt;
  std::vector<double> w;
  int* d_col = nullptr;     // device copies, uploaded by the first launch
  int* d_cnt = nullptr;
  double* d_w = nullptr;
  void** d_ptr = nullptr;   // source and destination pointer arrays of a launch
  int ptr_cap = 0;
};

namespace nsp {

namespace {

constexpr int TL = 32;       // axial modes per block (one warp along l)
constexpr int ROWS = 8;      // warps per block (destination radii in flight)
constexpr int MAX_IW = 8;

struct RemeshArgs {
  int NR, NT, NZ, Nrd, Ntd, Nzd, K;
  const int* col;       // [2][Nrd][K]
  const int* cnt;       // [2][Nrd]
  const double* w;      // [2][Nrd][K]
  const double2* const* src;  // per member: 3 components of NR*NT*NZ back to back
  double2* const* dst;        // per member: 3 components of Nrd*Ntd*Nzd back to back
};

__global__ void __launch_bounds__(TL* ROWS) remesh_k(RemeshArgs a) {
  extern __shared__ double2 line[];  // [NR][TL]
  const int f = blockIdx.z, mem = f / 3, comp = f - 3 * mem;
  const int itd = blockIdx.y;
  const int m = itd < a.Ntd / 2 ? itd : itd - a.Ntd;          // signed azimuthal mode
  const bool have = m >= -(a.NT / 2) && m < a.NT / 2;          // the source holds it
  const int it = m >= 0 ? m : m + a.NT;
  const int lx = threadIdx.x, l = blockIdx.x * TL + lx;
  const int L = min(a.NZ, a.Nzd);
  const bool live = have && l < L;
  const long long S = (long long)a.NR * a.NT * a.NZ, Sd = (long long)a.Nrd * a.Ntd * a.Nzd;
  if (have && blockIdx.x * TL < L) {
    const double2* s = a.src[mem] + comp * S + (long long)it * a.NZ + l;
    for (int j = threadIdx.y; j < a.NR; j += ROWS)
      line[j * TL + lx] = l < L ? s[(long long)j * a.NT * a.NZ] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  if (l >= a.Nzd) return;
  // parity table: u_r, u_theta (flag 1) even folding for odd m; u_z (flag 0) for even m (rmsh_k :17)
  const int flag = comp == 2 ? 0 : 1;
  const int p = abs((abs(m) & 1) - flag);
  double2* o = a.dst[mem] + comp * Sd + (long long)itd * a.Nzd + l;
  for (int i = threadIdx.y; i < a.Nrd; i += ROWS) {
    double2 v = make_double2(0.0, 0.0);
    if (live) {
      const int row = p * a.Nrd + i;
      const int n = a.cnt[row];
      for (int k = 0; k < n; k++) {
        const double wk = a.w[row * a.K + k];
        const double2 x = line[a.col[row * a.K + k] * TL + lx];
        v.x = fma(wk, x.x, v.x);
        v.y = fma(wk, x.y, v.y);
      }
      if (itd == 0 && l == 0) {  // mode (0,0): u_r = 0, Im u_theta = Im u_z = 0 (modeZZ_k :34-40)
        if (comp == 0) v.x = 0.0;
        v.y = 0.0;
      }
    }
    o[(long long)i * a.Ntd * a.Nzd] = v;
  }
}

// init_fd's grid (mod_remesh.cu:60-68, the same formula as mod_radialFD.cu:211-216).
std::vector<double> grid(int NR) {
  std::vector<double> r(NR);
  const int N_p = NR + (int)std::sqrt((double)NR);
  for (int i = N_p - NR; i < N_p; i++) {
    const int ir = N_p - i - 1;
    r[i - N_p + NR] = 0.5 * (1.0 + std::cos(0.5 * PI2 * ((double)ir / (double)N_p)));
  }
  for (int it = 0; it < 10; it++) {
    const double dr = 1.5 * r[0] - 0.5 * r[1];
    for (int j = 0; j < NR; j++) r[j] = r[j] * (1.0 + dr) - dr;
  }
  return r;
}

// Lagrange weights at x0 on x[0..n-1]: Fornberg's recursion at derivative order 0.
void lagrange(const double* x, int n, double x0, double* c) {
  c[0] = 1.0;
  for (int i = 1; i < n; i++) c[i] = 0.0;
  double c1 = 1.0, c4 = x[0] - x0;
  for (int i = 1; i < n; i++) {
    double c2 = 1.0;
    const double c5 = c4;
    c4 = x[i] - x0;
    for (int j = 0; j < i; j++) {
      const double c3 = x[i] - x[j];
      c2 = c2 * c3;
      if (j == i - 1) c[i] = -c1 * c5 * c[i - 1] / c2;
      c[j] = c4 * c[j] / c3;
    }
    c1 = c2;
  }
}

// RM[2][Nrd][NR] (mod_remesh.cu:70-115).  Mirrored stencil points (extended-grid index
// below iw) go to column iw-1-j, j counted from the stencil's first point, with a
// minus sign in the odd table -- as the tool assigns them, which for a stencil
// starting past the first mirrored point is not that point's own mirror column.
void build_matrix(nsp_remesh* p) {
  const int NR = p->NR, Nrd = p->Nrd, iw = p->iw;
  const std::vector<double> r_o = grid(NR), r_h = grid(Nrd);
  std::vector<double> rau(NR + iw);
  for (int i = 0; i < NR + iw; i++) rau[i] = i < iw ? -r_o[iw - i - 1] : r_o[i - iw];
  std::vector<double>& RM = p->RM;
  RM.assign((size_t)2 * Nrd * NR, 0.0);
  RM[(size_t)NR * Nrd - 1] = 1.0;  // wall point -> old wall point (:83)
  RM[(size_t)2 * NR * Nrd - 1] = 1.0;
  int jleft = 0;
  double c[2 * MAX_IW];
  for (int i = 0; i < Nrd - 1; i++) {
    const double x0 = r_h[i];
    for (int j = 0; j < NR + iw; j++)
      if (rau[j] >= x0) {
        jleft = j;
        break;
      }
    jleft -= iw;
    const int jright = std::min(NR + iw - 1, jleft + 2 * iw - 1);
    const int n = jright - jleft + 1;
    lagrange(&rau[jleft], n, x0, c);
    jleft -= iw;
    int jaux = jleft;
    for (int j = 0; j < n; j++) {
      if (jaux < 0) {
        const int jcol = iw - j - 1;
        jaux += 1;
        RM[(size_t)i * NR + jcol] += c[j];
        RM[(size_t)NR * Nrd + (size_t)i * NR + jcol] -= c[j];
      } else {
        const int jcol = jleft + j;
        RM[(size_t)i * NR + jcol] += c[j];
        RM[(size_t)NR * Nrd + (size_t)i * NR + jcol] += c[j];
      }
    }
  }
  // compressed rows
  p->K = 2 * iw;
  p->col.assign((size_t)2 * Nrd * p->K, 0);
  p->w.assign((size_t)2 * Nrd * p->K, 0.0);
  p->cnt.assign((size_t)2 * Nrd, 0);
  for (int row = 0; row < 2 * Nrd; row++) {
    int n = 0;
    for (int j = 0; j < NR; j++) {
      const double v = RM[(size_t)row * NR + j];
      if (v != 0.0) {
        p->col[(size_t)row * p->K + n] = j;
        p->w[(size_t)row * p->K + n] = v;
        n++;
      }
    }
    p->cnt[row] = n;
  }
}

int rfail(nsp_remesh*, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  set_host_error(buf);
  return code;
}

int cuda_fail(nsp_remesh* p, cudaError_t e, const char* what) {
  return rfail(p, NSP_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define RCK(call)                                       \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(p, e_, #call); \
  } while (0)

int upload(nsp_remesh* p, int count) {
  RCK(cudaSetDevice(p->device));
  if (!p->d_col) {
    RCK(cudaMalloc(&p->d_col, p->col.size() * sizeof(int)));
    RCK(cudaMalloc(&p->d_cnt, p->cnt.size() * sizeof(int)));
    RCK(cudaMalloc(&p->d_w, p->w.size() * sizeof(double)));
    RCK(cudaMemcpy(p->d_col, p->col.data(), p->col.size() * sizeof(int), cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(p->d_cnt, p->cnt.data(), p->cnt.size() * sizeof(int), cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(p->d_w, p->w.data(), p->w.size() * sizeof(double), cudaMemcpyHostToDevice));
    const size_t smem = (size_t)p->NR * TL * sizeof(double2);
    RCK(cudaFuncSetAttribute(remesh_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  if (p->ptr_cap < count) {
    if (p->d_ptr) RCK(cudaFree(p->d_ptr));
    p->d_ptr = nullptr;
    RCK(cudaMalloc(&p->d_ptr, 2 * (size_t)count * sizeof(void*)));
    p->ptr_cap = count;
  }
  return NSP_OK;
}

}  // namespace

// Launches the remesh of `count` members; src / dst are host arrays of device pointers.
// Synchronises the stream (the pointer array is reused by the next call).
int remesh_launch(nsp_remesh* p, int count, const void* const* src, void* const* dst, cudaStream_t st) {
  if (count <= 0) return NSP_OK;
  if (3LL * count > 65535) return rfail(p, NSP_ERR_ARG, "at most 21845 members per remesh call");
  for (int k = 0; k < count; k++)
    if (!src[k] || !dst[k]) return rfail(p, NSP_ERR_ARG, "null field pointer (member %d)", k);
  if (int rc = upload(p, count)) return rc;
  std::vector<const void*> ptrs(2 * (size_t)count);
  for (int k = 0; k < count; k++) {
    ptrs[k] = src[k];
    ptrs[count + k] = dst[k];
  }
  RCK(cudaMemcpyAsync(p->d_ptr, ptrs.data(), ptrs.size() * sizeof(void*), cudaMemcpyHostToDevice, st));
  RemeshArgs a{p->NR, p->NT, p->NZ, p->Nrd, p->Ntd, p->Nzd, p->K, p->d_col, p->d_cnt, p->d_w,
               reinterpret_cast<const double2* const*>(p->d_ptr), reinterpret_cast<double2* const*>(p->d_ptr + count)};
  dim3 grid_((p->Nzd + TL - 1) / TL, p->Ntd, 3 * count), block(TL, ROWS);
  remesh_k<<<grid_, block, (size_t)p->NR * TL * sizeof(double2), st>>>(a);
  RCK(cudaGetLastError());
  RCK(cudaStreamSynchronize(st));
  return NSP_OK;
}

void remesh_shape(const nsp_remesh* p, int* old3, int* new3) {
  old3[0] = p->NR, old3[1] = p->NT, old3[2] = p->NZ;
  new3[0] = p->Nrd, new3[1] = p->Ntd, new3[2] = p->Nzd;
}

int remesh_device(const nsp_remesh* p) { return p->device; }

}  // namespace nsp

using namespace nsp;

extern "C" {

int nsp_remesh_create(int NR, int NT, int NZ, int Nrd, int Ntd, int Nzd, int iw, int device, nsp_remesh** out) {
  if (!out) return rfail(nullptr, NSP_ERR_ARG, "null output");
  *out = nullptr;
  if (iw < 1 || iw > MAX_IW) return rfail(nullptr, NSP_ERR_ARG, "iw = %d outside [1, %d]", iw, MAX_IW);
  if (NR < std::max(2, iw) || Nrd < 2) return rfail(nullptr, NSP_ERR_ARG, "NR = %d, Nrd = %d: need NR >= max(2, iw), Nrd >= 2", NR, Nrd);
  if (NT < 2 || NT % 2 || Ntd < 2 || Ntd % 2) return rfail(nullptr, NSP_ERR_ARG, "NT = %d, Ntd = %d: need even values >= 2", NT, Ntd);
  if (NZ < 1 || Nzd < 1) return rfail(nullptr, NSP_ERR_ARG, "NZ = %d, Nzd = %d: need >= 1", NZ, Nzd);
  if ((size_t)NR * TL * sizeof(double2) > 227 * 1024) return rfail(nullptr, NSP_ERR_ARG, "NR = %d: the radial lines of a tile exceed shared memory", NR);
  if (device < 0) return rfail(nullptr, NSP_ERR_ARG, "device %d", device);
  nsp_remesh* p = new nsp_remesh;
  p->NR = NR, p->NT = NT, p->NZ = NZ, p->Nrd = Nrd, p->Ntd = Ntd, p->Nzd = Nzd, p->iw = iw, p->device = device;
  build_matrix(p);
  *out = p;
  return NSP_OK;
}

int nsp_remesh_matrix(const nsp_remesh* p, double* out) {
  if (!p || !out) return rfail(nullptr, NSP_ERR_ARG, "null argument");
  memcpy(out, p->RM.data(), p->RM.size() * sizeof(double));
  return NSP_OK;
}

int nsp_remesh_device(nsp_remesh* p, int count, const void* const* src, void* const* dst, void* stream) {
  if (!p || count < 0 || (count > 0 && (!src || !dst))) return rfail(p, NSP_ERR_ARG, "invalid arguments");
  return remesh_launch(p, count, src, dst, static_cast<cudaStream_t>(stream));
}

int nsp_remesh_files(nsp_remesh* p, const char* dir_in, const char* dir_out) {
  if (!p || !dir_in || !dir_out) return rfail(p, NSP_ERR_ARG, "null argument");
  const size_t S = (size_t)p->NR * p->NT * p->NZ, Sd = (size_t)p->Nrd * p->Ntd * p->Nzd;
  std::vector<double> h(2 * 3 * std::max(S, Sd));
  const char* comp = "rtz";
  for (int c = 0; c < 3; c++) {  // rBufferBinary of u?_o.bin (mod_remesh.cu:56-58)
    std::string f = std::string(dir_in) + "/u" + comp[c] + "_o.bin";
    FILE* fh = fopen(f.c_str(), "rb");
    if (!fh) return rfail(p, NSP_ERR_IO, "reading error: %s", f.c_str());
    size_t got = fread(h.data() + 2 * S * c, 16, S, fh);
    int extra = fgetc(fh);
    fclose(fh);
    if (got != S || extra != EOF) return rfail(p, NSP_ERR_IO, "reading error: %s is not %zu values", f.c_str(), S);
  }
  RCK(cudaSetDevice(p->device));
  void *d_in = nullptr, *d_out = nullptr;
  RCK(cudaMalloc(&d_in, 3 * S * sizeof(double2)));
  cudaError_t e = cudaMalloc(&d_out, 3 * Sd * sizeof(double2));
  int rc = NSP_OK;
  if (e != cudaSuccess) rc = cuda_fail(p, e, "cudaMalloc");
  if (rc == NSP_OK && (e = cudaMemcpy(d_in, h.data(), 3 * S * sizeof(double2), cudaMemcpyHostToDevice)) != cudaSuccess)
    rc = cuda_fail(p, e, "cudaMemcpy");
  if (rc == NSP_OK) rc = remesh_launch(p, 1, (const void* const*)&d_in, &d_out, 0);
  if (rc == NSP_OK && (e = cudaMemcpy(h.data(), d_out, 3 * Sd * sizeof(double2), cudaMemcpyDeviceToHost)) != cudaSuccess)
    rc = cuda_fail(p, e, "cudaMemcpy");
  cudaFree(d_in);
  cudaFree(d_out);
  if (rc) return rc;
  for (int c = 0; c < 3; c++) {  // wBufferBinary of u?_s.bin (main.cu:28-30)
    std::string f = std::string(dir_out) + "/u" + comp[c] + "_s.bin";
    FILE* fh = fopen(f.c_str(), "wb");
    if (!fh) return rfail(p, NSP_ERR_IO, "writing error: %s", f.c_str());
    size_t put = fwrite(h.data() + 2 * Sd * c, 16, Sd, fh);
    if (fclose(fh) != 0 || put != Sd) return rfail(p, NSP_ERR_IO, "writing error: %s", f.c_str());
  }
  return NSP_OK;
}

int nsp_remesh_destroy(nsp_remesh* p) {
  if (!p) return NSP_OK;
  if (p->d_col) {
    cudaSetDevice(p->device);
    cudaFree(p->d_col);
    cudaFree(p->d_cnt);
    cudaFree(p->d_w);
    if (p->d_ptr) cudaFree(p->d_ptr);
  }
  delete p;
  return NSP_OK;
}

}  // extern "C"
