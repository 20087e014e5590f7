// nsp_api.cu -- the C ABI (include/nspipe_gb300.h): contexts, operator upload,
// the CUDA-graph time step and state I/O.
//
// One nsp_step time step is one launch of a CUDA graph whose only node is a
// conditional WHILE node.  Its body evaluates, for every member group, the
// nonlinear term (3 kernels) and the predictor/corrector linear pass (1 kernel),
// then converge_k updates each member's phase and sets the loop condition.
// The first body iteration is the predictor of every member; later iterations
// are corrector iterations of the members that have not converged (the others
// skip their blocks), so each member keeps the reference's own iteration count
// (integrate, mod_integrate.cu:112-130) without any device-to-host round trip.
#include <sys/stat.h>

#include <cmath>
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "nsp_bounds.cuh"
#include "nsp_fft.cuh"
#include "nsp_internal.h"

namespace nsp {
void configure_transform_kernels();
void configure_linear_kernels();
bool transform_supported(int NTP, int NZR);
}  // namespace nsp

using namespace nsp;

namespace {

struct Group {
  nsp_params p;
  std::vector<int> users;   // user member indices, in slot order
  std::vector<double> sets; // distinct Re of the group (operator parameter sets)
  std::vector<int> mset;    // [slot] parameter set of each member
  HostOps ops;              // radial tables and set 0's flux response (host copy)
  bool device_setup = true; // mode tables built on the device (else on the host)
  Tables tb{};
  Bufs bf{};
};

}  // namespace

struct nsp_ctx {
  int device = 0;
  int precision = NSP_FP64;
  int nmem = 0;
  std::vector<nsp_params> prm;
  std::vector<int> grp, slot, internal;  // per user member
  std::vector<Group> groups;
  cudaStream_t st = nullptr;
  cudaStream_t own_st = nullptr;
  Ctl hctl{};
  Ctl* dctl = nullptr;
  int parity = 0;  // host mirror of ctl.parity
  bool setup_done = false;
  cudaGraphExec_t gexec = nullptr;
  bool use_graph = false;
  long long launches_last = 0;
  double2* scratch = nullptr;  // 2 x 3 x Smax, for nsp_nonlinear
  float2* scratch32 = nullptr; // 3 x Smax, FP32 input of nsp_nonlinear in the mixed form
  unsigned long long* diagbuf = nullptr;  // 2 ordered-bit maxima of the divergence diagnostic
  double* crossbuf = nullptr;             // per-level partials of the cross-section diagnostics
  size_t crossbuf_n = 0;
  // Parallel branches of the step graph: one per member group beyond the first.
  std::vector<cudaStream_t> side;
  cudaEvent_t ev_fork = nullptr;
  std::vector<cudaEvent_t> ev_join;
  // nsp_step_host: copy streams and per-chunk events (created on first use)
  cudaStream_t cp_in = nullptr, cp_out = nullptr;
  std::vector<cudaEvent_t> ev_in, ev_done;
  std::vector<cudaGraphExec_t> chunk_exec;  // step graphs of the member chunks
  std::vector<int> chunk_lo;                // their internal member bounds (K+1 values)
  long long Smax = 0;
  // Mixed form: U32/DR32[parity] hold the FP32 mirror of U[parity] (kept current by the
  // linear pass; cleared by every call that writes the state from outside).
  bool mirror_ok = false;
  // nsp_set_strict: a step whose corrector loop stopped at maxit with err > tol makes
  // nsp_step / nsp_step_host return NSP_ERR_MAXIT.
  bool strict = false;
  // Pinned host copy of the step history, then the members' status words, the fault
  // flag and the members' unconverged-step counts: read back after the steps with
  // asynchronous copies and one synchronisation.
  int* pin = nullptr;
  std::vector<void*> allocs;
  std::string err;
};

namespace {

int fail(nsp_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CK(call)                                                                                           \
  do {                                                                                                     \
    cudaError_t e_ = (call);                                                                               \
    if (e_ != cudaSuccess)                                                                                 \
      return fail(c, e_ == cudaErrorMemoryAllocation ? NSP_ERR_NOMEM : NSP_ERR_CUDA, "%s: %s (%s:%d)", #call, \
                  cudaGetErrorString(e_), __FILE__, __LINE__);                                             \
  } while (0)

template <typename X>
int dalloc(nsp_ctx* c, X** p, size_t bytes) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, bytes ? bytes : 16);
  if (e != cudaSuccess) return fail(c, NSP_ERR_NOMEM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  c->allocs.push_back(q);
  *p = (X*)q;
  return NSP_OK;
}

template <typename X>
int upload(nsp_ctx* c, const X** dst, const std::vector<X>& v) {
  X* d = nullptr;
  int rc = dalloc(c, &d, sizeof(X) * v.size());
  if (rc) return rc;
  CK(cudaMemcpy(d, v.data(), sizeof(X) * v.size(), cudaMemcpyHostToDevice));
  *dst = d;
  return NSP_OK;
}

bool smooth23(int n) {
  if (n < 2) return false;
  while (n % 2 == 0) n /= 2;
  while (n % 3 == 0) n /= 3;
  return n == 1;
}

// exp(-2 pi i e / n), exact at quarter turns, long-double accurate otherwise.
std::vector<double2> twiddles(int n) {
  std::vector<double2> w(n);
  const long double PI_L = 3.141592653589793238462643383279502884L;
  for (int e = 0; e < n; e++) {
    long long e4 = 4LL * e;
    if (e4 % n == 0) {
      static const double cx[4] = {1.0, 0.0, -1.0, 0.0}, sy[4] = {0.0, -1.0, 0.0, 1.0};
      int q = (int)(e4 / n) & 3;
      w[e] = make_double2(cx[q], sy[q]);
    } else {
      long double a = -2.0L * PI_L * (long double)e / (long double)n;
      w[e] = make_double2((double)cosl(a), (double)sinl(a));
    }
  }
  return w;
}

std::vector<float2> to_f32(const std::vector<double2>& v) {
  std::vector<float2> o(v.size());
  for (size_t i = 0; i < v.size(); i++) o[i] = make_float2((float)v[i].x, (float)v[i].y);
  return o;
}

// Members sharing everything but Re share one group (one launch per stage);
// their Re values become the group's operator parameter sets.
bool same_shape(const nsp_params& a, const nsp_params& b) {
  return a.NR == b.NR && a.NT == b.NT && a.NZ == b.NZ && a.LT == b.LT && a.LZ == b.LZ && a.dt == b.dt &&
         a.d_im == b.d_im && a.sten == b.sten && a.Qdes == b.Qdes && a.maxit == b.maxit && a.tol == b.tol;
}

// x = hi + lo with hi = fl32(x), lo = fl32(x - hi): the double-float form of a table.
static std::vector<float2> split_df_host(const std::vector<double>& v) {
  std::vector<float2> o(v.size());
  for (size_t e = 0; e < v.size(); e++) {
    const float hi = (float)v[e];
    o[e] = make_float2(hi, (float)(v[e] - (double)hi));
  }
  return o;
}

// Tables of one member's parameter set only (for single-member calls: nsp_nonlinear,
// nsp_lusolve), as a one-set view of its group's tables.
Tables member_view(const Group& g, int slot) {
  Tables t = g.tb;
  const int ps = g.mset[slot];
  t.fac += (size_t)ps * 4 * t.NR * NFAC * t.NTNZ;
  t.V += (size_t)ps * 3 * t.S;
  if (t.V32) t.V32 += (size_t)ps * 3 * t.S;
  if (t.facdf) t.facdf += (size_t)ps * 4 * t.NR * NFAC * t.NTNZ;
  if (t.fac32) t.fac32 += (size_t)ps * 4 * t.NR * NFAC * t.NTNZ;
  if (t.Vdf) t.Vdf += (size_t)ps * 2 * 3 * t.S;
  t.Luc += (size_t)ps * 2 * STEN * t.NR;
  t.Luc32 += (size_t)ps * 2 * STEN * t.NR;
  t.uc += (size_t)ps * t.NR;
  t.sscal += (size_t)4 * ps;
  t.nsets = 1;
  return t;
}

// The group's tables and buffers restricted to its members [a, b) (local slots): the
// kernels then cover only those members (chunked steps).
void range_view(const Group& g, bool mixed, int a, int b, Tables* t, Bufs* bf) {
  *t = g.tb;
  *bf = g.bf;
  t->nmem = b - a;
  t->mem0 = g.tb.mem0 + a;
  if (g.tb.nsets > 1) t->mset = g.tb.mset + a;
  const size_t s3 = (size_t)a * 3 * g.tb.S;
  for (int k = 0; k < 2; k++) {
    bf->U[k] += s3;
    if (bf->U32[k]) bf->U32[k] += s3;
    if (bf->DR32[k]) bf->DR32[k] += s3;
  }
  if (bf->RHSW) bf->RHSW += s3;
  if (bf->N) bf->N += s3;
  if (bf->N32) bf->N32 += s3;
  if (bf->RHSW32) bf->RHSW32 += s3;
  if (bf->NF) bf->NF += a;
  if (bf->RW00) bf->RW00 += (size_t)a * g.tb.NR;
  const size_t esz = mixed ? sizeof(float2) : sizeof(double2);
  const size_t plane = (size_t)g.tb.NR * g.tb.NTP * g.tb.NZ * esz;
  bf->G = static_cast<char*>(g.bf.G) + (size_t)a * 9 * plane;
  bf->H = static_cast<char*>(g.bf.H) + (size_t)a * 3 * plane;
  if (g.bf.MEAN) bf->MEAN = g.bf.MEAN + (size_t)a * g.tb.NR * MEAN_N;
}

int check_params(nsp_ctx* c, const nsp_params& p, int idx) {
  if (p.NR < 8 || p.NR > 1024) return fail(c, NSP_ERR_ARG, "member %d: NR=%d outside [8, 1024]", idx, p.NR);
  if (p.NT < 4 || p.NT % 2) return fail(c, NSP_ERR_ARG, "member %d: NT=%d must be even and >= 4", idx, p.NT);
  if (p.NZ < 3 || p.NZ % 2 == 0) return fail(c, NSP_ERR_ARG, "member %d: NZ=%d must be odd and >= 3", idx, p.NZ);
  if (p.sten != STEN) return fail(c, NSP_ERR_ARG, "member %d: sten=%d (only 7 is supported)", idx, p.sten);
  int NTP = 3 * p.NT / 2, NZR = 3 * (p.NZ - 1);
  if (!smooth23(NTP) || !smooth23(NZR))
    return fail(c, NSP_ERR_ARG, "member %d: transform lengths %d x %d must be of the form 2^a 3^b", idx, NTP, NZR);
  if (!transform_supported(NTP, NZR))
    return fail(c, NSP_ERR_ARG, "member %d: transform lengths %d x %d exceed the block size limits", idx, NTP, NZR);
  if (!(p.Re > 0) || !(p.dt > 0) || !(p.LT > 0) || !(p.LZ > 0) || p.maxit < 1 || !(p.tol >= 0) || !(p.Qdes == p.Qdes))
    return fail(c, NSP_ERR_ARG, "member %d: Re, dt, LT, LZ must be > 0, maxit >= 1, tol >= 0", idx);
  return NSP_OK;
}

int check_member(nsp_ctx* c, int m) {
  if (!c) return NSP_ERR_ARG;
  if (m < 0 || m >= c->nmem) return fail(c, NSP_ERR_ARG, "member %d out of range [0, %d)", m, c->nmem);
  return NSP_OK;
}

double2* state_ptr(nsp_ctx* c, int m, int comp) {
  Group& g = c->groups[c->grp[m]];
  return g.bf.U[c->parity] + ((size_t)c->slot[m] * 3 + comp) * g.tb.S;
}

// ------------------------------------------------------------ autotuner
// Picks the block shape of the linear pass per member group by timing every
// candidate on the context's own buffers (all members in corrector mode, CUDA
// events, best of 3 after a warm-up).  Choices are cached in a flat JSON object
// {"NRxNTxNZ:mM:pP": variant, ...} at $NSP_TUNE_CACHE (default
// $HOME/.cache/nspipe_gb300/tune.json); NSP_AUTOTUNE=0 keeps the defaults.
std::string tune_path() {
  const char* p = getenv("NSP_TUNE_CACHE");
  if (p && *p) return p;
  const char* h = getenv("HOME");
  return std::string(h ? h : "/tmp") + "/.cache/nspipe_gb300/tune.json";
}

std::map<std::string, int> tune_load() {
  std::map<std::string, int> m;
  FILE* f = fopen(tune_path().c_str(), "r");
  if (!f) return m;
  char key[256];
  int v;
  int ch;
  while ((ch = fgetc(f)) != EOF) {
    if (ch != '"') continue;
    if (fscanf(f, "%255[^\"]\": %d", key, &v) == 2) m[key] = v;
  }
  fclose(f);
  return m;
}

void tune_store(const std::map<std::string, int>& m) {
  std::string path = tune_path();
  for (size_t pos = path.find('/', 1); pos != std::string::npos; pos = path.find('/', pos + 1))
    mkdir(path.substr(0, pos).c_str(), 0755);  // existing directories are fine
  FILE* f = fopen(path.c_str(), "w");
  if (!f) return;
  fprintf(f, "{");
  size_t k = 0;
  for (auto& kv : m) fprintf(f, "%s\"%s\": %d", k++ ? ", " : "", kv.first.c_str(), kv.second);
  fprintf(f, "}\n");
  fclose(f);
}

// A kernel whose bounded wait ran out sets Ctl::fault (and abandons its work).
int check_fault(nsp_ctx* c) {
  int fault = 0;
  CK(cudaMemcpyAsync(&fault, &c->dctl->fault, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (fault) {
    CK(cudaMemsetAsync(&c->dctl->fault, 0, sizeof(int), c->st));
    return fail(c, NSP_ERR_DEVICE, "a device-side wait ran out; the call's results are invalid");
  }
  return NSP_OK;
}

int reset_control(nsp_ctx* c) {
  const int nm = c->nmem;
  std::vector<int> zeros(nm, 0);
  CK(cudaMemcpyAsync(c->hctl.phase, zeros.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemsetAsync(c->hctl.num, 0, sizeof(unsigned long long) * nm, c->st));
  CK(cudaMemsetAsync(c->hctl.den, 0, sizeof(unsigned long long) * nm, c->st));
  CK(cudaMemsetAsync(c->hctl.status, 0, sizeof(int) * nm, c->st));
  CK(cudaMemsetAsync(c->hctl.ite, 0, sizeof(int) * nm, c->st));
  CK(cudaMemcpyAsync(&c->dctl->parity, &c->parity, sizeof(int), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return NSP_OK;
}

// The z-stage kernel of each group (radix-stage or one of the two-pass splits compiled
// for its length and precision), timed like the linear pass: z stage alone on the
// group's buffers, best of 3 after a warm-up.  Cached per shape and precision,
// "z1:NRxNTxNZ:pP", not per member count: the kernels differ in rounding, and members
// of one shape give the same bits whatever ensemble they are stepped in.
int autotune_z(nsp_ctx* c, std::map<std::string, int>& cache, bool* dirty) {
  const bool mixed = c->precision == NSP_MIXED;
  const int nm = c->nmem;
  std::vector<int> zeros(nm, 0);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  for (auto& g : c->groups) {
    const int nv = z_variants(g.tb.NZR, g.tb.NTP, mixed);
    if (nv == 0) continue;
    char key[128];
    snprintf(key, sizeof key, "z1:%dx%dx%d:p%d", g.tb.NR, g.tb.NT, g.tb.NZ, c->precision);
    auto it = cache.find(key);
    if (it != cache.end() && it->second >= 0 && it->second <= nv) {
      g.tb.z_variant = it->second;
      continue;
    }
    CK(cudaMemcpyAsync(c->hctl.phase, zeros.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, c->st));
    float best = 1e30f;
    for (int v = 0; v <= nv; v++) {
      Tables tv = g.tb;
      tv.z_variant = v;
      launch_nonlinear(tv, g.bf, c->dctl, mixed, nullptr, nullptr, c->st, 2);
      float t = 1e30f;
      for (int r = 0; r < 3; r++) {
        CK(cudaEventRecord(e0, c->st));
        launch_nonlinear(tv, g.bf, c->dctl, mixed, nullptr, nullptr, c->st, 2);
        CK(cudaEventRecord(e1, c->st));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        t = std::min(t, ms);
      }
      CK(cudaGetLastError());
      if (t < best) { best = t; g.tb.z_variant = v; }
    }
    cache[key] = g.tb.z_variant;
    *dirty = true;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return NSP_OK;
}

int autotune(nsp_ctx* c) {
  for (auto& g : c->groups) {
    g.tb.lin_variant = g.tb.lin_variant_inc = linear_default_variant(g.tb.NR);
    g.tb.z_variant = z_default_variant(g.tb.NZR, g.tb.NTP, c->precision == NSP_MIXED);
  }
  const char* ev = getenv("NSP_AUTOTUNE");
  if (ev && ev[0] == '0') return NSP_OK;
  std::map<std::string, int> cache = tune_load();
  bool dirty = false;
  const int nm = c->nmem;
  std::vector<int> zeros(nm, 0), ones(nm, 1);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  for (auto& g : c->groups) {
    char key[128];
    snprintf(key, sizeof key, "v2:%dx%dx%d:m%d:p%d", g.tb.NR, g.tb.NT, g.tb.NZ, g.tb.nmem, c->precision);
    const std::string key_inc = std::string(key) + ":inc";
    auto it = cache.find(key), it_inc = cache.find(key_inc);
    const bool mixed = c->precision == NSP_MIXED;
    if (it != cache.end() && linear_variant_fits(it->second, g.tb.NR) &&
        (!mixed || (it_inc != cache.end() && linear_variant_fits(it_inc->second, g.tb.NR)))) {
      g.tb.lin_variant = it->second;
      if (mixed) g.tb.lin_variant_inc = it_inc->second;
      continue;
    }
    // A step is one predictor pass (phase 0) and usually one or two corrector passes
    // (phase 1): in the FP64 form one kernel takes both and each candidate is scored by
    // predictor + corrector time; in the mixed form the corrector is its own kernel
    // (the increment pass) and the two passes are tuned separately.
    float best = 1e30f, best_p[2] = {1e30f, 1e30f};
    for (int v = 0; v < LIN_VARIANTS; v++) {
      if (!linear_variant_fits(v, g.tb.NR)) continue;
      Tables tv = g.tb;
      tv.lin_variant = tv.lin_variant_inc = v;
      float score = 0.f;
      for (int phase = 0; phase < 2; phase++) {
        const std::vector<int>& ph = phase ? ones : zeros;
        const int which = phase ? LIN_CORR : LIN_PRED;
        CK(cudaMemcpyAsync(c->hctl.phase, ph.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, c->st));
        launch_linear(tv, g.bf, c->dctl, c->st, which);
        float t = 1e30f;
        for (int r = 0; r < 3; r++) {
          CK(cudaEventRecord(e0, c->st));
          launch_linear(tv, g.bf, c->dctl, c->st, which);
          CK(cudaEventRecord(e1, c->st));
          CK(cudaEventSynchronize(e1));
          float ms = 0.f;
          CK(cudaEventElapsedTime(&ms, e0, e1));
          t = std::min(t, ms);
        }
        score += t;
        if (mixed && t < best_p[phase]) {
          best_p[phase] = t;
          (phase ? g.tb.lin_variant_inc : g.tb.lin_variant) = v;
        }
      }
      CK(cudaGetLastError());
      if (!mixed && score < best) { best = score; g.tb.lin_variant = v; }
    }
    cache[key] = g.tb.lin_variant;
    if (mixed) cache[key_inc] = g.tb.lin_variant_inc;
    dirty = true;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const char* ez = getenv("NSP_Z2");
  if (!(ez && ez[0] == '0'))
    if (int rc = autotune_z(c, cache, &dirty)) return rc;
  if (dirty) tune_store(cache);
  return reset_control(c);
}

// The step graph of the members with internal index in [lo, hi) (all members: the
// context's step graph; a sub-range: a chunk graph of nsp_step_host) into *out.
int build_graph_range(nsp_ctx* c, int lo, int hi, cudaGraphExec_t* out) {
  if (*out) { cudaGraphExecDestroy(*out); *out = nullptr; }
  cudaGraph_t g = nullptr;
  CK(cudaGraphCreate(&g, 0));
  struct GraphOwner {  // destroys the step graph on every return path (instantiation copies it)
    cudaGraph_t g;
    ~GraphOwner() { cudaGraphDestroy(g); }
  } owner{g};
  cudaGraphConditionalHandle h;
  cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) {
    cudaGetLastError();
    c->use_graph = false;
    return NSP_OK;
  }
  // Member groups (different shapes) are independent until the convergence
  // bookkeeping: each group's kernels form their own branch of a pass so that groups
  // run concurrently, then converge_k joins them.
  const size_t ng = c->groups.size();
  if (c->side.size() + 1 < ng) {
    if (!c->ev_fork) CK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    while (c->side.size() + 1 < ng) {
      cudaStream_t s2;
      cudaEvent_t e2;
      CK(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&e2, cudaEventDisableTiming));
      c->side.push_back(s2);
      c->ev_join.push_back(e2);
    }
  }
  // One pass (the three transforms and the linear-pass kernel `which` per group, then
  // converge_k, which sets the loop condition when `cond`) captured into `into`.
  // A failure inside the capture still ends it, so that the context's stream is not
  // left capturing; the partial graph belongs to `into`, which the caller destroys.
  auto capture_body = [&](int which, bool cond) -> int {
    if (ng > 1) CK(cudaEventRecord(c->ev_fork, c->st));
    for (size_t k = 0; k < ng; k++) {
      Group& gr = c->groups[k];
      cudaStream_t sk = k == 0 ? c->st : c->side[k - 1];
      if (k > 0) CK(cudaStreamWaitEvent(sk, c->ev_fork, 0));
      const int a = std::max(lo, gr.tb.mem0) - gr.tb.mem0, b = std::min(hi, gr.tb.mem0 + gr.tb.nmem) - gr.tb.mem0;
      if (a < b) {  // (an empty branch still forks and joins)
        Tables t;
        Bufs bf;
        range_view(gr, c->precision == NSP_MIXED, a, b, &t, &bf);
        launch_nonlinear(t, bf, c->dctl, c->precision == NSP_MIXED, nullptr, nullptr, sk);
        launch_linear(t, bf, c->dctl, sk, which);
      }
      if (k > 0) CK(cudaEventRecord(c->ev_join[k - 1], sk));
    }
    for (size_t k = 1; k < ng; k++) CK(cudaStreamWaitEvent(c->st, c->ev_join[k - 1], 0));
    launch_converge(c->dctl, c->nmem, (unsigned long long)h, cond ? 1 : 0, c->st);
    return NSP_OK;
  };
  auto capture_pass = [&](cudaGraph_t into, int which, bool cond) -> int {
    CK(cudaStreamBeginCaptureToGraph(c->st, into, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    const int rc = capture_body(which, cond);
    cudaGraph_t cap = nullptr;
    const cudaError_t e_end = cudaStreamEndCapture(c->st, &cap);
    if (rc) {
      cudaGetLastError();  // (an invalidated capture also fails to end)
      return rc;
    }
    CK(e_end);
    return NSP_OK;
  };
  // The step: the predictor pass (a child graph), then the corrector passes in a
  // conditional WHILE node whose condition converge_k sets; the condition's default
  // value 1 makes at least one corrector pass, as in the reference.
  cudaGraph_t gp = nullptr;
  CK(cudaGraphCreate(&gp, 0));
  if (int rc = capture_pass(gp, LIN_PRED, false)) { cudaGraphDestroy(gp); return rc; }
  cudaGraphNode_t pnode;
  cudaError_t ec = cudaGraphAddChildGraphNode(&pnode, g, nullptr, 0, gp);  // (clones gp)
  cudaGraphDestroy(gp);
  CK(ec);
  cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, g, &pnode, nullptr, 1, &cp));
  if (int rc = capture_pass(cp.conditional.phGraph_out[0], LIN_CORR, true)) return rc;
  CK(cudaGraphInstantiate(out, g, 0));
  c->use_graph = true;
  return NSP_OK;
}

int build_graph(nsp_ctx* c) { return build_graph_range(c, 0, c->nmem, &c->gexec); }

}  // namespace

namespace nsp {
int ctx_fail(nsp_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  else set_host_error(msg);
  return code;
}

thread_local std::string g_host_err;
void set_host_error(const std::string& msg) { g_host_err = msg; }
}  // namespace nsp

extern "C" {

int nsp_default_params(nsp_params* p) {
  if (!p) return NSP_ERR_ARG;
  p->NR = 48; p->NT = 64; p->NZ = 257;
  p->LT = PI2; p->LZ = 100.0;
  p->Re = 1850.0;
  p->dt = 0.01; p->d_im = 0.51;
  p->maxit = 10; p->tol = 5e-8;
  p->sten = 7;
  p->Qdes = 0.5;
  return NSP_OK;
}

int nsp_create(const nsp_params* members, int n_members, int precision, int device, nsp_ctx** out) {
  if (!out || !members || n_members < 1) return NSP_ERR_ARG;
  *out = nullptr;
  if (precision != NSP_FP64 && precision != NSP_MIXED) return NSP_ERR_ARG;
  nsp_ctx* c = new nsp_ctx();
  *out = c;
  c->device = device;
  c->precision = precision;
  c->nmem = n_members;
  c->prm.assign(members, members + n_members);
  for (int m = 0; m < n_members; m++) {
    int rc = check_params(c, members[m], m);
    if (rc) return rc;
  }
  // Group members with identical operators; internal order is group-major.
  c->grp.assign(n_members, -1);
  c->slot.assign(n_members, -1);
  for (int m = 0; m < n_members; m++) {
    int gi = -1;
    for (size_t g = 0; g < c->groups.size(); g++)
      if (same_shape(c->groups[g].p, members[m])) { gi = (int)g; break; }
    if (gi < 0) {
      Group g;
      g.p = members[m];
      c->groups.push_back(g);
      gi = (int)c->groups.size() - 1;
    }
    Group& gr = c->groups[gi];
    c->grp[m] = gi;
    c->slot[m] = (int)gr.users.size();
    gr.users.push_back(m);
    int ps = -1;
    for (size_t k = 0; k < gr.sets.size(); k++)
      if (gr.sets[k] == members[m].Re) { ps = (int)k; break; }
    if (ps < 0) {
      gr.sets.push_back(members[m].Re);
      ps = (int)gr.sets.size() - 1;
    }
    gr.mset.push_back(ps);
  }
  c->internal.assign(n_members, 0);
  int base = 0;
  for (auto& g : c->groups) {
    for (size_t s = 0; s < g.users.size(); s++) c->internal[g.users[s]] = base + (int)s;
    base += (int)g.users.size();
  }
  CK(cudaSetDevice(device));
  CK(cudaStreamCreateWithFlags(&c->own_st, cudaStreamNonBlocking));
  c->st = c->own_st;
  // Member buffers.
  base = 0;
  for (auto& g : c->groups) {
    const nsp_params& p = g.p;
    Tables& tb = g.tb;
    tb.NR = p.NR; tb.NT = p.NT; tb.NZ = p.NZ;
    tb.NTP = 3 * p.NT / 2;
    tb.NZP = 3 * (p.NZ - 1) / 2 + 1;
    tb.NZR = 2 * tb.NZP - 2;
    tb.NTNZ = p.NT * p.NZ;
    tb.S = (long long)p.NR * tb.NTNZ;
    tb.nmem = (int)g.users.size();
    tb.mem0 = base;
    base += tb.nmem;
    size_t S3 = (size_t)tb.nmem * 3 * tb.S;
    size_t csz = (precision == NSP_MIXED) ? sizeof(float2) : sizeof(double2);
    size_t gsz = (size_t)tb.nmem * 9 * tb.NR * tb.NTP * tb.NZ * csz;
    size_t hsz = (size_t)tb.nmem * 3 * tb.NR * tb.NTP * tb.NZ * csz;
    int rc;
    if ((rc = dalloc(c, &g.bf.U[0], S3 * sizeof(double2)))) return rc;
    if ((rc = dalloc(c, &g.bf.U[1], S3 * sizeof(double2)))) return rc;
    g.bf.N = g.bf.RHSW = nullptr;
    g.bf.N32 = g.bf.RHSW32 = nullptr;
    g.bf.NF = g.bf.RW00 = nullptr;
    if (precision == NSP_MIXED) {
      if ((rc = dalloc(c, &g.bf.N32, S3 * sizeof(float2))) || (rc = dalloc(c, &g.bf.RHSW32, S3 * sizeof(float2))) ||
          (rc = dalloc(c, &g.bf.NF, sizeof(double) * tb.nmem)) ||
          (rc = dalloc(c, &g.bf.RW00, sizeof(double) * tb.nmem * (size_t)tb.NR)))
        return rc;
      CK(cudaMemset(g.bf.N32, 0, S3 * sizeof(float2)));
      CK(cudaMemset(g.bf.RHSW32, 0, S3 * sizeof(float2)));
      CK(cudaMemset(g.bf.NF, 0, sizeof(double) * tb.nmem));
      CK(cudaMemset(g.bf.RW00, 0, sizeof(double) * tb.nmem * (size_t)tb.NR));
    } else {
      if ((rc = dalloc(c, &g.bf.RHSW, S3 * sizeof(double2))) || (rc = dalloc(c, &g.bf.N, S3 * sizeof(double2))))
        return rc;
      CK(cudaMemset(g.bf.N, 0, S3 * sizeof(double2)));
      CK(cudaMemset(g.bf.RHSW, 0, S3 * sizeof(double2)));
    }
    if ((rc = dalloc(c, &g.bf.G, gsz))) return rc;
    if ((rc = dalloc(c, &g.bf.H, hsz))) return rc;
    CK(cudaMemset(g.bf.U[0], 0, S3 * sizeof(double2)));
    CK(cudaMemset(g.bf.U[1], 0, S3 * sizeof(double2)));
    CK(cudaMemset(g.bf.G, 0, gsz));
    CK(cudaMemset(g.bf.H, 0, hsz));
    g.bf.U32[0] = g.bf.U32[1] = nullptr;
    g.bf.DR32[0] = g.bf.DR32[1] = nullptr;
    g.bf.MEAN = nullptr;
    if (precision == NSP_MIXED) {
      if ((rc = dalloc(c, &g.bf.MEAN, sizeof(float) * MEAN_N * tb.nmem * (size_t)tb.NR))) return rc;
      CK(cudaMemset(g.bf.MEAN, 0, sizeof(float) * MEAN_N * tb.nmem * (size_t)tb.NR));
      for (int k = 0; k < 2; k++) {
        if ((rc = dalloc(c, &g.bf.U32[k], S3 * sizeof(float2)))) return rc;
        if ((rc = dalloc(c, &g.bf.DR32[k], S3 * sizeof(float2)))) return rc;
        CK(cudaMemset(g.bf.U32[k], 0, S3 * sizeof(float2)));
        CK(cudaMemset(g.bf.DR32[k], 0, S3 * sizeof(float2)));
      }
    }
    if (tb.S > c->Smax) c->Smax = tb.S;
  }
  if (int rc = dalloc(c, &c->scratch, sizeof(double2) * 6 * (size_t)c->Smax)) return rc;
  if (int rc = dalloc(c, &c->scratch32, sizeof(float2) * 3 * (size_t)c->Smax)) return rc;
  // Control block.
  Ctl& h = c->hctl;
  h.parity = 0; h.step = 0; h.any = 0; h.nmem = n_members;
  h.maxit = members[0].maxit;
  h.tol = members[0].tol;
  h.hist_cap = 1024;
  int rc;
  if ((rc = dalloc(c, &h.phase, sizeof(int) * n_members))) return rc;
  if ((rc = dalloc(c, &h.ite, sizeof(int) * n_members))) return rc;
  if ((rc = dalloc(c, &h.status, sizeof(int) * n_members))) return rc;
  if ((rc = dalloc(c, &h.num, sizeof(unsigned long long) * n_members))) return rc;
  if ((rc = dalloc(c, &h.den, sizeof(unsigned long long) * n_members))) return rc;
  if ((rc = dalloc(c, &h.err, sizeof(double) * n_members))) return rc;
  if ((rc = dalloc(c, &h.hist, sizeof(int) * n_members * (size_t)h.hist_cap))) return rc;
  if ((rc = dalloc(c, &h.unconv, sizeof(int) * n_members))) return rc;
  CK(cudaMemset(h.unconv, 0, sizeof(int) * n_members));
  CK(cudaMemset(h.phase, 0, sizeof(int) * n_members));
  CK(cudaMemset(h.ite, 0, sizeof(int) * n_members));
  CK(cudaMemset(h.status, 0, sizeof(int) * n_members));
  CK(cudaMemset(h.num, 0, sizeof(unsigned long long) * n_members));
  CK(cudaMemset(h.den, 0, sizeof(unsigned long long) * n_members));
  CK(cudaMemset(h.err, 0, sizeof(double) * n_members));
  if ((rc = dalloc(c, &c->dctl, sizeof(Ctl)))) return rc;
  CK(cudaMemcpy(c->dctl, &h, sizeof(Ctl), cudaMemcpyHostToDevice));
  // Bounds record of the bounds-checked build (nsp_bounds.cuh), shared by every group.
  unsigned long long* bc = nullptr;
  if ((rc = dalloc(c, &bc, 4 * sizeof(unsigned long long)))) return rc;
  CK(cudaMemset(bc, 0, 4 * sizeof(unsigned long long)));
  for (auto& g : c->groups) g.tb.bc = bc;
  CK(cudaMallocHost(&c->pin, sizeof(int) * ((size_t)(h.hist_cap + 2) * n_members + 1)));
  return NSP_OK;
}

int nsp_setup(nsp_ctx* c) {
  if (!c) return NSP_ERR_ARG;
  CK(cudaSetDevice(c->device));
  for (auto& g : c->groups) {
    // maxit/tol are per context in the device control block: all groups must agree.
    if (g.p.maxit != c->hctl.maxit || g.p.tol != c->hctl.tol)
      return fail(c, NSP_ERR_ARG, "all members must share maxit and tol");
    Tables& tb = g.tb;
    const nsp_params& p = g.p;
    HostOps& o = g.ops;
    // Radial tables of the group's shape, then every parameter set's (distinct Re)
    // scalars, flux response and explicit Laplacian, concatenated set-major.
    radial_fd(p.NR, o);
    const int nsets = (int)g.sets.size();
    std::vector<double> Luc_all, uc_all, sscal, c_im(nsets);
    for (int k = 0; k < nsets; k++) {
      nsp_params pk = p;
      pk.Re = g.sets[k];
      std::vector<double> uck;
      double Qck = 0.0;
      flux_response(pk, o, uck, Qck);
      const double c_ex = (1.0 - pk.d_im) / pk.Re;
      uc_all.insert(uc_all.end(), uck.begin(), uck.end());
      for (size_t e = 0; e < o.Lu.size(); e++) Luc_all.push_back(0.5 * (c_ex * o.Lu[e]));
      sscal.insert(sscal.end(), {c_ex, 2.0 / pk.Re, Qck, pk.Re});
      c_im[k] = pk.d_im / pk.Re;
      if (k == 0) {
        o.uc = uck;
        o.Qc = Qck;
      }
    }
    std::vector<double> rinv(p.NR), rinv2(p.NR);
    std::vector<float> D32(o.D.size());
    for (int i = 0; i < p.NR; i++) { rinv[i] = 1.0 / o.r[i]; rinv2[i] = 1.0 / (o.r[i] * o.r[i]); }
    for (size_t e = 0; e < o.D.size(); e++) D32[e] = (float)o.D[e];
    std::vector<float> Luc32(Luc_all.begin(), Luc_all.end()), rinv32(rinv.begin(), rinv.end());
    std::vector<double> Ddiv(o.D);  // stored row i holds columns left.. at offset i0; column i is the centre
    for (int tab = 0; tab < 2; tab++)
      for (int i = 0; i < p.NR; i++) {
        const int left = std::max(0, i - IW), right = std::min(i + IW, p.NR - 1), i0 = i + IW - right;
        Ddiv[(size_t)tab * STEN * p.NR + (size_t)STEN * i + i0 + (i - left)] += rinv[i];
      }
    int rc;
    if ((rc = upload(c, &tb.r, o.r)) || (rc = upload(c, &tb.rinv, rinv)) || (rc = upload(c, &tb.rinv2, rinv2)) ||
        (rc = upload(c, &tb.rdr, o.rdr)) || (rc = upload(c, &tb.uc, uc_all)) || (rc = upload(c, &tb.D, o.D)) ||
        (rc = upload(c, &tb.D32, D32)) || (rc = upload(c, &tb.Ddiv, Ddiv)) ||
        (rc = upload(c, &tb.Ddiv32, std::vector<float>(Ddiv.begin(), Ddiv.end()))) || (rc = upload(c, &tb.Lu, o.Lu)) || (rc = upload(c, &tb.Luc, Luc_all)) ||
        (rc = upload(c, &tb.Luc32, Luc32)) || (rc = upload(c, &tb.rinv32, rinv32)) ||
        (rc = upload(c, &tb.sscal, sscal)) || (rc = upload(c, &tb.mset, g.mset)))
      return rc;
    // Factors and correction profiles of every (set, mode): on the device by default,
    // one thread per (set, mode); NSP_DEVICE_SETUP=0 builds the same bits on the host.
    const size_t NTNZ = (size_t)p.NT * p.NZ;
    const size_t fac_n = (size_t)nsets * 4 * p.NR * NFAC * NTNZ, V_n = (size_t)nsets * 3 * p.NR * NTNZ;
    const char* se = getenv("NSP_DEVICE_SETUP");
    g.device_setup = !(se && se[0] == '0');
    if (g.device_setup) {
      double* fac = nullptr;
      double2* V = nullptr;
      const double* Lp = nullptr;
      if ((rc = dalloc(c, &fac, sizeof(double) * fac_n)) || (rc = dalloc(c, &V, sizeof(double2) * V_n)) ||
          (rc = upload(c, &Lp, o.Lp)))
        return rc;
      std::string err;
      if ((rc = launch_mode_tables(p, nsets, c_im.data(), tb.r, tb.D, tb.Lu, Lp, fac, V, c->st, &err)))
        return fail(c, rc, "%s", err.c_str());
      tb.fac = fac;
      tb.V = V;
    } else {
      std::vector<double> fac_all(fac_n);
      std::vector<double2> V_all(V_n);
      for (int k = 0; k < nsets; k++) {
        nsp_params pk = p;
        pk.Re = g.sets[k];
        mode_tables(pk, o, fac_all.data() + (size_t)k * 4 * p.NR * NFAC * NTNZ,
                    V_all.data() + (size_t)k * 3 * p.NR * NTNZ);
      }
      if ((rc = upload(c, &tb.fac, fac_all)) || (rc = upload(c, &tb.V, V_all))) return rc;
    }
    tb.nsets = nsets;
    tb.V32 = nullptr;
    tb.facdf = tb.Vdf = tb.Ddf = tb.Ddivdf = tb.rinvdf = nullptr;
    tb.fac32 = nullptr;
    if (c->precision == NSP_MIXED) {
      // the increment passes' FP32 correction profiles; the double-float factors, correction
      // profiles and stencils of the linear passes
      float2 *v32 = nullptr, *fdf = nullptr, *vdf = nullptr;
      float* f32 = nullptr;
      if ((rc = dalloc(c, &v32, sizeof(float2) * V_n)) || (rc = dalloc(c, &fdf, sizeof(float2) * fac_n)) ||
          (rc = dalloc(c, &vdf, sizeof(float2) * 2 * V_n)) || (rc = dalloc(c, &f32, sizeof(float) * fac_n)))
        return rc;
      launch_to_f32(tb.V, v32, (long long)V_n, c->st);
      launch_split_fac(tb.fac, fdf, f32, (long long)fac_n, (int)NTNZ, c->st);
      launch_split_df(reinterpret_cast<const double*>(tb.V), vdf, 2 * (long long)V_n, c->st);
      CK(cudaGetLastError());
      tb.V32 = v32;
      tb.facdf = fdf;
      tb.fac32 = f32;
      tb.Vdf = vdf;
      if ((rc = upload(c, &tb.Ddf, split_df_host(o.D))) || (rc = upload(c, &tb.Ddivdf, split_df_host(Ddiv))) ||
          (rc = upload(c, &tb.rinvdf, split_df_host(rinv))))
        return rc;
    }
    std::vector<double2> wt = twiddles(tb.NTP), wz = twiddles(tb.NZR);
    if ((rc = upload(c, &tb.tw_t, wt)) || (rc = upload(c, &tb.tw_z, wz)) || (rc = upload(c, &tb.tw_t32, to_f32(wt))) ||
        (rc = upload(c, &tb.tw_z32, to_f32(wz))))
      return rc;
    make_plan(tb.NTP, tb.pt);
    make_plan(tb.NZR, tb.pz);
    tb.kts = PI2 / p.LT;
    tb.kzs = PI2 / p.LZ;
    tb.inv_dt = 1.0 / p.dt;
    tb.c_ex = sscal[0];  // set 0's scalars; kernels read each member's from sscal
    tb.d_im = p.d_im;
    tb.one_m_dim = 1.0 - p.d_im;
    tb.two_re = sscal[1];
    tb.Qdes = p.Qdes;
    tb.Qc = sscal[2];
    tb.inv_norm = 1.0 / ((double)tb.NTP * (double)tb.NZR);
    tb.kts32 = (float)tb.kts;
    tb.kzs32 = (float)tb.kzs;
    tb.inv_norm32 = (float)tb.inv_norm;
    // Mixed form: theta transforms as tensor-core DFT GEMMs where the length has a
    // compiled tile shape (NSP_THETA_TC=0 keeps the FFT kernels).
    int dev_sms = 0;
    CK(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, c->device));
    tb.nsm = dev_sms;
    tb.tc_theta = 0;
    const char* te = getenv("NSP_THETA_TC");
    if (c->precision == NSP_MIXED && theta_tc_supported(tb.NT, tb.NTP) && !(te && te[0] == '0')) {
      if ((rc = upload(c, &tb.dft_inv, theta_dft_image(tb.NT, tb.NTP, true, 1.0))) ||
          (rc = upload(c, &tb.dft_fwd, theta_dft_image(tb.NT, tb.NTP, false, tb.inv_norm))))
        return rc;
      tb.tc_theta = 1;
    }
  }
  configure_transform_kernels();
  configure_linear_kernels();
  configure_theta_tc_kernels();
  CK(cudaGetLastError());
  if (int rc = autotune(c)) return rc;
  // NSP_GRAPH=0 selects the host-driven corrector loop (same kernels, one D2H flag
  // read per iteration) so that profilers can see every kernel launch.
  const char* ge = getenv("NSP_GRAPH");
  if (ge && ge[0] == '0') {
    c->use_graph = false;
  } else {
    int rc = build_graph(c);
    if (rc) return rc;
  }
  c->setup_done = true;
  return NSP_OK;
}

int nsp_load_state(nsp_ctx* c, int m, const char* fr, const char* ft, const char* fz) {
  if (int rc = check_member(c, m)) return rc;
  Group& g = c->groups[c->grp[m]];
  size_t n = (size_t)g.tb.S;
  std::vector<double> buf(2 * n * 3);
  const char* names[3] = {fr, ft, fz};
  for (int k = 0; k < 3; k++) {
    if (!names[k]) return fail(c, NSP_ERR_ARG, "null file name");
    FILE* f = fopen(names[k], "rb");
    if (!f) return fail(c, NSP_ERR_IO, "reading error: %s", names[k]);
    size_t got = fread(buf.data() + 2 * n * k, 16, n, f);
    int extra = fgetc(f);
    fclose(f);
    if (got != n) return fail(c, NSP_ERR_IO, "reading error: %s holds %zu of %zu values", names[k], got, n);
    if (extra != EOF) return fail(c, NSP_ERR_IO, "reading error: %s is longer than %zu values", names[k], n);
  }
  return nsp_set_state_host(c, m, buf.data(), buf.data() + 2 * n, buf.data() + 4 * n);
}

int nsp_save_state(nsp_ctx* c, int m, const char* fr, const char* ft, const char* fz) {
  if (int rc = check_member(c, m)) return rc;
  Group& g = c->groups[c->grp[m]];
  size_t n = (size_t)g.tb.S;
  std::vector<double> buf(2 * n * 3);
  if (int rc = nsp_get_state_host(c, m, buf.data(), buf.data() + 2 * n, buf.data() + 4 * n)) return rc;
  const char* names[3] = {fr, ft, fz};
  for (int k = 0; k < 3; k++) {
    if (!names[k]) return fail(c, NSP_ERR_ARG, "null file name");
    FILE* f = fopen(names[k], "wb");
    if (!f) return fail(c, NSP_ERR_IO, "writing error: %s", names[k]);
    size_t put = fwrite(buf.data() + 2 * n * k, 16, n, f);
    int cl = fclose(f);
    if (put != n || cl != 0) return fail(c, NSP_ERR_IO, "writing error: %s", names[k]);
  }
  return NSP_OK;
}

// A run of consecutive user members [m0, m0+n) stored in consecutive slots of one
// group: each component of the run is one pitched copy (host: the members' arrays back
// to back; device: member stride 3 S).
static int member_run(nsp_ctx* c, int m0, int mend) {
  int n = 1;
  while (m0 + n < mend && c->grp[m0 + n] == c->grp[m0] && c->slot[m0 + n] == c->slot[m0] + n) n++;
  return n;
}

// A member whose state is set from outside starts with a clean status.
static int clear_status(nsp_ctx* c, int m) {
  if (m < 0) CK(cudaMemsetAsync(c->hctl.status, 0, sizeof(int) * c->nmem, c->st));
  else CK(cudaMemsetAsync(c->hctl.status + c->internal[m], 0, sizeof(int), c->st));
  return NSP_OK;
}

static int copy_states(nsp_ctx* c, int m, double* const* host, bool to_device) {
  const int m0 = m < 0 ? 0 : m, mend = m < 0 ? c->nmem : m + 1;
  if (to_device) {
    c->mirror_ok = false;
    if (int rc = clear_status(c, m)) return rc;
  }
  size_t off = 0;  // doubles into each host component array
  for (int mm = m0; mm < mend;) {
    const int n = member_run(c, mm, mend);
    const size_t bytes = sizeof(double2) * (size_t)c->groups[c->grp[mm]].tb.S;
    for (int k = 0; k < 3; k++) {
      double* h = host[k] + off;
      double2* d = state_ptr(c, mm, k);
      if (to_device)
        CK(cudaMemcpy2DAsync(d, 3 * bytes, h, bytes, bytes, n, cudaMemcpyHostToDevice, c->st));
      else
        CK(cudaMemcpy2DAsync(h, bytes, d, 3 * bytes, bytes, n, cudaMemcpyDeviceToHost, c->st));
    }
    off += (size_t)n * bytes / sizeof(double);
    mm += n;
  }
  CK(cudaStreamSynchronize(c->st));
  return NSP_OK;
}

// Host transfers of one member, or of all members (member == NSP_ALL_MEMBERS) from/to
// arrays holding every member's component back to back in member order; one pitched
// copy per component per run of members stored together, one synchronisation per call.
int nsp_set_state_host(nsp_ctx* c, int m, const double* ur, const double* ut, const double* uz) {
  if (!c) return NSP_ERR_ARG;
  if (m != NSP_ALL_MEMBERS)
    if (int rc = check_member(c, m)) return rc;
  if (!ur || !ut || !uz) return fail(c, NSP_ERR_ARG, "null state pointer");
  double* src[3] = {const_cast<double*>(ur), const_cast<double*>(ut), const_cast<double*>(uz)};
  return copy_states(c, m, src, true);
}

int nsp_get_state_host(nsp_ctx* c, int m, double* ur, double* ut, double* uz) {
  if (!c) return NSP_ERR_ARG;
  if (m != NSP_ALL_MEMBERS)
    if (int rc = check_member(c, m)) return rc;
  if (!ur || !ut || !uz) return fail(c, NSP_ERR_ARG, "null state pointer");
  double* dst[3] = {ur, ut, uz};
  return copy_states(c, m, dst, false);
}

int nsp_set_state_device(nsp_ctx* c, int m, const void* ur, const void* ut, const void* uz) {
  if (int rc = check_member(c, m)) return rc;
  if (!ur || !ut || !uz) return fail(c, NSP_ERR_ARG, "null state pointer");
  size_t bytes = sizeof(double2) * (size_t)c->groups[c->grp[m]].tb.S;
  const void* src[3] = {ur, ut, uz};
  c->mirror_ok = false;
  if (int rc = clear_status(c, m)) return rc;
  for (int k = 0; k < 3; k++) CK(cudaMemcpyAsync(state_ptr(c, m, k), src[k], bytes, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return NSP_OK;
}

int nsp_get_state_device(nsp_ctx* c, int m, void* ur, void* ut, void* uz) {
  if (int rc = check_member(c, m)) return rc;
  if (!ur || !ut || !uz) return fail(c, NSP_ERR_ARG, "null state pointer");
  size_t bytes = sizeof(double2) * (size_t)c->groups[c->grp[m]].tb.S;
  void* dst[3] = {ur, ut, uz};
  for (int k = 0; k < 3; k++) CK(cudaMemcpyAsync(dst[k], state_ptr(c, m, k), bytes, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return NSP_OK;
}

// One step of every member whose phase is 0 at its start (members at -1 sit it out):
// the step graph, or the same kernels driven from the host (NSP_GRAPH=0).
static int run_step(nsp_ctx* c, int chunk = -1) {
  if (c->use_graph) {
    CK(cudaGraphLaunch(chunk < 0 ? c->gexec : c->chunk_exec[chunk], c->st));
    return NSP_OK;
  }
  const int lo = chunk < 0 ? 0 : c->chunk_lo[chunk], hi = chunk < 0 ? c->nmem : c->chunk_lo[chunk + 1];
  for (int it = 0; it <= c->hctl.maxit; it++) {
    for (auto& g : c->groups) {
      const int a = std::max(lo, g.tb.mem0) - g.tb.mem0, b = std::min(hi, g.tb.mem0 + g.tb.nmem) - g.tb.mem0;
      if (a >= b) continue;
      Tables t;
      Bufs bf;
      range_view(g, c->precision == NSP_MIXED, a, b, &t, &bf);
      launch_nonlinear(t, bf, c->dctl, c->precision == NSP_MIXED, nullptr, nullptr, c->st);
      launch_linear(t, bf, c->dctl, c->st);
    }
    launch_converge(c->dctl, c->nmem, 0ull, 0, c->st);
    CK(cudaGetLastError());
    int any = 1;
    CK(cudaMemcpyAsync(&any, &c->dctl->any, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    if (!any) break;
  }
  return NSP_OK;
}

// Copies between a member-major host array (each member's u_r, u_theta, u_z back to
// back, members in order) and the state buffers of parity `par`, for the members whose
// internal index is in [lo, hi): one copy per run of members stored together.
static int copy_chunk(nsp_ctx* c, int lo, int hi, int par, double* host, bool to_device, cudaStream_t st) {
  std::vector<size_t> off(c->nmem + 1, 0);
  for (int u = 0; u < c->nmem; u++) off[u + 1] = off[u] + 6 * (size_t)c->groups[c->grp[u]].tb.S;
  std::vector<int> users;
  for (int u = 0; u < c->nmem; u++)
    if (c->internal[u] >= lo && c->internal[u] < hi) users.push_back(u);
  for (size_t a = 0; a < users.size();) {
    size_t b = a + 1;
    while (b < users.size() && users[b] == users[b - 1] + 1 && c->grp[users[b]] == c->grp[users[a]] &&
           c->slot[users[b]] == c->slot[users[b - 1]] + 1)
      b++;
    const int u0 = users[a];
    Group& g = c->groups[c->grp[u0]];
    const size_t bytes = (b - a) * 3 * sizeof(double2) * (size_t)g.tb.S;
    double2* d = g.bf.U[par] + (size_t)c->slot[u0] * 3 * g.tb.S;
    if (to_device)
      CK(cudaMemcpyAsync(d, host + off[u0], bytes, cudaMemcpyHostToDevice, st));
    else
      CK(cudaMemcpyAsync(host + off[u0], d, bytes, cudaMemcpyDeviceToHost, st));
    a = b;
  }
  return NSP_OK;
}

// Mixed form: the FP32 mirror of the state for the members with internal index in [lo, hi).
static void mirror_range(nsp_ctx* c, int lo, int hi, int par, cudaStream_t st) {
  for (auto& g : c->groups) {
    const int a = std::max(lo, g.tb.mem0), b = std::min(hi, g.tb.mem0 + g.tb.nmem);
    if (a >= b) continue;
    Tables t = g.tb;
    t.nmem = b - a;
    const size_t o = (size_t)(a - g.tb.mem0) * 3 * g.tb.S;
    launch_mirror(t, g.bf.U[par] + o, g.bf.U32[par] + o, g.bf.DR32[par] + o, st);
  }
}

// Kernels launched per predictor or corrector pass: per group the three transform
// kernels and the linear pass, then converge_k.  The step graph launches the pass's
// own linear kernel; the host-driven loop launches both of the mixed form's (the
// full pass for the predictor, the increment pass for the correctors).
static long long kernels_per_pass(const nsp_ctx* c) {
  return (c->precision == NSP_MIXED && !c->use_graph ? 5LL : 4LL) * (long long)c->groups.size() + 1;
}

// The step history of the last `batch` steps into the pinned buffer; with `final` also
// the members' status words, the fault flag and the unconverged-step counts.  One
// synchronisation of the stream.
static int read_control(nsp_ctx* c, int batch, bool final) {
  const int nm = c->nmem;
  const size_t tail = (size_t)c->hctl.hist_cap * nm;
  if (batch > 0)
    CK(cudaMemcpyAsync(c->pin, c->hctl.hist, sizeof(int) * (size_t)batch * nm, cudaMemcpyDeviceToHost, c->st));
  if (final) {
    CK(cudaMemcpyAsync(c->pin + tail, c->hctl.status, sizeof(int) * nm, cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(c->pin + tail + nm, &c->dctl->fault, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(c->pin + tail + nm + 1, c->hctl.unconv, sizeof(int) * nm, cudaMemcpyDeviceToHost, c->st));
  }
  CK(cudaStreamSynchronize(c->st));
  return NSP_OK;
}

// After a final read_control: a device-side wait that ran out, then non-finite members.
static int control_verdict(nsp_ctx* c) {
  const int nm = c->nmem;
  const int* tail = c->pin + (size_t)c->hctl.hist_cap * nm;
  if (tail[nm]) {
    CK(cudaMemsetAsync(&c->dctl->fault, 0, sizeof(int), c->st));
    return fail(c, NSP_ERR_DEVICE, "a device-side wait ran out; the call's results are invalid");
  }
  for (int m = 0; m < nm; m++)
    if (tail[c->internal[m]] & NSP_ERR_NONFINITE)
      return fail(c, NSP_ERR_NONFINITE, "member %d: non-finite velocity or convergence measure", m);
  if (c->strict)
    for (int m = 0; m < nm; m++)
      if (const int n = tail[nm + 1 + c->internal[m]])
        return fail(c, NSP_ERR_MAXIT, "member %d: %d step(s) stopped at maxit = %d without convergence", m, n,
                    c->hctl.maxit);
  return NSP_OK;
}

int nsp_step(nsp_ctx* c, int nsteps, int* iters_out) {
  if (!c) return NSP_ERR_ARG;
  if (!c->setup_done) return fail(c, NSP_ERR_STATE, "nsp_step before nsp_setup");
  if (nsteps < 0) return fail(c, NSP_ERR_ARG, "nsteps < 0");
  CK(cudaSetDevice(c->device));
  const int nm = c->nmem;
  const int cap = c->hctl.hist_cap;
  long long launches = 0;
  const long long per_iter = kernels_per_pass(c);
  // Mixed form: the transforms read an FP32 mirror of the state and its radial
  // derivative, kept current by the linear pass; refresh them when the state was
  // written from outside since.
  if (c->precision == NSP_MIXED && nsteps > 0 && !c->mirror_ok)
    for (auto& g : c->groups) launch_mirror(g.tb, g.bf.U[c->parity], g.bf.U32[c->parity], g.bf.DR32[c->parity], c->st);
  c->mirror_ok = false;
  if (nsteps > 0) CK(cudaMemsetAsync(c->hctl.unconv, 0, sizeof(int) * nm, c->st));
  if (nsteps == 0)
    if (int rc = read_control(c, 0, true)) return rc;
  for (int done = 0; done < nsteps;) {
    int chunk = std::min(cap, nsteps - done);
    CK(cudaMemsetAsync(&c->dctl->step, 0, sizeof(int), c->st));
    for (int s = 0; s < chunk; s++)
      if (int rc = run_step(c)) return rc;
    CK(cudaGetLastError());
    if (int rc = read_control(c, chunk, done + chunk == nsteps)) return rc;
    const int* hist = c->pin;
    for (int s = 0; s < chunk; s++) {
      int mx = 0;
      for (int m = 0; m < nm; m++) mx = std::max(mx, hist[(size_t)s * nm + m]);
      launches += (1 + mx) * per_iter;
      if (iters_out)
        for (int m = 0; m < nm; m++) iters_out[(size_t)(done + s) * nm + m] = hist[(size_t)s * nm + c->internal[m]];
    }
    c->parity ^= (chunk & 1);
    done += chunk;
  }
  c->launches_last = launches;
  const int rc = control_verdict(c);
  c->mirror_ok = rc == NSP_OK && nsteps > 0;
  return rc;
}

int nsp_step_host(nsp_ctx* c, int nsteps, const double* in, double* out, int* iters_out) {
  if (!c) return NSP_ERR_ARG;
  if (!c->setup_done) return fail(c, NSP_ERR_STATE, "nsp_step_host before nsp_setup");
  if (nsteps < 0) return fail(c, NSP_ERR_ARG, "nsteps < 0");
  if (!in || !out) return fail(c, NSP_ERR_ARG, "null state pointer");
  CK(cudaSetDevice(c->device));
  const int nm = c->nmem;
  double* hin = const_cast<double*>(in);
  c->mirror_ok = false;
  if (nsteps == 0) {
    if (int rc = copy_chunk(c, 0, nm, c->parity, hin, true, c->st)) return rc;
    if (int rc = copy_chunk(c, 0, nm, c->parity, out, false, c->st)) return rc;
    CK(cudaStreamSynchronize(c->st));
    return NSP_OK;
  }
  // Member chunks (internal order), each with its own step graph: the first step copies
  // chunk k+1 in while chunk k steps, the last step copies chunk k out while chunk k+1 steps.
  // Chunk weights: with 16 or more members 1:4:3:1 -- short first and last chunks, whose
  // copy in and copy out are the exposed ones, and two long middle chunks (every chunk
  // step pays its kernels' fixed costs and partial last waves once).
  std::vector<int> wts = nm >= 16 ? std::vector<int>{1, 4, 3, 1} : (nm >= 4 ? std::vector<int>{1, 1} : std::vector<int>{1});
  if (const char* ke = getenv("NSP_HOST_CHUNKS")) {  // tuning override: "K" equal chunks, or weights "1:3:3:1"
    if (strchr(ke, ':')) {
      wts.clear();
      for (const char* q = ke; *q;) {
        const int w = atoi(q);
        if (w > 0 && (int)wts.size() < nm) wts.push_back(w);
        q = strchr(q, ':');
        if (!q) break;
        q++;
      }
      if (wts.empty()) wts.assign(1, 1);
    } else {
      wts.assign(std::max(1, std::min(nm, atoi(ke))), 1);
    }
  }
  std::vector<int> lo(1, 0);  // chunk bounds; a chunk that rounds to no member is dropped
  {
    int wsum = 0, acc = 0;
    for (int w : wts) wsum += w;
    for (int w : wts) {
      acc += w;
      const int b = (int)((long long)acc * nm / wsum);
      if (b > lo.back()) lo.push_back(b);
    }
  }
  const int K = (int)lo.size() - 1;
  if (c->chunk_lo != lo) {
    for (cudaGraphExec_t x : c->chunk_exec)
      if (x) cudaGraphExecDestroy(x);
    c->chunk_exec.assign(K, nullptr);
    c->chunk_lo = lo;
    if (c->use_graph)
      for (int k = 0; k < K; k++)
        if (int rc = build_graph_range(c, c->chunk_lo[k], c->chunk_lo[k + 1], &c->chunk_exec[k])) return rc;
  }
  if (!c->cp_in) {
    CK(cudaStreamCreateWithFlags(&c->cp_in, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&c->cp_out, cudaStreamNonBlocking));
  }
  while ((int)c->ev_in.size() < K) {
    cudaEvent_t e1, e2;
    CK(cudaEventCreateWithFlags(&e1, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&e2, cudaEventDisableTiming));
    c->ev_in.push_back(e1);
    c->ev_done.push_back(e2);
  }
  if (int rc = clear_status(c, NSP_ALL_MEMBERS)) return rc;  // every state comes from `in`
  CK(cudaMemsetAsync(c->hctl.unconv, 0, sizeof(int) * nm, c->st));
  // Copies in may start only once earlier work on the state is done.
  CK(cudaEventRecord(c->ev_done[0], c->st));
  CK(cudaStreamWaitEvent(c->cp_in, c->ev_done[0], 0));
  const int cap = c->hctl.hist_cap;
  const long long per_iter = kernels_per_pass(c);
  long long launches = 0;
  for (int done = 0; done < nsteps;) {
    const int batch = std::min(cap, nsteps - done);
    CK(cudaMemsetAsync(&c->dctl->step, 0, sizeof(int), c->st));
    std::vector<char> chunked(batch, 0);
    for (int s = 0; s < batch; s++) {
      const bool first = done + s == 0, last = done + s == nsteps - 1;
      const int p = c->parity;
      if (first || last) {
        chunked[s] = 1;
        // On a failure between chunks, put the control block back to its between-steps
        // state (no held parity, every member active) before reporting it.
        struct Restore {
          nsp_ctx* c;
          bool armed = true;
          ~Restore() {
            if (!armed) return;
            cudaMemsetAsync(&c->dctl->hold, 0, sizeof(int), c->st);
            cudaMemsetAsync(c->hctl.phase, 0, sizeof(int) * c->nmem, c->st);
            cudaStreamSynchronize(c->st);
          }
        } restore{c};
        CK(cudaMemsetAsync(&c->dctl->hold, 1, sizeof(int), c->st));
        for (int k = 0; k < K; k++) {
          const int lo = c->chunk_lo[k], hi = c->chunk_lo[k + 1];
          if (first) {
            // The chunk's copy in and its FP32 mirror run on the copy stream, beside the
            // previous chunk's step (other members' buffers).
            if (int rc = copy_chunk(c, lo, hi, p, hin, true, c->cp_in)) return rc;
            if (c->precision == NSP_MIXED) mirror_range(c, lo, hi, p, c->cp_in);
            CK(cudaEventRecord(c->ev_in[k], c->cp_in));
            CK(cudaStreamWaitEvent(c->st, c->ev_in[k], 0));
          }
          CK(cudaMemsetAsync(c->hctl.phase, 0xFF, sizeof(int) * nm, c->st));  // -1: sits this chunk out
          CK(cudaMemsetAsync(c->hctl.phase + lo, 0, sizeof(int) * (hi - lo), c->st));
          if (int rc = run_step(c, k)) return rc;
          if (last) {
            CK(cudaEventRecord(c->ev_done[k], c->st));
            CK(cudaStreamWaitEvent(c->cp_out, c->ev_done[k], 0));
            if (int rc = copy_chunk(c, lo, hi, p ^ 1, out, false, c->cp_out)) return rc;
          }
        }
        CK(cudaMemsetAsync(&c->dctl->hold, 0, sizeof(int), c->st));
        launch_finish_step(c->dctl, c->st);
        restore.armed = false;
      } else {
        if (int rc = run_step(c)) return rc;
      }
      CK(cudaGetLastError());
      c->parity ^= 1;
    }
    if (int rc = read_control(c, batch, done + batch == nsteps)) return rc;
    for (int s = 0; s < batch; s++) {
      const int* row = c->pin + (size_t)s * nm;
      if (chunked[s]) {
        for (int k = 0; k < K; k++)
          launches += (1 + *std::max_element(row + c->chunk_lo[k], row + c->chunk_lo[k + 1])) * per_iter;
      } else {
        launches += (1 + *std::max_element(row, row + nm)) * per_iter;
      }
      if (iters_out)
        for (int m = 0; m < nm; m++) iters_out[(size_t)(done + s) * nm + m] = row[c->internal[m]];
    }
    done += batch;
  }
  CK(cudaStreamSynchronize(c->cp_out));
  CK(cudaStreamSynchronize(c->cp_in));
  c->launches_last = launches;
  const int rc = control_verdict(c);
  c->mirror_ok = rc == NSP_OK;
  return rc;
}

int nsp_nonlinear(nsp_ctx* c, int m, const void* ur, const void* ut, const void* uz, void* nr, void* nt, void* nz) {
  if (int rc = check_member(c, m)) return rc;
  if (!c->setup_done) return fail(c, NSP_ERR_STATE, "nsp_nonlinear before nsp_setup");
  Group& g = c->groups[c->grp[m]];
  size_t S = (size_t)g.tb.S, bytes = sizeof(double2) * S;
  double2* in = c->scratch;
  double2* out = c->scratch + 3 * S;
  const void* src[3] = {ur, ut, uz};
  void* dst[3] = {nr, nt, nz};
  for (int k = 0; k < 3; k++) CK(cudaMemcpyAsync(in + k * S, src[k], bytes, cudaMemcpyDeviceToDevice, c->st));
  const bool mixed = c->precision == NSP_MIXED;
  if (mixed) launch_to_f32(in, c->scratch32, 3LL * (long long)S, c->st);
  const Tables tv = member_view(g, c->slot[m]);  // the member's 2/Re for the wall forcing
  launch_nonlinear(tv, g.bf, c->dctl, mixed, in, out, c->st, 7, mixed ? c->scratch32 : nullptr);
  CK(cudaGetLastError());
  for (int k = 0; k < 3; k++) CK(cudaMemcpyAsync(dst[k], out + k * S, bytes, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return check_fault(c);
}

int nsp_nonlinear_static(nsp_ctx* c, int m, const void* u3, void* n3) {
  if (int rc = check_member(c, m)) return rc;
  if (!c->setup_done) return fail(c, NSP_ERR_STATE, "nsp_nonlinear_static before nsp_setup");
  if (!u3 || !n3) return fail(c, NSP_ERR_ARG, "null field pointer");
  Group& g = c->groups[c->grp[m]];
  {  // the transforms read u3 until the last kernel writes n3 (the wall forcing reads u_z)
    const char *a = (const char*)u3, *b = (const char*)n3;
    const size_t fb = 3 * sizeof(double2) * (size_t)g.tb.S;
    if (a < b + fb && b < a + fb) return fail(c, NSP_ERR_ARG, "nsp_nonlinear_static: u3 and n3 overlap");
  }
  const bool mixed = c->precision == NSP_MIXED;
  const size_t csz = mixed ? sizeof(float2) : sizeof(double2);
  auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
  const size_t gsz = up((size_t)9 * g.tb.NR * g.tb.NTP * g.tb.NZ * csz);
  const size_t hsz = up((size_t)3 * g.tb.NR * g.tb.NTP * g.tb.NZ * csz);
  const size_t isz = mixed ? up((size_t)3 * g.tb.S * sizeof(float2)) : 0;
  const size_t need = gsz + hsz + isz;
  if (need > noalloc_scratch_bytes())
    return fail(c, NSP_ERR_ARG, "nsp_nonlinear_static: member %d needs %zu bytes of scratch, the fixed limit is %zu",
                m, need, noalloc_scratch_bytes());
  CK(cudaSetDevice(c->device));
  void* base = nullptr;
  CK(noalloc_scratch(c->device, &base));
  unsigned char* s = (unsigned char*)base;
  Bufs b = g.bf;
  b.G = s;
  b.H = s + gsz;
  float2* in32 = mixed ? (float2*)(s + gsz + hsz) : nullptr;
  if (mixed) launch_to_f32((const double2*)u3, in32, 3LL * g.tb.S, c->st);
  const Tables tv = member_view(g, c->slot[m]);
  launch_nonlinear(tv, b, c->dctl, mixed, (const double2*)u3, (double2*)n3, c->st, 7, in32);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  return check_fault(c);  // a tensor-core wait that ran out leaves n3 invalid
}

int nsp_lusolve(nsp_ctx* c, int m, int kind, const void* rhs, void* sol) {
  if (int rc = check_member(c, m)) return rc;
  if (!c->setup_done) return fail(c, NSP_ERR_STATE, "nsp_lusolve before nsp_setup");
  if (kind < 0 || kind > 7) return fail(c, NSP_ERR_ARG, "kind %d not in 0..7", kind);
  const Tables tv = member_view(c->groups[c->grp[m]], c->slot[m]);
  if (kind > 3 && !tv.facdf) return fail(c, NSP_ERR_ARG, "kind %d (double-float solve): mixed-form contexts only", kind);
  launch_lusolve(tv, kind, (const double2*)rhs, (double2*)sol, c->st);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  return NSP_OK;
}

// Friction diagnostics of one member from Re u_z(0,0)(r_i) (wrt_frc_k,
// mod_io_nonlinear.cu:40-52; flux as adj_flux, mod_cublasflux.cu:90-103).
static void friction(const HostOps& o, int NR, const double* uz0, double Re, nsp_diag_out* out) {
  double ucen = 0.0, du = 0.0, Q = 0.0;
  for (int i = 0; i <= IW; i++) ucen += uz0[i] * o.dr0[i];
  for (int i = 0; i < STEN; i++) du += uz0[NR - STEN + i] * o.D[(size_t)(NR - 1) * STEN + i];
  for (int i = 0; i < NR; i++) Q += o.rdr[i] * uz0[i];
  out->u_centre = ucen;
  out->u_tau = std::sqrt(std::fabs(du) / Re);
  out->flux = Q;
  out->re_tau = Re * out->u_tau;
}

static int ensure_diagbuf(nsp_ctx* c) {
  if (!c->diagbuf) {
    void* p = nullptr;
    if (int rc = dalloc(c, &p, 2 * sizeof(unsigned long long) * c->nmem)) return rc;
    c->diagbuf = static_cast<unsigned long long*>(p);
  }
  return NSP_OK;
}

static int ensure_crossbuf(nsp_ctx* c, size_t n) {
  if (c->crossbuf_n < n) {  // grows to the largest size asked for, then reused
    void* p = nullptr;
    if (int rc = dalloc(c, &p, n * sizeof(double))) return rc;
    c->crossbuf = static_cast<double*>(p);
    c->crossbuf_n = n;
  }
  return NSP_OK;
}

int nsp_diag(nsp_ctx* c, int m, nsp_diag_out* out) {
  if (int rc = check_member(c, m)) return rc;
  if (!out) return fail(c, NSP_ERR_ARG, "null output");
  if (!c->setup_done) return fail(c, NSP_ERR_STATE, "nsp_diag before nsp_setup");
  Group& g = c->groups[c->grp[m]];
  const int NR = g.tb.NR;
  std::vector<double2> uz(NR);
  CK(cudaMemcpy2DAsync(uz.data(), sizeof(double2), state_ptr(c, m, 2), sizeof(double2) * g.tb.NTNZ, sizeof(double2), NR,
                       cudaMemcpyDeviceToHost, c->st));
  int mi = c->internal[m];
  double err = 0.0;
  int status = 0;
  CK(cudaMemcpyAsync(&err, c->hctl.err + mi, sizeof(double), cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(&status, c->hctl.status + mi, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  int ite = 0, unconv = 0;
  CK(cudaMemcpyAsync(&ite, c->hctl.ite + mi, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(&unconv, c->hctl.unconv + mi, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  std::vector<double> uz0(NR);
  for (int i = 0; i < NR; i++) uz0[i] = uz[i].x;
  friction(g.ops, NR, uz0.data(), c->prm[m].Re, out);
  out->last_err = err;
  out->last_iters = ite;
  out->status = (status & NSP_ERR_NONFINITE) ? NSP_ERR_NONFINITE : NSP_OK;
  out->unconverged_steps = unconv;
  // Divergence of the state on the device.
  if (int rc = ensure_diagbuf(c)) return rc;
  CK(cudaMemsetAsync(c->diagbuf, 0, 2 * sizeof(unsigned long long), c->st));
  launch_diag_div(g.tb, state_ptr(c, m, 0), c->diagbuf, c->st);
  CK(cudaGetLastError());
  unsigned long long bits[2];
  CK(cudaMemcpyAsync(bits, c->diagbuf, sizeof bits, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  double dv[2];
  memcpy(dv, bits, sizeof dv);
  out->div_max = dv[0];
  out->div_wall = dv[1];
  return NSP_OK;
}

// Re u_z(0,0)(r) of every member into prof (internal order, each group's members
// NR_g values apiece) on the device, then to the host.  poff[g]: group offsets.
static int gather_means(nsp_ctx* c, std::vector<double>& prof, std::vector<size_t>& poff) {
  size_t n = 0;
  poff.assign(c->groups.size(), 0);
  for (size_t k = 0; k < c->groups.size(); k++) {
    poff[k] = n;
    n += (size_t)c->groups[k].tb.nmem * c->groups[k].tb.NR;
  }
  if (int rc = ensure_crossbuf(c, n)) return rc;
  for (size_t k = 0; k < c->groups.size(); k++) {
    const Group& g = c->groups[k];
    launch_gather_mean(g.tb, g.bf.U[c->parity], c->crossbuf + poff[k], g.tb.nmem, c->st);
  }
  CK(cudaGetLastError());
  prof.resize(n);
  CK(cudaMemcpyAsync(prof.data(), c->crossbuf, n * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return NSP_OK;
}

int nsp_diag_all(nsp_ctx* c, nsp_diag_out* out) {
  if (!c) return NSP_ERR_ARG;
  if (!out) return fail(c, NSP_ERR_ARG, "null output");
  if (!c->setup_done) return fail(c, NSP_ERR_STATE, "nsp_diag_all before nsp_setup");
  const int nm = c->nmem;
  if (int rc = ensure_diagbuf(c)) return rc;
  CK(cudaMemsetAsync(c->diagbuf, 0, 2 * sizeof(unsigned long long) * nm, c->st));
  for (const Group& g : c->groups)
    launch_diag_div(g.tb, g.bf.U[c->parity], c->diagbuf + 2 * g.tb.mem0, c->st, g.tb.nmem);
  CK(cudaGetLastError());
  std::vector<unsigned long long> bits(2 * (size_t)nm);
  std::vector<double> err(nm);
  std::vector<int> status(nm), ite(nm), unconv(nm);
  CK(cudaMemcpyAsync(bits.data(), c->diagbuf, sizeof(unsigned long long) * bits.size(), cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(unconv.data(), c->hctl.unconv, sizeof(int) * nm, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(err.data(), c->hctl.err, sizeof(double) * nm, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(status.data(), c->hctl.status, sizeof(int) * nm, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(ite.data(), c->hctl.ite, sizeof(int) * nm, cudaMemcpyDeviceToHost, c->st));
  std::vector<double> prof;
  std::vector<size_t> poff;
  if (int rc = gather_means(c, prof, poff)) return rc;  // synchronises the stream
  for (int m = 0; m < nm; m++) {
    const int gi = c->grp[m], mi = c->internal[m];
    const Group& g = c->groups[gi];
    friction(g.ops, g.tb.NR, prof.data() + poff[gi] + (size_t)c->slot[m] * g.tb.NR, c->prm[m].Re, out + m);
    out[m].last_err = err[mi];
    out[m].last_iters = ite[mi];
    out[m].status = (status[mi] & NSP_ERR_NONFINITE) ? NSP_ERR_NONFINITE : NSP_OK;
    out[m].unconverged_steps = unconv[mi];
    double dv[2];
    memcpy(dv, bits.data() + 2 * (size_t)mi, sizeof dv);
    out[m].div_max = dv[0];
    out[m].div_wall = dv[1];
  }
  return NSP_OK;
}

int nsp_mean_profile_all(nsp_ctx* c, double* out) {
  if (!c) return NSP_ERR_ARG;
  if (!out) return fail(c, NSP_ERR_ARG, "null output");
  std::vector<double> prof;
  std::vector<size_t> poff;
  if (int rc = gather_means(c, prof, poff)) return rc;
  size_t o = 0;
  for (int m = 0; m < c->nmem; m++) {
    const Group& g = c->groups[c->grp[m]];
    memcpy(out + o, prof.data() + poff[c->grp[m]] + (size_t)c->slot[m] * g.tb.NR, sizeof(double) * g.tb.NR);
    o += g.tb.NR;
  }
  return NSP_OK;
}

int nsp_cross_sections_all(nsp_ctx* c, double* q, double* u) {
  if (!c) return NSP_ERR_ARG;
  if (!q || !u) return fail(c, NSP_ERR_ARG, "null output");
  if (!c->setup_done) return fail(c, NSP_ERR_STATE, "nsp_cross_sections_all before nsp_setup");
  std::vector<size_t> poff(c->groups.size());
  size_t n = 0;
  for (size_t k = 0; k < c->groups.size(); k++) {
    poff[k] = n;
    n += (size_t)c->groups[k].tb.nmem * 2 * c->groups[k].tb.NR * c->groups[k].tb.NZR;
  }
  if (int rc = ensure_crossbuf(c, n)) return rc;
  for (size_t k = 0; k < c->groups.size(); k++) {
    const Group& g = c->groups[k];
    launch_diag_cross(g.tb, g.bf.U[c->parity], c->crossbuf + poff[k], c->st, g.tb.nmem);
  }
  CK(cudaGetLastError());
  std::vector<double> part(n);
  CK(cudaMemcpyAsync(part.data(), c->crossbuf, n * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  size_t o = 0;
  for (int m = 0; m < c->nmem; m++) {
    const Group& g = c->groups[c->grp[m]];
    const int NR = g.tb.NR, NZR = g.tb.NZR;
    const double* pm = part.data() + poff[c->grp[m]] + (size_t)c->slot[m] * 2 * NR * NZR;
    for (int z = 0; z < NZR; z++) {
      double sq = 0.0, su = 0.0;
      for (int i = 0; i < NR; i++) {  // the radial quadrature, in level order
        sq += pm[(size_t)i * NZR + z];
        su += pm[(size_t)(NR + i) * NZR + z];
      }
      q[o + z] = sq;
      u[o + z] = su;
    }
    o += NZR;
  }
  return NSP_OK;
}

int nsp_cross_sections(nsp_ctx* c, int m, double* q, double* u) {
  if (int rc = check_member(c, m)) return rc;
  if (!q || !u) return fail(c, NSP_ERR_ARG, "null output");
  if (!c->setup_done) return fail(c, NSP_ERR_STATE, "nsp_cross_sections before nsp_setup");
  const Group& g = c->groups[c->grp[m]];
  const int NR = g.tb.NR, NZR = g.tb.NZR;
  const size_t n = (size_t)2 * NR * NZR;
  if (int rc = ensure_crossbuf(c, n)) return rc;
  launch_diag_cross(g.tb, state_ptr(c, m, 0), c->crossbuf, c->st);
  CK(cudaGetLastError());
  std::vector<double> part(n);
  CK(cudaMemcpyAsync(part.data(), c->crossbuf, n * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  for (int z = 0; z < NZR; z++) {
    double sq = 0.0, su = 0.0;
    for (int i = 0; i < NR; i++) {  // the radial quadrature, in level order
      sq += part[(size_t)i * NZR + z];
      su += part[(size_t)(NR + i) * NZR + z];
    }
    q[z] = sq;
    u[z] = su;
  }
  return NSP_OK;
}

int nsp_mean_profile(nsp_ctx* c, int m, double* out) {
  if (int rc = check_member(c, m)) return rc;
  if (!out) return fail(c, NSP_ERR_ARG, "null output");
  const Group& g = c->groups[c->grp[m]];
  // Re u_z(0,0)(r_i): the first double of each radial row's (0,0) coefficient.
  CK(cudaMemcpy2DAsync(out, sizeof(double), state_ptr(c, m, 2), sizeof(double2) * g.tb.NTNZ, sizeof(double), g.tb.NR,
                       cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return NSP_OK;
}

int nsp_grid(nsp_ctx* c, int m, double* r, double* rdr) {
  if (int rc = check_member(c, m)) return rc;
  if (!c->setup_done) return fail(c, NSP_ERR_STATE, "nsp_grid before nsp_setup");
  const HostOps& o = c->groups[c->grp[m]].ops;
  if (r) memcpy(r, o.r.data(), sizeof(double) * o.r.size());
  if (rdr) memcpy(rdr, o.rdr.data(), sizeof(double) * o.rdr.size());
  return NSP_OK;
}

long long nsp_kernel_launches(nsp_ctx* c) { return c ? c->launches_last : 0; }

int nsp_describe(nsp_ctx* c, char* buf, int cap) {
  if (!c || !buf || cap <= 0) return NSP_ERR_ARG;
  std::string s = "{\"precision\": \"";
  s += c->precision == NSP_MIXED ? "mixed" : "fp64";
  s += "\", \"graph\": ";
  s += c->use_graph ? "true" : "false";
  // the arithmetic of the linear passes (the transforms' is each group's "theta"/"z_stage")
  s += c->precision == NSP_MIXED
           ? ", \"linear\": {\"predictor\": \"double-float (FP32 pairs) stencils, solves and corrections; FP64 state\", "
             "\"corrector\": \"increment pass: FP32 stencils, corrections and Helmholtz solves, double-float "
             "pressure solve, FP64 update\"}"
           : ", \"linear\": {\"predictor\": \"fp64\", \"corrector\": \"fp64\"}";
  s += ", \"groups\": [";
  for (size_t k = 0; k < c->groups.size(); k++) {
    const Tables& tb = c->groups[k].tb;
    int v = linear_variant_fits(tb.lin_variant, tb.NR) ? tb.lin_variant : linear_default_variant(tb.NR);
    int vi = linear_variant_fits(tb.lin_variant_inc, tb.NR) ? tb.lin_variant_inc : linear_default_variant(tb.NR);
    int LM = 0, NTH = 0, LMi = 0, NTHi = 0;
    linear_shape(v, &LM, &NTH);
    linear_shape(vi, &LMi, &NTHi);
    char inc[64] = "";
    if (c->precision == NSP_MIXED) snprintf(inc, sizeof inc, ", \"linear_block_corrector\": [%d, %d]", LMi, NTHi);
    char g[512];
    snprintf(g, sizeof(g),
             "%s{\"shape\": [%d, %d, %d], \"members\": %d, \"parameter_sets\": %d, \"linear_block\": [%d, %d]%s, "
             "\"theta\": \"%s\", \"z_stage\": \"%s\", \"setup\": \"%s\"}",
             k ? ", " : "", tb.NR, tb.NT, tb.NZ, tb.nmem, tb.nsets, LM, NTH, inc,
             c->precision != NSP_MIXED ? "fft-fp64" : (tb.tc_theta ? "tcgen05-3xtf32" : "fft-fp32"),
             z_variant_name(tb.NZR, tb.NTP, c->precision == NSP_MIXED, tb.z_variant).c_str(),
             c->groups[k].device_setup ? "device" : "host");
    s += g;
  }
  s += "]}";
  if ((int)s.size() + 1 > cap) return fail(c, NSP_ERR_ARG, "describe: buffer of %d bytes too small", cap);
  memcpy(buf, s.c_str(), s.size() + 1);
  return NSP_OK;
}

int nsp_set_stream(nsp_ctx* c, void* stream) {
  if (!c) return NSP_ERR_ARG;
  CK(cudaStreamSynchronize(c->st));
  c->st = stream ? (cudaStream_t)stream : c->own_st;
  return NSP_OK;
}

int nsp_bounds_report(nsp_ctx* c, long long* out) {
  if (!c || !out) return NSP_ERR_ARG;
  if (c->groups.empty() || !c->groups[0].tb.bc) return fail(c, NSP_ERR_STATE, "no bounds record");
  unsigned long long rec[4];
  CK(cudaStreamSynchronize(c->st));
  CK(cudaMemcpy(rec, c->groups[0].tb.bc, sizeof rec, cudaMemcpyDeviceToHost));
  for (int k = 0; k < 4; k++) out[k] = (long long)rec[k];
  out[4] = kBoundsCheck ? 1 : 0;
  return NSP_OK;
}

int nsp_set_strict(nsp_ctx* c, int strict) {
  if (!c) return NSP_ERR_ARG;
  c->strict = strict != 0;
  return NSP_OK;
}

int nsp_profile_stages(nsp_ctx* c, int reps, double* ms_out) {
  if (!c || !ms_out || reps < 1) return NSP_ERR_ARG;
  if (!c->setup_done) return fail(c, NSP_ERR_STATE, "nsp_profile_stages before nsp_setup");
  CK(cudaSetDevice(c->device));
  const int nm = c->nmem;
  std::vector<int> zeros(nm, 0), ones(nm, 1);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const bool mixed = c->precision == NSP_MIXED;
  for (int stage = 0; stage < 5; stage++) {
    auto launch = [&]() {
      if (stage < 3) {
        for (auto& g : c->groups) launch_nonlinear(g.tb, g.bf, c->dctl, mixed, nullptr, nullptr, c->st, 1 << stage);
      } else if (stage == 3) {
        for (auto& g : c->groups) launch_linear(g.tb, g.bf, c->dctl, c->st, LIN_PRED);  // phases are 0
      } else {
        launch_converge(c->dctl, nm, 0ull, 0, c->st);
      }
    };
    launch();  // warm-up
    CK(cudaEventRecord(e0, c->st));
    for (int r = 0; r < reps; r++) {
      launch();
      if (stage == 4) CK(cudaMemcpyAsync(c->hctl.phase, ones.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, c->st));
    }
    CK(cudaEventRecord(e1, c->st));
    CK(cudaGetLastError());
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    ms_out[stage] = ms / reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // Restore the step-boundary control state.
  return reset_control(c);
}

int nsp_profile_linear(nsp_ctx* c, int reps, double* ms_out) {
  if (!c || !ms_out || reps < 1) return NSP_ERR_ARG;
  if (!c->setup_done) return fail(c, NSP_ERR_STATE, "nsp_profile_linear before nsp_setup");
  CK(cudaSetDevice(c->device));
  const int nm = c->nmem;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  for (int pass = 0; pass < 2; pass++) {  // 0: every member in its predictor pass, 1: in a corrector pass
    std::vector<int> ph(nm, pass);
    CK(cudaMemcpyAsync(c->hctl.phase, ph.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, c->st));
    const int which = pass ? LIN_CORR : LIN_PRED;
    for (auto& g : c->groups) launch_linear(g.tb, g.bf, c->dctl, c->st, which);  // warm-up
    CK(cudaEventRecord(e0, c->st));
    for (int r = 0; r < reps; r++)
      for (auto& g : c->groups) launch_linear(g.tb, g.bf, c->dctl, c->st, which);
    CK(cudaEventRecord(e1, c->st));
    CK(cudaGetLastError());
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    ms_out[pass] = ms / reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return reset_control(c);
}

int nsp_measure_fp64_peak(nsp_ctx* c, double* tflops) {
  if (!c || !tflops) return NSP_ERR_ARG;
  CK(cudaSetDevice(c->device));
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, c->device));
  const int blocks = prop.multiProcessorCount * 8, threads = 256, iters = 4096;
  double* out = nullptr;
  CK(cudaMallocAsync(&out, sizeof(double) * blocks * threads, c->st));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  for (int w = 0; w < 2; w++) launch_fp64_peak(out, blocks, threads, iters, c->st);
  float best = 1e30f;
  for (int r = 0; r < 3; r++) {
    CK(cudaEventRecord(e0, c->st));
    launch_fp64_peak(out, blocks, threads, iters, c->st);
    CK(cudaEventRecord(e1, c->st));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    best = std::min(best, ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CK(cudaFreeAsync(out, c->st));
  CK(cudaStreamSynchronize(c->st));
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return NSP_OK;
}

int nsp_sync(nsp_ctx* c) {
  if (!c) return NSP_ERR_ARG;
  CK(cudaStreamSynchronize(c->st));
  return NSP_OK;
}

int nsp_get_params(nsp_ctx* c, int m, nsp_params* out) {
  if (int rc = check_member(c, m)) return rc;
  if (!out) return fail(c, NSP_ERR_ARG, "null output");
  *out = c->prm[m];
  return NSP_OK;
}

int nsp_info(nsp_ctx* c, int* n_members, int* precision) {
  if (!c) return NSP_ERR_ARG;
  if (n_members) *n_members = c->nmem;
  if (precision) *precision = c->precision;
  return NSP_OK;
}

int nsp_debug_inject(nsp_ctx* c, int flags) {
  if (!c) return NSP_ERR_ARG;
  CK(cudaMemcpyAsync(&c->dctl->inject, &flags, sizeof(int), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return NSP_OK;
}

const char* nsp_last_error(nsp_ctx* c) {
  if (c) return c->err.c_str();
  return g_host_err.empty() ? "null context" : g_host_err.c_str();
}

int nsp_remesh_members(nsp_remesh* rm, nsp_ctx* src, const int* src_members, nsp_ctx* dst, const int* dst_members,
                       int count) {
  if (!rm || !src || !dst || count < 0 || (count > 0 && (!src_members || !dst_members))) return NSP_ERR_ARG;
  int old3[3], new3[3];
  remesh_shape(rm, old3, new3);
  if (src->device != remesh_device(rm) || dst->device != remesh_device(rm))
    return fail(dst, NSP_ERR_ARG, "the remesh plan and both contexts must be on one device");
  std::vector<const void*> sp(count);
  std::vector<void*> dp(count);
  for (int k = 0; k < count; k++) {
    const int a = src_members[k], b = dst_members[k];
    if (int rc = check_member(src, a)) return rc == NSP_ERR_ARG && src != dst ? fail(dst, rc, "%s", src->err.c_str()) : rc;
    if (int rc = check_member(dst, b)) return rc;
    const nsp_params &ps = src->prm[a], &pd = dst->prm[b];
    if (ps.NR != old3[0] || ps.NT != old3[1] || ps.NZ != old3[2])
      return fail(dst, NSP_ERR_ARG, "source member %d is %dx%dx%d, the plan's source shape %dx%dx%d", a, ps.NR, ps.NT,
                  ps.NZ, old3[0], old3[1], old3[2]);
    if (pd.NR != new3[0] || pd.NT != new3[1] || pd.NZ != new3[2])
      return fail(dst, NSP_ERR_ARG, "destination member %d is %dx%dx%d, the plan's destination shape %dx%dx%d", b, pd.NR,
                  pd.NT, pd.NZ, new3[0], new3[1], new3[2]);
    sp[k] = state_ptr(src, a, 0);
    dp[k] = state_ptr(dst, b, 0);
  }
  for (int k = 0; k < count; k++)
    for (int q = 0; q < count; q++)
      if (sp[k] == dp[q]) return fail(dst, NSP_ERR_ARG, "a member is both a source and a destination");
  nsp_ctx* c = dst;  // CUDA failures are reported on the destination context
  c->mirror_ok = false;
  CK(cudaSetDevice(dst->device));
  CK(cudaStreamSynchronize(src->st));
  int rc = remesh_launch(rm, count, sp.data(), dp.data(), dst->st);
  if (rc) return fail(dst, rc, "%s", g_host_err.c_str());
  return NSP_OK;
}

int nsp_destroy(nsp_ctx* c) {
  if (!c) return NSP_OK;
  cudaSetDevice(c->device);
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  for (void* p : c->allocs) cudaFree(p);
  for (cudaStream_t s2 : c->side) cudaStreamDestroy(s2);
  for (cudaEvent_t e2 : c->ev_join) cudaEventDestroy(e2);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->cp_in) cudaStreamSynchronize(c->cp_in), cudaStreamDestroy(c->cp_in);
  if (c->cp_out) cudaStreamSynchronize(c->cp_out), cudaStreamDestroy(c->cp_out);
  for (cudaEvent_t e2 : c->ev_in) cudaEventDestroy(e2);
  for (cudaEvent_t e2 : c->ev_done) cudaEventDestroy(e2);
  for (cudaGraphExec_t x : c->chunk_exec)
    if (x) cudaGraphExecDestroy(x);
  if (c->own_st) cudaStreamDestroy(c->own_st);
  if (c->pin) cudaFreeHost(c->pin);
  delete c;
  return NSP_OK;
}

}  // extern "C"
