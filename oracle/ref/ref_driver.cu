// ref_driver.cu -- a driver main() for the reference nsPipe-CUDA build.
//
// TEST INFRASTRUCTURE.  Compiled together with the reference's own
// Main_Code/src/*.cu (except its main.cu) and a head.h whose #define
// parameters were patched per configuration.  It calls the reference's public
// entry points in the order of the reference main (main.cu:25-38):
// init_fd, setFft, setLinear, setCublasFlux, setDeriv, setNonlinear, setIO,
// setInt, setBCon, initField (restart=1 reads u?_s.bin), then integrate().
//
// Modes:
//   trace N LIST  : build with nsteps=1; calls integrate() N times and records
//                   the corrector iteration count of each step (the number of
//                   nonlinear() calls minus one, counted through a linker
//                   --wrap of nonlinear); writes ur_<s>.bin... after the steps
//                   s in the comma-separated LIST.
//   time  N       : build with nsteps=N; one untimed integrate() call (module
//                   loading, cuFFT/cuBLAS first use), the initial field put back,
//                   then one integrate() call timed with wall clock and
//                   cudaDeviceSynchronize on both sides.
#include "head.h"
#include <chrono>
#include <cstring>

static long g_nl_calls = 0;
extern "C" void __real__Z9nonlinear6vfieldS_(vfield u, vfield du);
extern "C" void __wrap__Z9nonlinear6vfieldS_(vfield u, vfield du) {
  g_nl_calls++;
  __real__Z9nonlinear6vfieldS_(u, du);
}

int main(int argc, const char* argv[]) {
  if (argc < 3) { fprintf(stderr, "usage: %s trace|time N [EVERY]\n", argv[0]); return 2; }
  const char* mode = argv[1];
  int N = atoi(argv[2]);
  const char* list = argc > 3 ? argv[3] : "";
  auto wanted = [&](int s) {
    char buf[32];
    snprintf(buf, sizeof buf, "%d", s);
    size_t n = strlen(buf);
    for (const char* p = list; (p = strstr(p, buf)) != nullptr; p += n)
      if ((p == list || p[-1] == ',') && (p[n] == ',' || p[n] == 0)) return true;
    return s == N;
  };
  CHECK_CUDART(cudaSetDevice(0));
  size_p sizes; sizes.Nr = NR; sizes.Nt = NT; sizes.Nz = NZ;
  double* r_h = (double*)malloc(NR * sizeof(double));
  double* Lu_h = (double*)malloc(2 * sten * NR * sizeof(double));
  double* Lp_h = (double*)malloc(2 * sten * NR * sizeof(double));
  double* rdr_h = (double*)malloc(NR * sizeof(double));
  init_fd(r_h, Lu_h, Lp_h, rdr_h);
  setFft(sizes); setLinear(r_h, Lu_h, Lp_h); setCublasFlux(rdr_h); setDeriv(r_h);
  setNonlinear(); setIO(r_h); setInt(); setBCon();
  vfield u, rhs; size_t sz = (size_t)NR * NT * NZ * sizeof(double2);
  CHECK_CUDART(cudaMalloc(&u.r, sz)); CHECK_CUDART(cudaMalloc(&rhs.r, sz));
  CHECK_CUDART(cudaMalloc(&u.t, sz)); CHECK_CUDART(cudaMalloc(&rhs.t, sz));
  CHECK_CUDART(cudaMalloc(&u.z, sz)); CHECK_CUDART(cudaMalloc(&rhs.z, sz));
  initField(u);
  CHECK_CUDART(cudaDeviceSynchronize());
  if (!strcmp(mode, "trace")) {
    FILE* f = fopen("iters.txt", "w");
    for (int s = 1; s <= N; s++) {
      long c0 = g_nl_calls;
      integrate(u, rhs);
      fprintf(f, "%d %ld\n", s, g_nl_calls - c0 - 1);
      if (wanted(s)) {
        char nm[3][64];
        snprintf(nm[0], 64, "ur_%d.bin", s); snprintf(nm[1], 64, "ut_%d.bin", s); snprintf(nm[2], 64, "uz_%d.bin", s);
        wBufferBinary((double*)u.r, nm[0], sizeof(double2), (size_t)NR * NT * NZ);
        wBufferBinary((double*)u.t, nm[1], sizeof(double2), (size_t)NR * NT * NZ);
        wBufferBinary((double*)u.z, nm[2], sizeof(double2), (size_t)NR * NT * NZ);
      }
    }
    fclose(f);
  } else {
    // warm-up: the same integrate() call once, untimed, from a saved copy of u
    vfield u0;
    CHECK_CUDART(cudaMalloc(&u0.r, sz)); CHECK_CUDART(cudaMalloc(&u0.t, sz)); CHECK_CUDART(cudaMalloc(&u0.z, sz));
    CHECK_CUDART(cudaMemcpy(u0.r, u.r, sz, cudaMemcpyDeviceToDevice));
    CHECK_CUDART(cudaMemcpy(u0.t, u.t, sz, cudaMemcpyDeviceToDevice));
    CHECK_CUDART(cudaMemcpy(u0.z, u.z, sz, cudaMemcpyDeviceToDevice));
    integrate(u, rhs);
    CHECK_CUDART(cudaMemcpy(u.r, u0.r, sz, cudaMemcpyDeviceToDevice));
    CHECK_CUDART(cudaMemcpy(u.t, u0.t, sz, cudaMemcpyDeviceToDevice));
    CHECK_CUDART(cudaMemcpy(u.z, u0.z, sz, cudaMemcpyDeviceToDevice));
    CHECK_CUDART(cudaDeviceSynchronize());
    long c0 = g_nl_calls;
    auto t0 = std::chrono::steady_clock::now();
    integrate(u, rhs);
    CHECK_CUDART(cudaDeviceSynchronize());
    auto t1 = std::chrono::steady_clock::now();
    double s = std::chrono::duration<double>(t1 - t0).count();
    long calls = g_nl_calls - c0;
    printf("\nREFTIME {\"steps\": %d, \"seconds\": %.9f, \"nonlinear_calls\": %ld}\n", nsteps, s, calls);
    wBufferBinary((double*)u.r, "ur.bin", sizeof(double2), (size_t)NR * NT * NZ);
    wBufferBinary((double*)u.t, "ut.bin", sizeof(double2), (size_t)NR * NT * NZ);
    wBufferBinary((double*)u.z, "uz.bin", sizeof(double2), (size_t)NR * NT * NZ);
  }
  return 0;
}
