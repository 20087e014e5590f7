// remesh_driver.cu -- a driver main() for the reference Re_Mesh tool.
//
// TEST INFRASTRUCTURE.  Compiled together with the tool's own
// tools/Re_Mesh/src/mod_remesh.cu and mod_io.cu and a head.h whose grid
// #defines (NR, NT, NZ, Nrd, Ntd, Nzd, iw; head.h:10-23) were patched.  It runs
// the sequence of the tool's main (main.cu:14-33): a zeroed destination field,
// re_mesh(u) (which reads ur_o.bin, ut_o.bin, uz_o.bin from the working
// directory), then ur_s.bin, ut_s.bin, uz_s.bin written by wBufferBinary -- on
// device 0, where the tool's main selects device 1 (main.cu:13).
#include "head.h"

int main() {
  CHECK_CUDART(cudaSetDevice(0));
  vfield u;
  size_t bytes = (size_t)Nrd * Ntd * Nzd * sizeof(double2);
  CHECK_CUDART(cudaMalloc(&u.r, bytes));
  CHECK_CUDART(cudaMalloc(&u.t, bytes));
  CHECK_CUDART(cudaMalloc(&u.z, bytes));
  CHECK_CUDART(cudaMemset(u.r, 0, bytes));
  CHECK_CUDART(cudaMemset(u.t, 0, bytes));
  CHECK_CUDART(cudaMemset(u.z, 0, bytes));
  re_mesh(u);
  CHECK_CUDART(cudaDeviceSynchronize());
  wBufferBinary((double*)u.r, "ur_s.bin", sizeof(double2), (size_t)Nrd * Ntd * Nzd);
  wBufferBinary((double*)u.t, "ut_s.bin", sizeof(double2), (size_t)Nrd * Ntd * Nzd);
  wBufferBinary((double*)u.z, "uz_s.bin", sizeof(double2), (size_t)Nrd * Ntd * Nzd);
  cudaFree(u.r);
  cudaFree(u.t);
  cudaFree(u.z);
  return 0;
}
