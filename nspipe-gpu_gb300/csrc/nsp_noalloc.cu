// nsp_noalloc.cu -- fixed device scratch for the allocation-free nonlinear entry point.
//
// nsp_nonlinear_static (nsp_api.cu) evaluates the same three transform kernels as
// nsp_nonlinear, but keeps their intermediates (the theta-inverse columns G, the
// z-forward products H and, in the mixed form, the FP32 copy of the input) in the
// file-scope array below instead of in memory obtained from cudaMalloc.  It is for
// callers that must not allocate device memory while they run: hosts with a
// device-memory budget fixed after start-up (real-time or embedded control loops
// driving the flow), applications whose own pool allocator owns the device memory,
// and loops that cannot afford cudaMalloc/cudaFree, which may synchronise the
// device and take unbounded time.
//
// The array is a plain __device__ symbol: every process that loads this library
// holds NOALLOC_SCRATCH_BYTES on each GPU it uses until it exits.  In host code
// the symbol's name is only a host-side stand-in, so its device address is looked
// up once per device with cudaGetSymbolAddress (with that device current) and
// cached; the first call on a device does this set-up.  The cached address belongs
// to the device's primary context: after cudaDeviceReset on that device the module
// is loaded again (possibly elsewhere), so a process that resets a device must not
// call the allocation-free entry point on it afterwards.
#include <mutex>
#include <string>

#include "nsp_internal.h"

namespace nsp {

constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(32) << 20;  // 32 MiB per device
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

size_t noalloc_scratch_bytes() { return NOALLOC_SCRATCH_BYTES; }

// Device address of the scratch array on `device` (which must be current).
cudaError_t noalloc_scratch(int device, void** ptr) {
  if (device < 0 || device >= NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[device] = p;
  }
  *ptr = g_noalloc_ptr[device];
  return cudaSuccess;
}

}  // namespace nsp
