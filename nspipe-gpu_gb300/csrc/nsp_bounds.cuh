// nsp_bounds.cuh -- the bounds-checked build of the step kernels.
//
// Compiled with -DNSP_BOUNDS_CHECK (nspipe-gpu_gb300/build.py --bounds-check, which
// makes libnspipe_gb300_bc.so), every global-memory access of the step kernels whose
// index is computed from the launch geometry is checked against the extent of the
// array (or member slab) it addresses.  An access outside it is skipped -- a load
// reads zero, a store is dropped -- and counted in the context's bounds record
// (Tables::bc): [0] violations, then the first violation's [1] site, [2] index and
// [3] extent (read with nsp_bounds_report).  In the normal build NSP_IN_BOUNDS is the
// constant true and every check compiles away.
#pragma once

#include "nsp_internal.h"

namespace nsp {

#ifdef NSP_BOUNDS_CHECK
constexpr bool kBoundsCheck = true;
__device__ __forceinline__ bool bounds_ok(unsigned long long* rec, long long idx, long long lim, int site) {
  if (idx >= 0 && idx < lim) return true;
  if (atomicAdd(rec, 1ull) == 0ull) {
    rec[1] = (unsigned long long)site;
    rec[2] = (unsigned long long)idx;
    rec[3] = (unsigned long long)lim;
  }
  return false;
}
#define NSP_IN_BOUNDS(tb, idx, lim, site) ::nsp::bounds_ok((tb).bc, (long long)(idx), (long long)(lim), (site))
#else
constexpr bool kBoundsCheck = false;
#define NSP_IN_BOUNDS(tb, idx, lim, site) true
#endif

// Check sites (the value recorded in bc[1]).
enum BoundsSite {
  BC_LIN_MEMBER = 1,   // linear pass: member index of the block
  BC_LIN_POINT,        // linear pass: point index of a member slab (state, N, RHSW, V, mirrors)
  BC_LIN_TAP,          // linear pass: stencil tap of the explicit Laplacian
  BC_LIN_FACTOR,       // linear pass: banded-factor row
  BC_THETA_IN,         // theta transforms: state / mirror / H load
  BC_THETA_OUT,        // theta transforms: G / N store
  BC_Z_IN,             // z stage: G load
  BC_Z_OUT,            // z stage: H store
  BC_MIRROR,           // FP32 mirror of an outside state
  BC_CONVERGE,         // convergence bookkeeping: member index
};

}  // namespace nsp
