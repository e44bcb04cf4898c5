// Host-side state and helpers shared by the C ABI translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pskel_gb300.h"

namespace pskel {

struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
};

// One per CUDA device, created on first use with that device current.
struct DeviceContext {
  int device = 0;
  int sms = 0;
  int smem_optin = 0;
  unsigned* err = nullptr;        // device error word (kernels atomicOr into it)
  unsigned* err_host = nullptr;   // pinned host copy of it, read after a stream's copy lands
  cudaStream_t stream = nullptr;  // stream of the *_host entry points
  cudaStream_t copy_in = nullptr, copy_out = nullptr;  // their overlapped copies
  DeviceBuffer host_in, host_out, host_u, host_v;  // staging for *_host
  DeviceBuffer partials;                           // 3D residual: per-CTA fp64 partial sums
  DeviceBuffer residuals;                          // 3D residual norms for *_host
  DeviceBuffer res_acc;                            // 3D wavefront: squared sums per reported step
  DeviceBuffer life_bits;                          // Life: the two bit planes of a run
  DeviceBuffer life_sync;                          // Life: item counter and per-tile pass counts
  DeviceBuffer fast2d_sync;                        // 2D multi-pass launches: item counter and per-tile pass counts
  DeviceBuffer tiles;                              // out-of-core runs: slab slots and both arrays' rings
  DeviceBuffer selftest;                           // the bounded-wait self-test's grids
};

pskel_status fail(pskel_status code, const char* fmt, ...);
pskel_status cuda_fail(cudaError_t e, const char* what);
void clear_error();
pskel_status get_context(DeviceContext** out);
pskel_status ensure_buffer(DeviceBuffer& b, size_t bytes);
pskel_status device_sync_check(DeviceContext* c, cudaStream_t s);
pskel_status check_mask(const pskel_mask& m, int dim, bool need_weights, int* max_off, int* ring);
pskel_status validate3d(const pskel_stencil* st, const void* in, const void* out, int64_t W, int64_t H, int64_t D,
                        int64_t iters, int64_t every, int* R);
// The 3D pass loop. With partials_override set, the residual partial sums go
// to that array (capacity partials_cap doubles) instead of c->partials, and
// nothing is allocated.
pskel_status iterate3d(const pskel_stencil& st, void* in, void* out, int64_t W, int64_t H, int64_t D, int64_t iters,
                       int R, const pskel_schedule* sched, int64_t every, double* residuals, double* partials_override,
                       int64_t partials_cap, DeviceContext* c, cudaStream_t s);

}  // namespace pskel
