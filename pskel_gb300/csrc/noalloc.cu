// pskel_iterate3d_noalloc: the 3D iterative stencil without any device
// allocation by the library.
//
// Some callers cannot let a library call cudaMalloc: a host application that
// owns every byte of device memory through its own pool and forbids plugins
// from allocating, or a latency-critical loop where cudaMalloc's implicit
// device synchronisation and unbounded latency are not acceptable. The regular
// entry point allocates its residual scratch, its error word and a stream on
// first use; this one takes all of them from file-scope device arrays of fixed
// size instead, and the caller passes the grids and the residual output.
#include <mutex>

#include "../../include/pskel_gb300.h"
#include "capi_internal.h"
#include "kernels.h"

namespace {

// Residual scratch: one fp64 partial sum per (fused step, CTA) of a pass.
// 16384 doubles = 128 KiB, enough for 8 fused steps on 2048 CTAs. Every GPU
// that loads the library holds this array (and the error word) until exit.
constexpr int64_t kNoAllocPartials = 16384;
static __device__ __align__(256) double g_noalloc_partials[kNoAllocPartials];
static __device__ __align__(256) unsigned g_noalloc_err[16];

struct NoAllocDevice {
  bool ready = false;
  double* partials = nullptr;  // device address of g_noalloc_partials on this device
  unsigned* err = nullptr;     // device address of g_noalloc_err on this device
  int sms = 0;
  int smem_optin = 0;
};

std::mutex g_mu;
NoAllocDevice g_dev[64];

// Once per device, with that device current: the device addresses of the
// file-scope arrays. In host code their names are host-side stand-ins, not
// device addresses, so they must never be passed to a kernel directly.
pskel_status setup(int dev, NoAllocDevice** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  NoAllocDevice& d = g_dev[dev];
  if (!d.ready) {
    cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&d.partials), g_noalloc_partials);
    if (e != cudaSuccess) return pskel::cuda_fail(e, "cudaGetSymbolAddress(residual scratch)");
    e = cudaGetSymbolAddress(reinterpret_cast<void**>(&d.err), g_noalloc_err);
    if (e != cudaSuccess) return pskel::cuda_fail(e, "cudaGetSymbolAddress(error word)");
    e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return pskel::cuda_fail(e, "cudaDeviceGetAttribute");
    e = cudaDeviceGetAttribute(&d.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return pskel::cuda_fail(e, "cudaDeviceGetAttribute");
    d.ready = true;
  }
  *out = &d;
  return PSKEL_OK;
}

}  // namespace

extern "C" PSKEL_API pskel_status pskel_iterate3d_noalloc(const pskel_stencil* st, void* in, void* out,
                                                          int64_t width, int64_t height, int64_t depth,
                                                          int64_t iterations, const pskel_schedule* sched,
                                                          int64_t residual_every, double* residuals, void* stream) {
  pskel::clear_error();
  int R = 0;
  if (pskel_status s = pskel::validate3d(st, in, out, width, height, depth, iterations, residual_every, &R)) return s;
  if (residual_every > 0 && iterations >= residual_every && !residuals)
    return pskel::fail(PSKEL_ERR_INVALID, "residual output pointer is NULL");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return pskel::cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) return pskel::fail(PSKEL_ERR_UNSUPPORTED, "device ordinal %d beyond 63", dev);
  NoAllocDevice* d = nullptr;
  if (pskel_status s = setup(dev, &d)) return s;
  if (iterations == 0) return PSKEL_OK;
  // a context that owns nothing: iterate3d only reads these fields when it is
  // given the scratch array (partials_override)
  pskel::DeviceContext c;
  c.device = dev;
  c.sms = d->sms;
  c.smem_optin = d->smem_optin;
  c.err = d->err;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (pskel_status q = pskel::iterate3d(*st, in, out, width, height, depth, iterations, R, sched, residual_every,
                                        residuals, d->partials, kNoAllocPartials, &c, s))
    return q;
  // the error word is read behind the run on the caller's stream, so only
  // that stream is waited for (no legacy-stream copy that would wait for
  // every other blocking stream of the device)
  unsigned word = 0;
  e = cudaMemcpyAsync(&word, d->err, sizeof(word), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return pskel::cuda_fail(e, "reading the device error word");
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return pskel::cuda_fail(e, "kernel execution");
  if (word) {
    e = cudaMemsetAsync(d->err, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return pskel::cuda_fail(e, "clearing the device error word");
    return pskel::fail(PSKEL_ERR_DEVICE, "device error word 0x%x (a bounded wait timed out)", word);
  }
  return PSKEL_OK;
}
