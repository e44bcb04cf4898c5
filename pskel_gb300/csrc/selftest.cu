// A self-test of the bounded waits every kernel of the library relies on: a
// kernel waits on an mbarrier phase that never completes, or on a device flag
// that nothing sets, with a short poll limit. It gives up, records the timeout
// in the device error word and returns, so the host reads PSKEL_ERR_DEVICE
// from pskel_sync and the context stays usable. Nothing faults, traps or hangs.
#include "../../include/pskel_gb300.h"
#include "capi_internal.h"
#include "common.cuh"

namespace pskel {
namespace {

__device__ unsigned g_never_set = 0;  // no code writes it

__global__ void selftest_wait_kernel(int which, unsigned limit, unsigned* err) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  if (which == 0) {
    // nobody arrives on the barrier: phase 0 never completes
    for (unsigned i = 0; i < limit; ++i)
      if (mbar_try_wait(&bar, 0u)) return;
    atomicOr(err, kDevErrTimeout);
  } else {
    for (unsigned i = 0; i < limit; ++i) {
      unsigned v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(&g_never_set) : "memory");
      if (v != 0u) return;
      __nanosleep(100);
    }
    atomicOr(err, kDevErrBarrier);
  }
}

}  // namespace
}  // namespace pskel

using namespace pskel;

extern "C" {

pskel_status pskel_selftest_bounded_wait(int32_t which, uint32_t polls, void* stream) {
  clear_error();
  if ((which != 0 && which != 1) || polls == 0 || polls > (1u << 20))
    return fail(PSKEL_ERR_INVALID, "selftest: which must be 0 or 1 and polls in 1..2^20");
  DeviceContext* c = nullptr;
  if (pskel_status s = get_context(&c)) return s;
  selftest_wait_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(which, polls, c->err);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PSKEL_OK : cuda_fail(e, "selftest launch");
}

}  // extern "C"
