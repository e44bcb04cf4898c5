// A self-test of the bounded waits every kernel of the library relies on: a
// kernel waits on an mbarrier phase that never completes, or on a device flag
// that nothing sets, with a short poll limit; or the persistent Life kernel
// itself is launched at pass 1 of a run whose pass 0 never ran, so the
// dependency wait of its first item runs out (likewise the multi-pass 2D
// kernel with its first pass skipped). The wait gives up, records the
// timeout in the device error word and returns (the Life kernel's other blocks
// see the latched word and stop), so the host reads PSKEL_ERR_DEVICE from
// pskel_sync and the context stays usable. Nothing faults, traps or hangs.
#include <algorithm>
#include <cstring>

#include "../../include/pskel_gb300.h"
#include "capi_internal.h"

#include "common.cuh"
#include "kernels.h"

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
  if (which < 0 || which > 3 || polls == 0 || polls > (1u << 20))
    return fail(PSKEL_ERR_INVALID, "selftest: which must be 0..3 and polls in 1..2^20");
  DeviceContext* c = nullptr;
  if (pskel_status s = get_context(&c)) return s;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (which < 2) {
    selftest_wait_kernel<<<1, 32, 0, s>>>(which, polls, c->err);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PSKEL_OK : cuda_fail(e, "selftest launch");
  }
  if (which == 3) {
    // the persistent multi-pass 2D kernel: Jacobi fp32 on a 256 x 256 grid of
    // zeros, two passes of 11 steps in one launch, items handed out from pass
    // 1 on: every item waits for pass 0, which never runs
    const int64_t n = 256;
    if (pskel_status q = ensure_buffer(c->selftest, 2 * n * n * sizeof(float))) return q;
    float* A = static_cast<float*>(c->selftest.ptr);
    const cudaError_t e = cudaMemsetAsync(A, 0, 2 * n * n * sizeof(float), s);
    if (e != cudaSuccess) return cuda_fail(e, "selftest set-up");
    static const int32_t offsets[8] = {-1, 0, 1, 0, 0, -1, 0, 1};
    static const float weights[4] = {0.25f, 0.25f, 0.25f, 0.25f};
    pskel_stencil st;
    memset(&st, 0, sizeof(st));
    st.op = PSKEL_OP_LINEAR;
    st.dtype = PSKEL_F32;
    st.mask.size = 4;
    st.mask.dimension = 2;
    st.mask.offsets = offsets;
    st.mask.weights = weights;
    pskel_schedule sch;
    memset(&sch, 0, sizeof(sch));
    sch.time_steps = 11;
    dep_wait_test() = DepWaitTest{polls, 1};
    const pskel_status q = pskel_iterate2d(&st, A, A + n * n, n, n, n, 22, &sch, stream);
    dep_wait_test() = DepWaitTest{0u, 0};
    return q;
  }
  // the Life kernel on a 512 x 512 grid of zeros, launched for pass 1 only with
  // cleared completion counts: every item waits for pass 0, which never ran
  const int W = 512, H = 512, T = 3;
  const int TH = life_bits_max_tile_h(T);
  const size_t plane = static_cast<size_t>(life_bits_words(W)) * H;
  if (pskel_status q = ensure_buffer(c->life_bits, 2 * plane * sizeof(uint32_t))) return q;
  if (pskel_status q = ensure_buffer(c->life_sync, life_bits_sync_bytes(W, H, TH))) return q;
  uint32_t* X = static_cast<uint32_t*>(c->life_bits.ptr);
  cudaError_t e = cudaMemsetAsync(X, 0, 2 * plane * sizeof(uint32_t), s);
  if (e == cudaSuccess) e = life_bits_clear_sync(c->life_sync.ptr, W, H, TH, s);
  if (e != cudaSuccess) return cuda_fail(e, "selftest set-up");
  LifeWindow win;
  memset(&win, 0, sizeof(win));
  win.pass0 = 1;
  win.np = 1;
  const int ctas = static_cast<int>(std::min<int64_t>(life_bits_tiles(W, H, TH),
                                                      static_cast<int64_t>(life_bits_persistent_ctas_per_sm(T)) * c->sms));
  e = life_bits_run_window(X, X + plane, W, H, 1, win, 1, 0, T, TH, ctas, c->life_sync.ptr, c->err, s, true, polls);
  return e == cudaSuccess ? PSKEL_OK : cuda_fail(e, "selftest launch");
}

}  // extern "C"
