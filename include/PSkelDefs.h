// PSkel drop-in for GB300: configuration macros and error handling.
//
// Mirrors the reference's PSkelDefs.h (PSkelDefs.h:36-70): MIN, __parallel__
// (host + device, always inline) and gpuErrchk (print "GPUassert" and exit
// with the error code, PSkelDefs.h:50-56). Library status codes are reported
// the same way.
#ifndef PSKEL_DEFS_H
#define PSKEL_DEFS_H

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>

#include "pskel_gb300.h"

#ifndef MIN
#define MIN(a, b) ((a) <= (b) ? (a) : (b))
#endif

#ifdef __CUDACC__
#define __parallel__ __host__ __device__ __forceinline__
#else
#define __parallel__ inline
#endif

namespace PSkel {

inline void gpuAssert(cudaError_t code, const char* file, int line, bool abort = false) {
  if (code != cudaSuccess) {
    std::fprintf(stderr, "GPUassert: %s %s %d\n", cudaGetErrorString(code), file, line);
    if (abort) std::exit(code);
  }
}

inline void pskelAssert(pskel_status code, const char* file, int line) {
  if (code != PSKEL_OK) {
    std::fprintf(stderr, "GPUassert: %s %s %d\n", pskel_last_error(), file, line);
    std::exit(code);
  }
}

#ifdef __CUDACC__
// An L2 prefetch hint for an address that a grid-stride kernel will read a
// few iterations later (generic address; a hint only: no value changes).
__device__ __forceinline__ void pskel_prefetch_l2(const void* p) { asm volatile("prefetch.L2 [%0];" ::"l"(p)); }
#endif

}  // namespace PSkel

#define gpuErrchk(ans) \
  { PSkel::gpuAssert(static_cast<cudaError_t>(ans), __FILE__, __LINE__, true); }
#define pskelErrchk(ans) \
  { PSkel::pskelAssert((ans), __FILE__, __LINE__); }

#endif  // PSKEL_DEFS_H
