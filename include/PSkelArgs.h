// PSkel drop-in for GB300: Args, Args2D, Args3D (extra per-cell data).
//
// Same interface as the reference (PSkelArgs.h:42-126, PSkelArgs.hpp): a
// handle to pinned host memory mapped into the device address space
// (cudaHostAllocWriteCombined | cudaHostAllocMapped) with an x-fastest
// accessor on host and device (PSkelArgs.hpp:108-115, 154-161). Unlike the
// reference's Args(int) (PSkelArgs.hpp:53) the constructor does not call
// cudaDeviceReset(), which would destroy every other allocation of the
// process; with unified virtual addressing the mapping needs no device flag.
#ifndef PSKEL_ARGS_H
#define PSKEL_ARGS_H

#include <cuda_runtime.h>

#include "PSkelDefs.h"

namespace PSkel {

namespace detail {
template <typename T>
inline void mapped_alloc(T** host, T** dev, size_t n) {
  gpuErrchk(cudaHostAlloc(reinterpret_cast<void**>(host), (n ? n : 1) * sizeof(T),
                          cudaHostAllocWriteCombined | cudaHostAllocMapped));
  gpuErrchk(cudaHostGetDevicePointer(reinterpret_cast<void**>(dev), *host, 0));
}
}  // namespace detail

template <typename T>
class Args {
 public:
  T* hostArray = nullptr;
  T* deviceArray = nullptr;
  int width = 0;
  Args() {}
  explicit Args(int w) : width(w) { detail::mapped_alloc(&hostArray, &deviceArray, static_cast<size_t>(w)); }
  __host__ __device__ int getWidth() const { return width; }
  __host__ __device__ __forceinline__ T& operator()(int x) const {
#ifdef __CUDA_ARCH__
    return deviceArray[x];
#else
    return hostArray[x];
#endif
  }
};

template <typename T>
class Args2D {
 public:
  T* hostArray = nullptr;
  T* deviceArray = nullptr;
  int width = 0, height = 0;
  Args2D() {}
  Args2D(int w, int h) : width(w), height(h) {
    detail::mapped_alloc(&hostArray, &deviceArray, static_cast<size_t>(w) * h);
  }
  __host__ __device__ int getWidth() const { return width; }
  __host__ __device__ int getHeight() const { return height; }
  __host__ __device__ __forceinline__ T& operator()(int x, int y) const {
#ifdef __CUDA_ARCH__
    return deviceArray[y * width + x];
#else
    return hostArray[y * width + x];
#endif
  }
};

template <typename T>
class Args3D {
 public:
  T* hostArray = nullptr;
  T* deviceArray = nullptr;
  int width = 0, height = 0, depth = 0;
  Args3D() {}
  Args3D(int w, int h, int d) : width(w), height(h), depth(d) {
    detail::mapped_alloc(&hostArray, &deviceArray, static_cast<size_t>(w) * h * d);
  }
  __host__ __device__ int getWidth() const { return width; }
  __host__ __device__ int getHeight() const { return height; }
  __host__ __device__ int getDepth() const { return depth; }
  __host__ __device__ __forceinline__ T& operator()(int x, int y, int z) const {
#ifdef __CUDA_ARCH__
    return deviceArray[(z * height + y) * width + x];
#else
    return hostArray[(z * height + y) * width + x];
#endif
  }
};

}  // namespace PSkel

#endif  // PSKEL_ARGS_H
