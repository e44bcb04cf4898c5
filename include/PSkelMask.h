// PSkel drop-in for GB300: Mask, Mask2D, Mask3D.
//
// Same interface as the reference (PSkelMask.h:48-262, PSkelMask.hpp): integer
// offsets hostMask[dimension * n + k] plus weights hostWeight[n], a halo value
// and a range; set/get/getWeight/getRange on host and device.
//  - Mask2D::get(n, a, h, w) returns a(h + dh, w + dw) with no bounds check
//    (PSkelMask.hpp:292-305);
//  - Mask3D::get returns the halo value for neighbours outside the array
//    (PSkelMask.hpp:186-199);
//  - getRange() is max |offset| unless a range was given (PSkelMask.hpp:201-229,
//    307-334).
#ifndef PSKEL_MASK_H
#define PSKEL_MASK_H

#include <cuda_runtime.h>

#include <cstdlib>

#include "PSkelArray.h"
#include "PSkelDefs.h"

namespace PSkel {

template <typename T>
class MaskBase {
 public:
  int* hostMask;
  int* deviceMask;
  T* hostWeight;
  T* deviceWeight;
  T haloValue;
  size_t size, dimension;
  size_t range;

 protected:
  MaskBase(size_t sz = 0, size_t dim = 0, T halo = T(0), size_t rng = 0)
      : hostMask(nullptr), deviceMask(nullptr), hostWeight(nullptr), deviceWeight(nullptr), haloValue(halo),
        size(sz), dimension(dim), range(rng) {
    if (sz > 0) hostAlloc();
  }

 public:
  void hostAlloc() {
    if (hostMask == nullptr && hostWeight == nullptr) {
      hostMask = static_cast<int*>(std::calloc(dimension * size, sizeof(int)));
      hostWeight = static_cast<T*>(std::calloc(size, sizeof(T)));
    }
  }
  void hostFree() {
    std::free(hostMask);
    std::free(hostWeight);
    hostMask = nullptr;
    hostWeight = nullptr;
  }
  void deviceAlloc() {
    if (deviceMask == nullptr) gpuErrchk(cudaMalloc(reinterpret_cast<void**>(&deviceMask), dimension * size * sizeof(int)));
    if (deviceWeight == nullptr) gpuErrchk(cudaMalloc(reinterpret_cast<void**>(&deviceWeight), size * sizeof(T)));
  }
  void copyToDevice() {
    gpuErrchk(cudaMemcpy(deviceMask, hostMask, dimension * size * sizeof(int), cudaMemcpyHostToDevice));
    gpuErrchk(cudaMemcpy(deviceWeight, hostWeight, size * sizeof(T), cudaMemcpyHostToDevice));
  }
  void deviceFree() {
    cudaFree(deviceMask);
    cudaFree(deviceWeight);
    deviceMask = nullptr;
    deviceWeight = nullptr;
  }
  size_t memSize() const { return dimension * size * sizeof(int) + size * sizeof(T); }

  __host__ __device__ __forceinline__ T& getWeight(size_t n) const {
#ifdef __CUDA_ARCH__
    return deviceWeight[n];
#else
    return hostWeight[n];
#endif
  }

  __host__ __device__ __forceinline__ const int* offsets() const {
#ifdef __CUDA_ARCH__
    return deviceMask;
#else
    return hostMask;
#endif
  }

  // max over entries of max |offset| (the reference's getRange without the
  // explicit range)
  __host__ __device__ size_t maxOffset() const {
    const int* p = offsets();
    size_t r = 0;
    for (size_t i = 0; i < size * dimension; ++i) {
      const size_t a = static_cast<size_t>(p[i] < 0 ? -p[i] : p[i]);
      if (a > r) r = a;
    }
    return r;
  }

  __host__ __device__ size_t getRange() {
    if (range > 0) return range;
    range = maxOffset();
    return range;
  }
};

template <typename T>
class Mask3D : public MaskBase<T> {
 public:
  Mask3D(size_t size = 0, T haloVal = T(0), size_t range = 0) : MaskBase<T>(size, 3, haloVal, range) {}
  __host__ __device__ void set(size_t n, int h, int w, int d, T weight = T(0)) {
#ifdef __CUDA_ARCH__
    int* m = this->deviceMask;
    T* wt = this->deviceWeight;
#else
    int* m = this->hostMask;
    T* wt = this->hostWeight;
#endif
    m[3 * n] = h;
    m[3 * n + 1] = w;
    m[3 * n + 2] = d;
    wt[n] = weight;
  }
  template <typename V>
  __host__ __device__ __forceinline__ T get(size_t n, const Array3D<V>& array, size_t h, size_t w, size_t d) const {
    const int* m = this->offsets();
    h += m[3 * n];
    w += m[3 * n + 1];
    d += m[3 * n + 2];
    return (w < array.getWidth() && h < array.getHeight() && d < array.getDepth()) ? T(array(h, w, d))
                                                                                    : this->haloValue;
  }
};

template <typename T>
class Mask2D : public MaskBase<T> {
 public:
  Mask2D(size_t size = 0, T haloVal = T(0), size_t range = 0) : MaskBase<T>(size, 2, haloVal, range) {}
  Mask2D(size_t size, int array[][2]) : MaskBase<T>(size, 2, T(0), 0) {
    for (size_t i = 0; i < size; ++i) set(i, array[i][0], array[i][1], T(1));
  }
  __host__ __device__ void set(size_t n, int h, int w, T weight = T(0)) {
#ifdef __CUDA_ARCH__
    int* m = this->deviceMask;
    T* wt = this->deviceWeight;
#else
    int* m = this->hostMask;
    T* wt = this->hostWeight;
#endif
    m[2 * n] = h;
    m[2 * n + 1] = w;
    wt[n] = weight;
  }
  template <typename V>
  __host__ __device__ __forceinline__ V& get(size_t n, const Array2D<V>& array, size_t h, size_t w) const {
    const int* m = this->offsets();
    return array(h + m[2 * n], w + m[2 * n + 1]);
  }
};

template <typename T>
class Mask : public MaskBase<T> {
 public:
  Mask(size_t size = 0, T haloVal = T(0), size_t range = 0) : MaskBase<T>(size, 1, haloVal, range) {}
  __host__ __device__ void set(size_t n, int i, T weight = T(0)) {
#ifdef __CUDA_ARCH__
    this->deviceMask[n] = i;
    this->deviceWeight[n] = weight;
#else
    this->hostMask[n] = i;
    this->hostWeight[n] = weight;
#endif
  }
  template <typename V>
  __host__ __device__ __forceinline__ T get(size_t n, const Array<V>& array, size_t i) const {
    i += this->offsets()[n];
    return (i < array.getWidth()) ? T(array(i)) : this->haloValue;
  }
};

}  // namespace PSkel

#endif  // PSKEL_MASK_H
