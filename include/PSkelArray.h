// PSkel drop-in for GB300: Array, Array2D, Array3D.
//
// Same interface as the reference (PSkelArray.h:53-384, PSkelArray.hpp):
// shallow value handles with public hostArray / deviceArray, real and virtual
// dimensions for slices, (h, w[, d]) access on host and device, explicit
// allocation and copies. Layouts: 2D [h][w], 3D [h][w][d] with d fastest
// (PSkelArray.hpp:349-352, 658-677).
//
// Device access goes through a view mapping (pskel_org_*, pskel_pitch_*):
// element (h, w, d) is deviceArray[((h - org_h) * pitch_w + (w - org_w)) *
// pitch_d + (d - org_d)]. For a plain device array the origin is 0 and the
// pitches are the dimensions; the tiled stencil kernels point deviceArray at
// a shared-memory tile and set the origin to the tile's corner, so a user
// functor's in(h, w) reads the tile without any change to user code.
#ifndef PSKEL_ARRAY_H
#define PSKEL_ARRAY_H

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "PSkelDefs.h"

namespace PSkel {

template <typename T>
class ArrayBase {
 public:
  typedef T value_type;
  T* deviceArray;
  T* hostArray;
  // view mapping used by device code (see the file comment)
  long pskel_org_h, pskel_org_w, pskel_org_d;
  long pskel_pitch_w, pskel_pitch_d;

 protected:
  size_t realWidth, realHeight, realDepth;
  size_t widthOffset, heightOffset, depthOffset;
  size_t width, height, depth;

  ArrayBase(size_t w, size_t h, size_t d) { init(w, h, d, true); }

  void init(size_t w, size_t h, size_t d, bool alloc) {
    width = realWidth = w;
    height = realHeight = h;
    depth = realDepth = d;
    widthOffset = heightOffset = depthOffset = 0;
    hostArray = nullptr;
    deviceArray = nullptr;
    reset_view();
    if (alloc && size() > 0) hostAlloc();
  }

 public:
  __host__ __device__ void reset_view() {
    pskel_org_h = pskel_org_w = pskel_org_d = 0;
    pskel_pitch_w = static_cast<long>(width);
    pskel_pitch_d = static_cast<long>(depth);
  }

  void deviceAlloc() {
    if (deviceArray == nullptr) gpuErrchk(cudaMalloc(reinterpret_cast<void**>(&deviceArray), size() * sizeof(T)));
    reset_view();
  }
  void deviceFree() {
    if (deviceArray != nullptr) {
      cudaFree(deviceArray);
      deviceArray = nullptr;
    }
  }
  void hostAlloc(size_t w, size_t h, size_t d) {
    init(w, h, d, false);
    hostAlloc();
  }
  void hostAlloc() {
    if (hostArray == nullptr) {
      void* p = nullptr;
      const size_t bytes = size() * sizeof(T);
      if (posix_memalign(&p, 64, bytes ? bytes : 64) != 0) p = nullptr;
      hostArray = static_cast<T*>(p);
    }
  }
  void hostFree() {
    if (hostArray != nullptr) {
      std::free(hostArray);
      hostArray = nullptr;
    }
  }

  __host__ __device__ size_t getWidth() const { return width; }
  __host__ __device__ size_t getHeight() const { return height; }
  __host__ __device__ size_t getDepth() const { return depth; }
  __host__ __device__ size_t getRealHeight() const { return realHeight; }
  __host__ __device__ size_t getWidthOffset() const { return widthOffset; }
  __host__ __device__ size_t getHeightOffset() const { return heightOffset; }
  __host__ __device__ size_t getDepthOffset() const { return depthOffset; }
  __host__ __device__ size_t memSize() const { return size() * sizeof(T); }
  __host__ __device__ size_t size() const { return height * width * depth; }
  __host__ __device__ size_t typeSize() const { return sizeof(T); }
  __host__ __device__ size_t realSize() const { return realHeight * realWidth * realDepth; }
  __host__ __device__ bool contiguous() const { return size() == realSize(); }

  T& hostGet(size_t h, size_t w, size_t d) const {
    return hostArray[((h + heightOffset) * realWidth + (w + widthOffset)) * realDepth + (d + depthOffset)];
  }

  // A view of a sub-block of `array` (shares its host memory).
  template <typename Arrays>
  void hostSlice(Arrays array, size_t wOff, size_t hOff, size_t dOff, size_t w, size_t h, size_t d) {
    if (deviceArray != nullptr && size() != w * h * d) deviceFree();
    width = w;
    height = h;
    depth = d;
    widthOffset = array.getWidthOffset() + wOff;
    heightOffset = array.getHeightOffset() + hOff;
    depthOffset = array.getDepthOffset() + dOff;
    realWidth = array.realWidth;
    realHeight = array.realHeight;
    realDepth = array.realDepth;
    hostArray = array.hostArray;
    reset_view();
  }

  // A new host array with a copy of `array`'s elements.
  template <typename Arrays>
  void hostClone(Arrays array) {
    init(array.getWidth(), array.getHeight(), array.getDepth(), false);
    hostAlloc();
    hostMemCopy(array);
  }

  // Element-wise copy of `array` (same virtual dimensions) into this array.
  template <typename Arrays>
  void hostMemCopy(Arrays array) {
    if (array.contiguous() && contiguous()) {
      std::memcpy(hostArray, array.hostArray, size() * sizeof(T));
      return;
    }
    for (size_t i = 0; i < height; ++i)
      for (size_t j = 0; j < width; ++j)
        for (size_t k = 0; k < depth; ++k) hostGet(i, j, k) = array.hostGet(i, j, k);
  }

  // Host -> device copy of the (possibly sliced) array into deviceArray.
  void copyToDevice() {
    if (contiguous()) {
      gpuErrchk(cudaMemcpy(deviceArray, hostArray, size() * sizeof(T), cudaMemcpyHostToDevice));
      return;
    }
    T* tmp = static_cast<T*>(std::malloc(size() * sizeof(T)));
    for (size_t h = 0; h < height; ++h)
      for (size_t w = 0; w < width; ++w)
        for (size_t d = 0; d < depth; ++d) tmp[(h * width + w) * depth + d] = hostGet(h, w, d);
    gpuErrchk(cudaMemcpy(deviceArray, tmp, size() * sizeof(T), cudaMemcpyHostToDevice));
    std::free(tmp);
  }

  // Device -> host copy of this array's deviceArray.
  void copyToHost() { copyFromDevice(*this); }

  // Device -> host copy of `array`'s deviceArray into this array's host memory.
  template <typename Arrays>
  void copyFromDevice(Arrays array) {
    if (contiguous()) {
      gpuErrchk(cudaMemcpy(hostArray, array.deviceArray, size() * sizeof(T), cudaMemcpyDeviceToHost));
      return;
    }
    T* tmp = static_cast<T*>(std::malloc(size() * sizeof(T)));
    gpuErrchk(cudaMemcpy(tmp, array.deviceArray, size() * sizeof(T), cudaMemcpyDeviceToHost));
    for (size_t h = 0; h < height; ++h)
      for (size_t w = 0; w < width; ++w)
        for (size_t d = 0; d < depth; ++d) hostGet(h, w, d) = tmp[(h * width + w) * depth + d];
    std::free(tmp);
  }

  __host__ __device__ operator bool() const {
#ifdef __CUDA_ARCH__
    return deviceArray != nullptr;
#else
    return hostArray != nullptr;
#endif
  }

  template <typename U>
  friend class ArrayBase;
};

template <typename T>
class Array3D : public ArrayBase<T> {
 public:
  Array3D() : ArrayBase<T>(0, 0, 0) {}
  Array3D(size_t width, size_t height, size_t depth) : ArrayBase<T>(width, height, depth) {}
  __host__ __device__ __forceinline__ T& operator()(size_t h, size_t w, size_t d) const {
#ifdef __CUDA_ARCH__
    return this->deviceArray[((static_cast<long>(h) - this->pskel_org_h) * this->pskel_pitch_w +
                              (static_cast<long>(w) - this->pskel_org_w)) *
                                 this->pskel_pitch_d +
                             (static_cast<long>(d) - this->pskel_org_d)];
#else
    return this->hostGet(h, w, d);
#endif
  }
};

template <typename T>
class Array2D : public ArrayBase<T> {
 public:
  Array2D() : ArrayBase<T>(0, 0, 0) {}
  Array2D(size_t width, size_t height) : ArrayBase<T>(width, height, 1) {}
  __host__ __device__ __forceinline__ T& operator()(size_t h, size_t w) const {
#ifdef __CUDA_ARCH__
    return this->deviceArray[(static_cast<long>(h) - this->pskel_org_h) * this->pskel_pitch_w +
                             (static_cast<long>(w) - this->pskel_org_w)];
#else
    return this->hostGet(h, w, 0);
#endif
  }
};

template <typename T>
class Array : public ArrayBase<T> {
 public:
  Array() : ArrayBase<T>(0, 0, 0) {}
  explicit Array(size_t size) : ArrayBase<T>(size, 1, 1) {}
  __host__ __device__ __forceinline__ T& operator()(size_t w) const {
#ifdef __CUDA_ARCH__
    return this->deviceArray[static_cast<long>(w) - this->pskel_org_w];
#else
    return this->hostGet(0, w, 0);
#endif
  }
};

}  // namespace PSkel

#endif  // PSKEL_ARRAY_H
