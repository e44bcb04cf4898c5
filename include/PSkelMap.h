// PSkel drop-in for GB300: the Map skeleton.
//
// Same class templates, constructors and run methods as the reference's
// PSkelMap.h (MapBase / Map / Map2D / Map3D, PSkelMap.h:44-164,
// PSkelMap.hpp:94-528): every element of the output is produced by the
// user's mapKernel functor, found in namespace PSkel as in the reference
// (PSkelMap.h:47-53):
//
//   mapKernel(Array<T> in, Array<T> out, Args args, size_t i)
//   mapKernel(Array2D<T> in, Array2D<T> out, Args args, size_t h, size_t w)
//   mapKernel(Array3D<T> in, Array3D<T> out, Args args, size_t h, size_t w, size_t d)
//
// runIterative* ping-pong between the input and the output like the
// reference (PSkelMap.hpp:185-243): iteration k maps the previous result; the
// host input is left unchanged and the output holds the result. The GPU
// methods generate one grid-stride kernel per functor (compile with nvcc for
// sm_103a); block sizes are hints and are ignored. Like the reference, this
// header is not included by PSkel.h.
#ifndef PSKEL_MAP_H
#define PSKEL_MAP_H

#include "PSkelArray.h"
#include "PSkelDefs.h"

#ifdef PSKEL_OMP
#include <omp.h>
#endif

namespace PSkel {

namespace detail {

#ifdef __CUDACC__
// One thread per element, grid-stride; (h, w, d) from the flat index with d
// fastest, the reference's layout (PSkelArray.hpp:349-352, 658-677). Where
// the input array is dense (flat index i at deviceArray[i]), each thread
// hints the input element of its iteration two ahead into L2: with one cell
// per thread and the user functor's store between loads, a thread otherwise
// has a single load in flight.
template <int Dim, class Arrays, class Args>
__global__ void map_kernel(Arrays in, Arrays out, Args args, size_t W, size_t H, size_t D) {
  const size_t n = W * H * D;
  const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  const bool dense = in.pskel_org_h == 0 && in.pskel_org_w == 0 && in.pskel_org_d == 0 &&
                     (Dim == 1 || in.pskel_pitch_w == static_cast<long>(W)) &&
                     (Dim < 3 || in.pskel_pitch_d == static_cast<long>(D));
  size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  if (dense && i + stride < n) pskel_prefetch_l2(in.deviceArray + i + stride);
  for (; i < n; i += stride) {
    if (dense && i + 2 * stride < n) pskel_prefetch_l2(in.deviceArray + i + 2 * stride);
    if constexpr (Dim == 1) {
      mapKernel(in, out, args, i);
    } else if constexpr (Dim == 2) {
      mapKernel(in, out, args, i / W, i % W);
    } else {
      const size_t d = i % D, hw = i / D;
      mapKernel(in, out, args, hw / W, hw % W, d);
    }
  }
}

template <int Dim, class Arrays, class Args>
void map_launch(Arrays in, Arrays out, Args args, size_t W, size_t H, size_t D) {
  int dev = 0, sms = 1;
  gpuErrchk(cudaGetDevice(&dev));
  gpuErrchk(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const size_t n = W * H * D;
  size_t blocks = (n + 255) / 256;
  if (blocks > static_cast<size_t>(sms) * 8) blocks = static_cast<size_t>(sms) * 8;
  if (blocks == 0) return;
  map_kernel<Dim><<<static_cast<unsigned>(blocks), 256>>>(in, out, args, W, H, D);
  gpuErrchk(cudaPeekAtLastError());
}
#endif

}  // namespace detail

template <class Arrays, class Args = int>
class MapBase {
 protected:
  Arrays input;
  Arrays output;
  Args args;

  virtual void runSeq(Arrays in, Arrays out) = 0;
#ifdef PSKEL_OMP
  virtual void runOpenMP(Arrays in, Arrays out, size_t numThreads) = 0;
#endif
  virtual void runCUDA(Arrays in, Arrays out) = 0;

 public:
  virtual ~MapBase() {}

  void runSequential() { runSeq(input, output); }
#ifdef PSKEL_OMP
  void runCPU(size_t numThreads = 0) { runOpenMP(input, output, numThreads); }
#endif
  void runGPU(size_t blockSize = 0) { runIterativeGPU(1, blockSize); }

  void runIterativeSequential(size_t iterations) {
    Arrays copy;
    copy.hostClone(input);
    for (size_t it = 0; it < iterations; ++it) {
      if (it % 2 == 0)
        runSeq(copy, output);
      else
        runSeq(output, copy);
    }
    if (iterations % 2 == 0) output.hostMemCopy(copy);
    copy.hostFree();
  }

#ifdef PSKEL_OMP
  void runIterativeCPU(size_t iterations, size_t numThreads = 0) {
    Arrays copy;
    copy.hostClone(input);
    for (size_t it = 0; it < iterations; ++it) {
      if (it % 2 == 0)
        runOpenMP(copy, output, numThreads);
      else
        runOpenMP(output, copy, numThreads);
    }
    if (iterations % 2 == 0) output.hostMemCopy(copy);
    copy.hostFree();
  }
#endif

  void runIterativeGPU(size_t iterations, size_t blockSize = 0) {
    (void)blockSize;
    Arrays in = input, out = output;
    in.deviceAlloc();
    out.deviceAlloc();
    in.copyToDevice();
    for (size_t it = 0; it < iterations; ++it) {
      if (it % 2 == 0)
        runCUDA(in, out);
      else
        runCUDA(out, in);
    }
    gpuErrchk(cudaDeviceSynchronize());
    if (iterations % 2 == 1)
      output.copyFromDevice(out);
    else
      output.copyFromDevice(in);
    in.deviceFree();
    out.deviceFree();
  }
};

template <class Arrays, class Args = int>
class Map : public MapBase<Arrays, Args> {
 public:
  Map() {}
  Map(Arrays input, Arrays output, Args args) {
    this->input = input;
    this->output = output;
    this->args = args;
  }

 protected:
  void runSeq(Arrays in, Arrays out) override {
    for (size_t i = 0; i < in.getWidth(); ++i) mapKernel(in, out, this->args, i);
  }
#ifdef PSKEL_OMP
  void runOpenMP(Arrays in, Arrays out, size_t numThreads) override {
    const int nt = numThreads ? static_cast<int>(numThreads) : omp_get_max_threads();
    const long n = static_cast<long>(in.getWidth());
#pragma omp parallel for num_threads(nt)
    for (long i = 0; i < n; ++i) mapKernel(in, out, this->args, static_cast<size_t>(i));
  }
#endif
  void runCUDA(Arrays in, Arrays out) override {
#ifdef __CUDACC__
    detail::map_launch<1>(in, out, this->args, in.getWidth(), 1, 1);
#else
    (void)in;
    (void)out;
#endif
  }
};

template <class Arrays, class Args = int>
class Map2D : public MapBase<Arrays, Args> {
 public:
  Map2D() {}
  Map2D(Arrays input, Arrays output, Args args) {
    this->input = input;
    this->output = output;
    this->args = args;
  }

 protected:
  void runSeq(Arrays in, Arrays out) override {
    for (size_t h = 0; h < in.getHeight(); ++h)
      for (size_t w = 0; w < in.getWidth(); ++w) mapKernel(in, out, this->args, h, w);
  }
#ifdef PSKEL_OMP
  void runOpenMP(Arrays in, Arrays out, size_t numThreads) override {
    const int nt = numThreads ? static_cast<int>(numThreads) : omp_get_max_threads();
    const long H = static_cast<long>(in.getHeight());
#pragma omp parallel for num_threads(nt)
    for (long h = 0; h < H; ++h)
      for (size_t w = 0; w < in.getWidth(); ++w) mapKernel(in, out, this->args, static_cast<size_t>(h), w);
  }
#endif
  void runCUDA(Arrays in, Arrays out) override {
#ifdef __CUDACC__
    detail::map_launch<2>(in, out, this->args, in.getWidth(), in.getHeight(), 1);
#else
    (void)in;
    (void)out;
#endif
  }
};

template <class Arrays, class Args = int>
class Map3D : public MapBase<Arrays, Args> {
 public:
  Map3D() {}
  Map3D(Arrays input, Arrays output, Args args) {
    this->input = input;
    this->output = output;
    this->args = args;
  }

 protected:
  void runSeq(Arrays in, Arrays out) override {
    for (size_t h = 0; h < in.getHeight(); ++h)
      for (size_t w = 0; w < in.getWidth(); ++w)
        for (size_t d = 0; d < in.getDepth(); ++d) mapKernel(in, out, this->args, h, w, d);
  }
#ifdef PSKEL_OMP
  void runOpenMP(Arrays in, Arrays out, size_t numThreads) override {
    const int nt = numThreads ? static_cast<int>(numThreads) : omp_get_max_threads();
    const long H = static_cast<long>(in.getHeight());
#pragma omp parallel for num_threads(nt)
    for (long h = 0; h < H; ++h)
      for (size_t w = 0; w < in.getWidth(); ++w)
        for (size_t d = 0; d < in.getDepth(); ++d) mapKernel(in, out, this->args, static_cast<size_t>(h), w, d);
  }
#endif
  void runCUDA(Arrays in, Arrays out) override {
#ifdef __CUDACC__
    detail::map_launch<3>(in, out, this->args, in.getWidth(), in.getHeight(), in.getDepth());
#else
    (void)in;
    (void)out;
#endif
  }
};

}  // namespace PSkel

#endif  // PSKEL_MAP_H
