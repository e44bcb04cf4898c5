// PSkel drop-in for GB300: the stencil skeleton (Stencil2D, Stencil3D).
//
// Same class templates and run methods as the reference (PSkelStencil.h:165-407,
// bodies PSkelStencil.hpp:708-2362):
//   Stencil2D<Array, Mask, Args> / Stencil3D<...>(input, output, mask, args)
//   runIterativeGPU(iterations, GPUBlockSizeX, GPUBlockSizeY)
//   runIterativeGPU(iterations, pyramidHeight, GPUBlockSizeX, GPUBlockSizeY)
//   runIterativeTilingGPU(iterations, tilingWidth, tilingHeight, tilingDepth,
//                         innerIterations = 1, GPUBlockSizeX = 0, GPUBlockSizeY = 0)
//   runIterativeAutoGPU(iterations, GPUBlockSize = 0)
//   runGPU(...), runTilingGPU(...), runAutoGPU(...)  (one iteration)
//   runIterativeCPU(iterations, numThreads), runCPU, runSequential,
//   runIterativeSequential  (host, only with -DPSKEL_OMP, like the reference)
//
// Results follow runIterativeCPU (PSkelStencil.hpp:880-938): after the run the
// host `output` array holds the final state; in 2D each array keeps its own
// ring (cells outside r <= h < H-r, r <= w < W-r, r = mask range), in 3D every
// cell is updated and out-of-grid neighbours read the mask halo value. The
// host `input` array is left unchanged by the GPU methods, as the reference's
// runIterativeGPU leaves it (it copies to the device and back from it).
//
// The block sizes are hints and are ignored; the schedule parameters mean:
//   pyramidHeight, innerIterations -> time steps fused per pass over the grid
//   tilingWidth/Height/Depth       -> on-chip core tile sizes
//   runIterativeAutoGPU            -> the library's tuned schedule
//
// Execution. The functor is the user's `stencilKernel` overload, found by
// argument-dependent lookup in namespace PSkel as in the reference
// (PSkelStencil.h:139-156). Two paths:
//  * Library kernels (precompiled sm_103a code in libpskel_gb300.so). An Args
//    type declares that its functor is one of the library's stencils by
//    deriving from (or being) one of the tags below, or by specialising
//    PSkel::StencilOp:
//      LinearStencil      out = sum_n weight_n * in(neighbour n), mask order
//      LifeStencil        Game of Life on the 8-neighbour mask (uint8 cells)
//      AdvectionArgs<T>   upwind advection-diffusion with per-cell winds
//    The functor itself is then not called on the GPU.
//  * Any other functor runs in a kernel generated in the user's translation
//    unit (compile it with nvcc): 2D grids are processed in shared-memory tiles
//    with the same temporal blocking as the library, the functor reading and
//    writing the tile through the Array2D views it is given; 3D grids run one
//    step per launch. The functor must read `input` only within the mask
//    range of the cell it updates.
#ifndef PSKEL_STENCIL_H
#define PSKEL_STENCIL_H

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#if defined(__CUDACC__) || __has_include(<cuda_bf16.h>)
#include <cuda_bf16.h>
#define PSKEL_HAVE_BF16 1
#endif

#include "PSkelArray.h"
#include "PSkelDefs.h"
#include "PSkelMask.h"
#include "PSkelStencilTiling.h"
#include "pskel_gb300.h"

namespace PSkel {

// ------------------------------------------------------------------ tags

// The functor computes out(h,w[,d]) = sum over mask entries of
// weight * neighbour, in mask order, without contraction.
struct LinearStencil {};
// The functor is the Game of Life rule on the Moore mask over 0/1 uint8 cells.
struct LifeStencil {};
// Upwind advection-diffusion (the reference's CLOUDSIM arithmetic,
// PSkelStencil.hpp:347-387) with per-cell winds wind_x(h,w), wind_y(h,w) and
// diffusivity K, time step dt, 1/dx.
template <typename T>
struct AdvectionArgs {
  Array2D<T> wind_x, wind_y;
  float K = 0.1f, dt = 0.2f, inv_dx = 10.0f;
};

enum StencilKind { kUserFunctor = -1, kLinear = PSKEL_OP_LINEAR, kLife = PSKEL_OP_LIFE, kAdvect = PSKEL_OP_ADVECT };

template <class Args, class Enable = void>
struct StencilOp {
  static constexpr int value = std::is_base_of<LinearStencil, Args>::value ? kLinear
                               : std::is_base_of<LifeStencil, Args>::value ? kLife
                                                                           : kUserFunctor;
};
template <typename T>
struct StencilOp<AdvectionArgs<T>> {
  static constexpr int value = kAdvect;
};

namespace detail {

template <typename T>
struct LibDtype {
  static constexpr int value = -1;
};
template <>
struct LibDtype<float> {
  static constexpr int value = PSKEL_F32;
};
template <>
struct LibDtype<uint8_t> {
  static constexpr int value = PSKEL_U8;
};
#ifdef PSKEL_HAVE_BF16
template <>
struct LibDtype<__nv_bfloat16> {
  static constexpr int value = PSKEL_BF16;
};
#endif

template <typename T>
inline float to_float(const T& v) {
  return static_cast<float>(v);
}
#ifdef PSKEL_HAVE_BF16
template <>
inline float to_float<__nv_bfloat16>(const __nv_bfloat16& v) {
  return __bfloat162float(v);
}
#endif

// A contiguous host copy of a (possibly sliced) array, or the array itself.
template <class Array>
struct Contig {
  typedef typename Array::value_type T;
  Array& a;
  std::vector<T> tmp;
  explicit Contig(Array& arr) : a(arr) {
    if (!a.contiguous()) {
      tmp.resize(a.size());
      for (size_t h = 0; h < a.getHeight(); ++h)
        for (size_t w = 0; w < a.getWidth(); ++w)
          for (size_t d = 0; d < a.getDepth(); ++d) tmp[(h * a.getWidth() + w) * a.getDepth() + d] = a.hostGet(h, w, d);
    }
  }
  T* data() { return a.contiguous() ? a.hostArray : tmp.data(); }
  void write_back() {
    if (a.contiguous()) return;
    for (size_t h = 0; h < a.getHeight(); ++h)
      for (size_t w = 0; w < a.getWidth(); ++w)
        for (size_t d = 0; d < a.getDepth(); ++d) a.hostGet(h, w, d) = tmp[(h * a.getWidth() + w) * a.getDepth() + d];
  }
};

template <class Mask>
pskel_mask describe_mask(Mask& m, std::vector<int32_t>& off, std::vector<float>& wt) {
  off.assign(m.hostMask, m.hostMask + m.size * m.dimension);
  wt.resize(m.size);
  for (size_t n = 0; n < m.size; ++n) wt[n] = to_float(m.hostWeight[n]);
  pskel_mask d;
  d.size = static_cast<int32_t>(m.size);
  d.dimension = static_cast<int32_t>(m.dimension);
  d.offsets = off.data();
  d.weights = wt.data();
  d.halo_value = to_float(m.haloValue);
  d.range = static_cast<int32_t>(m.range);
  return d;
}

inline pskel_schedule make_schedule(size_t tw, size_t th, size_t td, size_t steps) {
  pskel_schedule s;
  s.tile_w = static_cast<int32_t>(tw);
  s.tile_h = static_cast<int32_t>(th);
  s.tile_d = static_cast<int32_t>(td);
  s.time_steps = static_cast<int32_t>(steps);
  s.ctas = 0;
  return s;
}

// Device memory a run may use: the free memory, capped by the environment
// variable PSKEL_DEVICE_BYTES when it is set (to run out of core on purpose).
inline size_t device_budget() {
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    cudaGetLastError();
    fr = 0;
  }
  if (const char* e = std::getenv("PSKEL_DEVICE_BYTES")) {
    const unsigned long long cap = std::strtoull(e, nullptr, 10);
    if (cap > 0 && (fr == 0 || cap < fr)) fr = static_cast<size_t>(cap);
  }
  return fr;
}

// Rows [lo, hi) of a host array (whole rows; whole h-planes in 3D), copied to
// or from the device memory `dev`. A sliced array goes through its own
// element-wise copy. Used by the out-of-core runs of user functors.
template <class Array>
void rows_to_device(const Array& a, size_t lo, size_t hi, typename Array::value_type* dev) {
  typedef typename Array::value_type V;
  const size_t row = a.getWidth() * a.getDepth();
  if (a.contiguous()) {
    gpuErrchk(cudaMemcpy(dev, a.hostArray + lo * row, (hi - lo) * row * sizeof(V), cudaMemcpyHostToDevice));
    return;
  }
  Array s = a;
  s.deviceArray = nullptr;  // never free the parent's device memory
  s.hostSlice(a, 0, lo, 0, a.getWidth(), hi - lo, a.getDepth());
  s.deviceArray = dev;
  s.copyToDevice();
}

template <class Array>
void rows_to_host(Array& a, size_t lo, size_t hi, const typename Array::value_type* dev) {
  typedef typename Array::value_type V;
  const size_t row = a.getWidth() * a.getDepth();
  if (a.contiguous()) {
    gpuErrchk(cudaMemcpy(a.hostArray + lo * row, dev, (hi - lo) * row * sizeof(V), cudaMemcpyDeviceToHost));
    return;
  }
  Array s = a;
  s.deviceArray = nullptr;
  s.hostSlice(a, 0, lo, 0, a.getWidth(), hi - lo, a.getDepth());
  Array src = s;
  src.deviceArray = const_cast<V*>(dev);
  s.copyFromDevice(src);
}

// Core rows of an out-of-core slab: the tiling height when given, else
// the most that fit `budget` bytes as `buffers` device buffers of the slab
// and its halo (90 % of the budget), at least one and at most `extent`.
inline size_t slab_rows(size_t given, size_t budget, size_t row_bytes, size_t buffers, size_t halo_rows,
                        size_t extent) {
  size_t s = given;
  if (s == 0) {
    const size_t fit = budget > 0 ? (budget / 10 * 9) / (buffers * row_bytes) : extent;
    s = fit > 2 * halo_rows ? fit - 2 * halo_rows : 1;
  }
  if (s < 1) s = 1;
  if (s > extent) s = extent;
  return s;
}

#ifdef __CUDACC__
// ------------------------------------------------ user-functor GPU kernels

// One pass of `steps` steps of a user functor on 2D shared-memory tiles.
// Same scheme as the library kernels: a (TW + 2RT) x (TH + 2RT) tile, a
// shrinking computed region per step, tiles that reach the ring also stage
// the destination's ring, the core written back for interior cells only.
// The buffers hold H rows of the grid starting at grid row `row0` (0 for a
// whole grid; a slab of an out-of-core run otherwise): the functor sees grid
// coordinates, and the buffers' first and last `ring` rows are not updated
// (the grid's ring, or a slab edge whose rows the caller does not keep).
template <class Array, class Mask, class Args>
__global__ void __launch_bounds__(256) functor2d_pass(Array in, Array out, Mask mask, Args args, int W, int H,
                                                      int ring, int R, int steps, int T, int TW, int TH,
                                                      int tiles_x, int tiles_y, int row0) {
  typedef typename Array::value_type V;
  typedef typename std::remove_reference<decltype(mask.getWeight(0))>::type WT;
  extern __shared__ __align__(16) unsigned char pskel_smem[];
  const int HX = R * T, HY = R * T;
  const int LW = TW + 2 * HX, LH = TH + 2 * HY;
  const size_t tile_bytes = (static_cast<size_t>(LW) * LH * sizeof(V) + 15) & ~size_t(15);
  V* A = reinterpret_cast<V*>(pskel_smem);
  V* B = reinterpret_cast<V*>(pskel_smem + tile_bytes);
  int* s_off = reinterpret_cast<int*>(pskel_smem + 2 * tile_bytes);
  WT* s_wt = reinterpret_cast<WT*>(s_off + ((mask.size * mask.dimension + 3) & ~size_t(3)));
  for (size_t i = threadIdx.x; i < mask.size * mask.dimension; i += blockDim.x) s_off[i] = mask.deviceMask[i];
  for (size_t i = threadIdx.x; i < mask.size; i += blockDim.x) s_wt[i] = mask.deviceWeight[i];
  __syncthreads();
  mask.deviceMask = s_off;
  mask.deviceWeight = s_wt;
  const V* gsrc = in.deviceArray;
  V* gdst = out.deviceArray;
  const int ntiles = tiles_x * tiles_y;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
    const int gy0 = ty * TH - HY, gx0 = tx * TW - HX;
    const bool touches_ring = (gy0 < ring) || (gy0 + LH > H - ring) || (gx0 < ring) || (gx0 + LW > W - ring);
    for (int i = threadIdx.x; i < LW * LH; i += blockDim.x) {
      const int y = i / LW, x = i - y * LW;
      const int gy = gy0 + y, gx = gx0 + x;
      const bool inside = gy >= 0 && gy < H && gx >= 0 && gx < W;
      A[i] = inside ? gsrc[static_cast<long>(gy) * W + gx] : V();
      if (touches_ring && steps >= 2) B[i] = inside ? gdst[static_cast<long>(gy) * W + gx] : V();
    }
    __syncthreads();
    Array va = in, vb = out;
    va.deviceArray = A;
    vb.deviceArray = B;
    va.pskel_org_h = vb.pskel_org_h = gy0 + row0;
    va.pskel_org_w = vb.pskel_org_w = gx0;
    va.pskel_pitch_w = vb.pskel_pitch_w = LW;
    for (int s = 1; s <= steps; ++s) {
      const Array& vin = (s & 1) ? va : vb;
      const Array& vout = (s & 1) ? vb : va;
      const int e = R * (steps - s);
      const int ylo = HY - e, yhi = HY + TH + e, xlo = HX - e, xhi = HX + TW + e;
      const int rw = xhi - xlo;
      for (int i = threadIdx.x; i < (yhi - ylo) * rw; i += blockDim.x) {
        const int y = ylo + i / rw, x = xlo + i % rw;
        const int gy = gy0 + y, gx = gx0 + x;
        if (gy >= ring && gy < H - ring && gx >= ring && gx < W - ring)
          stencilKernel(vin, vout, mask, args, static_cast<size_t>(gy + row0), static_cast<size_t>(gx));
      }
      __syncthreads();
    }
    const V* fin = (steps & 1) ? B : A;
    for (int i = threadIdx.x; i < TW * TH; i += blockDim.x) {
      const int y = HY + i / TW, x = HX + i % TW;
      const int gy = gy0 + y, gx = gx0 + x;
      if (gy >= ring && gy < H - ring && gx >= ring && gx < W - ring) gdst[static_cast<long>(gy) * W + gx] = fin[y * LW + x];
    }
    __syncthreads();
  }
}

// One step of a user functor on a 1D array: every cell, grid-stride.
template <class Array, class Mask, class Args>
__global__ void __launch_bounds__(256) functor1d_step(Array in, Array out, Mask mask, Args args, size_t W) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < W;
       i += static_cast<size_t>(gridDim.x) * blockDim.x)
    stencilKernel(in, out, mask, args, i);
}

// One step of a user functor on a 3D grid: every cell of the planes
// [h0, h1), d fastest across lanes (grid coordinates; an out-of-core slab
// passes its own planes).
template <class Array, class Mask, class Args>
__global__ void __launch_bounds__(128) functor3d_step(Array in, Array out, Mask mask, Args args, int W, int h0, int h1,
                                                      int D) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= D) return;
  for (int h = h0 + static_cast<int>(blockIdx.z); h < h1; h += gridDim.z)
    for (int w = blockIdx.y; w < W; w += gridDim.y)
      stencilKernel(in, out, mask, args, static_cast<size_t>(h), static_cast<size_t>(w), static_cast<size_t>(d));
}
#endif  // __CUDACC__

}  // namespace detail

// ------------------------------------------------------------ StencilBase

template <class Array, class Mask, class Args = int>
class StencilBase {
 protected:
  Array input;
  Array output;
  Args args;
  Mask mask;
  bool outOfCore = false;

  virtual void runGPUSchedule(size_t iterations, pskel_schedule sched) = 0;
#ifdef PSKEL_OMP
  virtual void runOpenMP(Array in, Array out, size_t numThreads) = 0;
#endif
  // Device bytes an in-core run holds (the reference's test in runAutoGPU,
  // PSkelStencil.hpp:832: input + output + mask below 99.8% of free memory).
  virtual size_t inCoreBytes() { return input.memSize() + output.memSize() + 4096; }
  bool fitsDevice(size_t budget) {
    return budget == 0 || static_cast<double>(inCoreBytes()) < 0.998 * static_cast<double>(budget);
  }
  // Out-of-core run of a library stencil; false when there is none (user
  // functors), and the caller then runs in core.
  virtual bool runOutOfCore(size_t iterations, size_t slabRows, size_t innerIterations, size_t budget) {
    (void)iterations;
    (void)slabRows;
    (void)innerIterations;
    (void)budget;
    return false;
  }

 public:
  virtual ~StencilBase() {}

  // ---- GPU (PSkelStencil.h:258-306)
  void runIterativeGPU(size_t iterations, size_t GPUBlockSizeX, size_t GPUBlockSizeY) {
    (void)GPUBlockSizeX;
    (void)GPUBlockSizeY;
    runGPUSchedule(iterations, detail::make_schedule(0, 0, 0, 0));
  }
  void runIterativeGPU(size_t iterations, size_t pyramidHeight, size_t GPUBlockSizeX, size_t GPUBlockSizeY) {
    (void)GPUBlockSizeX;
    (void)GPUBlockSizeY;
    runGPUSchedule(iterations, detail::make_schedule(0, 0, 0, pyramidHeight));
  }
  // Arrays that fit in device memory run there, the tiling parameters sizing
  // on-chip tiles; arrays that do not (the reference's reason for host tiles,
  // PSkelStencil.hpp:829-861) run out of core: slabs of tilingHeight rows
  // (h-planes in 3D) streamed through the device, innerIterations steps per
  // visit.
  void runIterativeTilingGPU(size_t iterations, size_t tilingWidth, size_t tilingHeight, size_t tilingDepth,
                             size_t innerIterations = 1, size_t GPUBlockSizeX = 0, size_t GPUBlockSizeY = 0) {
    (void)GPUBlockSizeX;
    (void)GPUBlockSizeY;
    const size_t budget = detail::device_budget();
    outOfCore = !fitsDevice(budget) && runOutOfCore(iterations, tilingHeight, innerIterations, budget);
    if (!outOfCore)
      runGPUSchedule(iterations, detail::make_schedule(tilingWidth, tilingHeight, tilingDepth, innerIterations));
  }
  void runIterativeAutoGPU(size_t iterations, size_t GPUBlockSize = 0) {
    (void)GPUBlockSize;
    const size_t budget = detail::device_budget();
    outOfCore = !fitsDevice(budget) && runOutOfCore(iterations, 0, 0, budget);
    if (!outOfCore) runGPUSchedule(iterations, autoSchedule(iterations));
  }
  // An explicit schedule (a tuner's pick, for example).
  void runIterativeGPU(size_t iterations, const pskel_schedule& sched) { runGPUSchedule(iterations, sched); }
  // Whether the last runIterativeTilingGPU / runIterativeAutoGPU ran out of core.
  bool ranOutOfCore() const { return outOfCore; }

  void runGPU(size_t GPUBlockSizeX = 0, size_t GPUBlockSizeY = 0) { runIterativeGPU(1, GPUBlockSizeX, GPUBlockSizeY); }
  void runTilingGPU(size_t tilingWidth, size_t tilingHeight, size_t tilingDepth, size_t GPUBlockSizeX = 0,
                    size_t GPUBlockSizeY = 0) {
    runIterativeTilingGPU(1, tilingWidth, tilingHeight, tilingDepth, 1, GPUBlockSizeX, GPUBlockSizeY);
  }
  void runAutoGPU(size_t GPUBlockSize = 0) { runIterativeAutoGPU(1, GPUBlockSize); }

  // The schedule runIterativeAutoGPU uses: the library's tuned default.
  virtual pskel_schedule autoSchedule(size_t iterations) {
    (void)iterations;
    return detail::make_schedule(0, 0, 0, 0);
  }

#ifdef PSKEL_OMP
  // ---- host (PSkelStencil.hpp:864-938): ping-pong over the host arrays;
  // with an even number of iterations the input is copied into the output.
  void runIterativeCPU(size_t iterations, size_t numThreads = 0) {
    for (size_t it = 0; it < iterations; ++it) {
      if (it % 2 == 0)
        runOpenMP(input, output, numThreads);
      else
        runOpenMP(output, input, numThreads);
    }
    if (iterations % 2 == 0) output.hostMemCopy(input);
  }
  void runIterativeSequential(size_t iterations) { runIterativeCPU(iterations, 1); }
  void runCPU(size_t numThreads = 0) { runOpenMP(input, output, numThreads); }
  void runSequential() { runOpenMP(input, output, 1); }
#endif
};

// ------------------------------------------------------------- Stencil2D

template <class Array, class Mask, class Args>
class Stencil2D : public StencilBase<Array, Mask, Args> {
  typedef typename Array::value_type T;

 public:
  Stencil2D() {}
  Stencil2D(Array _input, Array _output, Mask _mask, Args _args) {
    this->input = _input;
    this->output = _output;
    this->mask = _mask;
    this->args = _args;
  }

  // runIterativeAutoGPU's schedule for the library's stencils: the pick of the
  // registered cost model (pskel_set_cost_model or the PSKEL_COST_MODEL file)
  // among the library's candidates, else the library default.
  pskel_schedule autoSchedule(size_t iterations) override {
    constexpr int op = StencilOp<Args>::value;
    constexpr int dt = detail::LibDtype<T>::value;
    pskel_schedule s = detail::make_schedule(0, 0, 0, 0);
    if constexpr (op != kUserFunctor && dt >= 0) {
      std::vector<int32_t> off;
      std::vector<float> wt;
      pskel_stencil st;
      std::memset(&st, 0, sizeof(st));
      st.op = static_cast<pskel_op>(op);
      st.dtype = static_cast<pskel_dtype>(dt);
      st.mask = detail::describe_mask(this->mask, off, wt);
      pskelErrchk(pskel_auto_schedule2d(&st, static_cast<int64_t>(this->input.getWidth()),
                                        static_cast<int64_t>(this->input.getHeight()),
                                        static_cast<int64_t>(iterations), &s));
    }
    return s;
  }

 protected:
  void runGPUSchedule(size_t iterations, pskel_schedule sched) override {
    constexpr int op = StencilOp<Args>::value;
    constexpr int dt = detail::LibDtype<T>::value;
    if constexpr (op != kUserFunctor && dt >= 0) {
      runLibrary(iterations, sched);
    } else {
      runFunctor(iterations, sched);
    }
  }

  size_t inCoreBytes() override {
    const size_t grid = this->input.memSize();
    return (StencilOp<Args>::value == kAdvect ? 4 : 2) * grid + 4096;
  }

  bool runOutOfCore(size_t iterations, size_t slabRows, size_t innerIterations, size_t budget) override {
    constexpr int op = StencilOp<Args>::value;
    constexpr int dt = detail::LibDtype<T>::value;
    if constexpr (op != kUserFunctor && dt >= 0) {
      runLibrary(iterations, detail::make_schedule(0, 0, 0, 0), true, slabRows, innerIterations, budget);
      return true;
    } else {
#ifdef __CUDACC__
      runFunctorOutOfCore(iterations, slabRows, innerIterations, budget);
      return true;
#else
      (void)iterations;
      (void)slabRows;
      (void)innerIterations;
      (void)budget;
      return false;
#endif
    }
  }

#ifdef __CUDACC__
  // A user functor on arrays larger than the device memory: the reference's
  // host tiling (runIterativeTilingGPU, PSkelStencil.hpp:1663-1760) with
  // full-width slabs of `slabRows` core rows (sized from the budget when 0)
  // and `innerIterations` steps per visit. Each pass (odd length, so every
  // step sees the ring the step-by-step run sees) reads one host array and
  // writes the other: per slab, the source and destination rows of the slab
  // and a halo of R x steps rows go to the device, the generated tile kernel
  // runs the pass on them with grid coordinates (rows beyond the slab's halo
  // are never read; the halo absorbs what its edge rows get wrong), and the
  // slab's core rows come back. As in the reference, the passes ping-pong
  // between a host copy of the input and the output, and the input array is
  // left as it was.
  void runFunctorOutOfCore(size_t iterations, size_t slabRows, size_t innerIterations, size_t budget) {
    const int W = static_cast<int>(this->input.getWidth()), H = static_cast<int>(this->input.getHeight());
    const int ring = static_cast<int>(this->mask.getRange());
    const int reach = static_cast<int>(this->mask.maxOffset());
    const int R = ring > reach ? ring : reach;
    int TB = innerIterations > 0 ? static_cast<int>(innerIterations) : 5;
    if (R == 0) TB = 1;
    std::vector<int32_t> passes(static_cast<size_t>(iterations) + 1);
    const int np = pskel_plan_passes(static_cast<int64_t>(iterations), TB, passes.data(),
                                     static_cast<int32_t>(passes.size()));
    TB = 1;
    for (int i = 0; i < np; ++i) TB = passes[i] > TB ? passes[i] : TB;
    const size_t halo = static_cast<size_t>(R) * TB;
    const size_t S = detail::slab_rows(slabRows, budget, static_cast<size_t>(W) * sizeof(T), 2, halo,
                                       static_cast<size_t>(H));
    const size_t cap = S + 2 * halo < static_cast<size_t>(H) ? S + 2 * halo : static_cast<size_t>(H);
    T* din = nullptr;
    T* dout = nullptr;
    gpuErrchk(cudaMalloc(reinterpret_cast<void**>(&din), cap * W * sizeof(T)));
    gpuErrchk(cudaMalloc(reinterpret_cast<void**>(&dout), cap * W * sizeof(T)));
    this->mask.deviceAlloc();
    this->mask.copyToDevice();
    const int TW = 64, TH = 32;
    typedef typename std::remove_reference<decltype(this->mask.getWeight(0))>::type WT;
    const size_t tile_bytes =
        ((static_cast<size_t>(TW + 2 * R * TB) * (TH + 2 * R * TB) * sizeof(T)) + 15) & ~size_t(15);
    const size_t smem = 2 * tile_bytes + ((this->mask.size * this->mask.dimension + 3) & ~size_t(3)) * sizeof(int) +
                        this->mask.size * sizeof(WT) + 16;
    auto kern = detail::functor2d_pass<Array, Mask, Args>;
    gpuErrchk(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    int dev = 0, sms = 0, per_sm = 0;
    gpuErrchk(cudaGetDevice(&dev));
    gpuErrchk(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    gpuErrchk(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem));
    Array copy;
    copy.hostClone(this->input);  // the reference's inputCopy: the input array is not written
    for (int i = 0; i < np; ++i) {
      Array& src = (i % 2 == 0) ? copy : this->output;
      Array& dst = (i % 2 == 0) ? this->output : copy;
      for (size_t c0 = 0; c0 < static_cast<size_t>(H); c0 += S) {
        const size_t c1 = c0 + S < static_cast<size_t>(H) ? c0 + S : static_cast<size_t>(H);
        const size_t lo = c0 > halo ? c0 - halo : 0;
        const size_t hi = c1 + halo < static_cast<size_t>(H) ? c1 + halo : static_cast<size_t>(H);
        const int Hs = static_cast<int>(hi - lo);
        detail::rows_to_device(src, lo, hi, din);
        detail::rows_to_device(dst, lo, hi, dout);  // its ring is read by every second step
        Array vin = src, vout = dst;
        vin.deviceArray = din;
        vout.deviceArray = dout;
        const int tiles_x = (W + TW - 1) / TW, tiles_y = (Hs + TH - 1) / TH;
        int ctas = (per_sm > 0 ? per_sm : 1) * sms;
        if (ctas > tiles_x * tiles_y) ctas = tiles_x * tiles_y;
        kern<<<ctas, 256, smem>>>(vin, vout, this->mask, this->args, W, Hs, ring, R, passes[i], TB, TW, TH, tiles_x,
                                  tiles_y, static_cast<int>(lo));
        gpuErrchk(cudaPeekAtLastError());
        detail::rows_to_host(dst, c0, c1, dout + (c0 - lo) * W);
      }
    }
    // an even number of passes ends in the copy (with the input's ring, as the
    // step-by-step run leaves it)
    if (np % 2 == 0) this->output.hostMemCopy(copy);
    copy.hostFree();
    gpuErrchk(cudaFree(din));
    gpuErrchk(cudaFree(dout));
    this->mask.deviceFree();
  }
#endif

  void runLibrary(size_t iterations, pskel_schedule sched, bool tiled = false, size_t slabRows = 0,
                  size_t innerIterations = 0, size_t budget = 0) {
    constexpr int op = StencilOp<Args>::value;
    std::vector<int32_t> off;
    std::vector<float> wt;
    pskel_stencil st;
    std::memset(&st, 0, sizeof(st));
    st.op = static_cast<pskel_op>(op);
    st.dtype = static_cast<pskel_dtype>(detail::LibDtype<T>::value);
    st.mask = detail::describe_mask(this->mask, off, wt);
    detail::Contig<Array> in(this->input), out(this->output);
    if constexpr (op == kAdvect) {
      detail::Contig<Array> u(this->args.wind_x), v(this->args.wind_y);
      st.wind_u = u.data();
      st.wind_v = v.data();
      st.diffusivity = this->args.K;
      st.dt = this->args.dt;
      st.inv_dx = this->args.inv_dx;
      run2d(st, in.data(), out.data(), iterations, sched, tiled, slabRows, innerIterations, budget);
    } else {
      run2d(st, in.data(), out.data(), iterations, sched, tiled, slabRows, innerIterations, budget);
    }
    out.write_back();
  }

  void run2d(const pskel_stencil& st, const T* in, T* out, size_t iterations, const pskel_schedule& sched,
             bool tiled, size_t slabRows, size_t innerIterations, size_t budget) {
    const int64_t W = static_cast<int64_t>(this->input.getWidth()), H = static_cast<int64_t>(this->input.getHeight());
    if (tiled) {
      pskelErrchk(pskel_run2d_host_tiled(&st, in, out, W, H, static_cast<int64_t>(iterations),
                                         static_cast<int64_t>(slabRows), static_cast<int32_t>(innerIterations),
                                         static_cast<int64_t>(budget), nullptr));
    } else {
      pskelErrchk(pskel_run2d_host(&st, in, out, W, H, static_cast<int64_t>(iterations), &sched));
    }
  }

  void runFunctor(size_t iterations, pskel_schedule sched) {
#ifdef __CUDACC__
    const int W = static_cast<int>(this->input.getWidth()), H = static_cast<int>(this->input.getHeight());
    const int ring = static_cast<int>(this->mask.getRange());
    const int reach = static_cast<int>(this->mask.maxOffset());
    const int R = ring > reach ? ring : reach;
    int TB = sched.time_steps > 0 ? sched.time_steps : 5;
    if (R == 0) TB = 1;
    const int TW = sched.tile_w > 0 ? sched.tile_w : 64;
    const int TH = sched.tile_h > 0 ? sched.tile_h : 32;
    Array in = this->input, out = this->output;
    in.deviceAlloc();
    out.deviceAlloc();
    this->mask.deviceAlloc();
    this->mask.copyToDevice();
    in.copyToDevice();
    out.copyToDevice();  // its ring is read by every second step
    std::vector<int32_t> passes(static_cast<size_t>(iterations) + 1);
    const int np = pskel_plan_passes(static_cast<int64_t>(iterations), TB, passes.data(),
                                     static_cast<int32_t>(passes.size()));
    TB = 1;
    for (int i = 0; i < np; ++i) TB = passes[i] > TB ? passes[i] : TB;
    typedef typename std::remove_reference<decltype(this->mask.getWeight(0))>::type WT;
    const size_t tile_bytes =
        ((static_cast<size_t>(TW + 2 * R * TB) * (TH + 2 * R * TB) * sizeof(T)) + 15) & ~size_t(15);
    const size_t smem = 2 * tile_bytes + ((this->mask.size * this->mask.dimension + 3) & ~size_t(3)) * sizeof(int) +
                        this->mask.size * sizeof(WT) + 16;
    auto kern = detail::functor2d_pass<Array, Mask, Args>;
    gpuErrchk(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    int dev = 0, sms = 0, per_sm = 0;
    gpuErrchk(cudaGetDevice(&dev));
    gpuErrchk(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    gpuErrchk(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem));
    const int tiles_x = (W + TW - 1) / TW, tiles_y = (H + TH - 1) / TH;
    int ctas = (per_sm > 0 ? per_sm : 1) * sms;
    if (ctas > tiles_x * tiles_y) ctas = tiles_x * tiles_y;
    if (ctas < 1) ctas = 1;
    for (int i = 0; i < np; ++i) {
      const bool fwd = (i % 2 == 0);
      kern<<<ctas, 256, smem>>>(fwd ? in : out, fwd ? out : in, this->mask, this->args, W, H, ring, R, passes[i], TB,
                                TW, TH, tiles_x, tiles_y, 0);
      gpuErrchk(cudaPeekAtLastError());
    }
    gpuErrchk(cudaDeviceSynchronize());
    if (iterations % 2 == 1)
      this->output.copyFromDevice(out);
    else
      this->output.copyFromDevice(in);
    in.deviceFree();
    out.deviceFree();
    this->mask.deviceFree();
#else
    (void)iterations;
    (void)sched;
    static_assert(StencilOp<Args>::value != kUserFunctor || sizeof(Args) == 0,
                  "a user stencilKernel runs on the GPU only when this file is compiled with nvcc");
#endif
  }

#ifdef PSKEL_OMP
  void runOpenMP(Array in, Array out, size_t numThreads) override {
    const size_t r = this->mask.getRange();
    const size_t H = in.getHeight(), W = in.getWidth();
    const long hr = static_cast<long>(H) - static_cast<long>(r);
    const int nt = numThreads ? static_cast<int>(numThreads) : omp_get_max_threads();
#pragma omp parallel for num_threads(nt)
    for (long h = static_cast<long>(r); h < hr; ++h)
      for (size_t w = r; w + r < W; ++w) stencilKernel(in, out, this->mask, this->args, static_cast<size_t>(h), w);
  }
#endif
};

// ------------------------------------------------------------- Stencil (1D)

// The 1D skeleton (PSkelStencil.h:384-407, PSkelStencil.hpp:2303-2327): every
// cell i in [0, width) is updated each step by the user functor
// stencilKernel(in, out, mask, args, i); Mask::get reads the halo value
// outside the array. The GPU methods run one generated grid-stride kernel per
// step, ping-ponging on the device; the result is copied into `output`.
template <class Array, class Mask, class Args>
class Stencil : public StencilBase<Array, Mask, Args> {
 public:
  Stencil() {}
  Stencil(Array _input, Array _output, Mask _mask, Args _args) {
    this->input = _input;
    this->output = _output;
    this->mask = _mask;
    this->args = _args;
  }

 protected:
  void runGPUSchedule(size_t iterations, pskel_schedule sched) override {
    (void)sched;
#ifdef __CUDACC__
    const size_t W = this->input.getWidth();
    Array in = this->input, out = this->output;
    in.deviceAlloc();
    out.deviceAlloc();
    this->mask.deviceAlloc();
    this->mask.copyToDevice();
    in.copyToDevice();
    int dev = 0, sms = 1;
    gpuErrchk(cudaGetDevice(&dev));
    gpuErrchk(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    size_t blocks = (W + 255) / 256;
    if (blocks > static_cast<size_t>(sms) * 8) blocks = static_cast<size_t>(sms) * 8;
    if (blocks < 1) blocks = 1;
    for (size_t it = 0; it < iterations; ++it) {
      if (it % 2 == 0)
        detail::functor1d_step<<<static_cast<unsigned>(blocks), 256>>>(in, out, this->mask, this->args, W);
      else
        detail::functor1d_step<<<static_cast<unsigned>(blocks), 256>>>(out, in, this->mask, this->args, W);
      gpuErrchk(cudaPeekAtLastError());
    }
    gpuErrchk(cudaDeviceSynchronize());
    if (iterations % 2 == 1)
      this->output.copyFromDevice(out);
    else
      this->output.copyFromDevice(in);
    in.deviceFree();
    out.deviceFree();
    this->mask.deviceFree();
#else
    (void)iterations;
    static_assert(sizeof(Args) == 0, "the 1D stencil runs on the GPU only when this file is compiled with nvcc");
#endif
  }

#ifdef PSKEL_OMP
  void runOpenMP(Array in, Array out, size_t numThreads) override {
    const long W = static_cast<long>(in.getWidth());
    const int nt = numThreads ? static_cast<int>(numThreads) : omp_get_max_threads();
#pragma omp parallel for num_threads(nt)
    for (long i = 0; i < W; ++i) stencilKernel(in, out, this->mask, this->args, static_cast<size_t>(i));
  }
#endif
};

// ------------------------------------------------------------- Stencil3D

template <class Array, class Mask, class Args>
class Stencil3D : public StencilBase<Array, Mask, Args> {
  typedef typename Array::value_type T;

 public:
  Stencil3D() {}
  Stencil3D(Array _input, Array _output, Mask _mask, Args _args) {
    this->input = _input;
    this->output = _output;
    this->mask = _mask;
    this->args = _args;
  }

  // fp64 residual norms ||u_k - u_{k-1}||_2 recorded by the next GPU run at
  // every k that is a multiple of `every` (library path only; 0 disables).
  void setResidualInterval(size_t every) { residualEvery = every; }
  const std::vector<double>& residuals() const { return residualNorms; }

 protected:
  size_t residualEvery = 0;
  std::vector<double> residualNorms;

  // Out of core the residual norms are not recorded (residuals() is empty).
  bool runOutOfCore(size_t iterations, size_t slabRows, size_t innerIterations, size_t budget) override {
    constexpr int op = StencilOp<Args>::value;
    constexpr int dt = detail::LibDtype<T>::value;
    if constexpr (op == kLinear && dt >= 0 && dt != PSKEL_U8) {
      std::vector<int32_t> off;
      std::vector<float> wt;
      pskel_stencil st;
      std::memset(&st, 0, sizeof(st));
      st.op = PSKEL_OP_LINEAR;
      st.dtype = static_cast<pskel_dtype>(dt);
      st.mask = detail::describe_mask(this->mask, off, wt);
      detail::Contig<Array> in(this->input), out(this->output);
      residualNorms.clear();
      pskelErrchk(pskel_run3d_host_tiled(&st, in.data(), out.data(), static_cast<int64_t>(this->input.getWidth()),
                                         static_cast<int64_t>(this->input.getHeight()),
                                         static_cast<int64_t>(this->input.getDepth()),
                                         static_cast<int64_t>(iterations), static_cast<int64_t>(slabRows),
                                         static_cast<int32_t>(innerIterations), static_cast<int64_t>(budget),
                                         nullptr));
      out.write_back();
      return true;
    } else {
#ifdef __CUDACC__
      runFunctorOutOfCore(iterations, slabRows, innerIterations, budget);
      return true;
#else
      (void)iterations;
      (void)slabRows;
      (void)innerIterations;
      (void)budget;
      return false;
#endif
    }
  }

#ifdef __CUDACC__
  // A user functor on 3D arrays larger than the device memory: slabs of
  // `slabRows` h-planes (sized from the budget when 0) with a halo of
  // R x steps planes, `innerIterations` steps per visit (the reference's host
  // tiling, PSkelStencil.hpp:1663-1760, in full (w, d) planes). Every cell is
  // updated each step (Stencil3D semantics); the slab buffers carry R guard
  // planes on each side so that the functor's reads through Mask3D::get at
  // the slab's edge planes stay inside them (those planes are halo: the
  // values they get are not kept). The passes ping-pong between a host copy
  // of the input and the output; the input array is left as it was.
  void runFunctorOutOfCore(size_t iterations, size_t slabRows, size_t innerIterations, size_t budget) {
    const int W = static_cast<int>(this->input.getWidth()), H = static_cast<int>(this->input.getHeight());
    const int D = static_cast<int>(this->input.getDepth());
    const int R = static_cast<int>(this->mask.maxOffset());
    const int TB = innerIterations > 0 ? static_cast<int>(innerIterations) : 4;
    const size_t plane = static_cast<size_t>(W) * D;
    const size_t halo = static_cast<size_t>(R) * TB, G = static_cast<size_t>(R);
    const size_t S = detail::slab_rows(slabRows, budget, plane * sizeof(T), 2, halo + G, static_cast<size_t>(H));
    const size_t cap = (S + 2 * halo < static_cast<size_t>(H) ? S + 2 * halo : static_cast<size_t>(H)) + 2 * G;
    T* buf[2] = {nullptr, nullptr};
    for (T*& b : buf) {
      gpuErrchk(cudaMalloc(reinterpret_cast<void**>(&b), cap * plane * sizeof(T)));
      gpuErrchk(cudaMemset(b, 0, cap * plane * sizeof(T)));
    }
    this->mask.deviceAlloc();
    this->mask.copyToDevice();
    Array copy;
    copy.hostClone(this->input);  // the reference's inputCopy: the input array is not written
    const dim3 block(128);
    size_t np = 0;
    for (size_t done = 0; done < iterations; ++np) {
      const int steps = static_cast<int>(iterations - done < static_cast<size_t>(TB) ? iterations - done : TB);
      Array& src = (np % 2 == 0) ? copy : this->output;
      Array& dst = (np % 2 == 0) ? this->output : copy;
      for (size_t c0 = 0; c0 < static_cast<size_t>(H); c0 += S) {
        const size_t c1 = c0 + S < static_cast<size_t>(H) ? c0 + S : static_cast<size_t>(H);
        const size_t lo = c0 > halo ? c0 - halo : 0;
        const size_t hi = c1 + halo < static_cast<size_t>(H) ? c1 + halo : static_cast<size_t>(H);
        detail::rows_to_device(src, lo, hi, buf[0] + G * plane);
        const int Hs = static_cast<int>(hi - lo);
        const dim3 grid((D + 127) / 128, W < 65535 ? W : 65535, Hs < 65535 ? Hs : 65535);
        for (int s = 0; s < steps; ++s) {
          // views with grid coordinates: plane h sits at buffer plane h - lo + G
          Array vin = src, vout = dst;
          vin.deviceArray = buf[s % 2] + G * plane;
          vout.deviceArray = buf[(s + 1) % 2] + G * plane;
          vin.reset_view();
          vout.reset_view();
          vin.pskel_org_h = vout.pskel_org_h = static_cast<long>(lo);
          detail::functor3d_step<<<grid, block>>>(vin, vout, this->mask, this->args, W, static_cast<int>(lo),
                                                  static_cast<int>(hi), D);
          gpuErrchk(cudaPeekAtLastError());
        }
        detail::rows_to_host(dst, c0, c1, buf[steps % 2] + (G + c0 - lo) * plane);
      }
      done += static_cast<size_t>(steps);
    }
    if (np % 2 == 0) this->output.hostMemCopy(copy);
    copy.hostFree();
    for (T* b : buf) gpuErrchk(cudaFree(b));
    this->mask.deviceFree();
  }
#endif

  void runGPUSchedule(size_t iterations, pskel_schedule sched) override {
    constexpr int op = StencilOp<Args>::value;
    constexpr int dt = detail::LibDtype<T>::value;
    if constexpr (op == kLinear && dt >= 0 && dt != PSKEL_U8) {
      std::vector<int32_t> off;
      std::vector<float> wt;
      pskel_stencil st;
      std::memset(&st, 0, sizeof(st));
      st.op = PSKEL_OP_LINEAR;
      st.dtype = static_cast<pskel_dtype>(dt);
      st.mask = detail::describe_mask(this->mask, off, wt);
      detail::Contig<Array> in(this->input), out(this->output);
      const int64_t every = static_cast<int64_t>(residualEvery);
      residualNorms.assign(every > 0 ? iterations / residualEvery : 0, 0.0);
      pskelErrchk(pskel_run3d_host(&st, in.data(), out.data(), static_cast<int64_t>(this->input.getWidth()),
                                   static_cast<int64_t>(this->input.getHeight()),
                                   static_cast<int64_t>(this->input.getDepth()), static_cast<int64_t>(iterations),
                                   &sched, every, residualNorms.empty() ? nullptr : residualNorms.data()));
      out.write_back();
    } else {
      runFunctor(iterations);
    }
  }

  void runFunctor(size_t iterations) {
#ifdef __CUDACC__
    const int W = static_cast<int>(this->input.getWidth()), H = static_cast<int>(this->input.getHeight());
    const int D = static_cast<int>(this->input.getDepth());
    Array in = this->input, out = this->output;
    in.deviceAlloc();
    out.deviceAlloc();
    this->mask.deviceAlloc();
    this->mask.copyToDevice();
    in.copyToDevice();
    const dim3 block(128);
    const dim3 grid((D + 127) / 128, W < 65535 ? W : 65535, H < 65535 ? H : 65535);
    for (size_t it = 0; it < iterations; ++it) {
      if (it % 2 == 0)
        detail::functor3d_step<<<grid, block>>>(in, out, this->mask, this->args, W, 0, H, D);
      else
        detail::functor3d_step<<<grid, block>>>(out, in, this->mask, this->args, W, 0, H, D);
      gpuErrchk(cudaPeekAtLastError());
    }
    gpuErrchk(cudaDeviceSynchronize());
    if (iterations % 2 == 1)
      this->output.copyFromDevice(out);
    else
      this->output.copyFromDevice(in);
    in.deviceFree();
    out.deviceFree();
    this->mask.deviceFree();
#else
    (void)iterations;
    static_assert(StencilOp<Args>::value == kLinear || sizeof(Args) == 0,
                  "a user stencilKernel runs on the GPU only when this file is compiled with nvcc");
#endif
  }

#ifdef PSKEL_OMP
  void runOpenMP(Array in, Array out, size_t numThreads) override {
    const long H = static_cast<long>(in.getHeight());
    const int nt = numThreads ? static_cast<int>(numThreads) : omp_get_max_threads();
#pragma omp parallel for num_threads(nt)
    for (long h = 0; h < H; ++h)
      for (size_t w = 0; w < in.getWidth(); ++w)
        for (size_t d = 0; d < in.getDepth(); ++d)
          stencilKernel(in, out, this->mask, this->args, static_cast<size_t>(h), w, d);
  }
#endif
};

}  // namespace PSkel

#endif  // PSKEL_STENCIL_H
