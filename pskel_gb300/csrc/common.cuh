// Shared device helpers: TMA tile loads, mbarriers with bounded waits, bf16
// storage conversions and the device error word.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace pskel {

// Device error word written by kernels instead of trapping. Bits:
enum DeviceError : unsigned {
  kDevErrTimeout = 1u,    // an mbarrier wait ran out of iterations
  kDevErrValue = 2u,      // an input value outside the kernel's domain (Life: cell not 0/1)
  kDevErrBarrier = 4u,    // a dependency wait between tiles or passes ran out of iterations
  kDevErrAlign = 8u,      // dynamic shared memory not 128-byte aligned (kernel did nothing)
};

// Bits after which the persistent kernels stop: a wait that ran out means a
// producer never arrived, and every item that depends on it would wait its
// full limit too. (kDevErrValue is only reported.)
constexpr unsigned kDevErrStop = kDevErrTimeout | kDevErrBarrier;

// True once a stop bit is latched in the error word (by this launch or an
// earlier one of the call): persistent kernels then take no more items and
// abandon their dependency waits, so one lost tile costs one wait limit, not
// one per dependent item.
__device__ __forceinline__ bool error_latched(const unsigned* err) {
  return (*reinterpret_cast<const volatile unsigned*>(err) & kDevErrStop) != 0u;
}

// Upper bound on mbarrier polls before a kernel gives up on a TMA load. A load
// of one tile completes in microseconds; 2^26 polls is seconds.
constexpr unsigned kMbarSpinLimit = 1u << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Orders this thread's earlier generic-proxy accesses of global memory (and
// those it has observed) before its later async-proxy (TMA) accesses.
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Wait for phase `phase` of `bar`; false (and the error word set) if the wait
// ran out of polls. Never spins unboundedly.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, unsigned* err) {
  for (unsigned i = 0; i < kMbarSpinLimit; ++i) {
    if (mbar_try_wait(bar, phase)) return true;
  }
  if (err) atomicOr(err, kDevErrTimeout);
  return false;
}

// 2D tiled TMA load of box (x, y) into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// 3D tiled TMA load of box (x, y, z) into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Sum of squared differences sum((a_i - b_i)^2) over fp32 pairs in
// double-float arithmetic, so the fp64 pipe (slow on this part) is used once
// per thread instead of per cell. Error-free transformations: the difference
// is split exactly into hi + lo (Knuth's TwoSum), hi^2 exactly into p + e
// (FMA), and p is added to the running (s, c) pair with TwoSum; the 2*hi*lo
// term and the pair's low part are added in fp32. Relative error of the sum is
// about 2^-44 per term; flush() hands the pair to an fp64 sum every plane.
struct SqDiffAcc {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float a, float b) {
    const float hi = __fsub_rn(a, b);
    const float bp = __fsub_rn(hi, a);  // about -b
    const float ap = __fsub_rn(hi, bp);  // about a
    const float lo = __fsub_rn(__fsub_rn(a, ap), __fadd_rn(b, bp));
    const float p = __fmul_rn(hi, hi);
    const float e = __fmaf_rn(hi, hi, -p);
    const float t = __fadd_rn(s, p);
    const float tb = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, tb)), __fsub_rn(p, tb));
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, __fadd_rn(e, __fmul_rn(__fmul_rn(2.0f, hi), lo))));
  }
  __device__ __forceinline__ double value() const { return static_cast<double>(s) + static_cast<double>(c); }
  // Moves the pair into an fp64 sum and restarts it. Called once per plane,
  // so that a pair sums a few dozen terms and the fp64 pipe adds once per
  // thread and plane.
  __device__ __forceinline__ void flush(double& total) {
    total += value();
    s = 0.0f;
    c = 0.0f;
  }
};

// Storage conversions. fp32 storage is the identity; bf16 storage widens on
// load and rounds to nearest even on store.
template <class TS> struct Storage;
template <> struct Storage<float> {
  static __device__ __forceinline__ float load(float v) { return v; }
  static __device__ __forceinline__ float store(float v) { return v; }
};
template <> struct Storage<__nv_bfloat16> {
  static __device__ __forceinline__ float load(__nv_bfloat16 v) { return __bfloat162float(v); }
  static __device__ __forceinline__ __nv_bfloat16 store(float v) { return __float2bfloat16_rn(v); }
};

// 16 bytes of cells (4 fp32 or 8 bf16) kept packed in four 32-bit registers,
// widened to fp32 on use.
template <class TS>
struct Vec16 {
  static constexpr int V = 16 / sizeof(TS);  // cells per vector
  uint32_t r[4];                             // raw 16 bytes
  __device__ __forceinline__ float at(int c) const {
    if constexpr (sizeof(TS) == 4) {
      return __uint_as_float(r[c]);
    } else {
      return (c & 1) ? __uint_as_float(r[c >> 1] & 0xFFFF0000u) : __uint_as_float(r[c >> 1] << 16);
    }
  }
  __device__ __forceinline__ void load(const TS* p) {
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(p));
    r[0] = v.x;
    r[1] = v.y;
    r[2] = v.z;
    r[3] = v.w;
  }
  __device__ __forceinline__ void fill(uint32_t h) { r[0] = r[1] = r[2] = r[3] = h; }
};

// The one edge cell a lane needs from a staged row laid out as a 16-byte
// west halo vector, 32 core vectors (one per lane) and a 16-byte east halo
// vector: lane 0 the cell before the first core cell (the last cell of the
// west vector, in bytes 12..15), lane 31 the cell after the last one (the
// first cell of the east vector, at byte 16 + 32*16). Every lane issues the
// same one 4-byte shared load (lanes 1..30 take lane 0's word, a broadcast,
// and ignore it) and, for bf16, one byte permute that widens its half of the
// word -- instead of two predicated loads and widenings per row.
template <class TS>
struct EdgeCell {
  int off;       // byte offset of the lane's word within the row
  uint32_t sel;  // __byte_perm selector: the cell's 16 bits to the top, zeros below
  __device__ __forceinline__ explicit EdgeCell(int lane)
      : off(lane == 31 ? 16 + 32 * 16 : 12), sel(lane == 31 ? 0x1044u : 0x3244u) {}
  __device__ __forceinline__ float get(const uint8_t* row) const {
    const uint32_t w = *reinterpret_cast<const uint32_t*>(row + off);
    if constexpr (sizeof(TS) == 4) {
      return __uint_as_float(w);
    } else {
      return __uint_as_float(__byte_perm(w, 0u, sel));
    }
  }
};

// Paired fp32 arithmetic (Blackwell's add/sub/fma.f32x2): two lanes per
// instruction, each rounded to nearest like the scalar .rn forms, so every lane
// matches the reference's unfused scalar arithmetic bit for bit -- provided no
// product is fused into the sum it feeds. ptxas does fuse a paired product
// (mul.rn.f32x2, or fma.rn.f32x2 with a constant -0 addend) into a paired sum,
// .rn and -fmad=false notwithstanding, so a product is written as
// fma(a, b, z) with z = (-0, -0) formed at run time from a kernel parameter
// (neg_zero2): fma(a, b, -0) rounds exactly like a*b, signed zeros included,
// and fma(a, b, z) + c is no single multiply-add.
__device__ __forceinline__ unsigned long long f2_bits(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 f2_from(unsigned long long v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
// guard: a kernel parameter that is always 0 (the zero-initialised
// fuse_guard field of the launch parameters)
__device__ __forceinline__ float2 neg_zero2(uint32_t guard) {
  const float z = __uint_as_float(guard ^ 0x80000000u);
  return make_float2(z, z);
}
__device__ __forceinline__ float2 fmul2_rn(float2 a, float2 b, float2 nz) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)), "l"(f2_bits(nz)));
  return f2_from(d);
}
__device__ __forceinline__ float2 fadd2_rn(float2 a, float2 b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_from(d);
}
__device__ __forceinline__ float2 fsub2_rn(float2 a, float2 b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_from(d);
}
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }

// The 7-point weighted sum of the reference's order (centre, h-1, h+1, w-1,
// w+1, d-1, d+1; products and sums unfused) for the V cells of one vector row.
// kPaired: two neighbouring cells per instruction (fmul2_rn / fadd2_rn round
// each lane exactly as __fmul_rn / __fadd_rn, so every cell gets the scalar
// result); wt2[n] holds (wt[n], wt[n]), nz is neg_zero2 of the launch. The
// d-neighbour products are formed one lane at a time: the pair (c[k-1], c[k])
// straddles two register pairs, and two scalar products cost less than
// gathering it. Without kPaired, one cell per instruction (the fp32 one-step
// kernel, bound by HBM, measured faster so: 788 against 732 GCells/s).
template <bool kPaired, class Vt>
__device__ __forceinline__ void cross7_row(const float* wt, const float2* wt2, float2 nz, const Vt& c, const Vt& dn,
                                           const Vt& up, const Vt& a, const Vt& b, float dl, float dr,
                                           float (&res)[Vt::V]) {
  constexpr int V = Vt::V;
  if constexpr (kPaired) {
#pragma unroll
    for (int k = 0; k < V; k += 2) {
      const float c0 = c.at(k), c1 = c.at(k + 1);
      const float l0 = k == 0 ? dl : c.at(k - 1);
      const float r1 = k + 2 == V ? dr : c.at(k + 2);
      float2 acc = fmul2_rn(wt2[0], make_float2(c0, c1), nz);
      acc = fadd2_rn(acc, fmul2_rn(wt2[1], make_float2(dn.at(k), dn.at(k + 1)), nz));
      acc = fadd2_rn(acc, fmul2_rn(wt2[2], make_float2(up.at(k), up.at(k + 1)), nz));
      acc = fadd2_rn(acc, fmul2_rn(wt2[3], make_float2(a.at(k), a.at(k + 1)), nz));
      acc = fadd2_rn(acc, fmul2_rn(wt2[4], make_float2(b.at(k), b.at(k + 1)), nz));
      acc = fadd2_rn(acc, make_float2(__fmul_rn(wt[5], l0), __fmul_rn(wt[5], c0)));
      acc = fadd2_rn(acc, make_float2(__fmul_rn(wt[6], c1), __fmul_rn(wt[6], r1)));
      res[k] = acc.x;
      res[k + 1] = acc.y;
    }
  } else {
#pragma unroll
    for (int k = 0; k < V; ++k) {
      const float l = (k == 0) ? dl : c.at(k - 1);
      const float r = (k == V - 1) ? dr : c.at(k + 1);
      float acc = __fmul_rn(wt[0], c.at(k));
      acc = __fadd_rn(acc, __fmul_rn(wt[1], dn.at(k)));
      acc = __fadd_rn(acc, __fmul_rn(wt[2], up.at(k)));
      acc = __fadd_rn(acc, __fmul_rn(wt[3], a.at(k)));
      acc = __fadd_rn(acc, __fmul_rn(wt[4], b.at(k)));
      acc = __fadd_rn(acc, __fmul_rn(wt[5], l));
      acc = __fadd_rn(acc, __fmul_rn(wt[6], r));
      res[k] = acc;
    }
  }
}

}  // namespace pskel
