// 2D fp32 / bf16-storage stencils, temporally blocked in shared memory.
//
// One pass advances the grid by `steps` time steps. Each persistent CTA walks
// core tiles of TW x TH cells; per tile it stages the halo tile of
// (TW + 2HX) x (TH + 2HY) elements (HY = R*T, HX = R*T rounded up to 16 bytes)
// with a TMA load (plus the two wind tiles for advection), then runs the steps
// ping-ponging between two shared buffers on a shrinking region (redundant
// halo recompute), and finally writes the core with 128-bit stores.
//
// Update rule per cell, as Stencil2D::runOpenMP (PSkelStencil.hpp:2197-2257):
// cells with r <= h < H-r and r <= w < W-r take the stencil value; all other
// cells keep their value (and are never written to global memory).
//
// Arithmetic is fp32 with explicit round-to-nearest intrinsics (__fmul_rn,
// __fadd_rn) so nothing is contracted into an FMA and the operation order is
// exactly the oracle's. bf16 storage rounds every step's result to bf16.
#include "common.cuh"
#include "kernels.h"

namespace pskel {
namespace {

template <class TS, Op2D OP> struct Layout {
  static constexpr int kBufs = (OP == Op2D::Advect) ? 4 : 2;  // A, B [, U, V]
  static __host__ __device__ size_t buf_bytes(int LW, int LH) {
    return (static_cast<size_t>(LW) * LH * sizeof(TS) + 127) & ~size_t(127);
  }
  static __host__ __device__ size_t total(int LW, int LH) { return 128 + kBufs * buf_bytes(LW, LH) + 16; }
};

template <class TS, int NM>
__device__ __forceinline__ float linear_value(const TS* in, int idx, const Stencil2DParams& p, const int* s_off,
                                              const float* s_wt) {
  using S = Storage<TS>;
  if constexpr (NM > 0) {
    float acc = __fmul_rn(p.wt[0], S::load(in[idx + p.off[0]]));
#pragma unroll
    for (int n = 1; n < NM; ++n) acc = __fadd_rn(acc, __fmul_rn(p.wt[n], S::load(in[idx + p.off[n]])));
    return acc;
  } else {
    float acc = __fmul_rn(s_wt[0], S::load(in[idx + s_off[0]]));
    for (int n = 1; n < p.nm; ++n) acc = __fadd_rn(acc, __fmul_rn(s_wt[n], S::load(in[idx + s_off[n]])));
    return acc;
  }
}

// Upwind advection + diffusion: the arithmetic of PSkelStencil.hpp:347-387
// with K, dt and 1/dx as parameters.
template <class TS>
__device__ __forceinline__ float advect_value(const TS* in, const TS* U, const TS* V, int idx, int LW,
                                              const Stencil2DParams& p) {
  using S = Storage<TS>;
  const float c = S::load(in[idx]);
  const float n = S::load(in[idx - LW]);
  const float e = S::load(in[idx + 1]);
  const float wv = S::load(in[idx - 1]);
  const float s = S::load(in[idx + LW]);
  const float sum = __fsub_rn(__fmul_rn(4.0f, c), __fadd_rn(__fadd_rn(__fadd_rn(n, e), wv), s));
  const float xw = S::load(U[idx]);
  const float yw = S::load(V[idx]);
  const int xf = (xw > 0.0f) ? 1 : -1;
  const int yf = (yw > 0.0f) ? 1 : -1;
  const float cvy = __fmul_rn(static_cast<float>(yf), yw);
  const float cvx = __fmul_rn(static_cast<float>(xf), xw);
  const float nbx = S::load(in[idx + xf]);
  const float nby = S::load(in[idx + yf * LW]);
  const float temp_wind = __fsub_rn(__fmul_rn(-cvx, __fmul_rn(__fsub_rn(c, nbx), p.inv_dx)),
                                    __fmul_rn(cvy, __fmul_rn(__fsub_rn(c, nby), p.inv_dx)));
  const float cond = __fmul_rn(__fmul_rn(-p.K, __fmul_rn(sum, 0.25f)), p.dt);
  const float result = __fadd_rn(c, cond);
  return __fadd_rn(result, __fmul_rn(temp_wind, p.dt));
}

template <class TS>
__device__ __forceinline__ void coop_load(TS* dst, const TS* src, int gy0, int gx0, int LW, int LH, int W, int H,
                                          int64_t pitch) {
  for (int i = threadIdx.x; i < LW * LH; i += blockDim.x) {
    const int y = i / LW, x = i - y * LW;
    const int gy = gy0 + y, gx = gx0 + x;
    TS v;
    if (gy >= 0 && gy < H && gx >= 0 && gx < W) {
      v = src[static_cast<int64_t>(gy) * pitch + gx];
    } else {
      v = Storage<TS>::store(0.0f);
    }
    dst[i] = v;
  }
}

template <class TS, Op2D OP, bool kTma, int NM>
__global__ void __launch_bounds__(kStencil2DThreads)
    stencil2d_kernel(const __grid_constant__ CUtensorMap map_src, const __grid_constant__ CUtensorMap map_dst,
                     const __grid_constant__ CUtensorMap map_u,
                     const __grid_constant__ CUtensorMap map_v, const __grid_constant__ Stencil2DParams p) {
  using S = Storage<TS>;
  using L = Layout<TS, OP>;
  // dynamic shared memory, 128-byte aligned for TMA; derived pointers stay
  // in the shared window (no integer round trip), so accesses compile to
  // shared-memory instructions
  extern __shared__ __align__(128) uint8_t smem_raw[];
  uint8_t* base = smem_raw;
  if ((smem_u32(smem_raw) & 127u) != 0) {
    if (threadIdx.x == 0) atomicOr(p.err, kDevErrAlign);
    return;
  }
  const int LW = p.LW, LH = p.LH;
  const size_t bb = L::buf_bytes(LW, LH);
  TS* bufA = reinterpret_cast<TS*>(base);
  TS* bufB = reinterpret_cast<TS*>(base + bb);
  TS* bufU = reinterpret_cast<TS*>(base + 2 * bb);
  TS* bufV = reinterpret_cast<TS*>(base + 3 * bb);
  uint64_t* bar = reinterpret_cast<uint64_t*>(base + L::kBufs * bb);

  __shared__ int s_off[kMaxMask2D];
  __shared__ float s_wt[kMaxMask2D];

  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  constexpr int kWarps = kStencil2DThreads / 32;
  if (NM == 0 && tid < p.nm) {
    s_off[tid] = p.off[tid];
    s_wt[tid] = p.wt[tid];
  }
  if (kTma && tid == 0) {
    mbar_init(bar, 1);
    fence_barrier_init();
    prefetch_tensormap(&map_src);
    prefetch_tensormap(&map_dst);
    if (OP == Op2D::Advect) {
      prefetch_tensormap(&map_u);
      prefetch_tensormap(&map_v);
    }
  }
  __syncthreads();

  const TS* src = static_cast<const TS*>(p.src);
  TS* dst = static_cast<TS*>(p.dst);
  uint32_t phase = 0;
  const int ntiles = p.tiles_x * p.tiles_y;
  constexpr int kVec = 16 / sizeof(TS);

  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int ty = tile / p.tiles_x;
    const int tx = tile - ty * p.tiles_x;
    const int gy0 = ty * p.TH - p.HY;
    const int gx0 = tx * p.TW - p.HX;

    // Ring cells are never written, so each global buffer keeps its own ring
    // and the odd steps of a pass read the destination buffer's ring. Tiles
    // that reach the ring stage the destination tile into bufB for that.
    const bool touches_ring = (gy0 < p.ring) || (gy0 + LH > p.H - p.ring) || (gx0 < p.ring) ||
                              (gx0 + LW > p.W - p.ring);
    const bool stage_dst = touches_ring && p.steps >= 2;
    if (kTma) {
      if (tid == 0) {
        fence_proxy_async();
        const uint32_t tile_bytes = static_cast<uint32_t>(LW * LH * sizeof(TS));
        const uint32_t ntile = 1u + (stage_dst ? 1u : 0u) + (OP == Op2D::Advect ? 2u : 0u);
        mbar_arrive_expect_tx(bar, ntile * tile_bytes);
        tma_load_2d(bufA, &map_src, gx0, gy0, bar);
        if (stage_dst) tma_load_2d(bufB, &map_dst, gx0, gy0, bar);
        if (OP == Op2D::Advect) {
          tma_load_2d(bufU, &map_u, gx0, gy0, bar);
          tma_load_2d(bufV, &map_v, gx0, gy0, bar);
        }
      }
      int ok = 1;
      if (tid == 0) ok = mbar_wait_bounded(bar, phase, p.err) ? 1 : 0;
      phase ^= 1u;
      if (!__syncthreads_and(ok)) return;
    } else {
      coop_load(bufA, src, gy0, gx0, LW, LH, p.W, p.H, p.pitch);
      if (stage_dst) coop_load(bufB, static_cast<const TS*>(p.dst), gy0, gx0, LW, LH, p.W, p.H, p.pitch);
      if (OP == Op2D::Advect) {
        coop_load(bufU, static_cast<const TS*>(p.u), gy0, gx0, LW, LH, p.W, p.H, p.pitch);
        coop_load(bufV, static_cast<const TS*>(p.v), gy0, gx0, LW, LH, p.W, p.H, p.pitch);
      }
      __syncthreads();
    }

    for (int s = 1; s <= p.steps; ++s) {
      const TS* in = (s & 1) ? bufA : bufB;
      TS* out = (s & 1) ? bufB : bufA;
      const int e = p.R * (p.steps - s);
      const int y_lo = p.HY - e, y_hi = p.HY + p.TH + e;
      const int x_lo = p.HX - e, x_hi = p.HX + p.TW + e;
      for (int y = y_lo + warp; y < y_hi; y += kWarps) {
        const int gy = gy0 + y;
        const bool row_in = (gy >= p.ring) && (gy < p.H - p.ring);
        for (int x = x_lo + lane; x < x_hi; x += 32) {
          const int idx = y * LW + x;
          const int gx = gx0 + x;
          if (row_in && gx >= p.ring && gx < p.W - p.ring) {
            float v;
            if constexpr (OP == Op2D::Linear) {
              v = linear_value<TS, NM>(in, idx, p, s_off, s_wt);
            } else {
              v = advect_value<TS>(in, bufU, bufV, idx, LW, p);
            }
            out[idx] = S::store(v);
          }
        }
      }
      __syncthreads();
    }

    // core -> global, interior cells only
    const TS* fin = (p.steps & 1) ? bufB : bufA;
    const int vec_per_row = p.TW / kVec;
    for (int i = tid; i < p.TH * vec_per_row; i += kStencil2DThreads) {
      const int r = i / vec_per_row;
      const int cv = i - r * vec_per_row;
      const int y = p.HY + r, x = p.HX + cv * kVec;
      const int gy = gy0 + y, gx = gx0 + x;
      if (gy < p.ring || gy >= p.H - p.ring) continue;
      if (gx + kVec <= p.ring || gx >= p.W - p.ring) continue;
      TS* d = dst + static_cast<int64_t>(gy) * p.pitch + gx;
      const TS* sp = fin + y * LW + x;
      if (gx >= p.ring && gx + kVec <= p.W - p.ring && (reinterpret_cast<uintptr_t>(d) & 15) == 0) {
        *reinterpret_cast<uint4*>(d) = *reinterpret_cast<const uint4*>(sp);
      } else {
#pragma unroll
        for (int k = 0; k < kVec; ++k) {
          const int xx = gx + k;
          if (xx >= p.ring && xx < p.W - p.ring) d[k] = sp[k];
        }
      }
    }
    __syncthreads();
  }
}

template <class TS, Op2D OP, bool kTma, int NM>
cudaError_t launch_one(const CUtensorMap* ms, const CUtensorMap* md, const CUtensorMap* mu, const CUtensorMap* mv,
                       const Stencil2DParams& p, int ctas, cudaStream_t s) {
  const size_t smem = Layout<TS, OP>::total(p.LW, p.LH);
  auto kern = stencil2d_kernel<TS, OP, kTma, NM>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  kern<<<ctas, kStencil2DThreads, smem, s>>>(*ms, *md, *mu, *mv, p);
  return cudaGetLastError();
}

template <class TS, Op2D OP, bool kTma>
cudaError_t dispatch_nm(const CUtensorMap* ms, const CUtensorMap* md, const CUtensorMap* mu, const CUtensorMap* mv,
                        const Stencil2DParams& p, int ctas, cudaStream_t s) {
  if (OP == Op2D::Advect) return launch_one<TS, OP, kTma, 0>(ms, md, mu, mv, p, ctas, s);
  switch (p.nm) {
    case 4: return launch_one<TS, OP, kTma, 4>(ms, md, mu, mv, p, ctas, s);
    case 5: return launch_one<TS, OP, kTma, 5>(ms, md, mu, mv, p, ctas, s);
    case 9: return launch_one<TS, OP, kTma, 9>(ms, md, mu, mv, p, ctas, s);
    default: return launch_one<TS, OP, kTma, 0>(ms, md, mu, mv, p, ctas, s);
  }
}

template <class TS, Op2D OP>
cudaError_t dispatch_tma(bool tma, const CUtensorMap* ms, const CUtensorMap* md, const CUtensorMap* mu,
                         const CUtensorMap* mv,
                         const Stencil2DParams& p, int ctas, cudaStream_t s) {
  return tma ? dispatch_nm<TS, OP, true>(ms, md, mu, mv, p, ctas, s) : dispatch_nm<TS, OP, false>(ms, md, mu, mv, p, ctas, s);
}

}  // namespace

size_t stencil2d_smem_bytes(Op2D op, int dtype, int LW, int LH) {
  if (dtype == 2) {
    return op == Op2D::Advect ? Layout<__nv_bfloat16, Op2D::Advect>::total(LW, LH)
                              : Layout<__nv_bfloat16, Op2D::Linear>::total(LW, LH);
  }
  return op == Op2D::Advect ? Layout<float, Op2D::Advect>::total(LW, LH) : Layout<float, Op2D::Linear>::total(LW, LH);
}

int stencil2d_max_ctas_per_sm(Op2D op, int dtype, int nm, int LW, int LH) {
  const size_t smem = stencil2d_smem_bytes(op, dtype, LW, LH);
  int dev = 0;
  cudaGetDevice(&dev);
  int per_sm = 0;
  cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  int per_block = 0;
  cudaDeviceGetAttribute(&per_block, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (smem > static_cast<size_t>(per_block)) return 0;
  // each CTA also reserves ~1 KB of system shared memory and 256 B of static arrays
  const int by_smem = static_cast<int>(per_sm / (smem + 1024 + 2 * kMaxMask2D * 4));
  const int by_threads = 2048 / kStencil2DThreads;
  (void)nm;
  return by_smem < by_threads ? by_smem : by_threads;
}

cudaError_t stencil2d_pass(Op2D op, int dtype, bool use_tma, const CUtensorMap* map_src, const CUtensorMap* map_dst,
                           const CUtensorMap* map_u,
                           const CUtensorMap* map_v, const Stencil2DParams& p, int ctas, cudaStream_t s) {
  if (dtype == 2) {
    return op == Op2D::Advect
               ? dispatch_tma<__nv_bfloat16, Op2D::Advect>(use_tma, map_src, map_dst, map_u, map_v, p, ctas, s)
               : dispatch_tma<__nv_bfloat16, Op2D::Linear>(use_tma, map_src, map_dst, map_u, map_v, p, ctas, s);
  }
  return op == Op2D::Advect ? dispatch_tma<float, Op2D::Advect>(use_tma, map_src, map_dst, map_u, map_v, p, ctas, s)
                            : dispatch_tma<float, Op2D::Linear>(use_tma, map_src, map_dst, map_u, map_v, p, ctas, s);
}

}  // namespace pskel
