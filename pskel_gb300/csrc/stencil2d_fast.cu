// 2D fp32 / bf16-storage stencils of reach 1 with a known mask shape
// (weights at run time) and the advection-diffusion op: register-windowed
// temporal blocking.
//
// Same tiling and semantics as stencil2d.cu (TMA-staged halo tiles, T steps
// per pass ping-ponging between two shared buffers, the destination's ring
// staged for ring tiles, interior cells only written back), but each thread
// owns one 4-cell column vector of a strip of S rows
// and reads every shared-memory row once per step with one vector load (128
// bits fp32, 64 bits bf16) plus its two edge neighbours, keeping a
// (S + 2)-row window in registers. The tile is 128 cells wide and
// 16 * S + 2 rows high (16 warps of S rows each);
// every step computes the whole tile minus its outer row, and garbage from the
// tile edges advances one cell per step into the halo, which the core never
// reaches in T <= halo steps.
//
// Arithmetic is the oracle's: products and sums in mask order with
// __fmul_rn/__fadd_rn (no contraction), bf16 results rounded every step.
#include "common.cuh"
#include "kernels.h"

namespace pskel {
namespace {

template <class TS>
struct Vec;
template <>
struct Vec<float> {
  static constexpr int N = 4;
};
template <>
struct Vec<__nv_bfloat16> {
  static constexpr int N = 4;
};

__device__ __forceinline__ void ld_vec(const float* p, float* r) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  r[0] = v.x;
  r[1] = v.y;
  r[2] = v.z;
  r[3] = v.w;
}
__device__ __forceinline__ void ld_vec(const __nv_bfloat16* p, float* r) {
  const uint2 v = *reinterpret_cast<const uint2*>(p);
  r[0] = __uint_as_float(v.x << 16);
  r[1] = __uint_as_float(v.x & 0xFFFF0000u);
  r[2] = __uint_as_float(v.y << 16);
  r[3] = __uint_as_float(v.y & 0xFFFF0000u);
}
__device__ __forceinline__ void st_vec(float* p, const float* r) {
  *reinterpret_cast<float4*>(p) = make_float4(r[0], r[1], r[2], r[3]);
}
__device__ __forceinline__ void st_vec(__nv_bfloat16* p, const float* r) {
  const uint32_t a = __bfloat16_as_ushort(__float2bfloat16_rn(r[0]));
  const uint32_t b = __bfloat16_as_ushort(__float2bfloat16_rn(r[1]));
  const uint32_t c = __bfloat16_as_ushort(__float2bfloat16_rn(r[2]));
  const uint32_t d = __bfloat16_as_ushort(__float2bfloat16_rn(r[3]));
  *reinterpret_cast<uint2*>(p) = make_uint2(a | (b << 16), c | (d << 16));
}
__device__ __forceinline__ float ld1(const float* p) { return *p; }
__device__ __forceinline__ float ld1(const __nv_bfloat16* p) { return __bfloat162float(*p); }

// Mask shapes of reach 1, entries in summation order.
template <int K>
struct Shape {
  int n;
  int dh[9];
  int dw[9];
};
template <int K>
__host__ __device__ constexpr Shape<K> shape_of() {
  if constexpr (K == 0) return Shape<0>{4, {-1, 1, 0, 0}, {0, 0, -1, 1}};
  if constexpr (K == 1) return Shape<1>{5, {0, -1, 1, 0, 0}, {0, 0, 0, -1, 1}};
  if constexpr (K == 2) return Shape<2>{9, {-1, -1, -1, 0, 0, 0, 1, 1, 1}, {-1, 0, 1, -1, 0, 1, -1, 0, 1}};
}

// OpK: 0..2 linear shapes above, 3 = advection.
constexpr int kFastThreads = 512;
constexpr int kFastBufs = 3;  // rotating tile buffers: source, partner, next source

// Wind vector at (gy, gx..gx+3) straight from global memory (read-only path;
// the tile's winds stay in L1 across the steps of a pass). Zero outside the grid.
template <class TS>
__device__ __forceinline__ void ld_wind(const TS* f, int64_t pitch, int gy, int gx, int W, int H, float* r) {
  if (gy >= 0 && gy < H && gx >= 0 && gx + 4 <= W) {
    const TS* q = f + static_cast<int64_t>(gy) * pitch + gx;
    if constexpr (sizeof(TS) == 4) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(q));
      r[0] = v.x;
      r[1] = v.y;
      r[2] = v.z;
      r[3] = v.w;
    } else {
      const uint2 v = __ldg(reinterpret_cast<const uint2*>(q));
      r[0] = __uint_as_float(v.x << 16);
      r[1] = __uint_as_float(v.x & 0xFFFF0000u);
      r[2] = __uint_as_float(v.y << 16);
      r[3] = __uint_as_float(v.y & 0xFFFF0000u);
    }
  } else {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int x = gx + c;
      r[c] = (gy >= 0 && gy < H && x >= 0 && x < W) ? ld1(f + static_cast<int64_t>(gy) * pitch + x) : 0.0f;
    }
  }
}

template <class TS, int OpK, int S>
__global__ void __launch_bounds__(kFastThreads, S <= 4 ? 2 : 1)
    fast2d_kernel(const __grid_constant__ CUtensorMap map_src, const __grid_constant__ CUtensorMap map_dst,
                  const __grid_constant__ CUtensorMap map_u, const __grid_constant__ CUtensorMap map_v,
                  const __grid_constant__ Stencil2DParams p) {
  constexpr int N = Vec<TS>::N;
  constexpr int LW = 32 * N;
  constexpr int LH = (kFastThreads / 32) * S + 2;
  constexpr bool kAdvect = (OpK == 3);
  constexpr size_t kBuf = (static_cast<size_t>(LW) * LH * sizeof(TS) + 127) & ~size_t(127);
  constexpr uint32_t kTileBytes = static_cast<uint32_t>(LW * LH * sizeof(TS));
  // dynamic shared memory, 128-byte aligned for TMA; derived pointers stay
  // in the shared window (no integer round trip), so accesses compile to
  // shared-memory instructions
  extern __shared__ __align__(128) uint8_t smem_raw[];
  uint8_t* base = smem_raw;
  if ((smem_u32(smem_raw) & 127u) != 0) {
    if (threadIdx.x == 0) atomicOr(p.err, kDevErrAlign);
    return;
  }
  auto buf = [&](int i) { return reinterpret_cast<TS*>(base + static_cast<size_t>(i) * kBuf); };
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + kFastBufs * kBuf);  // one per buffer
  (void)map_u;
  (void)map_v;

  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int x0 = lane * N;           // this thread's column vector
  const int yb = 1 + warp * S;       // first row of this warp's strip
  if (tid == 0) {
    for (int i = 0; i < kFastBufs; ++i) mbar_init(&bars[i], 1);
    fence_barrier_init();
    prefetch_tensormap(&map_src);
    prefetch_tensormap(&map_dst);
  }
  __syncthreads();

  constexpr auto shp = shape_of<(OpK < 3 ? OpK : 0)>();
  float wt[9];
#pragma unroll
  for (int n = 0; n < 9; ++n) wt[n] = (n < shp.n) ? p.wt[n] : 0.0f;

  TS* dst = static_cast<TS*>(p.dst);
  const TS* wu = static_cast<const TS*>(p.u);
  const TS* wv = static_cast<const TS*>(p.v);
  uint32_t phase_bits = 0;  // bit i: parity of the next completion of bars[i]
  const int ntiles = p.tiles_x * p.tiles_y;
  auto origin = [&](int t, int& gy0, int& gx0) {
    const int ty = t / p.tiles_x;
    gy0 = ty * p.TH - p.HY;
    gx0 = (t - ty * p.tiles_x) * p.TW - p.HX;
  };
  auto load = [&](int b, const CUtensorMap* m, int gy0, int gx0) {
    fence_proxy_async();
    mbar_arrive_expect_tx(&bars[b], kTileBytes);
    tma_load_2d(buf(b), m, gx0, gy0, &bars[b]);
  };
  // one thread waits on a buffer's barrier; the block barrier that follows
  // publishes the tile to the other threads
  auto wait1 = [&](int b) -> bool { return mbar_wait_bounded(&bars[b], (phase_bits >> b) & 1u, p.err); };

  if (tid == 0 && static_cast<int>(blockIdx.x) < ntiles) {
    int gy0, gx0;
    origin(blockIdx.x, gy0, gx0);
    load(0, &map_src, gy0, gx0);
  }
  int it = 0;  // tiles processed by this CTA: buffer rotation
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int bs = it % 3, bp = (it + 2) % 3, bn = (it + 1) % 3;  // source, partner, next source
    int gy0, gx0;
    origin(tile, gy0, gx0);
    const bool ring_tile = (gy0 < p.ring) || (gy0 + LH > p.H - p.ring) || (gx0 < p.ring) || (gx0 + LW > p.W - p.ring);
    const bool stage_dst = ring_tile && p.steps >= 2;
    if (tid == 0) {
      // the partner buffer was last read by the previous tile's write-back
      if (stage_dst) load(bp, &map_dst, gy0, gx0);
      const int next = tile + static_cast<int>(gridDim.x);
      if (next < ntiles) {
        int ny0, nx0;
        origin(next, ny0, nx0);
        load(bn, &map_src, ny0, nx0);
      }
    }
    int ok = 1;
    if (tid == 0) ok = (wait1(bs) && (!stage_dst || wait1(bp))) ? 1 : 0;
    phase_bits ^= (1u << bs);
    if (stage_dst) phase_bits ^= (1u << bp);
    if (!__syncthreads_and(ok)) return;

    const int gxv = gx0 + x0;
    for (int s = 1; s <= p.steps; ++s) {
      const TS* in = buf((s & 1) ? bs : bp);
      TS* out = buf((s & 1) ? bp : bs);
      // window: rows yb-1 .. yb+S, each [left, v0..v3, right]; the left and
      // right neighbours come from the adjacent lanes (one warp spans a row)
      float win[S + 2][N + 2];
#pragma unroll
      for (int k = 0; k < S + 2; ++k) {
        ld_vec(in + (yb - 1 + k) * LW + x0, &win[k][1]);
        win[k][0] = __shfl_up_sync(0xFFFFFFFFu, win[k][N], 1);
        win[k][N + 1] = __shfl_down_sync(0xFFFFFFFFu, win[k][1], 1);
      }
#pragma unroll
      for (int k = 1; k <= S; ++k) {
        const int y = yb - 1 + k;
        float res[N];
        if constexpr (!kAdvect) {
#pragma unroll
          for (int c = 0; c < N; ++c) {
            float acc = __fmul_rn(wt[0], win[k + shp.dh[0]][1 + c + shp.dw[0]]);
#pragma unroll
            for (int n = 1; n < shp.n; ++n) acc = __fadd_rn(acc, __fmul_rn(wt[n], win[k + shp.dh[n]][1 + c + shp.dw[n]]));
            res[c] = acc;
          }
        } else {
          float uu[N], vv[N];
          ld_wind(wu, p.pitch, gy0 + y, gxv, p.W, p.H, uu);
          ld_wind(wv, p.pitch, gy0 + y, gxv, p.W, p.H, vv);
#pragma unroll
          for (int c = 0; c < N; ++c) {
            const float cc = win[k][1 + c];
            const float n_ = win[k - 1][1 + c];
            const float e_ = win[k][2 + c];
            const float w_ = win[k][c];
            const float s_ = win[k + 1][1 + c];
            const float sum = __fsub_rn(__fmul_rn(4.0f, cc), __fadd_rn(__fadd_rn(__fadd_rn(n_, e_), w_), s_));
            const float xw = uu[c], yw = vv[c];
            const float cvy = (yw > 0.0f) ? yw : -yw;  // yf * yw with yf = +-1
            const float cvx = (xw > 0.0f) ? xw : -xw;
            const float nbx = (xw > 0.0f) ? e_ : w_;
            const float nby = (yw > 0.0f) ? s_ : n_;
            const float temp_wind = __fsub_rn(__fmul_rn(-cvx, __fmul_rn(__fsub_rn(cc, nbx), p.inv_dx)),
                                              __fmul_rn(cvy, __fmul_rn(__fsub_rn(cc, nby), p.inv_dx)));
            const float cond = __fmul_rn(__fmul_rn(-p.K, __fmul_rn(sum, 0.25f)), p.dt);
            res[c] = __fadd_rn(__fadd_rn(cc, cond), __fmul_rn(temp_wind, p.dt));
          }
        }
        TS* o = out + y * LW + x0;
        if (ring_tile) {
          // cells outside r <= h < H-r, r <= w < W-r keep this buffer's value
          const int gy = gy0 + y;
          const bool row_in = gy >= p.ring && gy < p.H - p.ring;
          float old[N];
          ld_vec(o, old);
#pragma unroll
          for (int c = 0; c < N; ++c) {
            const int gx = gxv + c;
            if (!(row_in && gx >= p.ring && gx < p.W - p.ring)) res[c] = old[c];
          }
        }
        st_vec(o, res);
      }
      __syncthreads();
    }

    // core -> global, interior cells only, vector stores
    const TS* fin = buf((p.steps & 1) ? bp : bs);
    const int vpr = p.TW / N;
    for (int i = tid; i < p.TH * vpr; i += kFastThreads) {
      const int r = i / vpr;
      const int cv = i - r * vpr;
      const int y = p.HY + r, x = p.HX + cv * N;
      const int gy = gy0 + y, gx = gx0 + x;
      if (gy < p.ring || gy >= p.H - p.ring) continue;
      if (gx + N <= p.ring || gx >= p.W - p.ring) continue;
      TS* d = dst + static_cast<int64_t>(gy) * p.pitch + gx;
      const TS* sp = fin + y * LW + x;
      constexpr int kVecBytes = N * static_cast<int>(sizeof(TS));
      if (gx >= p.ring && gx + N <= p.W - p.ring && (reinterpret_cast<uintptr_t>(d) & (kVecBytes - 1)) == 0) {
        if constexpr (kVecBytes == 16)
          *reinterpret_cast<uint4*>(d) = *reinterpret_cast<const uint4*>(sp);
        else
          *reinterpret_cast<uint2*>(d) = *reinterpret_cast<const uint2*>(sp);
      } else {
#pragma unroll
        for (int k = 0; k < N; ++k) {
          const int xx = gx + k;
          if (xx >= p.ring && xx < p.W - p.ring) d[k] = sp[k];
        }
      }
    }
    __syncthreads();
  }
}

template <class TS, int OpK, int S>
cudaError_t launch_fast(const CUtensorMap* ms, const CUtensorMap* md, const CUtensorMap* mu, const CUtensorMap* mv,
                        const Stencil2DParams& p, int ctas, cudaStream_t s) {
  const size_t smem = fast2d_smem_bytes(OpK == 3, sizeof(TS) == 2 ? 2 : 1, S);
  auto kern = fast2d_kernel<TS, OpK, S>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  // persistent CTAs: no more than can be resident (registers or shared memory)
  static int resident = 0;
  if (resident == 0) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFastThreads, smem);
    resident = (per_sm > 0 ? per_sm : 1) * sms;
  }
  if (ctas > resident) ctas = resident;
  kern<<<ctas, kFastThreads, smem, s>>>(*ms, *md, *mu, *mv, p);
  return cudaGetLastError();
}

template <class TS, int S>
cudaError_t dispatch_op(int opk, const CUtensorMap* ms, const CUtensorMap* md, const CUtensorMap* mu,
                        const CUtensorMap* mv, const Stencil2DParams& p, int ctas, cudaStream_t s) {
  switch (opk) {
    case 0: return launch_fast<TS, 0, S>(ms, md, mu, mv, p, ctas, s);
    case 1: return launch_fast<TS, 1, S>(ms, md, mu, mv, p, ctas, s);
    case 2: return launch_fast<TS, 2, S>(ms, md, mu, mv, p, ctas, s);
    default: return launch_fast<TS, 3, S>(ms, md, mu, mv, p, ctas, s);
  }
}

}  // namespace

int fast2d_shape(const int* offsets, int n) {
  for (int k = 0; k < 3; ++k) {
    int sn = 0;
    const int* dh = nullptr;
    const int* dw = nullptr;
    static const int j_dh[4] = {-1, 1, 0, 0}, j_dw[4] = {0, 0, -1, 1};
    static const int c_dh[5] = {0, -1, 1, 0, 0}, c_dw[5] = {0, 0, 0, -1, 1};
    static const int b_dh[9] = {-1, -1, -1, 0, 0, 0, 1, 1, 1}, b_dw[9] = {-1, 0, 1, -1, 0, 1, -1, 0, 1};
    if (k == 0) { sn = 4; dh = j_dh; dw = j_dw; }
    if (k == 1) { sn = 5; dh = c_dh; dw = c_dw; }
    if (k == 2) { sn = 9; dh = b_dh; dw = b_dw; }
    if (sn != n) continue;
    bool same = true;
    for (int i = 0; i < n && same; ++i) same = offsets[2 * i] == dh[i] && offsets[2 * i + 1] == dw[i];
    if (same) return k;
  }
  return -1;
}

size_t fast2d_smem_bytes(bool advect, int dtype, int S) {
  (void)advect;
  const size_t esz = (dtype == 2) ? 2 : 4;
  const size_t lw = 128;
  const size_t lh = 16 * S + 2;
  const size_t buf = (lw * lh * esz + 127) & ~size_t(127);
  return 128 + kFastBufs * buf + 8 * kFastBufs;
}

int fast2d_max_ctas_per_sm(bool advect, int dtype, int S) {
  const size_t smem = fast2d_smem_bytes(advect, dtype, S);
  int dev = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  const int by_smem = static_cast<int>(per_sm / (smem + 1024));
  return by_smem < 8 ? by_smem : 8;
}

cudaError_t fast2d_pass(int opk, int dtype, int S, const CUtensorMap* ms, const CUtensorMap* md,
                        const CUtensorMap* mu, const CUtensorMap* mv, const Stencil2DParams& p, int ctas,
                        cudaStream_t s) {
  if (dtype == 2)
    return S == 8 ? dispatch_op<__nv_bfloat16, 8>(opk, ms, md, mu, mv, p, ctas, s)
                  : dispatch_op<__nv_bfloat16, 4>(opk, ms, md, mu, mv, p, ctas, s);
  return S == 8 ? dispatch_op<float, 8>(opk, ms, md, mu, mv, p, ctas, s)
                : dispatch_op<float, 4>(opk, ms, md, mu, mv, p, ctas, s);
}

}  // namespace pskel
