// 3D weighted-mask stencils (fp32 / bf16 storage), 2.5D streaming with
// temporal blocking, and the fused fp64 residual norm.
//
// Layout is the reference's (PSkelArray.hpp:349-352): element (h, w, d) at
// [(h * W + w) * D + d], d fastest. Every cell is updated; a neighbour outside
// the grid reads the mask's halo value (Mask3D::get, PSkelMask.hpp:186-199;
// Stencil3D::runOpenMP visits every cell, PSkelStencil.hpp:2104-2113).
//
// Each persistent CTA owns a (w, d) tile column and marches along h. For a
// pass of `steps` time steps it keeps, per time level k < steps, a ring of
// 2R+1 planes of the tile window in shared memory. At march position i, level
// 0 receives input plane i (one 3D TMA load of a one-plane box, prefetched a
// plane ahead), and level k computes plane i - k*R from level k-1's planes
// i - k*R - R .. i - k*R + R. Level `steps` goes straight to global memory.
// The (w, d) region computed at level k shrinks by R per level: the halo of
// R*T cells is recomputed redundantly by neighbouring tiles.
//
// Residual: when global step g (1-based) is a multiple of `every`, the CTA
// accumulates sum((u_g - u_{g-1})^2) over its core cells in fp64 and writes
// one partial per (reported step, CTA) to a scratch array; reduce3d_residual
// then adds the partials of each reported step in a fixed order, so the norm
// does not depend on thread timing.
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "kernels.h"

namespace pskel {
namespace {

template <class TS>
__host__ __device__ inline size_t plane_bytes(int LW, int LD) {
  return (static_cast<size_t>(LW) * LD * sizeof(TS) + 127) & ~size_t(127);
}

template <class TS>
__device__ __forceinline__ void fill_plane(TS* pl, int n, TS v) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) pl[i] = v;
}

template <class TS, int NM, bool kTma>
__global__ void __launch_bounds__(kStencil3DThreads)
    stencil3d_kernel(const __grid_constant__ CUtensorMap map_src, const __grid_constant__ Stencil3DParams p) {
  using S = Storage<TS>;
  // dynamic shared memory, 128-byte aligned for TMA; planes are addressed by
  // element offsets from `sm`, so every access is a shared-memory access
  extern __shared__ __align__(128) uint8_t smem_raw[];
  if ((smem_u32(smem_raw) & 127u) != 0) {
    if (threadIdx.x == 0) atomicOr(p.err, kDevErrAlign);
    return;
  }
  TS* sm = reinterpret_cast<TS*>(smem_raw);
  const int LW = p.LW, LD = p.LD, NP = p.NP, R = p.R;
  const int plane_elems = LW * LD;
  const int pe = static_cast<int>(plane_bytes<TS>(LW, LD) / sizeof(TS));  // plane stride in elements
  // level 0 ring has kPrefetch3D extra slots: the next planes load while the
  // current ones are still read; levels 1..steps-1 have NP slots each. Each
  // level-0 slot has its own mbarrier.
  const int NP0 = NP + kPrefetch3D;
  auto level_off = [&](int k, int slot) -> int { return (k == 0 ? slot : NP0 + (k - 1) * NP + slot) * pe; };
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + static_cast<size_t>(NP0 + (p.T - 1) * NP) * pe * sizeof(TS));

  // fp64 residual partials per (level of this pass, warp); each warp adds
  // its own reduced sums in march order, so the partials are deterministic
  __shared__ double s_part[kMax3DSteps][kStencil3DThreads / 32];

  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  constexpr int kWarps = kStencil3DThreads / 32;
  constexpr int kM = NM > 0 ? NM : kMaxMask3D;
  for (int i = tid; i < kMax3DSteps * kWarps; i += kStencil3DThreads) (&s_part[0][0])[i] = 0.0;
  // mask entries in registers: weights, plane offsets dh, in-plane offsets
  float wt[kM];
  int offh[kM], offp[kM];
  const int nm = NM > 0 ? NM : p.nm;
#pragma unroll
  for (int n = 0; n < kM; ++n) {
    wt[n] = n < nm ? p.wt[n] : 0.0f;
    offh[n] = n < nm ? p.off_h[n] : 0;
    offp[n] = n < nm ? p.off_plane[n] : 0;
  }
  if (kTma && tid == 0) {
    for (int b = 0; b < NP0; ++b) mbar_init(&bars[b], 1);
    fence_barrier_init();
    prefetch_tensormap(&map_src);
  }
  __syncthreads();

  const TS halo = S::store(p.halo);
  const TS* src = static_cast<const TS*>(p.src);
  TS* dst = static_cast<TS*>(p.dst);
  const int ncols = p.tiles_w * p.tiles_d;
  const int ntiles = ncols * p.hchunks;
  const int steps = p.steps;
  uint32_t phase_bits = 0;  // bit b: parity of the next completion of bars[b]
  auto wrap = [](int x, int n) { return x < 0 ? x + n : (x >= n ? x - n : x); };  // |x| < 2n
  auto modn = [](int x, int n) { const int r = x % n; return r < 0 ? r + n : r; };

  // Work items: a (w, d) tile column over a chunk [h0, h1) of output planes.
  // The march starts steps * R planes early to warm the level rings up.
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int hc = tile / ncols;
    const int col = tile - hc * ncols;
    const int tw = col / p.tiles_d;
    const int td = col - tw * p.tiles_d;
    const int h0 = hc * p.HC;
    const int h1 = min(p.H, h0 + p.HC);
    const int first = max(0, h0 - steps * R);
    const int last = h1 - 1 + steps * R;
    const int gw0 = tw * p.TW - p.HW;  // global w of local w 0
    const int gd0 = td * p.TD - p.HD;  // global d of local d 0
    const bool edge = (gw0 < 0) || (gw0 + LW > p.W) || (gd0 < 0) || (gd0 + LD > p.D);

    // planes before the grid read the halo value at every level
    for (int k = 0; k < steps; ++k)
      for (int q = -R; q < 0; ++q) {
        TS* pl = sm + level_off(k, modn(q, k == 0 ? NP0 : NP));
        for (int e = tid; e < plane_elems; e += kStencil3DThreads) pl[e] = halo;
      }
    __syncthreads();

    auto issue = [&](int plane) {
      const int b = modn(plane, NP0);
      fence_proxy_async();
      mbar_arrive_expect_tx(&bars[b], static_cast<uint32_t>(plane_elems * sizeof(TS)));
      tma_load_3d(sm + level_off(0, b), &map_src, gd0, gw0, plane, &bars[b]);
    };
    if (kTma && tid == 0)
      for (int j = first; j < first + kPrefetch3D && j < p.H && j <= last; ++j) issue(j);

    int s0 = modn(first, NP0);  // level-0 slot of plane i
    int sN = modn(first, NP);   // plane i modulo NP (levels >= 1)
    for (int i = first; i <= last; ++i, s0 = (s0 + 1 == NP0 ? 0 : s0 + 1), sN = (sN + 1 == NP ? 0 : sN + 1)) {
      // ---- level 0: input plane i
      TS* pl0 = sm + level_off(0, s0);
      if (i < p.H && !kTma) {
        for (int e = tid; e < plane_elems; e += kStencil3DThreads) {
          const int lw = e / LD, ld = e - lw * LD;
          const int gw = gw0 + lw, gd = gd0 + ld;
          pl0[e] = (gw < 0 || gw >= p.W || gd < 0 || gd >= p.D) ? halo
                                                                : src[(static_cast<int64_t>(i) * p.W + gw) * p.D + gd];
        }
      } else if (i < p.H) {
        // one thread waits for the plane; the barrier below publishes it
        int ok = 1;
        if (tid == 0) {
          ok = mbar_wait_bounded(&bars[s0], (phase_bits >> s0) & 1u, p.err) ? 1 : 0;
        }
        phase_bits ^= (1u << s0);
        if (!__syncthreads_and(ok)) return;
        if (edge && S::load(halo) != 0.0f) {
          for (int e = tid; e < plane_elems; e += kStencil3DThreads) {
            const int lw = e / LD, ld = e - lw * LD;
            const int gw = gw0 + lw, gd = gd0 + ld;
            if (gw < 0 || gw >= p.W || gd < 0 || gd >= p.D) pl0[e] = halo;
          }
        }
      } else {
        for (int e = tid; e < plane_elems; e += kStencil3DThreads) pl0[e] = halo;
      }
      __syncthreads();
      // plane i+P's slot held plane i+P-NP0 = i-2R-1, which no level reads any more
      if (kTma && tid == 0 && i + kPrefetch3D < p.H && i + kPrefetch3D <= last) issue(i + kPrefetch3D);

      // ---- levels 1..steps
      for (int k = 1; k <= steps; ++k) {
        const int q = i - k * R;
        // planes this level must produce for the chunk's output planes
        if (q < max(0, h0 - (steps - k) * R) || q >= h1 + (steps - k) * R) continue;
        // slot of plane q at level k (q mod NP) and at level k-1
        const int slot_q = modn(sN - k * R, NP);
        const int slot_q0 = modn(i - k * R, NP0);  // for level 0 (NP0 slots)
        if (k < steps && q >= p.H) {
          TS* pl = sm + level_off(k, slot_q);
          for (int e = tid; e < plane_elems; e += kStencil3DThreads) pl[e] = halo;
          __syncthreads();
          continue;
        }
        if (q >= p.H) continue;
        const int e = R * (steps - k);
        const int w_lo = p.HW - e, w_hi = p.HW + p.TW + e;
        const int d_lo = p.HD - e, d_hi = p.HD + p.TD + e;
        // neighbour planes q + dh of level k-1, as element offsets
        int nb[kM];
#pragma unroll
        for (int n = 0; n < kM; ++n) {
          if (n < nm) {
            const int sl = (k == 1) ? wrap(slot_q0 + offh[n], NP0) : wrap(slot_q + offh[n], NP);
            nb[n] = level_off(k - 1, sl) + offp[n];
          }
        }
        const int prev = level_off(k - 1, k == 1 ? slot_q0 : slot_q);
        const int outo = (k < steps) ? level_off(k, slot_q) : 0;
        const bool report = p.every > 0 && ((p.step0 + k) % p.every) == 0 && q >= h0 && q < h1;
        double acc_res = 0.0;
        for (int lw = w_lo + warp; lw < w_hi; lw += kWarps) {
          const int gw = gw0 + lw;
          const bool w_in = gw >= 0 && gw < p.W;
          const bool w_core = lw >= p.HW && lw < p.HW + p.TW;
          for (int ld = d_lo + lane; ld < d_hi; ld += 32) {
            const int gd = gd0 + ld;
            const int idx = lw * LD + ld;
            TS v;
            if (w_in && gd >= 0 && gd < p.D) {
              float acc = __fmul_rn(wt[0], S::load(sm[nb[0] + idx]));
#pragma unroll
              for (int n = 1; n < kM; ++n)
                if (n < nm) acc = __fadd_rn(acc, __fmul_rn(wt[n], S::load(sm[nb[n] + idx])));
              v = S::store(acc);
              const bool core = w_core && ld >= p.HD && ld < p.HD + p.TD;
              if (core) {
                if (report) {
                  const double dlt = static_cast<double>(S::load(v)) - static_cast<double>(S::load(sm[prev + idx]));
                  acc_res += dlt * dlt;
                }
                if (k == steps) dst[(static_cast<int64_t>(q) * p.W + gw) * p.D + gd] = v;
              }
            } else {
              v = halo;
            }
            if (k < steps) sm[outo + idx] = v;
          }
        }
        if (report) {
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) acc_res += __shfl_down_sync(0xFFFFFFFFu, acc_res, o);
          if (lane == 0) s_part[k - 1][warp] += acc_res;
        }
        __syncthreads();
      }
    }
    __syncthreads();
  }

  // ---- fp64 residual partials: one per (reported level, CTA)
  if (p.every > 0 && tid == 0) {
    for (int k = 1; k <= steps; ++k) {
      if (((p.step0 + k) % p.every) != 0) continue;
      double t = 0.0;
      for (int w = 0; w < kWarps; ++w) t += s_part[k - 1][w];
      p.partials[static_cast<size_t>(k - 1) * gridDim.x + blockIdx.x] = t;
    }
  }
}

// One step without temporal blocking: each thread owns a (w, d) column of a
// 32 x 8 block and marches along a chunk of h, reading its neighbours through
// the read-only cache (the three planes a block touches stay in L1), so every
// cell is read from DRAM about once and written once. Lanes run along d, the
// contiguous axis, so every load and store of a warp is one 128-byte line.
template <class TS, int NM>
__global__ void __launch_bounds__(256)
    stream3d_kernel(const __grid_constant__ Stencil3DParams p) {
  using S = Storage<TS>;
  constexpr int kM = NM > 0 ? NM : kMaxMask3D;
  __shared__ double s_part[8];
  const int nm = NM > 0 ? NM : p.nm;
  float wt[kM];
  int oh[kM], ow[kM], od[kM];
  int64_t off[kM];
  const int64_t plane = static_cast<int64_t>(p.W) * p.D;
#pragma unroll
  for (int n = 0; n < kM; ++n) {
    wt[n] = n < nm ? p.wt[n] : 0.0f;
    oh[n] = n < nm ? p.off_h[n] : 0;
    ow[n] = n < nm ? p.off_w[n] : 0;
    od[n] = n < nm ? p.off_d[n] : 0;
    off[n] = oh[n] * plane + static_cast<int64_t>(ow[n]) * p.D + od[n];
  }
  const TS* __restrict__ src = static_cast<const TS*>(p.src);
  TS* __restrict__ dst = static_cast<TS*>(p.dst);
  const float halo = p.halo;
  const int d = blockIdx.x * 32 + (threadIdx.x & 31);
  const int w = blockIdx.y * 8 + (threadIdx.x >> 5);
  const int h0 = blockIdx.z * p.HC;
  const int h1 = min(p.H, h0 + p.HC);
  const bool col_ok = d < p.D && w < p.W;
  // columns whose every neighbour column is inside the grid skip the checks
  const bool col_inner = col_ok && d >= p.R && d + p.R < p.D && w >= p.R && w + p.R < p.W;
  const bool report = p.every > 0 && ((p.step0 + 1) % p.every) == 0;
  double acc_res = 0.0;
  if (col_ok) {
    for (int h = h0; h < h1; ++h) {
      const int64_t c = h * plane + static_cast<int64_t>(w) * p.D + d;
      float acc;
      if (col_inner && h >= p.R && h + p.R < p.H) {
        acc = __fmul_rn(wt[0], S::load(__ldg(src + c + off[0])));
#pragma unroll
        for (int n = 1; n < kM; ++n)
          if (n < nm) acc = __fadd_rn(acc, __fmul_rn(wt[n], S::load(__ldg(src + c + off[n]))));
      } else {
        acc = 0.0f;
#pragma unroll
        for (int n = 0; n < kM; ++n) {
          if (n < nm) {
            const unsigned hh = static_cast<unsigned>(h + oh[n]), ww = static_cast<unsigned>(w + ow[n]);
            const unsigned dd = static_cast<unsigned>(d + od[n]);
            const bool in = hh < static_cast<unsigned>(p.H) && ww < static_cast<unsigned>(p.W) &&
                            dd < static_cast<unsigned>(p.D);
            const float v = in ? S::load(__ldg(src + c + off[n])) : halo;
            const float t = __fmul_rn(wt[n], v);
            acc = (n == 0) ? t : __fadd_rn(acc, t);
          }
        }
      }
      const TS out = S::store(acc);
      dst[c] = out;
      if (report) {
        const double dl = static_cast<double>(S::load(out)) - static_cast<double>(S::load(__ldg(src + c)));
        acc_res += dl * dl;
      }
    }
  }
  if (p.every > 0) {
    // deterministic: fixed shuffle tree per warp, warps added in order
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc_res += __shfl_down_sync(0xFFFFFFFFu, acc_res, o);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = acc_res;
    __syncthreads();
    if (threadIdx.x == 0 && report) {
      double t = 0.0;
      for (int i = 0; i < 8; ++i) t += s_part[i];
      const int cta = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
      p.partials[cta] = t;
    }
  }
}

// The 7-point cross (centre, h-1, h+1, w-1, w+1, d-1, d+1, summed in that
// order), one step per launch, with the planes staged in shared memory by TMA.
// A persistent block owns work items of 32 vectors of d (128 fp32 / 256 bf16
// cells) x 16 w rows x p.HC planes. A producer warp streams the planes h0-1 ..
// h1 of its items, one 3D TMA copy per plane of the 34-vector x 18-row box
// (a vector and a row of halo on each side; positions outside the grid are
// zero-filled), into a ring of slots. Each slot has a "full"
// mbarrier (the copy landed) and an "empty" one (all consumer warps have read
// it), so consumer warps run independently of each other, up to the ring's
// depth. Every wait is bounded. With a zero halo value the zero fill is the
// halo; otherwise out-of-grid positions are replaced by it. A consumer warp
// owns kRW consecutive w rows of the item (16 / kRW consumer warps): more rows
// per warp convert and load each staged row fewer times per output cell, and
// spread the per-plane waits over more cells: with 4 rows the issue-bound bf16
// variant runs 8 % faster than with 2, the HBM-bound fp32 one the same.
constexpr int kS3BoxX = 34;                 // 16-byte vectors per staged row
constexpr int kS3RowBytes = kS3BoxX * 16;   // 544
constexpr int kS3BoxY = 18;                 // 16 rows + one each side
constexpr int kS3PlaneBytes = (kS3RowBytes * kS3BoxY + 127) & ~127;
constexpr int kS3MaxConsumers = 8;

// Ring depth and residency per storage type, measured on GB300 (512^3 heat):
// fp32 is HBM-bound and gains from a fourth resident block (4 slots, 4 blocks
// per SM: 93 % of the measured copy bandwidth against 80 % with 6 slots and 3
// blocks); bf16 is issue-bound and needs the registers of 3 blocks (6 slots).
template <class TS>
struct S3Rows {
  static constexpr int kRW = 4;                            // w rows per consumer warp
  static constexpr int kCons = 16 / kRW;                   // consumer warps
  static constexpr int kThreads = 32 * (kCons + 1);        // + the producer warp
  static constexpr int kSlots = sizeof(TS) == 4 ? 4 : 6;   // staged planes in the ring
  static constexpr int kMinBlocks = sizeof(TS) == 4 ? 4 : 3;
  static constexpr size_t kSmem = kSlots * static_cast<size_t>(kS3PlaneBytes) + 16 * kSlots;
};


// barrier among the consumer warps only (the producer warp may have left)
template <int kCons>
__device__ __forceinline__ void consumers_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(32 * kCons) : "memory");
}

template <class TS, bool kReport, bool kZeroHalo>
__global__ void __launch_bounds__(S3Rows<TS>::kThreads, S3Rows<TS>::kMinBlocks)
    stream3d_tma_kernel(const __grid_constant__ CUtensorMap map, const __grid_constant__ Stencil3DParams p) {
  using S = Storage<TS>;
  using Vt = Vec16<TS>;
  constexpr int V = Vt::V;
  constexpr int kRW = S3Rows<TS>::kRW;
  constexpr int kS3Consumers = S3Rows<TS>::kCons;
  constexpr int kS3Slots = S3Rows<TS>::kSlots;
  extern __shared__ __align__(128) uint8_t smem_raw[];
  __shared__ double s_part[kS3MaxConsumers];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if ((smem_u32(smem_raw) & 127u) != 0) {
    if (tid == 0) atomicOr(p.err, kDevErrAlign);
    return;
  }
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + kS3Slots * kS3PlaneBytes);
  uint64_t* empty = full + kS3Slots;
  if (tid == 0) {
    for (int i = 0; i < kS3Slots; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], kS3Consumers);
    }
    fence_barrier_init();
  }
  __syncthreads();

  const int H = p.H, W = p.W, D = p.D;
  const int hbeg = p.hbeg, hend = p.hend > 0 ? p.hend : H;  // planes written by this launch
  const int dblocks = (D + 32 * V - 1) / (32 * V), wblocks = (W + 15) / 16;
  const int64_t items = static_cast<int64_t>(dblocks) * wblocks * p.hchunks;
  auto geometry = [&](int64_t it, int& d0, int& w0, int& h0, int& h1) {
    const int db = static_cast<int>(it % dblocks);
    const int64_t r = it / dblocks;
    d0 = db * 32 * V;
    w0 = static_cast<int>(r % wblocks) * 16;
    h0 = hbeg + static_cast<int>(r / wblocks) * p.HC;
    h1 = min(hend, h0 + p.HC);
  };

  if (warp == kS3Consumers) {
    // ---- producer: planes h0-1 .. h1 of every item, in order
    if (lane == 0) {
      prefetch_tensormap(&map);
      int slot = 0;
      uint32_t use = 0;
      for (int64_t it = blockIdx.x; it < items; it += gridDim.x) {
        int d0, w0, h0, h1;
        geometry(it, d0, w0, h0, h1);
        // the map addresses the grid as 32-bit words (a box row of 136 words)
        const int x = (d0 - V) * static_cast<int>(sizeof(TS)) / 4;
        for (int q = h0 - 1; q <= h1; ++q) {
          if (use > 0 && !mbar_wait_bounded(&empty[slot], (use - 1) & 1u, p.err)) return;
          fence_proxy_async();
          mbar_arrive_expect_tx(&full[slot], static_cast<uint32_t>(kS3RowBytes * kS3BoxY));
          tma_load_3d(smem_raw + slot * kS3PlaneBytes, &map, x, w0 - 1, q, &full[slot]);
          if (++slot == kS3Slots) {
            slot = 0;
            ++use;
          }
        }
      }
    }
    return;
  }

  // ---- consumers
  const int64_t plane = static_cast<int64_t>(W) * D;
  TS* __restrict__ dst = static_cast<TS*>(p.dst);
  const float halo = p.halo;
  uint32_t hraw;
  if constexpr (sizeof(TS) == 4) {
    hraw = __float_as_uint(halo);
  } else {
    const uint32_t hb = __bfloat16_as_ushort(__float2bfloat16_rn(halo));
    hraw = hb | (hb << 16);
  }
  // this thread's staged rows: row 0 of the box is w0-1
  const int r0 = kRW * warp + 1;
  const uint8_t* const sbase = smem_raw;
  const int o_row0 = r0 * kS3RowBytes + (lane + 1) * 16;
  const EdgeCell<TS> edge(lane);  // d0-1 (lane 0) and d0+32V (lane 31) of a staged row
  const int o_el = r0 * kS3RowBytes + (V - 1) * static_cast<int>(sizeof(TS));  // d0-1
  const int o_er = r0 * kS3RowBytes + 33 * 16;                                  // d0+32V
  SqDiffAcc acc_res;
  double acc_total = 0.0;
  float2 wt2[5];
#pragma unroll
  for (int n = 0; n < 5; ++n) wt2[n] = make_float2(p.wt[n], p.wt[n]);
  const float2 nz = neg_zero2(p.fuse_guard);
  auto ld = [&](int slot, int off, Vt& v) {
    const uint4 x = *reinterpret_cast<const uint4*>(sbase + slot * kS3PlaneBytes + off);
    v.r[0] = x.x;
    v.r[1] = x.y;
    v.r[2] = x.z;
    v.r[3] = x.w;
  };
  auto ld1 = [&](int slot, int off) -> float {
    return S::load(*reinterpret_cast<const TS*>(sbase + slot * kS3PlaneBytes + off));
  };
  auto next = [](int s) { return s + 1 == kS3Slots ? 0 : s + 1; };
  bool alive = true;
  // slot and phase parity of the next plane in the sequence
  int s_next = 0;
  uint32_t ph_next = 0;
  auto wait_full = [&](int slot, uint32_t ph) -> bool { return mbar_wait_bounded(&full[slot], ph, p.err); };

  for (int64_t it = blockIdx.x; it < items && alive; it += gridDim.x) {
    int d0, w0, h0, h1;
    geometry(it, d0, w0, h0, h1);
    const int d = d0 + lane * V;
    const int w = w0 + warp * kRW;
    const bool d_ok = d < D;
    bool row_ok[kRW];
#pragma unroll
    for (int j = 0; j < kRW; ++j) row_ok[j] = d_ok && w + j < W;
    // general halo: which staged values lie outside the grid
    const bool wm_in = row_ok[0] && w > 0, wp_in = row_ok[kRW - 1] && w + kRW < W;
    const bool el_in = d0 > 0, er_in = d0 + 32 * V < D;
    int s_dn = s_next, s_cur = next(s_dn), s_up = next(s_cur);
    uint32_t ph_dn = ph_next, ph_cur = ph_next ^ (s_cur == 0 ? 1u : 0u), ph_up = ph_cur ^ (s_up == 0 ? 1u : 0u);
    if (!wait_full(s_dn, ph_dn) || !wait_full(s_cur, ph_cur)) {
      alive = false;
      break;
    }
    for (int h = h0; h < h1; ++h) {
      if (!wait_full(s_up, ph_up)) {
        alive = false;
        break;
      }
      Vt dn[kRW], cur[kRW], up[kRW], wm, wp;
#pragma unroll
      for (int j = 0; j < kRW; ++j) {
        ld(s_dn, o_row0 + j * kS3RowBytes, dn[j]);
        ld(s_cur, o_row0 + j * kS3RowBytes, cur[j]);
        ld(s_up, o_row0 + j * kS3RowBytes, up[j]);
      }
      ld(s_cur, o_row0 - kS3RowBytes, wm);
      ld(s_cur, o_row0 + kRW * kS3RowBytes, wp);
      // lane 0: cell d0-1 of row j (el); lane 31: cell d0+32V (er). bf16 rows
      // take one load and permute per lane (EdgeCell): 1383 against 1305
      // GCells/s on 512^3; fp32 rows, bound by HBM, keep the two predicated
      // loads, which measured 785 against 746.
      float el[kRW], er[kRW];
      if constexpr (sizeof(TS) == 2) {
#pragma unroll
        for (int j = 0; j < kRW; ++j) {
          el[j] = edge.get(sbase + s_cur * kS3PlaneBytes + (r0 + j) * kS3RowBytes);
          er[j] = el[j];
        }
      } else {
#pragma unroll
        for (int j = 0; j < kRW; ++j) {
          el[j] = 0.0f;
          er[j] = 0.0f;
        }
        if (lane == 0) {
#pragma unroll
          for (int j = 0; j < kRW; ++j) el[j] = ld1(s_cur, o_el + j * kS3RowBytes);
        }
        if (lane == 31) {
#pragma unroll
          for (int j = 0; j < kRW; ++j) er[j] = ld1(s_cur, o_er + j * kS3RowBytes);
        }
      }
      // plane h-1 is read for the last time
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s_dn]);
      if constexpr (!kZeroHalo) {
#pragma unroll
        for (int j = 0; j < kRW; ++j) {
          if (h - 1 < 0) dn[j].fill(hraw);
          if (h + 1 >= H) up[j].fill(hraw);
          if (!row_ok[j]) {
            dn[j].fill(hraw);
            cur[j].fill(hraw);
            up[j].fill(hraw);
          }
          if (!el_in) el[j] = halo;
          if (!er_in) er[j] = halo;
        }
        if (!wm_in) wm.fill(hraw);
        if (!wp_in) wp.fill(hraw);
      }
      TS* out = dst + (h * plane + static_cast<int64_t>(w) * D + d);
#pragma unroll
      for (int j = 0; j < kRW; ++j) {
        float dl = __shfl_up_sync(0xFFFFFFFFu, cur[j].at(V - 1), 1);
        float dr = __shfl_down_sync(0xFFFFFFFFu, cur[j].at(0), 1);
        if (lane == 0) dl = el[j];
        if (lane == 31) dr = er[j];
        const Vt& a = (j == 0) ? wm : cur[j > 0 ? j - 1 : 0];
        const Vt& b = (j == kRW - 1) ? wp : cur[j < kRW - 1 ? j + 1 : 0];
        float res[V], stored[V];
        cross7_row<sizeof(TS) == 2>(p.wt, wt2, nz, cur[j], dn[j], up[j], a, b, dl, dr, res);
        uint32_t o[4];
        if constexpr (sizeof(TS) == 4) {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            o[k] = __float_as_uint(res[k]);
            stored[k] = res[k];
          }
        } else {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const __nv_bfloat162 bb = __floats2bfloat162_rn(res[2 * k], res[2 * k + 1]);
            o[k] = *reinterpret_cast<const uint32_t*>(&bb);
            stored[2 * k] = __uint_as_float(o[k] << 16);
            stored[2 * k + 1] = __uint_as_float(o[k] & 0xFFFF0000u);
          }
        }
        if (kReport && row_ok[j]) {
#pragma unroll
          for (int k = 0; k < V; ++k) acc_res.add(stored[k], cur[j].at(k));
        }
        if (row_ok[j]) *reinterpret_cast<uint4*>(out + j * D) = make_uint4(o[0], o[1], o[2], o[3]);
      }
      if (kReport) acc_res.flush(acc_total);
      s_dn = s_cur;
      ph_dn = ph_cur;
      s_cur = s_up;
      ph_cur = ph_up;
      s_up = next(s_up);
      ph_up ^= (s_up == 0) ? 1u : 0u;
    }
    if (!alive) break;
    // planes h1-1 and h1 are released at the end of the item
    __syncwarp();
    if (lane == 0) {
      mbar_arrive(&empty[s_dn]);
      mbar_arrive(&empty[s_cur]);
    }
    s_next = s_up;
    ph_next = ph_up;
  }
  if constexpr (kReport) {
    double v = acc_total;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    if (lane == 0) s_part[warp] = v;
    consumers_sync<kS3Consumers>();
    if (tid == 0) {
      double t = 0.0;
      for (int i = 0; i < kS3Consumers; ++i) t += s_part[i];
      p.partials[blockIdx.x] = t;
    }
  }
}

// Sums the per-CTA partials of each reported step in CTA order and stores
// the square root at residuals[slot0 + j].
__global__ void reduce3d_residual(const double* __restrict__ partials, int nctas, int steps, int64_t step0, int every,
                                  double* __restrict__ residuals) {
  const int k = blockIdx.x + 1;  // level within the pass
  if (k > steps || ((step0 + k) % every) != 0) return;
  __shared__ double s[256];
  double t = 0.0;
  // fixed assignment of partials to threads and a fixed tree: deterministic
  for (int c = threadIdx.x; c < nctas; c += blockDim.x) t += partials[static_cast<size_t>(k - 1) * nctas + c];
  s[threadIdx.x] = t;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) residuals[(step0 + k) / every - 1] = sqrt(s[0]);
}

// Adds the CTA partials of one reported step to *acc (fixed order).
__global__ void reduce3d_accumulate(const double* __restrict__ partials, int nctas, double* __restrict__ acc) {
  __shared__ double s[256];
  double t = 0.0;
  for (int c = threadIdx.x; c < nctas; c += blockDim.x) t += partials[c];
  s[threadIdx.x] = t;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *acc += s[0];
}

__global__ void finish3d_residuals(const double* __restrict__ acc, int n, double* __restrict__ residuals) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) residuals[i] = sqrt(acc[i]);
}

template <class TS, int NM, bool kTma>
cudaError_t launch3d(const CUtensorMap* map, const Stencil3DParams& p, int ctas, cudaStream_t s) {
  const size_t smem = stencil3d_smem_bytes(p.TW + 2 * p.HW, p.TD + 2 * p.HD, p.NP, p.T, sizeof(TS));
  auto kern = stencil3d_kernel<TS, NM, kTma>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  kern<<<ctas, kStencil3DThreads, smem, s>>>(*map, p);
  e = cudaGetLastError();
  if (e != cudaSuccess || p.every <= 0) return e;
  bool any = false;
  for (int k = 1; k <= p.steps; ++k) any = any || ((p.step0 + k) % p.every) == 0;
  if (!any) return cudaSuccess;
  reduce3d_residual<<<p.steps, 256, 0, s>>>(p.partials, ctas, p.steps, p.step0, p.every, p.residuals);
  return cudaGetLastError();
}

template <class TS, int NM>
cudaError_t launch_stream(const Stencil3DParams& p, cudaStream_t s) {
  const dim3 grid((p.D + 31) / 32, (p.W + 7) / 8, p.hchunks);
  stream3d_kernel<TS, NM><<<grid, 256, 0, s>>>(p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || p.every <= 0 || ((p.step0 + 1) % p.every) != 0) return e;
  const int nctas = static_cast<int>(grid.x * grid.y * grid.z);
  reduce3d_residual<<<1, 256, 0, s>>>(p.partials, nctas, 1, p.step0, p.every, p.residuals);
  return cudaGetLastError();
}

}  // namespace

bool stream3d_is_cross7(const int* offsets, int n, int64_t D, int esize) {
  static const int k[7][3] = {{0, 0, 0}, {-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
  if (n != 7 || D % (16 / esize) != 0) return false;
  for (int i = 0; i < 7; ++i)
    for (int j = 0; j < 3; ++j)
      if (offsets[3 * i + j] != k[i][j]) return false;
  return true;
}

int64_t stream3d_ctas(int W, int D, int hchunks) {
  return static_cast<int64_t>((D + 31) / 32) * ((W + 7) / 8) * hchunks;
}

size_t stream3d_tma_smem_bytes(int dtype) {
  return dtype == 2 ? S3Rows<__nv_bfloat16>::kSmem : S3Rows<float>::kSmem;
}

template <class TS>
int tma_blocks_per_sm() {
  const size_t smem = S3Rows<TS>::kSmem;
  void* ks[4] = {reinterpret_cast<void*>(stream3d_tma_kernel<TS, false, false>),
                 reinterpret_cast<void*>(stream3d_tma_kernel<TS, false, true>),
                 reinterpret_cast<void*>(stream3d_tma_kernel<TS, true, false>),
                 reinterpret_cast<void*>(stream3d_tma_kernel<TS, true, true>)};
  int best = 1 << 30;
  for (void* k : ks) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, S3Rows<TS>::kThreads, smem) != cudaSuccess) n = 1;
    best = std::min(best, n);
  }
  return std::max(1, best);
}

int stream3d_tma_blocks_per_sm(int dtype) {
  return dtype == 2 ? tma_blocks_per_sm<__nv_bfloat16>() : tma_blocks_per_sm<float>();
}

int64_t stream3d_tma_items(int W, int D, int hchunks, int esize) {
  const int kD = 32 * (16 / esize);
  return static_cast<int64_t>((D + kD - 1) / kD) * ((W + 15) / 16) * hchunks;
}

template <class TS>
void launch_tma(const CUtensorMap* map, const Stencil3DParams& p, int ctas, bool report, cudaStream_t s) {
  const size_t smem = S3Rows<TS>::kSmem;
  uint32_t hbits;
  std::memcpy(&hbits, &p.halo, sizeof(hbits));
  const bool zero = hbits == 0u;  // +0.0 exactly: the TMA zero fill is the halo
  if (report && zero)
    stream3d_tma_kernel<TS, true, true><<<ctas, S3Rows<TS>::kThreads, smem, s>>>(*map, p);
  else if (report)
    stream3d_tma_kernel<TS, true, false><<<ctas, S3Rows<TS>::kThreads, smem, s>>>(*map, p);
  else if (zero)
    stream3d_tma_kernel<TS, false, true><<<ctas, S3Rows<TS>::kThreads, smem, s>>>(*map, p);
  else
    stream3d_tma_kernel<TS, false, false><<<ctas, S3Rows<TS>::kThreads, smem, s>>>(*map, p);
}

cudaError_t stream3d_tma_band(int dtype, const CUtensorMap* map, const Stencil3DParams& p, int ctas, double* acc,
                              cudaStream_t s) {
  if (dtype == 2)
    launch_tma<__nv_bfloat16>(map, p, ctas, acc != nullptr, s);
  else
    launch_tma<float>(map, p, ctas, acc != nullptr, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || acc == nullptr) return e;
  reduce3d_accumulate<<<1, 256, 0, s>>>(p.partials, ctas, acc);
  return cudaGetLastError();
}

cudaError_t stream3d_accumulate(const double* partials, int n, double* acc, cudaStream_t s) {
  reduce3d_accumulate<<<1, 256, 0, s>>>(partials, n, acc);
  return cudaGetLastError();
}

cudaError_t stream3d_finish_residuals(const double* acc, int n, double* residuals, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  finish3d_residuals<<<(n + 255) / 256, 256, 0, s>>>(acc, n, residuals);
  return cudaGetLastError();
}

cudaError_t stream3d_tma_step(int dtype, const CUtensorMap* map, const Stencil3DParams& p, int ctas,
                              cudaStream_t s) {
  const bool report = p.every > 0 && ((p.step0 + 1) % p.every) == 0;
  if (dtype == 2)
    launch_tma<__nv_bfloat16>(map, p, ctas, report, s);
  else
    launch_tma<float>(map, p, ctas, report, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !report) return e;
  reduce3d_residual<<<1, 256, 0, s>>>(p.partials, ctas, 1, p.step0, p.every, p.residuals);
  return cudaGetLastError();
}

cudaError_t stream3d_reduce_residuals(const double* partials, int ctas, int steps, int64_t step0, int every,
                                      double* residuals, cudaStream_t s) {
  reduce3d_residual<<<steps, 256, 0, s>>>(partials, ctas, steps, step0, every, residuals);
  return cudaGetLastError();
}

cudaError_t stream3d_step(int dtype, const Stencil3DParams& p, cudaStream_t s) {
  if (dtype == 2) return p.nm == 7 ? launch_stream<__nv_bfloat16, 7>(p, s) : launch_stream<__nv_bfloat16, 0>(p, s);
  return p.nm == 7 ? launch_stream<float, 7>(p, s) : launch_stream<float, 0>(p, s);
}

size_t stencil3d_smem_bytes(int LW, int LD, int NP, int T, size_t esize) {
  const size_t pb = (static_cast<size_t>(LW) * LD * esize + 127) & ~size_t(127);
  return (static_cast<size_t>(NP + kPrefetch3D) + static_cast<size_t>(T - 1) * NP) * pb + 8 * (NP + kPrefetch3D);
}

int stencil3d_max_ctas_per_sm(size_t smem) {
  int dev = 0;
  cudaGetDevice(&dev);
  int per_sm = 0, per_block = 0;
  cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&per_block, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (smem > static_cast<size_t>(per_block)) return 0;
  const size_t static_smem = 3 * kMaxMask3D * 4 + 8 * 8 + 1024;
  const int by_smem = static_cast<int>(per_sm / (smem + static_smem));
  const int by_threads = 2048 / kStencil3DThreads;
  return by_smem < by_threads ? by_smem : by_threads;
}

cudaError_t stencil3d_pass(int dtype, bool use_tma, const CUtensorMap* map_src, const Stencil3DParams& p, int ctas,
                           cudaStream_t s) {
  if (dtype == 2) {
    if (use_tma)
      return p.nm == 7 ? launch3d<__nv_bfloat16, 7, true>(map_src, p, ctas, s)
                       : launch3d<__nv_bfloat16, 0, true>(map_src, p, ctas, s);
    return p.nm == 7 ? launch3d<__nv_bfloat16, 7, false>(map_src, p, ctas, s)
                     : launch3d<__nv_bfloat16, 0, false>(map_src, p, ctas, s);
  }
  if (use_tma)
    return p.nm == 7 ? launch3d<float, 7, true>(map_src, p, ctas, s) : launch3d<float, 0, true>(map_src, p, ctas, s);
  return p.nm == 7 ? launch3d<float, 7, false>(map_src, p, ctas, s) : launch3d<float, 0, false>(map_src, p, ctas, s);
}

}  // namespace pskel
