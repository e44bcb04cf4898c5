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
// order) without temporal blocking, vectorised: each thread owns one 16-byte
// vector of d cells (4 fp32 or 8 bf16, kept packed in registers) in each of
// two adjacent w rows and marches along h keeping the planes of its cells in
// registers. Loads run one plane ahead of the arithmetic: while plane h is
// computed, plane h+2 of the thread's rows, the w-neighbour rows of plane h+1
// and the d-edge values of plane h+1 (lanes 0 and 31; the other lanes get the
// d-1 / d+V neighbours from their neighbours by shuffles) are in flight. Four
// plane slots and two neighbour slots rotate through a four-way unrolled
// march, so no values move between registers. Requires D % V == 0.
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

template <class TS, bool kReport>
__global__ void __launch_bounds__(256, 3) stream3d_cross7_kernel(const __grid_constant__ Stencil3DParams p) {
  using S = Storage<TS>;
  using Vt = Vec16<TS>;
  constexpr int V = Vt::V;
  __shared__ double s_part[8];
  // the weights (p.wt) stay in the parameter bank: instruction operands, no registers
  const TS* __restrict__ src = static_cast<const TS*>(p.src);
  TS* __restrict__ dst = static_cast<TS*>(p.dst);
  const float halo = p.halo;
  // the halo value as raw storage bits (packed twice for bf16)
  uint32_t hraw;
  if constexpr (sizeof(TS) == 4) {
    hraw = __float_as_uint(halo);
  } else {
    const uint32_t hb = __bfloat16_as_ushort(__float2bfloat16_rn(halo));
    hraw = hb | (hb << 16);
  }
  const int lane = threadIdx.x & 31;
  const int d = (blockIdx.x * 32 + lane) * V;
  const int w = blockIdx.y * 16 + (threadIdx.x >> 5) * 2;
  const int h0 = blockIdx.z * p.HC;
  const int h1 = min(p.H, h0 + p.HC);
  const int H = p.H, D = p.D;
  const bool d_ok = d < D;
  const bool row0 = d_ok && w < p.W, row1 = d_ok && w + 1 < p.W;
  const bool wm_ok = row0 && w > 0, wp_ok = row1 && w + 2 < p.W;
  const bool el_ok = lane == 0 && d > 0, er_ok = lane == 31 && d + V < D;
  const int64_t plane = static_cast<int64_t>(p.W) * D;
  constexpr bool report = kReport;  // this launch's step is a reported one
  SqDiffAcc acc_res;
  const int64_t col = static_cast<int64_t>(w) * D + d;

  // loads of plane q: the thread's two rows, the outer w neighbours, the d edges
  auto ld_rows = [&](int q, Vt (&r)[2]) {
    const bool in = q >= 0 && q < H;
    const TS* at = src + (col + q * plane);
    if (in && row0) r[0].load(at); else r[0].fill(hraw);
    if (in && row1) r[1].load(at + D); else r[1].fill(hraw);
  };
  auto ld_side = [&](int q, Vt (&r)[2], float (&e)[2][2]) {
    const bool in = q >= 0 && q < H;
    const TS* at = src + (col + q * plane);
    if (in && wm_ok) r[0].load(at - D); else r[0].fill(hraw);
    if (in && wp_ok) r[1].load(at + 2 * D); else r[1].fill(hraw);
    e[0][0] = (in && el_ok && row0) ? S::load(at[-1]) : halo;
    e[1][0] = (in && el_ok && row1) ? S::load(at[D - 1]) : halo;
    e[0][1] = (in && er_ok && row0) ? S::load(at[V]) : halo;
    e[1][1] = (in && er_ok && row1) ? S::load(at[D + V]) : halo;
  };
  // one plane: prefetch h+2 / h+1, then compute plane h from dn, cur, up
  auto step = [&](int h, Vt (&dn)[2], Vt (&cur)[2], Vt (&up)[2], Vt (&nx)[2], Vt (&sc)[2], Vt (&sn)[2],
                  float (&ec)[2][2], float (&en)[2][2]) {
    ld_rows(h + 2, nx);
    ld_side(h + 1, sn, en);
    TS* out = dst + (col + h * plane);
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      // every lane takes part in the shuffles; lanes past D hold the halo value
      float dl = __shfl_up_sync(0xFFFFFFFFu, cur[j].at(V - 1), 1);
      float dr = __shfl_down_sync(0xFFFFFFFFu, cur[j].at(0), 1);
      if (lane == 0) dl = ec[j][0];
      if (lane == 31) dr = ec[j][1];
      const Vt& wm = (j == 0) ? sc[0] : cur[0];
      const Vt& wp = (j == 0) ? cur[1] : sc[1];
      const bool row_ok = (j == 0) ? row0 : row1;
      // four cells at a time; results are packed to storage as they come
      uint32_t o[4];
#pragma unroll
      for (int g = 0; g < V / 4; ++g) {
        float res[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int c = 4 * g + k;
          const float l = (c == 0) ? dl : cur[j].at(c - 1);
          const float r = (c == V - 1) ? dr : cur[j].at(c + 1);
          float acc = __fmul_rn(p.wt[0], cur[j].at(c));
          acc = __fadd_rn(acc, __fmul_rn(p.wt[1], dn[j].at(c)));
          acc = __fadd_rn(acc, __fmul_rn(p.wt[2], up[j].at(c)));
          acc = __fadd_rn(acc, __fmul_rn(p.wt[3], wm.at(c)));
          acc = __fadd_rn(acc, __fmul_rn(p.wt[4], wp.at(c)));
          acc = __fadd_rn(acc, __fmul_rn(p.wt[5], l));
          acc = __fadd_rn(acc, __fmul_rn(p.wt[6], r));
          res[k] = acc;
        }
        float stored[4];
        if constexpr (sizeof(TS) == 4) {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            o[k] = __float_as_uint(res[k]);
            stored[k] = res[k];
          }
        } else {
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            const __nv_bfloat162 b = __floats2bfloat162_rn(res[2 * k], res[2 * k + 1]);
            o[2 * g + k] = *reinterpret_cast<const uint32_t*>(&b);
            stored[2 * k] = __uint_as_float(o[2 * g + k] << 16);
            stored[2 * k + 1] = __uint_as_float(o[2 * g + k] & 0xFFFF0000u);
          }
        }
        if (report && row_ok) {
#pragma unroll
          for (int k = 0; k < 4; ++k) acc_res.add(stored[k], cur[j].at(4 * g + k));
        }
      }
      if (row_ok) *reinterpret_cast<uint4*>(out + j * D) = make_uint4(o[0], o[1], o[2], o[3]);
    }
  };

  Vt A[2], B[2], C[2], E[2], sA[2], sB[2];
  float eA[2][2], eB[2][2];
  ld_rows(h0 - 1, A);
  ld_rows(h0, B);
  ld_rows(h0 + 1, C);
  ld_side(h0, sA, eA);
  for (int h = h0; h < h1; h += 4) {
    step(h, A, B, C, E, sA, sB, eA, eB);
    if (h + 1 >= h1) break;
    step(h + 1, B, C, E, A, sB, sA, eB, eA);
    if (h + 2 >= h1) break;
    step(h + 2, C, E, A, B, sA, sB, eA, eB);
    if (h + 3 >= h1) break;
    step(h + 3, E, A, B, C, sB, sA, eB, eA);
  }
  if constexpr (kReport) {
    double v = acc_res.value();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    if (lane == 0) s_part[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int i = 0; i < 8; ++i) t += s_part[i];
      const int cta = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
      p.partials[cta] = t;
    }
  }
}

// The same 7-point cross, one step per launch, with the planes staged in
// shared memory by TMA. A persistent block owns a work item of 32 vectors of
// d (128 fp32 / 256 bf16 cells) x 16 w rows x p.HC planes; one 3D TMA copy
// per plane brings the 34-vector x 18-row box (one vector and one row of
// halo on each side) into a ring of kS3Slots plane slots. The producer
// (thread 0) runs up to three planes ahead of the plane being computed and
// across work items; each slot has an mbarrier, and a slot is reused only
// after the block barrier that follows its last read. Out-of-grid positions
// (zero-filled by TMA) are replaced by the mask halo value.
constexpr int kS3Slots = 6;
constexpr int kS3BoxX = 34;                 // 16-byte vectors per staged row
constexpr int kS3RowBytes = kS3BoxX * 16;   // 544
constexpr int kS3BoxY = 18;                 // 16 rows + one each side
constexpr int kS3PlaneBytes = (kS3RowBytes * kS3BoxY + 127) & ~127;
constexpr int kS3Threads = 256;

template <class TS, bool kReport>
__global__ void __launch_bounds__(kS3Threads, 3)
    stream3d_tma_kernel(const __grid_constant__ CUtensorMap map, const __grid_constant__ Stencil3DParams p) {
  using S = Storage<TS>;
  using Vt = Vec16<TS>;
  constexpr int V = Vt::V;
  extern __shared__ __align__(128) uint8_t smem_raw[];
  __shared__ double s_part[kS3Threads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if ((smem_u32(smem_raw) & 127u) != 0) {
    if (tid == 0) atomicOr(p.err, kDevErrAlign);
    return;
  }
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + kS3Slots * kS3PlaneBytes);
  if (tid == 0) {
    for (int i = 0; i < kS3Slots; ++i) mbar_init(&full[i], 1);
    fence_barrier_init();
    prefetch_tensormap(&map);
  }
  __syncthreads();

  const int H = p.H, W = p.W, D = p.D;
  const int dblocks = (D + 32 * V - 1) / (32 * V), wblocks = (W + 15) / 16;
  const int64_t items = static_cast<int64_t>(dblocks) * wblocks * p.hchunks;
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
  SqDiffAcc acc_res;

  // in-grid planes of an item: qlo .. qhi (planes h0-1 .. h1 clipped to the grid)
  auto item_planes = [&](int64_t it, int& d0, int& w0, int& h0, int& h1, int& qlo, int& qhi) {
    const int db = static_cast<int>(it % dblocks);
    const int64_t r = it / dblocks;
    const int wb = static_cast<int>(r % wblocks);
    const int ch = static_cast<int>(r / wblocks);
    d0 = db * 32 * V;
    w0 = wb * 16;
    h0 = ch * p.HC;
    h1 = min(H, h0 + p.HC);
    qlo = max(h0 - 1, 0);
    qhi = min(h1, H - 1);
  };

  // producer state (thread 0): the next plane to issue and the sequence count
  int64_t p_item = blockIdx.x;
  int p_q = 0, p_qhi = -1, p_d0 = 0, p_w0 = 0;
  uint32_t issued = 0;
  auto p_load_item = [&]() {
    int h0, h1;
    if (p_item < items) item_planes(p_item, p_d0, p_w0, h0, h1, p_q, p_qhi);
  };
  auto produce_upto = [&](uint32_t limit) {
    while (issued < limit && p_item < items) {
      const int slot = static_cast<int>(issued % kS3Slots);
      fence_proxy_async();
      mbar_arrive_expect_tx(&full[slot], static_cast<uint32_t>(kS3RowBytes * kS3BoxY));
      // the map addresses the grid as 32-bit words (a box row of 136 words)
      tma_load_3d(smem_raw + slot * kS3PlaneBytes, &map, (p_d0 - V) * static_cast<int>(sizeof(TS)) / 4, p_w0 - 1,
                  p_q, &full[slot]);
      ++issued;
      if (++p_q > p_qhi) {
        p_item += gridDim.x;
        p_load_item();
      }
    }
  };
  if (tid == 0) {
    p_load_item();
    produce_upto(kS3Slots);
  }

  uint32_t seq_base = 0;  // sequence number of the current item's plane qlo
  bool ok_all = true;
  for (int64_t it = blockIdx.x; it < items && ok_all; it += gridDim.x) {
    int d0, w0, h0, h1, qlo, qhi;
    item_planes(it, d0, w0, h0, h1, qlo, qhi);
    const int d = d0 + lane * V;
    const int w = w0 + warp * 2;
    const bool d_ok = d < D;
    const bool row0 = d_ok && w < W, row1 = d_ok && w + 1 < W;
    const bool wm_ok = row0 && w > 0, wp_ok = row1 && w + 2 < W;
    const bool el_ok = lane == 0 && d > 0, er_ok = lane == 31 && d + V < D;
    auto seq_of = [&](int q) { return seq_base + static_cast<uint32_t>(q - qlo); };
    auto in_grid = [&](int q) { return q >= 0 && q < H; };
    // wait (thread 0) for plane q, publish to the block with the barrier
    auto wait_plane = [&](int q) -> bool {
      int ok = 1;
      if (tid == 0 && in_grid(q)) {
        const uint32_t k = seq_of(q);
        ok = mbar_wait_bounded(&full[k % kS3Slots], (k / kS3Slots) & 1u, p.err) ? 1 : 0;
      }
      return __syncthreads_and(ok) != 0;
    };
    auto row_ptr = [&](int q, int r) -> const uint8_t* {
      return smem_raw + (seq_of(q) % kS3Slots) * kS3PlaneBytes + r * kS3RowBytes;
    };
    auto rd = [&](int q, int r, bool ok, Vt& v) {
      if (ok && in_grid(q)) {
        const uint4 x = *reinterpret_cast<const uint4*>(row_ptr(q, r) + (lane + 1) * 16);
        v.r[0] = x.x;
        v.r[1] = x.y;
        v.r[2] = x.z;
        v.r[3] = x.w;
      } else {
        v.fill(hraw);
      }
    };
    auto rd_edge = [&](int q, int r, bool ok, int vec, int c) -> float {
      if (!(ok && in_grid(q))) return halo;
      const TS* e = reinterpret_cast<const TS*>(row_ptr(q, r) + vec * 16);
      return S::load(e[c]);
    };

    if (!wait_plane(h0 - 1) || !wait_plane(h0)) {
      ok_all = false;
      break;
    }
    const int r0 = 2 * warp + 1;  // staged row of the thread's first w row
    for (int h = h0; h < h1; ++h) {
      if (!wait_plane(h + 1)) {
        ok_all = false;
        break;
      }
      // planes below h-1 are no longer read: their slots may be refilled
      if (tid == 0) produce_upto(seq_of(max(h - 1, qlo)) + kS3Slots);
      Vt dn[2], cur[2], up[2], wm, wp;
      rd(h - 1, r0, row0, dn[0]);
      rd(h - 1, r0 + 1, row1, dn[1]);
      rd(h, r0, row0, cur[0]);
      rd(h, r0 + 1, row1, cur[1]);
      rd(h + 1, r0, row0, up[0]);
      rd(h + 1, r0 + 1, row1, up[1]);
      rd(h, r0 - 1, wm_ok, wm);
      rd(h, r0 + 2, wp_ok, wp);
      const float el0 = rd_edge(h, r0, el_ok && row0, 0, V - 1), el1 = rd_edge(h, r0 + 1, el_ok && row1, 0, V - 1);
      const float er0 = rd_edge(h, r0, er_ok && row0, 33, 0), er1 = rd_edge(h, r0 + 1, er_ok && row1, 33, 0);
      TS* out = dst + (h * plane + static_cast<int64_t>(w) * D + d);
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        float dl = __shfl_up_sync(0xFFFFFFFFu, cur[j].at(V - 1), 1);
        float dr = __shfl_down_sync(0xFFFFFFFFu, cur[j].at(0), 1);
        if (lane == 0) dl = (j == 0) ? el0 : el1;
        if (lane == 31) dr = (j == 0) ? er0 : er1;
        const Vt& a = (j == 0) ? wm : cur[0];
        const Vt& b = (j == 0) ? cur[1] : wp;
        const bool row_ok = (j == 0) ? row0 : row1;
        uint32_t o[4];
#pragma unroll
        for (int g = 0; g < V / 4; ++g) {
          float res[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int c = 4 * g + k;
            const float l = (c == 0) ? dl : cur[j].at(c - 1);
            const float r = (c == V - 1) ? dr : cur[j].at(c + 1);
            float acc = __fmul_rn(p.wt[0], cur[j].at(c));
            acc = __fadd_rn(acc, __fmul_rn(p.wt[1], dn[j].at(c)));
            acc = __fadd_rn(acc, __fmul_rn(p.wt[2], up[j].at(c)));
            acc = __fadd_rn(acc, __fmul_rn(p.wt[3], a.at(c)));
            acc = __fadd_rn(acc, __fmul_rn(p.wt[4], b.at(c)));
            acc = __fadd_rn(acc, __fmul_rn(p.wt[5], l));
            acc = __fadd_rn(acc, __fmul_rn(p.wt[6], r));
            res[k] = acc;
          }
          float stored[4];
          if constexpr (sizeof(TS) == 4) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              o[k] = __float_as_uint(res[k]);
              stored[k] = res[k];
            }
          } else {
#pragma unroll
            for (int k = 0; k < 2; ++k) {
              const __nv_bfloat162 bb = __floats2bfloat162_rn(res[2 * k], res[2 * k + 1]);
              o[2 * g + k] = *reinterpret_cast<const uint32_t*>(&bb);
              stored[2 * k] = __uint_as_float(o[2 * g + k] << 16);
              stored[2 * k + 1] = __uint_as_float(o[2 * g + k] & 0xFFFF0000u);
            }
          }
          if (kReport && row_ok) {
#pragma unroll
            for (int k = 0; k < 4; ++k) acc_res.add(stored[k], cur[j].at(4 * g + k));
          }
        }
        if (row_ok) *reinterpret_cast<uint4*>(out + j * D) = make_uint4(o[0], o[1], o[2], o[3]);
      }
    }
    if (!ok_all) break;
    // every plane of the item has been read once the block passes this barrier
    __syncthreads();
    seq_base += static_cast<uint32_t>(qhi - qlo + 1);
    if (tid == 0) produce_upto(seq_base + kS3Slots);
  }
  if constexpr (kReport) {
    double v = acc_res.value();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    if (lane == 0) s_part[warp] = v;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int i = 0; i < kS3Threads / 32; ++i) t += s_part[i];
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
cudaError_t launch_stream(const Stencil3DParams& p, bool cross7, cudaStream_t s) {
  constexpr int kD = 32 * (16 / static_cast<int>(sizeof(TS)));  // d cells per cross7 block
  const dim3 grid(cross7 ? (p.D + kD - 1) / kD : (p.D + 31) / 32, cross7 ? (p.W + 15) / 16 : (p.W + 7) / 8,
                  p.hchunks);
  const bool report = p.every > 0 && ((p.step0 + 1) % p.every) == 0;
  if (cross7 && report)
    stream3d_cross7_kernel<TS, true><<<grid, 256, 0, s>>>(p);
  else if (cross7)
    stream3d_cross7_kernel<TS, false><<<grid, 256, 0, s>>>(p);
  else
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

int64_t stream3d_ctas(int W, int D, int hchunks, bool cross7, int esize) {
  const int kD = 32 * (16 / esize);
  return static_cast<int64_t>(cross7 ? (D + kD - 1) / kD : (D + 31) / 32) * (cross7 ? (W + 15) / 16 : (W + 7) / 8) *
         hchunks;
}

size_t stream3d_tma_smem_bytes() { return kS3Slots * kS3PlaneBytes + 8 * kS3Slots; }

int stream3d_tma_blocks_per_sm(int dtype) {
  const size_t smem = stream3d_tma_smem_bytes();
  auto k = (dtype == 2) ? stream3d_tma_kernel<__nv_bfloat16, false> : stream3d_tma_kernel<float, false>;
  auto kr = (dtype == 2) ? stream3d_tma_kernel<__nv_bfloat16, true> : stream3d_tma_kernel<float, true>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  cudaFuncSetAttribute(kr, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  int n = 0, nr = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kS3Threads, smem) != cudaSuccess) n = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nr, kr, kS3Threads, smem) != cudaSuccess) nr = 1;
  return std::max(1, std::min(n, nr));
}

int64_t stream3d_tma_items(int W, int D, int hchunks, int esize) {
  const int kD = 32 * (16 / esize);
  return static_cast<int64_t>((D + kD - 1) / kD) * ((W + 15) / 16) * hchunks;
}

cudaError_t stream3d_tma_step(int dtype, const CUtensorMap* map, const Stencil3DParams& p, int ctas,
                              cudaStream_t s) {
  const bool report = p.every > 0 && ((p.step0 + 1) % p.every) == 0;
  const size_t smem = stream3d_tma_smem_bytes();
  if (dtype == 2) {
    if (report)
      stream3d_tma_kernel<__nv_bfloat16, true><<<ctas, kS3Threads, smem, s>>>(*map, p);
    else
      stream3d_tma_kernel<__nv_bfloat16, false><<<ctas, kS3Threads, smem, s>>>(*map, p);
  } else {
    if (report)
      stream3d_tma_kernel<float, true><<<ctas, kS3Threads, smem, s>>>(*map, p);
    else
      stream3d_tma_kernel<float, false><<<ctas, kS3Threads, smem, s>>>(*map, p);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !report) return e;
  reduce3d_residual<<<1, 256, 0, s>>>(p.partials, ctas, 1, p.step0, p.every, p.residuals);
  return cudaGetLastError();
}

cudaError_t stream3d_step(int dtype, const Stencil3DParams& p, bool cross7, cudaStream_t s) {
  if (dtype == 2)
    return p.nm == 7 ? launch_stream<__nv_bfloat16, 7>(p, cross7, s) : launch_stream<__nv_bfloat16, 0>(p, cross7, s);
  return p.nm == 7 ? launch_stream<float, 7>(p, cross7, s) : launch_stream<float, 0>(p, cross7, s);
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
