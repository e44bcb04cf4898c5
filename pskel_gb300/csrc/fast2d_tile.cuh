// Device code shared by the register-windowed 2D kernel and the batched
// persistent kernel: vector helpers, mask shapes and the per-tile routine.
#pragma once

#include "common.cuh"
#include "kernels.h"

namespace pskel {
namespace fast2d {

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

constexpr int kFastThreads = 512;
constexpr int kFastBufs = 3;  // rotating tile buffers: source, partner, next source
constexpr int kFastWarps = kFastThreads / 32;

// Warp w of the tile routine and warp w+1 share named barrier 1 + w (ids
// 1..15; 0 is the block barrier). Between two steps a warp meets its two
// neighbours only -- the warps whose rows it reads and who read its rows --
// in two rounds: even warps first with the warp below, odd warps first with
// the warp above, so pairs (0,1), (2,3), ... meet first and (1,2), (3,4), ...
// second, and no chain of waits runs through the block.
static_assert(kFastWarps <= 16, "one named barrier per neighbouring pair, ids 1..15");
__device__ __forceinline__ void pair_barrier(int id) { asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory"); }
__device__ __forceinline__ void neighbours_barrier(int w) {
  if ((w & 1) == 0) {
    if (w + 1 < kFastWarps) pair_barrier(1 + w);
    if (w > 0) pair_barrier(w);
  } else {
    pair_barrier(w);
    if (w + 1 < kFastWarps) pair_barrier(1 + w);
  }
}

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

// One advection-diffusion update (the reference's CLOUDSIM arithmetic,
// PSkelStencil.hpp:347-387): centre cc, neighbours north n_ (row above), east
// e_, west w_, south s_ (row below), winds xw, yw; no contraction.
__device__ __forceinline__ float advect_cell(float cc, float n_, float e_, float w_, float s_, float xw, float yw,
                                             float K, float dt, float inv_dx) {
  const float sum = __fsub_rn(__fmul_rn(4.0f, cc), __fadd_rn(__fadd_rn(__fadd_rn(n_, e_), w_), s_));
  const float cvy = (yw > 0.0f) ? yw : -yw;  // yf * yw with yf = +-1
  const float cvx = (xw > 0.0f) ? xw : -xw;
  const float nbx = (xw > 0.0f) ? e_ : w_;
  const float nby = (yw > 0.0f) ? s_ : n_;
  const float temp_wind = __fsub_rn(__fmul_rn(-cvx, __fmul_rn(__fsub_rn(cc, nbx), inv_dx)),
                                    __fmul_rn(cvy, __fmul_rn(__fsub_rn(cc, nby), inv_dx)));
  const float cond = __fmul_rn(__fmul_rn(-K, __fmul_rn(sum, 0.25f)), dt);
  return __fadd_rn(__fadd_rn(cc, cond), __fmul_rn(temp_wind, dt));
}

// advect_cell for two horizontally neighbouring cells at once (x in lane .x,
// x+1 in lane .y), the same operations in the same order per lane, two cells
// per instruction where the operands come in register pairs. The east and
// west pairs straddle two register pairs (east of x is the centre of x+1), so
// the first two sums of the neighbourhood take one instruction per lane. nz:
// neg_zero2 of the launch.
__device__ __forceinline__ float2 advect_pair(float2 cc, float2 n_, float2 e_, float2 w_, float2 s_, float2 xw,
                                              float2 yw, float K, float dt, float inv_dx, float2 nz) {
  const float2 new_ = make_float2(__fadd_rn(__fadd_rn(n_.x, e_.x), w_.x), __fadd_rn(__fadd_rn(n_.y, e_.y), w_.y));
  const float2 sum = fsub2_rn(fmul2_rn(dup2(4.0f), cc, nz), fadd2_rn(new_, s_));
  const float2 cvy = make_float2((yw.x > 0.0f) ? yw.x : -yw.x, (yw.y > 0.0f) ? yw.y : -yw.y);
  const float2 ncvx = make_float2((xw.x > 0.0f) ? -xw.x : xw.x, (xw.y > 0.0f) ? -xw.y : xw.y);  // -cvx
  const float2 nbx = make_float2((xw.x > 0.0f) ? e_.x : w_.x, (xw.y > 0.0f) ? e_.y : w_.y);
  const float2 nby = make_float2((yw.x > 0.0f) ? s_.x : n_.x, (yw.y > 0.0f) ? s_.y : n_.y);
  const float2 temp_wind = fsub2_rn(fmul2_rn(ncvx, fmul2_rn(fsub2_rn(cc, nbx), dup2(inv_dx), nz), nz),
                                    fmul2_rn(cvy, fmul2_rn(fsub2_rn(cc, nby), dup2(inv_dx), nz), nz));
  const float2 cond = fmul2_rn(fmul2_rn(dup2(-K), fmul2_rn(sum, dup2(0.25f), nz), nz), dup2(dt), nz);
  return fadd2_rn(fadd2_rn(cc, cond), fmul2_rn(temp_wind, dup2(dt), nz));
}

// Geometry and op parameters of one tile's grid (passed in registers).
struct TileGeom {
  int W, H, ring, steps;
  int TW, TH, HX, HY;
  int64_t pitch;
  float K, dt, inv_dx;
  const void* u;
  const void* v;
};

// The tile routine for a tile that touches no ring cell (its whole window
// lies in the interior): every warp keeps its S rows, and the rows above and
// below them, in registers for all the steps, with west and east neighbours by
// shuffles, updates the rows in place top to bottom (the old row above kept
// aside), and after each step exchanges only its first and last rows with
// the two neighbouring warps through `xch` (two parities, so one meeting per
// step suffices, as in the Life kernel). bf16 rows are rounded to bf16 every
// step, as storing them would. The core rows go from registers to dst.
template <class TS, int OpK, int S>
__device__ __forceinline__ void fast2d_run_tile_regs(const TS* sbuf, TS* xch, TS* dst, const TileGeom& g, int gy0,
                                                     int gx0, const float* wt, const float2* wt2, float2 nz) {
  constexpr int N = Vec<TS>::N;
  constexpr int LW = 32 * N;
  constexpr int LH = kFastWarps * S + 2;
  constexpr bool kAdvect = (OpK == 3);
  constexpr auto shp = shape_of<(OpK < 3 ? OpK : 0)>();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int x0 = lane * N;
  const int yb = 1 + warp * S;  // window row of this warp's row 1
  const TS* wu = static_cast<const TS*>(g.u);
  const TS* wv = static_cast<const TS*>(g.v);
  const int gxv = gx0 + x0;
  float r[S + 2][N];  // window rows yb-1 .. yb+S
#pragma unroll
  for (int k = 0; k < S + 2; ++k) ld_vec(sbuf + (yb - 1 + k) * LW + x0, r[k]);
  int par = 0;
  for (int s = 1; s <= g.steps; ++s) {
    // after step s only rows [s, LH - s) are exact; a warp with none of them
    // computes nothing (it still meets its neighbours below)
    if (!(yb + S <= s || yb >= LH - s)) {
      float a[N];  // the row above, as it was before this step
      float aw, ae, cw, ce;  // west / east neighbours of the row above and of this row
#pragma unroll
      for (int c = 0; c < N; ++c) a[c] = r[0][c];
      aw = __shfl_up_sync(0xFFFFFFFFu, r[0][N - 1], 1);
      ae = __shfl_down_sync(0xFFFFFFFFu, r[0][0], 1);
      cw = __shfl_up_sync(0xFFFFFFFFu, r[1][N - 1], 1);
      ce = __shfl_down_sync(0xFFFFFFFFu, r[1][0], 1);
#pragma unroll
      for (int k = 1; k <= S; ++k) {
        const float bw = __shfl_up_sync(0xFFFFFFFFu, r[k + 1][N - 1], 1);
        const float be = __shfl_down_sync(0xFFFFFFFFu, r[k + 1][0], 1);
        const int y = yb - 1 + k;
        const bool live = y >= s && y < LH - s;
        float res[N];
        if (live) {
          // cell c + dw of the row dh below this one (dh, dw in -1..1)
          auto at = [&](int dh, int cc) -> float {
            if (dh < 0) return cc < 0 ? aw : (cc >= N ? ae : a[cc < 0 ? 0 : (cc >= N ? N - 1 : cc)]);
            if (dh > 0) return cc < 0 ? bw : (cc >= N ? be : r[k + 1][cc < 0 ? 0 : (cc >= N ? N - 1 : cc)]);
            return cc < 0 ? cw : (cc >= N ? ce : r[k][cc < 0 ? 0 : (cc >= N ? N - 1 : cc)]);
          };
          if constexpr (!kAdvect) {
#pragma unroll
            for (int c = 0; c < N; c += 2) {
              float2 acc;
#pragma unroll
              for (int n = 0; n < shp.n; ++n) {
                const int dh = shp.dh[n], dw = shp.dw[n];
                const float2 t = (dw == 0) ? fmul2_rn(wt2[n], make_float2(at(dh, c), at(dh, c + 1)), nz)
                                           : make_float2(__fmul_rn(wt[n], at(dh, c + dw)),
                                                         __fmul_rn(wt[n], at(dh, c + 1 + dw)));
                acc = (n == 0) ? t : fadd2_rn(acc, t);
              }
              res[c] = acc.x;
              res[c + 1] = acc.y;
            }
          } else {
            float uu[N], vv[N];
            ld_wind(wu, g.pitch, gy0 + y, gxv, g.W, g.H, uu);
            ld_wind(wv, g.pitch, gy0 + y, gxv, g.W, g.H, vv);
#pragma unroll
            for (int c = 0; c < N; c += 2) {
              const float2 r2 = advect_pair(make_float2(at(0, c), at(0, c + 1)), make_float2(at(-1, c), at(-1, c + 1)),
                                            make_float2(at(0, c + 1), at(0, c + 2)),
                                            make_float2(at(0, c - 1), at(0, c)),
                                            make_float2(at(1, c), at(1, c + 1)), make_float2(uu[c], uu[c + 1]),
                                            make_float2(vv[c], vv[c + 1]), g.K, g.dt, g.inv_dx, nz);
              res[c] = r2.x;
              res[c + 1] = r2.y;
            }
          }
          if constexpr (sizeof(TS) == 2) {
#pragma unroll
            for (int c = 0; c < N; ++c)
              res[c] = __uint_as_float(static_cast<uint32_t>(__bfloat16_as_ushort(__float2bfloat16_rn(res[c]))) << 16);
          }
        }
        // this row, before the step, is the row above the next one
#pragma unroll
        for (int c = 0; c < N; ++c) a[c] = r[k][c];
        aw = cw;
        ae = ce;
        if (live) {
#pragma unroll
          for (int c = 0; c < N; ++c) r[k][c] = res[c];
        }
        cw = bw;
        ce = be;
      }
    }
    if (s < g.steps) {
      // first and last rows to the neighbours; theirs back
      TS* xb = xch + par * (2 * kFastWarps * LW);
      st_vec(xb + (2 * warp) * LW + x0, r[1]);
      st_vec(xb + (2 * warp + 1) * LW + x0, r[S]);
      neighbours_barrier(warp);
      if (warp > 0) ld_vec(xb + (2 * (warp - 1) + 1) * LW + x0, r[0]);
      if (warp < kFastWarps - 1) ld_vec(xb + (2 * (warp + 1)) * LW + x0, r[S + 1]);
      par ^= 1;
    }
  }
  // core rows [HY, HY + TH), columns [HX, HX + TW) to dst: a lane's N cells
  // lie all inside or all outside (HX and TW are multiples of N)
  if (x0 >= g.HX && x0 < g.HX + g.TW) {
#pragma unroll
    for (int k = 1; k <= S; ++k) {
      const int y = yb - 1 + k;
      if (y >= g.HY && y < g.HY + g.TH) st_vec(dst + static_cast<int64_t>(gy0 + y) * g.pitch + gxv, r[k]);
    }
  }
}

// Runs g.steps steps on a staged tile (source tile in sbuf, the partner
// buffer pbuf holding the destination's ring when the tile touches it), then
// writes the core's interior cells to dst. All threads of the block call it.
// An fp32 tile clear of the ring takes the register-resident routine above
// (pbuf, unused then, holds its row exchange). Measured on GB300 against this
// shared-memory routine (GCells/s): advection 4096^2 T=5 453 -> 476, batched
// Jacobi fp32 813 -> 846, Jacobi 1024^2 fp32 708 -> 703; bf16 (rounded in
// registers every step) Jacobi 653 -> 626, batch 782 -> 783, so bf16 keeps
// the shared-memory routine.
template <class TS, int OpK, int S>
__device__ __forceinline__ void fast2d_run_tile(TS* sbuf, TS* pbuf, TS* dst, const TileGeom& g, int gy0, int gx0,
                                                bool ring_tile, const float* wt, float2 nz) {
  constexpr int N = Vec<TS>::N;
  constexpr int LW = 32 * N;
  constexpr bool kAdvect = (OpK == 3);
  constexpr auto shp = shape_of<(OpK < 3 ? OpK : 0)>();
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int x0 = lane * N;
  const int yb = 1 + warp * S;
  constexpr int LH = (kFastThreads / 32) * S + 2;
  const TS* wu = static_cast<const TS*>(g.u);
  const TS* wv = static_cast<const TS*>(g.v);
  const int gxv = gx0 + x0;
  float2 wt2[shp.n > 0 ? shp.n : 1];
#pragma unroll
  for (int n = 0; n < shp.n; ++n) wt2[n] = make_float2(wt[n], wt[n]);
  if constexpr (sizeof(TS) == 4) {
    if (!ring_tile) {
      fast2d_run_tile_regs<TS, OpK, S>(sbuf, pbuf, dst, g, gy0, gx0, wt, wt2, nz);
      return;
    }
  }
  for (int s = 1; s <= g.steps; ++s) {
    const TS* in = ((s & 1) ? sbuf : pbuf);
    TS* out = ((s & 1) ? pbuf : sbuf);
    // After step s only rows [s, LH - s) are exact (the tile edges feed
    // garbage in one row per step) and only they are read by step s + 1 and
    // by the write-back (core rows [HY, LH - HY), HY >= steps). Rows outside
    // are not computed: whatever the buffer holds there is never used, and a
    // ring cell there keeps the buffer's value as a computed one would. The
    // test is uniform per warp; a warp with no such row skips the step.
    if (yb + S <= s || yb >= LH - s) {
      neighbours_barrier(warp);
      continue;
    }
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
      if (y < s || y >= LH - s) continue;
      float res[N];
      // two neighbouring cells per instruction (cells c, c+1: lanes .x, .y)
      if constexpr (!kAdvect) {
#pragma unroll
        for (int c = 0; c < N; c += 2) {
          float2 acc;
#pragma unroll
          for (int n = 0; n < shp.n; ++n) {
            const int dh = shp.dh[n], dw = shp.dw[n];
            // a row neighbour (dw != 0) straddles two register pairs: one
            // product per lane
            const float2 t = (dw == 0) ? fmul2_rn(wt2[n], make_float2(win[k + dh][1 + c], win[k + dh][2 + c]), nz)
                                       : make_float2(__fmul_rn(wt[n], win[k + dh][1 + c + dw]),
                                                     __fmul_rn(wt[n], win[k + dh][2 + c + dw]));
            acc = (n == 0) ? t : fadd2_rn(acc, t);
          }
          res[c] = acc.x;
          res[c + 1] = acc.y;
        }
      } else {
        float uu[N], vv[N];
        ld_wind(wu, g.pitch, gy0 + y, gxv, g.W, g.H, uu);
        ld_wind(wv, g.pitch, gy0 + y, gxv, g.W, g.H, vv);
#pragma unroll
        for (int c = 0; c < N; c += 2) {
          const float2 r2 = advect_pair(
              make_float2(win[k][1 + c], win[k][2 + c]), make_float2(win[k - 1][1 + c], win[k - 1][2 + c]),
              make_float2(win[k][2 + c], win[k][3 + c]), make_float2(win[k][c], win[k][1 + c]),
              make_float2(win[k + 1][1 + c], win[k + 1][2 + c]), make_float2(uu[c], uu[c + 1]),
              make_float2(vv[c], vv[c + 1]), g.K, g.dt, g.inv_dx, nz);
          res[c] = r2.x;
          res[c + 1] = r2.y;
        }
      }
      TS* o = out + y * LW + x0;
      if (ring_tile) {
        // cells outside r <= h < H-r, r <= w < W-r keep this buffer's value
        const int gy = gy0 + y;
        const bool row_in = gy >= g.ring && gy < g.H - g.ring;
        float old[N];
        ld_vec(o, old);
#pragma unroll
        for (int c = 0; c < N; ++c) {
          const int gx = gxv + c;
          if (!(row_in && gx >= g.ring && gx < g.W - g.ring)) res[c] = old[c];
        }
      }
      st_vec(o, res);
    }
    // a step's rows are read by the warps above and below at the next step,
    // and overwritten one step later only after they have met again
    neighbours_barrier(warp);
  }
  __syncthreads();  // the write-back reads every warp's rows

  // core -> global, interior cells only, vector stores
  const TS* fin = ((g.steps & 1) ? pbuf : sbuf);
  const int vpr = g.TW / N;
  for (int i = tid; i < g.TH * vpr; i += kFastThreads) {
    const int r = i / vpr;
    const int cv = i - r * vpr;
    const int y = g.HY + r, x = g.HX + cv * N;
    const int gy = gy0 + y, gx = gx0 + x;
    if (gy < g.ring || gy >= g.H - g.ring) continue;
    if (gx + N <= g.ring || gx >= g.W - g.ring) continue;
    TS* d = dst + static_cast<int64_t>(gy) * g.pitch + gx;
    const TS* sp = fin + y * LW + x;
    constexpr int kVecBytes = N * static_cast<int>(sizeof(TS));
    if (gx >= g.ring && gx + N <= g.W - g.ring && (reinterpret_cast<uintptr_t>(d) & (kVecBytes - 1)) == 0) {
      if constexpr (kVecBytes == 16)
        *reinterpret_cast<uint4*>(d) = *reinterpret_cast<const uint4*>(sp);
      else
        *reinterpret_cast<uint2*>(d) = *reinterpret_cast<const uint2*>(sp);
    } else {
#pragma unroll
      for (int k = 0; k < N; ++k) {
        const int xx = gx + k;
        if (xx >= g.ring && xx < g.W - g.ring) d[k] = sp[k];
      }
    }
  }
}

}  // namespace fast2d
}  // namespace pskel
