// 2D fp32 / bf16-storage stencils of reach 1 (a known linear shape, or the
// advection-diffusion op), one step per launch, streaming: the path for
// schedules of one time step per pass, where a step moves every cell through
// HBM once and temporal blocking has nothing to reuse.
//
// Each warp owns 128 columns (four cells per lane: 16 bytes of fp32, 8 of
// bf16) of a chunk of rows and marches down them, keeping rows h-1, h, h+1 in
// registers and loading row h+2 (and the winds of row h+1) while row h is
// computed (bf16: rows h+3 and winds h+2), with the row slots rotated by an
// unrolled march, so no value moves between registers. West/east neighbours come from
// the adjacent lanes by shuffles; the warp's edge lanes load theirs with the
// row. Only cells with ring <= h < H-ring and ring <= w < W-ring are written,
// so each buffer keeps its own ring, as in Stencil2D::runOpenMP
// (PSkelStencil.hpp:2197-2257).
//
// Arithmetic is the oracle's: products and sums in mask order with
// __fmul_rn/__fadd_rn (no contraction), bf16 results rounded every step.
#include "fast2d_tile.cuh"

namespace pskel {
namespace {

using fast2d::advect_cell;
using fast2d::shape_of;

constexpr int kStreamThreads = 256;

// four cells per lane for either storage type: the same lanes-per-cell as
// fp32 keeps bf16 warps as many and as light as fp32 ones
template <class TS>
using LaneVec = Vec4c<TS>;

template <class TS>
struct Row {
  LaneVec<TS> v;
  float l, r;  // the cells west of the first and east of the last element (edge lanes only)
};

// OpK: 0..2 linear shapes (fast2d::shape_of), 3 = advection.
template <class TS, int OpK>
__global__ void __launch_bounds__(kStreamThreads, sizeof(TS) == 2 ? 4 : 3) stream2d_kernel(const __grid_constant__ Stencil2DParams p) {
  using Vt = LaneVec<TS>;
  constexpr int V = Vt::V;
  constexpr bool kAdvect = (OpK == 3);
  constexpr int kShape = OpK < 3 ? OpK : 0;
  constexpr int kTerms = shape_of<kShape>().n;
  // rows loaded ahead of the one computed: bf16 rows carry half the bytes, so
  // they run one row further ahead to keep as many bytes in flight
  constexpr int kPD = sizeof(TS) == 2 ? 2 : 1;
  const int lane = threadIdx.x & 31;
  const int64_t gw = static_cast<int64_t>(blockIdx.x) * (kStreamThreads / 32) + (threadIdx.x >> 5);
  const int cols = (p.W + 32 * V - 1) / (32 * V);
  const int64_t items = static_cast<int64_t>(cols) * p.tiles_y;
  if (gw >= items) return;  // whole warps leave together
  const int cb = static_cast<int>(gw % cols);
  const int rc = static_cast<int>(gw / cols);
  const int W = p.W, H = p.H, ring = p.ring;
  const int c = cb * 32 * V + lane * V;
  const int hs = max(rc * p.TH, ring);
  const int he = min(min(rc * p.TH + p.TH, H), H - ring);
  if (hs >= he) return;
  const TS* __restrict__ src = static_cast<const TS*>(p.src);
  TS* __restrict__ dst = static_cast<TS*>(p.dst);
  const TS* __restrict__ wu = static_cast<const TS*>(p.u);
  const TS* __restrict__ wv = static_cast<const TS*>(p.v);
  const bool c_ok = c < W;
  const bool l_ok = lane == 0 && c > 0 && c_ok;
  const bool r_ok = lane == 31 && c + V < W;
  const int64_t pitch = p.pitch;

  auto ld_row = [&](int q, Row<TS>& r) {
    const bool in = q >= 0 && q < H;
    const TS* at = src + (static_cast<int64_t>(q) * pitch + c);
    if (in && c_ok) r.v.load(at); else r.v.fill(0u);
    r.l = (in && l_ok) ? Storage<TS>::load(at[-1]) : 0.0f;
    r.r = (in && r_ok) ? Storage<TS>::load(at[V]) : 0.0f;
  };
  auto ld_wind = [&](int q, Vt& u, Vt& v) {
    if constexpr (kAdvect) {
      const bool in = q >= 0 && q < H && c_ok;
      const int64_t o = static_cast<int64_t>(q) * pitch + c;
      if (in) u.load(wu + o); else u.fill(0u);
      if (in) v.load(wv + o); else v.fill(0u);
    }
  };
  // the value of a row at element k (k = -1 and V reach the neighbours)
  auto val = [&](const Row<TS>& r, float west, float east, int k) -> float {
    return (k < 0) ? west : (k >= V ? east : r.v.at(k));
  };
  // the computed row h goes to its interior columns only
  const int wlo = ring, whi = W - ring;
  const bool full_vec = c >= wlo && c + V <= whi;
  auto store_row = [&](int h, const float* res) {
    TS* o = dst + (static_cast<int64_t>(h) * pitch + c);
    if (full_vec) {
      if constexpr (sizeof(TS) == 4) {
        *reinterpret_cast<float4*>(o) = make_float4(res[0], res[1], res[2], res[3]);
      } else {
        const __nv_bfloat162 b0 = __floats2bfloat162_rn(res[0], res[1]);
        const __nv_bfloat162 b1 = __floats2bfloat162_rn(res[2], res[3]);
        *reinterpret_cast<uint2*>(o) =
            make_uint2(*reinterpret_cast<const uint32_t*>(&b0), *reinterpret_cast<const uint32_t*>(&b1));
      }
    } else {
#pragma unroll
      for (int k = 0; k < V; ++k)
        if (c + k >= wlo && c + k < whi) o[k] = Storage<TS>::store(res[k]);
    }
  };

  // one row: load row h+1+kPD (and the winds of row h+kPD), then compute row h
  auto step = [&](int h, Row<TS>& dn, Row<TS>& cur, Row<TS>& up, Row<TS>& nx, Vt& uc, Vt& vc, Vt& un, Vt& vn) {
    ld_row(h + 1 + kPD, nx);
    ld_wind(h + kPD, un, vn);
    // west / east neighbours of the three rows: adjacent lanes, or the edge loads
    float wd = __shfl_up_sync(0xFFFFFFFFu, dn.v.at(V - 1), 1), ed = __shfl_down_sync(0xFFFFFFFFu, dn.v.at(0), 1);
    float wc = __shfl_up_sync(0xFFFFFFFFu, cur.v.at(V - 1), 1), ec = __shfl_down_sync(0xFFFFFFFFu, cur.v.at(0), 1);
    float wup = __shfl_up_sync(0xFFFFFFFFu, up.v.at(V - 1), 1), eup = __shfl_down_sync(0xFFFFFFFFu, up.v.at(0), 1);
    if (lane == 0) {
      wd = dn.l;
      wc = cur.l;
      wup = up.l;
    }
    if (lane == 31) {
      ed = dn.r;
      ec = cur.r;
      eup = up.r;
    }
    float res[V];
#pragma unroll
    for (int k = 0; k < V; ++k) {
      if constexpr (kAdvect) {
        res[k] = advect_cell(cur.v.at(k), dn.v.at(k), val(cur, wc, ec, k + 1), val(cur, wc, ec, k - 1), up.v.at(k),
                             uc.at(k), vc.at(k), p.K, p.dt, p.inv_dx);
      } else {
        float acc = 0.0f;
#pragma unroll
        for (int n = 0; n < kTerms; ++n) {
          const int dh = shape_of<kShape>().dh[n], dw = shape_of<kShape>().dw[n];
          const float x = (dh < 0) ? val(dn, wd, ed, k + dw)
                                   : (dh > 0 ? val(up, wup, eup, k + dw) : val(cur, wc, ec, k + dw));
          const float t = __fmul_rn(p.wt[n], x);
          acc = (n == 0) ? t : __fadd_rn(acc, t);
        }
        res[k] = acc;
      }
    }
    if (c_ok) store_row(h, res);
  };

  // row slots A..E (winds aligned with them), rotated by unrolling the march
  // 3 + kPD times: no value moves between registers
  Row<TS> A, B, C, D, E;
  Vt uA, vA, uB, vB, uC, vC, uD, vD, uE, vE;
  ld_row(hs - 1, A);
  ld_row(hs, B);
  ld_row(hs + 1, C);
  ld_wind(hs, uB, vB);
  if constexpr (kPD == 1) {
    for (int h = hs; h < he; h += 4) {
      step(h, A, B, C, D, uB, vB, uC, vC);
      if (h + 1 >= he) break;
      step(h + 1, B, C, D, A, uC, vC, uD, vD);
      if (h + 2 >= he) break;
      step(h + 2, C, D, A, B, uD, vD, uA, vA);
      if (h + 3 >= he) break;
      step(h + 3, D, A, B, C, uA, vA, uB, vB);
    }
  } else {
    ld_row(hs + 2, D);
    ld_wind(hs + 1, uC, vC);
    for (int h = hs; h < he; h += 5) {
      step(h, A, B, C, E, uB, vB, uD, vD);
      if (h + 1 >= he) break;
      step(h + 1, B, C, D, A, uC, vC, uE, vE);
      if (h + 2 >= he) break;
      step(h + 2, C, D, E, B, uD, vD, uA, vA);
      if (h + 3 >= he) break;
      step(h + 3, D, E, A, C, uE, vE, uB, vB);
      if (h + 4 >= he) break;
      step(h + 4, E, A, B, D, uA, vA, uC, vC);
    }
  }
}

template <class TS>
cudaError_t launch(int opk, const Stencil2DParams& p, int blocks, cudaStream_t s) {
  switch (opk) {
    case 0: stream2d_kernel<TS, 0><<<blocks, kStreamThreads, 0, s>>>(p); break;
    case 1: stream2d_kernel<TS, 1><<<blocks, kStreamThreads, 0, s>>>(p); break;
    case 2: stream2d_kernel<TS, 2><<<blocks, kStreamThreads, 0, s>>>(p); break;
    default: stream2d_kernel<TS, 3><<<blocks, kStreamThreads, 0, s>>>(p); break;
  }
  return cudaGetLastError();
}

}  // namespace

int64_t stream2d_warps(int W, int H, int HC, int dtype) {
  (void)dtype;
  const int V = 4;
  return static_cast<int64_t>((W + 32 * V - 1) / (32 * V)) * ((H + HC - 1) / HC);
}

cudaError_t stream2d_step(int opk, int dtype, const Stencil2DParams& p, cudaStream_t s) {
  const int64_t warps = stream2d_warps(p.W, p.H, p.TH, dtype);
  const int blocks = static_cast<int>((warps + kStreamThreads / 32 - 1) / (kStreamThreads / 32));
  if (blocks <= 0) return cudaSuccess;
  return dtype == 2 ? launch<__nv_bfloat16>(opk, p, blocks, s) : launch<float>(opk, p, blocks, s);
}

}  // namespace pskel
