// 2D fp32 / bf16-storage stencils of reach 1 (a known linear shape, or the
// advection-diffusion op), one step per launch, streaming: the path for
// schedules of one time step per pass, where a step moves every cell through
// HBM once and temporal blocking has nothing to reuse. Only cells with
// ring <= h < H-ring and ring <= w < W-ring are written, so each buffer keeps
// its own ring, as in Stencil2D::runOpenMP (PSkelStencil.hpp:2197-2257).
//
// Arithmetic is the oracle's: products and sums in mask order, unfused
// (two neighbouring cells per instruction with the paired fp32 forms of
// common.cuh), bf16 results rounded every step.
#include "fast2d_tile.cuh"

namespace pskel {
namespace {

using fast2d::advect_pair;
using fast2d::shape_of;

// Rows are staged by TMA. A persistent block owns work items of 32 16-byte
// vectors of columns (128 fp32 / 256 bf16 cells) x p.TH rows. A producer warp streams boxes of 8 rows (the row above
// the group first) and 16 bytes of halo columns each side -- and, for
// advection, the 8 rows of winds beside them -- into a ring of slots; the
// consumer warps compute the 8 rows of a group, kRW consecutive rows each,
// reading the kRW + 2 source rows once from shared memory and sharing their
// conversions and neighbour shuffles between the rows. Each slot has a "full"
// and an "empty" mbarrier; every wait is bounded.
constexpr int kR2Slots = 4;
constexpr int kR2Rows = 8;                    // rows per box and per group
constexpr int kR2PhiBytes = (16 + 512 + 16) * kR2Rows;   // 4352
constexpr int kR2WindBytes = 512 * kR2Rows;             // 4096
constexpr int kR2RW = 2;                      // rows per consumer warp
constexpr int kR2Cons = kR2Rows / kR2RW;      // consumer warps
constexpr int kR2Threads = 32 * (kR2Cons + 1);

template <bool kAdvect>
struct R2Slot {
  static constexpr int kBytes = kAdvect ? kR2PhiBytes + 2 * kR2WindBytes : kR2PhiBytes;
  static constexpr int kStride = (kBytes + 127) & ~127;
};

__device__ __forceinline__ void mbar_arrive1(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

template <class TS, int OpK>
__global__ void __launch_bounds__(kR2Threads, 4) stream2d_tma_kernel(const __grid_constant__ CUtensorMap map_phi,
                                                                  const __grid_constant__ CUtensorMap map_u,
                                                                  const __grid_constant__ CUtensorMap map_v,
                                                                  const __grid_constant__ Stencil2DParams p) {
  using Vt = Vec16<TS>;
  constexpr int V = Vt::V;
  constexpr int ES = static_cast<int>(sizeof(TS));
  constexpr bool kAdvect = (OpK == 3);
  constexpr int kShape = OpK < 3 ? OpK : 0;
  constexpr int kTerms = shape_of<kShape>().n;
  constexpr int kStride = R2Slot<kAdvect>::kStride;
  extern __shared__ __align__(128) uint8_t smem_raw[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if ((smem_u32(smem_raw) & 127u) != 0) {
    if (tid == 0) atomicOr(p.err, kDevErrAlign);
    return;
  }
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + kR2Slots * kStride);
  uint64_t* empty = full + kR2Slots;
  if (tid == 0) {
    for (int i = 0; i < kR2Slots; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], kR2Cons);
    }
    fence_barrier_init();
  }
  __syncthreads();
  const int W = p.W, H = p.H, ring = p.ring;
  float2 wt2[kTerms > 0 ? kTerms : 1];
#pragma unroll
  for (int n = 0; n < kTerms; ++n) wt2[n] = make_float2(p.wt[n], p.wt[n]);
  const float2 nz = neg_zero2(p.fuse_guard);
  const int strips = (W + 32 * V - 1) / (32 * V);
  const int64_t items = static_cast<int64_t>(strips) * p.tiles_y;
  // rows of an item that are written: [hs, he)
  auto item = [&](int64_t it, int& c0, int& hs, int& he) {
    const int sb = static_cast<int>(it % strips);
    const int rc = static_cast<int>(it / strips);
    c0 = sb * 32 * V;
    hs = max(rc * p.TH, ring);
    he = min(min(rc * p.TH + p.TH, H), H - ring);
  };
  auto groups_of = [](int hs, int he) { return he > hs ? (he - hs + kR2Rows - 1) / kR2Rows : 0; };

  if (warp == kR2Cons) {
    // ---- producer: boxes 0 .. groups of every item (box k: rows hs+8k-1 ..)
    if (lane == 0) {
      prefetch_tensormap(&map_phi);
      if constexpr (kAdvect) {
        prefetch_tensormap(&map_u);
        prefetch_tensormap(&map_v);
      }
      int slot = 0;
      uint32_t use = 0;
      for (int64_t it = blockIdx.x; it < items; it += gridDim.x) {
        int c0, hs, he;
        item(it, c0, hs, he);
        const int ng = groups_of(hs, he);
        if (ng == 0) continue;
        const int xp = (c0 * ES - 16) / 4;  // 32-bit words, 16 bytes before c0
        const int xw = c0 * ES / 4;
        for (int k = 0; k <= ng; ++k) {
          if (use > 0 && !mbar_wait_bounded(&empty[slot], (use - 1) & 1u, p.err)) return;
          uint8_t* dst = smem_raw + slot * kStride;
          fence_proxy_async();
          mbar_arrive_expect_tx(&full[slot], static_cast<uint32_t>(R2Slot<kAdvect>::kBytes));
          tma_load_2d(dst, &map_phi, xp, hs + kR2Rows * k - 1, &full[slot]);
          if constexpr (kAdvect) {
            tma_load_2d(dst + kR2PhiBytes, &map_u, xw, hs + kR2Rows * k, &full[slot]);
            tma_load_2d(dst + kR2PhiBytes + kR2WindBytes, &map_v, xw, hs + kR2Rows * k, &full[slot]);
          }
          if (++slot == kR2Slots) {
            slot = 0;
            ++use;
          }
        }
      }
    }
    return;
  }

  // ---- consumers: warp w computes rows hs + 8k + kR2RW*w .. + kR2RW-1 of group k
  TS* __restrict__ dst = static_cast<TS*>(p.dst);
  const int64_t pitch = p.pitch;
  auto next = [](int s) { return s + 1 == kR2Slots ? 0 : s + 1; };
  int s_next = 0;
  uint32_t ph_next = 0;
  // the row `r` (0..7, or 8+ for the next box) of the group's staged phi rows
  // and the row's edge cell for lane 0 (west) / lane 31 (east)
  const EdgeCell<TS> edge(lane);
  auto ld_row = [&](int slot_a, int slot_b, int r, Vt& v, float& h) {
    const int sl = (r < kR2Rows) ? slot_a : slot_b;
    const int rr = (r < kR2Rows) ? r : r - kR2Rows;
    const uint8_t* row = smem_raw + sl * kStride + rr * (16 + 512 + 16);
    const uint4 x = *reinterpret_cast<const uint4*>(row + 16 + lane * 16);
    v.r[0] = x.x;
    v.r[1] = x.y;
    v.r[2] = x.z;
    v.r[3] = x.w;
    h = edge.get(row);
  };
  bool alive = true;
  for (int64_t it = blockIdx.x; it < items && alive; it += gridDim.x) {
    int c0, hs, he;
    item(it, c0, hs, he);
    const int ng = groups_of(hs, he);
    if (ng == 0) continue;
    const int c = c0 + lane * V;
    const bool c_ok = c < W;
    const int wlo = ring, whi = W - ring;
    const bool full_vec = c >= wlo && c + V <= whi;
    int s_a = s_next;
    uint32_t ph_a = ph_next;
    if (!mbar_wait_bounded(&full[s_a], ph_a, p.err)) {
      alive = false;
      break;
    }
    for (int k = 0; k < ng; ++k) {
      const int s_b = next(s_a);
      const uint32_t ph_b = ph_a ^ ((s_b == 0) ? 1u : 0u);
      if (!mbar_wait_bounded(&full[s_b], ph_b, p.err)) {
        alive = false;
        break;
      }
      const int rbase = hs + kR2Rows * k + warp * kR2RW;
      // staged rows rbase-1 .. rbase+kR2RW, with their west and east neighbours
      Vt rows[kR2RW + 2];
      float rh[kR2RW + 2];
#pragma unroll
      for (int q = 0; q < kR2RW + 2; ++q) ld_row(s_a, s_b, warp * kR2RW + q, rows[q], rh[q]);
      Vt uu[kR2RW], vv[kR2RW];
      if constexpr (kAdvect) {
#pragma unroll
        for (int j = 0; j < kR2RW; ++j) {
          const uint8_t* wrow = smem_raw + s_a * kStride + kR2PhiBytes + (warp * kR2RW + j) * 512 + lane * 16;
          const uint4 a = *reinterpret_cast<const uint4*>(wrow);
          const uint4 b = *reinterpret_cast<const uint4*>(wrow + kR2WindBytes);
          uu[j].r[0] = a.x; uu[j].r[1] = a.y; uu[j].r[2] = a.z; uu[j].r[3] = a.w;
          vv[j].r[0] = b.x; vv[j].r[1] = b.y; vv[j].r[2] = b.z; vv[j].r[3] = b.w;
        }
      }
      // box k (slot a) is done: group k-1 and this group were its readers
      __syncwarp();
      if (lane == 0) mbar_arrive1(&empty[s_a]);
      float wq[kR2RW + 2], eq[kR2RW + 2];
#pragma unroll
      for (int q = 0; q < kR2RW + 2; ++q) {
        wq[q] = __shfl_up_sync(0xFFFFFFFFu, rows[q].at(V - 1), 1);
        eq[q] = __shfl_down_sync(0xFFFFFFFFu, rows[q].at(0), 1);
        if (lane == 0) wq[q] = rh[q];
        if (lane == 31) eq[q] = rh[q];
      }
      auto val = [&](int q, int kk) -> float {
        return (kk < 0) ? wq[q] : (kk >= V ? eq[q] : rows[q].at(kk));
      };
#pragma unroll
      for (int j = 0; j < kR2RW; ++j) {
        const int r = rbase + j;
        if (!(r < he && c_ok)) continue;
        // two neighbouring cells per instruction (cells kk, kk+1: lanes .x, .y)
        float res[V];
#pragma unroll
        for (int kk = 0; kk < V; kk += 2) {
          auto pr = [&](int q, int k0) { return make_float2(val(q, k0), val(q, k0 + 1)); };
          float2 r2;
          if constexpr (kAdvect) {
            r2 = advect_pair(pr(j + 1, kk), pr(j, kk), pr(j + 1, kk + 1), pr(j + 1, kk - 1), pr(j + 2, kk),
                             make_float2(uu[j].at(kk), uu[j].at(kk + 1)), make_float2(vv[j].at(kk), vv[j].at(kk + 1)),
                             p.K, p.dt, p.inv_dx, nz);
          } else {
#pragma unroll
            for (int n = 0; n < kTerms; ++n) {
              const int dh = shape_of<kShape>().dh[n], dw = shape_of<kShape>().dw[n];
              // a row neighbour (dw != 0) straddles two register pairs: one
              // product per lane
              const float2 t = (dw == 0) ? fmul2_rn(wt2[n], pr(j + 1 + dh, kk), nz)
                                         : make_float2(__fmul_rn(p.wt[n], val(j + 1 + dh, kk + dw)),
                                                       __fmul_rn(p.wt[n], val(j + 1 + dh, kk + 1 + dw)));
              r2 = (n == 0) ? t : fadd2_rn(r2, t);
            }
          }
          res[kk] = r2.x;
          res[kk + 1] = r2.y;
        }
        TS* o = dst + (static_cast<int64_t>(r) * pitch + c);
        if (full_vec) {
          uint32_t w4[4];
          if constexpr (ES == 4) {
#pragma unroll
            for (int q = 0; q < 4; ++q) w4[q] = __float_as_uint(res[q]);
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const __nv_bfloat162 b2 = __floats2bfloat162_rn(res[2 * q], res[2 * q + 1]);
              w4[q] = *reinterpret_cast<const uint32_t*>(&b2);
            }
          }
          *reinterpret_cast<uint4*>(o) = make_uint4(w4[0], w4[1], w4[2], w4[3]);
        } else {
#pragma unroll
          for (int q = 0; q < V; ++q)
            if (c + q >= wlo && c + q < whi) o[q] = Storage<TS>::store(res[q]);
        }
      }
      s_a = s_b;
      ph_a = ph_b;
    }
    if (!alive) break;
    // the item's last box (rows below its last group) is released here
    __syncwarp();
    if (lane == 0) mbar_arrive1(&empty[s_a]);
    s_next = next(s_a);
    ph_next = ph_a ^ ((s_next == 0) ? 1u : 0u);
  }
}

template <class TS, int OpK>
void* tma_kernel_ptr() {
  return reinterpret_cast<void*>(stream2d_tma_kernel<TS, OpK>);
}

void* tma_kernel(int opk, int dtype) {
  if (dtype == 2) {
    switch (opk) {
      case 0: return tma_kernel_ptr<__nv_bfloat16, 0>();
      case 1: return tma_kernel_ptr<__nv_bfloat16, 1>();
      case 2: return tma_kernel_ptr<__nv_bfloat16, 2>();
      default: return tma_kernel_ptr<__nv_bfloat16, 3>();
    }
  }
  switch (opk) {
    case 0: return tma_kernel_ptr<float, 0>();
    case 1: return tma_kernel_ptr<float, 1>();
    case 2: return tma_kernel_ptr<float, 2>();
    default: return tma_kernel_ptr<float, 3>();
  }
}

size_t tma_smem(int opk) {
  const size_t stride = (opk == 3) ? R2Slot<true>::kStride : R2Slot<false>::kStride;
  return kR2Slots * stride + 16 * kR2Slots;
}

}  // namespace

int stream2d_tma_blocks_per_sm(int opk, int dtype) {
  void* k = tma_kernel(opk, dtype);
  const size_t smem = tma_smem(opk);
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kR2Threads, smem) != cudaSuccess) n = 1;
  return n > 0 ? n : 1;
}

int64_t stream2d_tma_items(int W, int H, int HC, int dtype) {
  const int V = dtype == 2 ? 8 : 4;
  return static_cast<int64_t>((W + 32 * V - 1) / (32 * V)) * ((H + HC - 1) / HC);
}

cudaError_t stream2d_tma_step(int opk, int dtype, const CUtensorMap* phi, const CUtensorMap* u, const CUtensorMap* v,
                              const Stencil2DParams& p, int ctas, cudaStream_t s) {
  void* k = tma_kernel(opk, dtype);
  const size_t smem = tma_smem(opk);
  void* args[] = {const_cast<CUtensorMap*>(phi), const_cast<CUtensorMap*>(u), const_cast<CUtensorMap*>(v),
                  const_cast<Stencil2DParams*>(&p)};
  return cudaLaunchKernel(k, dim3(ctas), dim3(kR2Threads), args, smem, s);
}

}  // namespace pskel
