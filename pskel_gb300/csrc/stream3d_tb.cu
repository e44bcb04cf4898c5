// The 7-point 3D cross, TWO steps per launch: the plane-streaming kernel of
// stencil3d.cu with a second time level fused behind the first.
//
// A persistent block owns work items of 32 vectors of d (128 fp32 / 256 bf16
// cells) x 16 w rows x HC planes, as the one-step kernel does. A producer
// warp streams the source planes h0-2 .. h1+1 of its items by 3D TMA (boxes
// of 34 vectors x 20 rows: two rows and a vector of halo on each side, zero
// outside the grid) into a ring of 4 slots. For each plane p = h0-1 .. h1
// the block computes the first step (level 1) of plane p over 18 rows
// (w0-1 .. w0+16) and the two edge cells d0-1 and d0+32V of the 16 core rows
// into a ring of 3 level-1 planes in shared memory, and then the second step
// (level 2) of plane p-1 over the core from level-1 planes p-2, p-1, p, which
// goes to HBM. HBM therefore sees one read and one write of the grid per two
// steps. Level-1 values are rounded to the storage type, as the step-by-step
// run stores them, and cells outside the grid hold the halo value, so the
// second step reads exactly what the first step of a step-by-step run wrote.
//
// Warps: 4 consumer warps (level 1 and level 2 of 4 core rows each), an edge
// warp (level 1 of the rows w0-1 and w0+16 and of the 32 edge cells), the
// producer. Two named barriers per plane: between level 1 and level 2, and
// after level 2, before level 1 of the next plane overwrites the oldest of the
// three level-1 slots. Every wait is bounded.
//
// Arithmetic: the reference's order (centre, h-1, h+1, w-1, w+1, d-1, d+1),
// __fmul_rn / __fadd_rn (two cells per instruction in the vector rows,
// cross7_row), no contraction: bit-identical to two launches of the
// one-step kernel.
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "kernels.h"

namespace pskel {
namespace {

constexpr int kTbBoxX = 34;                  // 16-byte vectors per staged row
constexpr int kTbRowBytes = kTbBoxX * 16;    // 544
constexpr int kTbL0Rows = 20;                // w0-2 .. w0+17
constexpr int kTbL1Rows = 18;                // w0-1 .. w0+16
constexpr int kTbL0Bytes = (kTbRowBytes * kTbL0Rows + 127) & ~127;
constexpr int kTbL1Bytes = (kTbRowBytes * kTbL1Rows + 127) & ~127;
constexpr int kTbL0Slots = 4;
constexpr int kTbL1Slots = 3;
constexpr int kTbCons = 4;                   // consumer warps, 4 core rows each
constexpr int kTbRW = 4;
constexpr int kTbEdge = kTbCons;             // warp index of the edge warp
constexpr int kTbProd = kTbCons + 1;         // warp index of the producer
constexpr int kTbThreads = 32 * (kTbCons + 2);
constexpr int kTbSync = 32 * (kTbCons + 1);  // consumers + edge warp
constexpr size_t kTbSmem = static_cast<size_t>(kTbL0Slots) * kTbL0Bytes +
                           static_cast<size_t>(kTbL1Slots) * kTbL1Bytes + 16 * kTbL0Slots;

__device__ __forceinline__ void tb_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kTbSync) : "memory"); }

// 7-point weighted sum in the reference's order, unfused.
__device__ __forceinline__ float cross7(const float* wt, float c, float dn, float up, float a, float b, float l,
                                        float r) {
  float acc = __fmul_rn(wt[0], c);
  acc = __fadd_rn(acc, __fmul_rn(wt[1], dn));
  acc = __fadd_rn(acc, __fmul_rn(wt[2], up));
  acc = __fadd_rn(acc, __fmul_rn(wt[3], a));
  acc = __fadd_rn(acc, __fmul_rn(wt[4], b));
  acc = __fadd_rn(acc, __fmul_rn(wt[5], l));
  acc = __fadd_rn(acc, __fmul_rn(wt[6], r));
  return acc;
}

// A 16-byte vector read from / written to shared memory.
template <class TS>
__device__ __forceinline__ void lds(const uint8_t* p, Vec16<TS>& v) {
  const uint4 x = *reinterpret_cast<const uint4*>(p);
  v.r[0] = x.x;
  v.r[1] = x.y;
  v.r[2] = x.z;
  v.r[3] = x.w;
}
__device__ __forceinline__ void sts(uint8_t* p, const uint32_t (&o)[4]) {
  *reinterpret_cast<uint4*>(p) = make_uint4(o[0], o[1], o[2], o[3]);
}

template <class TS>
__device__ __forceinline__ float ld_cell(const uint8_t* p) {
  return Storage<TS>::load(*reinterpret_cast<const TS*>(p));
}
template <class TS>
__device__ __forceinline__ void st_cell(uint8_t* p, float v) {
  *reinterpret_cast<TS*>(p) = Storage<TS>::store(v);
}

// Rounds V results to the storage type: packed words `o`, and the stored
// values widened back (what the next step reads) in `stored`.
template <class TS>
__device__ __forceinline__ void pack_row(const float (&res)[16 / sizeof(TS)], uint32_t (&o)[4],
                                         float (&stored)[16 / sizeof(TS)]) {
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
}



// kRep: bit 0 reports ||u_1 - u_0|| (the first step of the pass), bit 1
// ||u_2 - u_1|| (the second), as one fp64 partial per block each.
template <class TS, bool kZeroHalo, int kRep>
__global__ void __launch_bounds__(kTbThreads, 3)
    stream3d_tb2_kernel(const __grid_constant__ CUtensorMap map, const __grid_constant__ Stencil3DParams p) {
  using Vt = Vec16<TS>;
  constexpr int V = Vt::V;
  constexpr int ES = static_cast<int>(sizeof(TS));
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ double s_part[2][kTbCons];
  __shared__ int s_abort;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if ((smem_u32(smem) & 127u) != 0) {  // uniform across the block
    if (tid == 0) atomicOr(p.err, kDevErrAlign);
    return;
  }
  uint8_t* const l0 = smem;
  uint8_t* const l1 = smem + kTbL0Slots * kTbL0Bytes;
  uint64_t* full = reinterpret_cast<uint64_t*>(l1 + kTbL1Slots * kTbL1Bytes);
  uint64_t* empty = full + kTbL0Slots;
  if (tid == 0) {
    for (int i = 0; i < kTbL0Slots; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], kTbCons + 1);
    }
    fence_barrier_init();
    s_abort = 0;
  }
  __syncthreads();

  const int H = p.H, W = p.W, D = p.D;
  const int dblocks = (D + 32 * V - 1) / (32 * V), wblocks = (W + 15) / 16;
  const int64_t items = static_cast<int64_t>(dblocks) * wblocks * p.hchunks;
  auto geometry = [&](int64_t it, int& d0, int& w0, int& h0, int& h1) {
    const int db = static_cast<int>(it % dblocks);
    const int64_t r = it / dblocks;
    d0 = db * 32 * V;
    w0 = static_cast<int>(r % wblocks) * 16;
    h0 = static_cast<int>(r / wblocks) * p.HC;
    h1 = min(H, h0 + p.HC);
  };

  if (warp == kTbProd) {
    // ---- producer: source planes h0-2 .. h1+1 of every item, in order
    if (lane == 0) {
      prefetch_tensormap(&map);
      uint32_t n0 = 0;
      for (int64_t it = blockIdx.x; it < items; it += gridDim.x) {
        int d0, w0, h0, h1;
        geometry(it, d0, w0, h0, h1);
        const int x = (d0 - V) * ES / 4;  // the map addresses the grid as 32-bit words
        for (int q = h0 - 2; q <= h1 + 1; ++q, ++n0) {
          const int slot = static_cast<int>(n0 % kTbL0Slots);
          if (n0 >= kTbL0Slots && !mbar_wait_bounded(&empty[slot], ((n0 / kTbL0Slots) - 1) & 1u, p.err)) return;
          fence_proxy_async();
          mbar_arrive_expect_tx(&full[slot], static_cast<uint32_t>(kTbRowBytes * kTbL0Rows));
          tma_load_3d(l0 + slot * kTbL0Bytes, &map, x, w0 - 2, q, &full[slot]);
        }
      }
    }
    return;
  }

  // ---- consumers (warps 0..3) and the edge warp (warp 4)
  const float halo = p.halo;
  uint32_t hraw;
  if constexpr (ES == 4) {
    hraw = __float_as_uint(halo);
  } else {
    const uint32_t hb = __bfloat16_as_ushort(__float2bfloat16_rn(halo));
    hraw = hb | (hb << 16);
  }
  const float hst = Storage<TS>::load(Storage<TS>::store(halo));  // the halo as stored
  float wt[7];
#pragma unroll
  for (int n = 0; n < 7; ++n) wt[n] = p.wt[n];
  float2 wt2[5];
#pragma unroll
  for (int n = 0; n < 5; ++n) wt2[n] = make_float2(wt[n], wt[n]);
  const float2 nz = neg_zero2(p.fuse_guard);
  TS* __restrict__ dst = static_cast<TS*>(p.dst);
  const int64_t plane = static_cast<int64_t>(W) * D;
  const bool edge = warp == kTbEdge;
  SqDiffAcc acc1, acc2;
  double tot1 = 0.0, tot2 = 0.0;
  uint32_t n0 = 0, n1 = 0;  // source planes consumed / level-1 planes computed by this block
  auto l0p = [&](uint32_t n) -> const uint8_t* { return l0 + (n % kTbL0Slots) * kTbL0Bytes; };
  auto l1p = [&](uint32_t n) -> uint8_t* { return l1 + (n % kTbL1Slots) * kTbL1Bytes; };
  auto wait_l0 = [&](uint32_t n) -> bool {
    return mbar_wait_bounded(&full[n % kTbL0Slots], (n / kTbL0Slots) & 1u, p.err);
  };
  const int vo = (lane + 1) * 16;  // this lane's vector in a staged row

  for (int64_t it = blockIdx.x; it < items; it += gridDim.x) {
    int d0, w0, h0, h1;
    geometry(it, d0, w0, h0, h1);
    const int d = d0 + lane * V;
    const bool d_ok = d < D;
    const bool el_in = d0 > 0, er_in = d0 + 32 * V < D;
    int ok = wait_l0(n0) && wait_l0(n0 + 1);
    for (int pl = h0 - 1; pl <= h1; ++pl) {
      const uint32_t i0 = n0 + static_cast<uint32_t>(pl - (h0 - 1));  // source plane pl-1
      if (ok) ok = wait_l0(i0 + 2);
      if (!ok) s_abort = 1;
      const uint8_t* Ldn = l0p(i0);
      const uint8_t* Lcur = l0p(i0 + 1);
      const uint8_t* Lup = l0p(i0 + 2);
      uint8_t* L1w = l1p(n1);
      const bool plane_in = pl >= 0 && pl < H;
      const bool dn_in = pl - 1 >= 0, up_in = pl + 1 < H;
      // ---------------- level 1 of plane pl
      if (ok && !edge) {
        // rows r = 4 warp + j (0..15), one at a time with a rolling window of
        // three centre-plane rows (staged rows r+1 .. r+3): few vectors live
        const int rb = kTbRW * warp;
        Vt a, c;
        lds(Lcur + (rb + 1) * kTbRowBytes + vo, a);
        lds(Lcur + (rb + 2) * kTbRowBytes + vo, c);
        if constexpr (!kZeroHalo) {
          if (!d_ok || w0 + rb - 1 < 0 || w0 + rb - 1 >= W) a.fill(hraw);
          if (!d_ok || w0 + rb >= W) c.fill(hraw);
        }
#pragma unroll
        for (int j = 0; j < kTbRW; ++j) {
          const int w = w0 + rb + j;
          Vt b, dn, up;
          lds(Lcur + (rb + 3 + j) * kTbRowBytes + vo, b);
          lds(Ldn + (rb + 2 + j) * kTbRowBytes + vo, dn);
          lds(Lup + (rb + 2 + j) * kTbRowBytes + vo, up);
          float el = ld_cell<TS>(Lcur + (rb + 2 + j) * kTbRowBytes + (V - 1) * ES);
          float er = ld_cell<TS>(Lcur + (rb + 2 + j) * kTbRowBytes + 33 * 16);
          if constexpr (!kZeroHalo) {
            if (!d_ok || w + 1 >= W) b.fill(hraw);
            if (!dn_in || !d_ok || w >= W) dn.fill(hraw);
            if (!up_in || !d_ok || w >= W) up.fill(hraw);
            if (!el_in) el = halo;
            if (!er_in) er = halo;
          }
          float dl = __shfl_up_sync(0xFFFFFFFFu, c.at(V - 1), 1);
          float dr = __shfl_down_sync(0xFFFFFFFFu, c.at(0), 1);
          if (lane == 0) dl = el;
          if (lane == 31) dr = er;
          float res[V], stored[V];
          cross7_row<true>(wt, wt2, nz, c, dn, up, a, b, dl, dr, res);
          uint32_t o[4];
          pack_row<TS>(res, o, stored);
          const bool valid = plane_in && d_ok && w < W;
          if (!valid) {
            o[0] = o[1] = o[2] = o[3] = hraw;
          } else if ((kRep & 1) && pl >= h0 && pl < h1) {
#pragma unroll
            for (int k = 0; k < V; ++k) acc1.add(stored[k], c.at(k));
          }
          sts(L1w + (rb + 1 + j) * kTbRowBytes + vo, o);
          a = c;
          c = b;
        }
        if (kRep & 1) acc1.flush(tot1);
      } else if (ok) {
        // the edge warp: rows w0-1 and w0+16 of level 1 ...
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int r = e ? 16 : -1;  // core-relative row; staged row r+2, level-1 row r+1
          const int w = w0 + r;
          Vt c, a, b, dn, up;
          lds(Lcur + (r + 1) * kTbRowBytes + vo, a);
          lds(Lcur + (r + 2) * kTbRowBytes + vo, c);
          lds(Lcur + (r + 3) * kTbRowBytes + vo, b);
          lds(Ldn + (r + 2) * kTbRowBytes + vo, dn);
          lds(Lup + (r + 2) * kTbRowBytes + vo, up);
          float el = ld_cell<TS>(Lcur + (r + 2) * kTbRowBytes + (V - 1) * ES);
          float er = ld_cell<TS>(Lcur + (r + 2) * kTbRowBytes + 33 * 16);
          if constexpr (!kZeroHalo) {
            if (!d_ok || w - 1 < 0 || w - 1 >= W) a.fill(hraw);
            if (!d_ok || w < 0 || w >= W) c.fill(hraw);
            if (!d_ok || w + 1 < 0 || w + 1 >= W) b.fill(hraw);
            if (!dn_in || !d_ok || w < 0 || w >= W) dn.fill(hraw);
            if (!up_in || !d_ok || w < 0 || w >= W) up.fill(hraw);
            if (!el_in) el = halo;
            if (!er_in) er = halo;
          }
          float dl = __shfl_up_sync(0xFFFFFFFFu, c.at(V - 1), 1);
          float dr = __shfl_down_sync(0xFFFFFFFFu, c.at(0), 1);
          if (lane == 0) dl = el;
          if (lane == 31) dr = er;
          float res[V], stored[V];
          cross7_row<true>(wt, wt2, nz, c, dn, up, a, b, dl, dr, res);
          uint32_t o[4];
          pack_row<TS>(res, o, stored);
          if (!(plane_in && d_ok && w >= 0 && w < W)) o[0] = o[1] = o[2] = o[3] = hraw;
          sts(L1w + (r + 1) * kTbRowBytes + vo, o);
        }
        // ... and the cells d0-1 (lanes 0..15) and d0+32V (lanes 16..31) of the core rows
        {
          const int r = lane & 15, side = lane >> 4;
          const int w = w0 + r;
          const int dd = side ? d0 + 32 * V : d0 - 1;
          const int oc = side ? 33 * 16 : (V - 1) * ES;       // the cell
          const int ol = side ? 32 * 16 + (V - 1) * ES : (V - 2) * ES;  // its d-1 neighbour
          const int orr = side ? 33 * 16 + ES : 16;           // its d+1 neighbour
          const uint8_t* rc = Lcur + (r + 2) * kTbRowBytes;
          float c = ld_cell<TS>(rc + oc);
          float a = ld_cell<TS>(rc - kTbRowBytes + oc);
          float b = ld_cell<TS>(rc + kTbRowBytes + oc);
          float dn = ld_cell<TS>(Ldn + (r + 2) * kTbRowBytes + oc);
          float up = ld_cell<TS>(Lup + (r + 2) * kTbRowBytes + oc);
          float l = ld_cell<TS>(rc + ol);
          float rr = ld_cell<TS>(rc + orr);
          const bool cell_in = plane_in && w < W && dd >= 0 && dd < D;
          if constexpr (!kZeroHalo) {
            if (w - 1 < 0) a = halo;
            if (w + 1 >= W) b = halo;
            if (!dn_in) dn = halo;
            if (!up_in) up = halo;
            if (dd - 1 < 0) l = halo;
            if (dd + 1 >= D) rr = halo;
          }
          const float v = cell_in ? Storage<TS>::load(Storage<TS>::store(cross7(wt, c, dn, up, a, b, l, rr))) : hst;
          st_cell<TS>(L1w + (r + 1) * kTbRowBytes + oc, v);
        }
      }
      // the source plane pl-1 is read for the last time
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[i0 % kTbL0Slots]);
      tb_sync();
      if (s_abort) break;
      // ---------------- level 2 of plane pl-1 from level-1 planes pl-2, pl-1, pl
      if (!edge && pl > h0) {
        const uint8_t* Mdn = l1p(n1 - 2);
        const uint8_t* Mcur = l1p(n1 - 1);
        const uint8_t* Mup = l1p(n1);
        const int rb = kTbRW * warp;
        // level-1 rows are stored at row index r+1; cells outside the grid hold
        // the halo value already
        Vt a, c;
        lds(Mcur + rb * kTbRowBytes + vo, a);
        lds(Mcur + (rb + 1) * kTbRowBytes + vo, c);
        TS* out = dst + (static_cast<int64_t>(pl - 1) * plane + static_cast<int64_t>(w0 + rb) * D + d);
#pragma unroll
        for (int j = 0; j < kTbRW; ++j) {
          Vt b, dn, up;
          lds(Mcur + (rb + 2 + j) * kTbRowBytes + vo, b);
          lds(Mdn + (rb + 1 + j) * kTbRowBytes + vo, dn);
          lds(Mup + (rb + 1 + j) * kTbRowBytes + vo, up);
          const float el = ld_cell<TS>(Mcur + (rb + 1 + j) * kTbRowBytes + (V - 1) * ES);
          const float er = ld_cell<TS>(Mcur + (rb + 1 + j) * kTbRowBytes + 33 * 16);
          float dl = __shfl_up_sync(0xFFFFFFFFu, c.at(V - 1), 1);
          float dr = __shfl_down_sync(0xFFFFFFFFu, c.at(0), 1);
          if (lane == 0) dl = el;
          if (lane == 31) dr = er;
          float res[V], stored[V];
          cross7_row<true>(wt, wt2, nz, c, dn, up, a, b, dl, dr, res);
          uint32_t o[4];
          pack_row<TS>(res, o, stored);
          if (d_ok && w0 + rb + j < W) {
            *reinterpret_cast<uint4*>(out + j * D) = make_uint4(o[0], o[1], o[2], o[3]);
            if (kRep & 2) {
#pragma unroll
              for (int k = 0; k < V; ++k) acc2.add(stored[k], c.at(k));
            }
          }
          a = c;
          c = b;
        }
        if (kRep & 2) acc2.flush(tot2);
      }
      // every level-1 plane of the ring has been read before the next one is
      // written over the oldest
      tb_sync();
      ++n1;
    }
    if (s_abort) break;
    // source planes h1 and h1+1 are released at the end of the item
    const uint32_t last = n0 + static_cast<uint32_t>(h1 - h0 + 2);
    __syncwarp();
    if (lane == 0) {
      mbar_arrive(&empty[last % kTbL0Slots]);
      mbar_arrive(&empty[(last + 1) % kTbL0Slots]);
    }
    n0 += static_cast<uint32_t>(h1 - h0 + 4);
  }
  if constexpr (kRep != 0) {
    double v1 = tot1, v2 = tot2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v1 += __shfl_down_sync(0xFFFFFFFFu, v1, o);
      v2 += __shfl_down_sync(0xFFFFFFFFu, v2, o);
    }
    if (lane == 0 && !edge) {
      s_part[0][warp] = v1;
      s_part[1][warp] = v2;
    }
    tb_sync();
    if (tid == 0) {
      double t1 = 0.0, t2 = 0.0;
      for (int i = 0; i < kTbCons; ++i) {
        t1 += s_part[0][i];
        t2 += s_part[1][i];
      }
      // the layout reduce3d_residual reads: step k of the pass at (k-1) * ctas
      if (kRep & 1) p.partials[blockIdx.x] = t1;
      if (kRep & 2) p.partials[gridDim.x + blockIdx.x] = t2;
    }
  }
}


template <class TS, bool kZero>
void launch_tb2(const CUtensorMap* map, const Stencil3DParams& p, int ctas, int rep, cudaStream_t s) {
  switch (rep) {
    case 0: stream3d_tb2_kernel<TS, kZero, 0><<<ctas, kTbThreads, kTbSmem, s>>>(*map, p); break;
    case 1: stream3d_tb2_kernel<TS, kZero, 1><<<ctas, kTbThreads, kTbSmem, s>>>(*map, p); break;
    case 2: stream3d_tb2_kernel<TS, kZero, 2><<<ctas, kTbThreads, kTbSmem, s>>>(*map, p); break;
    default: stream3d_tb2_kernel<TS, kZero, 3><<<ctas, kTbThreads, kTbSmem, s>>>(*map, p); break;
  }
}

template <class TS>
int tb2_blocks_per_sm() {
  void* ks[8] = {reinterpret_cast<void*>(stream3d_tb2_kernel<TS, false, 0>),
                 reinterpret_cast<void*>(stream3d_tb2_kernel<TS, false, 1>),
                 reinterpret_cast<void*>(stream3d_tb2_kernel<TS, false, 2>),
                 reinterpret_cast<void*>(stream3d_tb2_kernel<TS, false, 3>),
                 reinterpret_cast<void*>(stream3d_tb2_kernel<TS, true, 0>),
                 reinterpret_cast<void*>(stream3d_tb2_kernel<TS, true, 1>),
                 reinterpret_cast<void*>(stream3d_tb2_kernel<TS, true, 2>),
                 reinterpret_cast<void*>(stream3d_tb2_kernel<TS, true, 3>)};
  int best = 1 << 30;
  for (void* k : ks) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kTbSmem));
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kTbThreads, kTbSmem) != cudaSuccess) n = 1;
    best = std::min(best, n);
  }
  return std::max(1, best);
}

}  // namespace

int stream3d_tb2_blocks_per_sm(int dtype) {
  static int cached[3] = {0, 0, 0};  // per storage type; the same on every device of a process
  const int k = dtype == 2 ? 2 : 1;
  if (cached[k] == 0) cached[k] = dtype == 2 ? tb2_blocks_per_sm<__nv_bfloat16>() : tb2_blocks_per_sm<float>();
  return cached[k];
}

uint32_t stream3d_tb2_box_rows() { return kTbL0Rows; }

cudaError_t stream3d_tb2_pass(int dtype, const CUtensorMap* map, const Stencil3DParams& p, int ctas,
                              cudaStream_t s) {
  int rep = 0;
  if (p.every > 0) {
    if ((p.step0 + 1) % p.every == 0) rep |= 1;
    if ((p.step0 + 2) % p.every == 0) rep |= 2;
  }
  uint32_t hbits;
  std::memcpy(&hbits, &p.halo, sizeof(hbits));
  const bool zero = hbits == 0u;  // +0.0 exactly: the TMA zero fill is the halo
  if (dtype == 2) {
    if (zero) launch_tb2<__nv_bfloat16, true>(map, p, ctas, rep, s);
    else launch_tb2<__nv_bfloat16, false>(map, p, ctas, rep, s);
  } else {
    if (zero) launch_tb2<float, true>(map, p, ctas, rep, s);
    else launch_tb2<float, false>(map, p, ctas, rep, s);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || rep == 0) return e;
  return stream3d_reduce_residuals(p.partials, ctas, 2, p.step0, p.every, p.residuals, s);
}

cudaError_t stream3d_tb2_band(int dtype, const CUtensorMap* map, const Stencil3DParams& p, int ctas, double* acc1,
                              double* acc2, cudaStream_t s) {
  const int rep = (acc1 ? 1 : 0) | (acc2 ? 2 : 0);
  uint32_t hbits;
  std::memcpy(&hbits, &p.halo, sizeof(hbits));
  const bool zero = hbits == 0u;  // +0.0 exactly: the TMA zero fill is the halo
  if (dtype == 2) {
    if (zero) launch_tb2<__nv_bfloat16, true>(map, p, ctas, rep, s);
    else launch_tb2<__nv_bfloat16, false>(map, p, ctas, rep, s);
  } else {
    if (zero) launch_tb2<float, true>(map, p, ctas, rep, s);
    else launch_tb2<float, false>(map, p, ctas, rep, s);
  }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && acc1) e = stream3d_accumulate(p.partials, ctas, acc1, s);
  if (e == cudaSuccess && acc2) e = stream3d_accumulate(p.partials + ctas, ctas, acc2, s);
  return e;
}

}  // namespace pskel
