// Game of Life, temporally blocked and bit-sliced.
//
// One pass advances the whole grid by up to 16 steps. Each persistent CTA
// walks tiles of 224 x TH core cells: it stages the (TH + 2T) x 256 byte halo
// tile into shared memory with one TMA load, packs the 0/1 bytes into 32-cell
// bit words, runs the steps on the bit planes (neighbour counts with
// bit-sliced full adders; one word = 32 cells per ~15 integer ops), then
// unpacks the core and writes it with 128-bit coalesced stores. Ring cells
// (outside r <= h < H-r, r <= w < W-r) are never updated and never written,
// the semantics of Stencil2D::runOpenMP (PSkelStencil.hpp:2197-2257) that the
// reference's GPU kernel also follows (guard at PSkelStencil.hpp:576).
//
// Redundant halo work: the tile carries T rows and 16 columns of halo on each
// side; garbage entering from the tile edge advances one cell per step, so
// the core is exact after T <= 16 steps.
#include "common.cuh"
#include "kernels.h"

namespace pskel {
namespace {

constexpr int kWords = kLifeLW / 32;  // 8 bit words per tile row
// Bit planes hold 256 tile rows plus a zero row above and below, and each row
// holds a zero word on either side of its 8 words, so the step loop reads
// neighbours without bounds checks. Pitch 11: the 8-row strips of one warp
// land on distinct banks.
constexpr int kBitRows = 256;
constexpr int kBitPitch = 11;
constexpr int kBitPlaneWords = (kBitRows + 2) * kBitPitch;
constexpr int kRowsPerStrip = kBitRows / (kLifeThreads / kWords);  // 8

__device__ __forceinline__ int bit_index(int row, int word) { return (row + 1) * kBitPitch + word + 1; }

// 16 cells (one byte each, value 0/1) -> 16 bits, cell i at bit i.
__device__ __forceinline__ uint32_t pack16(uint4 v) {
  const uint32_t n0 = (v.x * 0x01020408u) >> 24;
  const uint32_t n1 = (v.y * 0x01020408u) >> 24;
  const uint32_t n2 = (v.z * 0x01020408u) >> 24;
  const uint32_t n3 = (v.w * 0x01020408u) >> 24;
  return n0 | (n1 << 4) | (n2 << 8) | (n3 << 12);
}

// 16 bits -> 16 bytes of 0/1.
__device__ __forceinline__ uint4 unpack16(uint32_t h) {
  uint4 v;
  v.x = ((h & 0xFu) * 0x00204081u) & 0x01010101u;
  v.y = (((h >> 4) & 0xFu) * 0x00204081u) & 0x01010101u;
  v.z = (((h >> 8) & 0xFu) * 0x00204081u) & 0x01010101u;
  v.w = (((h >> 12) & 0xFu) * 0x00204081u) & 0x01010101u;
  return v;
}

__device__ __forceinline__ uint32_t bit_range(int lo, int hi) {
  lo = max(0, min(32, lo));
  hi = max(0, min(32, hi));
  if (hi <= lo) return 0u;
  const uint32_t upto_hi = (hi == 32) ? 0xFFFFFFFFu : ((1u << hi) - 1u);
  const uint32_t below_lo = (lo == 32) ? 0xFFFFFFFFu : ((1u << lo) - 1u);
  return upto_hi & ~below_lo;
}

// One step for a strip of 8 rows of one word column: the neighbour count of
// each cell is (w + c + e of the row above) + (w + e of its row) + (w + c + e
// of the row below), summed with bit-sliced full adders and kept mod 8
// (a count of 8 aliases to 0, which is dead either way).
template <bool kMasked>
__device__ __forceinline__ void life_strip(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, int y0, int j,
                                           uint32_t colmask, int gy0, int ring, int H) {
  uint32_t c[kRowsPerStrip + 2], t0[kRowsPerStrip + 2], t1[kRowsPerStrip + 2];
  uint32_t p0[kRowsPerStrip + 2], p1[kRowsPerStrip + 2];
  const uint32_t* base = in + bit_index(y0 - 1, j);
#pragma unroll
  for (int k = 0; k < kRowsPerStrip + 2; ++k) {
    const uint32_t* r = base + k * kBitPitch;
    const uint32_t l = r[-1], cc = r[0], e = r[1];
    const uint32_t we = __funnelshift_l(l, cc, 1);  // bit b = cell b-1
    const uint32_t ea = __funnelshift_r(cc, e, 1);  // bit b = cell b+1
    c[k] = cc;
    t0[k] = we ^ cc ^ ea;
    t1[k] = (we & cc) | (we & ea) | (cc & ea);
    p0[k] = we ^ ea;
    p1[k] = we & ea;
  }
  uint32_t* o = out + bit_index(y0, j);
#pragma unroll
  for (int k = 1; k <= kRowsPerStrip; ++k) {
    const uint32_t s0 = t0[k - 1] ^ p0[k] ^ t0[k + 1];
    const uint32_t k0 = (t0[k - 1] & p0[k]) | (t0[k - 1] & t0[k + 1]) | (p0[k] & t0[k + 1]);
    const uint32_t x1 = t1[k - 1] ^ p1[k] ^ t1[k + 1];
    const uint32_t y1 = (t1[k - 1] & p1[k]) | (t1[k - 1] & t1[k + 1]) | (p1[k] & t1[k + 1]);
    const uint32_t s1 = x1 ^ k0;
    const uint32_t s2 = y1 ^ (x1 & k0);
    const uint32_t alive = s1 & ~s2 & (s0 | c[k]);  // count 3, or count 2 and alive
    uint32_t* dst = o + (k - 1) * kBitPitch;
    if (kMasked) {
      // cells outside r <= h < H-r, r <= w < W-r keep the value this plane holds
      const int gy = gy0 + y0 + k - 1;
      const uint32_t m = (gy >= ring && gy < H - ring) ? colmask : 0u;
      *dst = (alive & m) | (*dst & ~m);
    } else {
      *dst = alive;
    }
  }
}

template <bool kTma>
__global__ void __launch_bounds__(kLifeThreads, 2)
    life_kernel(const __grid_constant__ CUtensorMap map, const __grid_constant__ CUtensorMap map_dst,
                const uint8_t* __restrict__ src, uint8_t* __restrict__ dst,
                int W, int H, int64_t pitch, int ring, int steps, int T, int TH, int LH, int tiles_x, int tiles_y,
                unsigned* err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* bytes = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  uint32_t* bitsA = reinterpret_cast<uint32_t*>(bytes + LH * kLifeLW);
  uint32_t* bitsB = bitsA + kBitPlaneWords;
  uint64_t* bar = reinterpret_cast<uint64_t*>(bitsB + kBitPlaneWords);

  const int tid = threadIdx.x;
  // zero both planes once: the padding rows/words are never written again and
  // rows at or beyond LH stay zero until the first tile's steps run over them
  for (int i = tid; i < 2 * kBitPlaneWords; i += kLifeThreads) bitsA[i] = 0u;
  if (kTma && tid == 0) {
    mbar_init(bar, 1);
    fence_barrier_init();
    prefetch_tensormap(&map);
    prefetch_tensormap(&map_dst);
  }
  __syncthreads();

  uint32_t phase = 0;
  bool bad_value = false;
  const int ntiles = tiles_x * tiles_y;
  const int j = tid & (kWords - 1);
  const int y0 = (tid >> 3) * kRowsPerStrip;  // 32 strips of 8 rows

  // The byte tile is free again as soon as it is packed into bits, so the
  // next tile's TMA load is issued before this tile's steps run.
  auto issue_load = [&](int t, const CUtensorMap* m) {
    const int ty = t / tiles_x;
    const int tx = t - ty * tiles_x;
    fence_proxy_async();
    mbar_arrive_expect_tx(bar, static_cast<uint32_t>(LH * kLifeLW));
    tma_load_2d(bytes, m, tx * kLifeTW - kLifeHX, ty * TH - T, bar);
  };
  if (kTma && tid == 0 && static_cast<int>(blockIdx.x) < ntiles) issue_load(blockIdx.x, &map);

  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int ty = tile / tiles_x;
    const int tx = tile - ty * tiles_x;
    const int gy0 = ty * TH - T;          // global row of local row 0
    const int gx0 = tx * kLifeTW - kLifeHX;  // global column of local column 0

    // Ring cells (outside r <= h < H-r, r <= w < W-r) are never written, so
    // each global buffer keeps its own ring and step k reads the ring of the
    // buffer it reads from. Tiles that reach the ring therefore also stage the
    // destination buffer: its ring is what the odd steps of the pass read.
    const bool touches_ring = (gy0 < ring) || (gy0 + LH > H - ring) || (gx0 < ring) || (gx0 + kLifeLW > W - ring);
    const int nstage = (touches_ring && steps >= 2) ? 2 : 1;
    for (int k = 0; k < nstage; ++k) {
      if (k == 1) {
        __syncthreads();  // the byte tile is reused
        if (kTma && tid == 0) issue_load(tile, &map_dst);
      }
      if (kTma) {
        if (!mbar_wait_bounded(bar, phase, err)) return;
        phase ^= 1u;
      } else {
        const uint8_t* from = (k == 0) ? src : dst;
        for (int i = tid; i < LH * 16; i += kLifeThreads) {
          const int row = i >> 4, c = i & 15;
          const int gy = gy0 + row, gx = gx0 + c * 16;
          uint4 v = make_uint4(0, 0, 0, 0);
          if (gy >= 0 && gy < H) {
            const uint8_t* p = from + static_cast<int64_t>(gy) * pitch + gx;
            if (gx >= 0 && gx + 16 <= W && (reinterpret_cast<uintptr_t>(p) & 15) == 0) {
              v = *reinterpret_cast<const uint4*>(p);
            } else {
              uint8_t tmp[16];
#pragma unroll
              for (int b = 0; b < 16; ++b) tmp[b] = (gx + b >= 0 && gx + b < W) ? p[b] : 0;
              v.x = tmp[0] | (tmp[1] << 8) | (tmp[2] << 16) | (uint32_t(tmp[3]) << 24);
              v.y = tmp[4] | (tmp[5] << 8) | (tmp[6] << 16) | (uint32_t(tmp[7]) << 24);
              v.z = tmp[8] | (tmp[9] << 8) | (tmp[10] << 16) | (uint32_t(tmp[11]) << 24);
              v.w = tmp[12] | (tmp[13] << 8) | (tmp[14] << 16) | (uint32_t(tmp[15]) << 24);
            }
          }
          *reinterpret_cast<uint4*>(bytes + row * kLifeLW + c * 16) = v;
        }
        __syncthreads();
      }
      // bytes -> bit words (LH is even, so each warp's trip count is uniform)
      uint32_t* plane = (k == 0) ? bitsA : bitsB;
      for (int i = tid; i < LH * 16; i += kLifeThreads) {
        const int row = i >> 4, c = i & 15;
        uint4 v = *reinterpret_cast<const uint4*>(bytes + row * kLifeLW + c * 16);
        if ((v.x | v.y | v.z | v.w) & 0xFEFEFEFEu) {
          if (k == 0) {
            bad_value = true;  // every source cell is state
          } else {
            // only the destination's ring is read; its interior may hold anything
            const int gy = gy0 + row, gx = gx0 + c * 16;
            const bool row_ring = (gy < ring) || (gy >= H - ring);
            const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
            for (int b = 0; b < 16; ++b) {
              const uint32_t byte = (w4[b >> 2] >> ((b & 3) * 8)) & 0xFFu;
              if (byte > 1u && (row_ring || gx + b < ring || gx + b >= W - ring)) bad_value = true;
            }
          }
          v.x &= 0x01010101u;
          v.y &= 0x01010101u;
          v.z &= 0x01010101u;
          v.w &= 0x01010101u;
        }
        const uint32_t half = pack16(v);
        const uint32_t other = __shfl_xor_sync(0xFFFFFFFFu, half, 1);
        if ((c & 1) == 0) plane[bit_index(row, c >> 1)] = half | (other << 16);
      }
      // rows [LH, 256) of the plane restart from zero for every tile
      for (int i = LH * kWords + tid; i < kBitRows * kWords; i += kLifeThreads)
        plane[bit_index(i >> 3, i & 7)] = 0u;
    }
    __syncthreads();
    if (kTma && tid == 0 && tile + static_cast<int>(gridDim.x) < ntiles) issue_load(tile + gridDim.x, &map);

    // ---- the steps, on bit planes. Rows at or beyond LH are computed too
    // (from zeros); like the tile edges they only feed the halo.
    const uint32_t colmask = bit_range(ring - (gx0 + 32 * j), (W - ring) - (gx0 + 32 * j));
    for (int s = 0; s < steps; ++s) {
      const uint32_t* in = (s & 1) ? bitsB : bitsA;
      uint32_t* out = (s & 1) ? bitsA : bitsB;
      if (touches_ring) {
        life_strip<true>(in, out, y0, j, colmask, gy0, ring, H);
      } else {
        life_strip<false>(in, out, y0, j, colmask, gy0, ring, H);
      }
      __syncthreads();
    }

    // ---- core bits -> bytes -> global (interior cells only)
    const uint32_t* fin = (steps & 1) ? bitsB : bitsA;
    for (int i = tid; i < TH * 16; i += kLifeThreads) {
      const int c = i & 15;
      if (c == 0 || c == 15) continue;
      const int row = T + (i >> 4);
      const int gy = gy0 + row;
      if (gy < ring || gy >= H - ring) continue;
      const int gx = gx0 + c * 16;
      if (gx + 16 <= ring || gx >= W - ring) continue;
      const uint32_t word = fin[bit_index(row, c >> 1)];
      const uint4 v = unpack16((c & 1) ? (word >> 16) : (word & 0xFFFFu));
      uint8_t* d = dst + static_cast<int64_t>(gy) * pitch + gx;
      if (gx >= ring && gx + 16 <= W - ring && (reinterpret_cast<uintptr_t>(d) & 15) == 0) {
        *reinterpret_cast<uint4*>(d) = v;
      } else {
        const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int b = 0; b < 16; ++b) {
          const int x = gx + b;
          if (x >= ring && x < W - ring) d[b] = static_cast<uint8_t>(w4[b >> 2] >> ((b & 3) * 8));
        }
      }
    }
    __syncthreads();
  }
  if (bad_value) atomicOr(err, kDevErrValue);
}

}  // namespace

size_t life_smem_bytes(int LH) {
  return 128 + static_cast<size_t>(LH) * kLifeLW + 2 * static_cast<size_t>(kBitPlaneWords) * 4 + 16;
}

int life_max_ctas_per_sm(int LH) {
  int n = 0;
  const size_t smem = life_smem_bytes(LH);
  cudaFuncSetAttribute(life_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  cudaFuncSetAttribute(life_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, life_kernel<true>, kLifeThreads, smem) != cudaSuccess) return 1;
  return n > 0 ? n : 1;
}

cudaError_t life_pass(const CUtensorMap* map_src, const CUtensorMap* map_dst, bool use_tma, const uint8_t* src, uint8_t* dst, int W, int H,
                      int64_t pitch, int ring, int steps, const LifeGeom& g, unsigned* err, cudaStream_t s) {
  const size_t smem = life_smem_bytes(g.LH);
  CUtensorMap dummy;
  memset(&dummy, 0, sizeof(dummy));
  const CUtensorMap& m = use_tma ? *map_src : dummy;
  const CUtensorMap& md = use_tma ? *map_dst : dummy;
  if (use_tma) {
    life_kernel<true><<<g.ctas, kLifeThreads, smem, s>>>(m, md, src, dst, W, H, pitch, ring, steps, g.T, g.TH, g.LH,
                                                         g.tiles_x, g.tiles_y, err);
  } else {
    life_kernel<false><<<g.ctas, kLifeThreads, smem, s>>>(m, md, src, dst, W, H, pitch, ring, steps, g.T, g.TH, g.LH,
                                                          g.tiles_x, g.tiles_y, err);
  }
  return cudaGetLastError();
}

}  // namespace pskel
