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

// Three-input boolean functions as single LOP3 instructions. The truth-table
// immediate is f(0xF0, 0xCC, 0xAA) for inputs (a, b, c).
template <uint32_t kLut>
__device__ __forceinline__ uint32_t lop3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm("lop3.b32 %0, %1, %2, %3, %4;" : "=r"(d) : "r"(a), "r"(b), "r"(c), "n"(kLut));
  return d;
}
constexpr uint32_t kXor3 = 0x96;      // a ^ b ^ c
constexpr uint32_t kMaj = 0xE8;       // at least two of a, b, c
constexpr uint32_t kNotAAndBxC = 0x06;  // ~a & (b ^ c)
constexpr uint32_t kAAndBorC = 0xE0;  // a & (b | c)
constexpr uint32_t kSelect = 0xCA;    // a ? b : c, bitwise

// One step for a strip of 8 rows of one word column. The neighbour count of
// each cell is (w + c + e of the row above) + (w + e of its row) + (w + c + e
// of the row below); each term is a 2-bit bit-sliced number, and the three are
// added with full adders: s0 = low bit, k0 = its carry, x1/y1 = sum/carry of
// the twos. With k0 folded in, count in {2, 3} <=> ~y1 & (x1 ^ k0), and the
// cell lives iff that holds and (s0 | alive): count 3, or count 2 and alive.
// A count of 8 leaves y1 set, so it is dead as it must be.
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
    t0[k] = lop3<kXor3>(we, cc, ea);
    t1[k] = lop3<kMaj>(we, cc, ea);
    p0[k] = we ^ ea;
    p1[k] = we & ea;
  }
  uint32_t* o = out + bit_index(y0, j);
#pragma unroll
  for (int k = 1; k <= kRowsPerStrip; ++k) {
    const uint32_t s0 = lop3<kXor3>(t0[k - 1], p0[k], t0[k + 1]);
    const uint32_t k0 = lop3<kMaj>(t0[k - 1], p0[k], t0[k + 1]);
    const uint32_t x1 = lop3<kXor3>(t1[k - 1], p1[k], t1[k + 1]);
    const uint32_t y1 = lop3<kMaj>(t1[k - 1], p1[k], t1[k + 1]);
    const uint32_t two_or_three = lop3<kNotAAndBxC>(y1, x1, k0);
    const uint32_t alive = lop3<kAAndBorC>(two_or_three, s0, c[k]);
    uint32_t* dst = o + (k - 1) * kBitPitch;
    if (kMasked) {
      // cells outside r <= h < H-r, r <= w < W-r keep the value this plane holds
      const int gy = gy0 + y0 + k - 1;
      const uint32_t m = (gy >= ring && gy < H - ring) ? colmask : 0u;
      *dst = lop3<kSelect>(m, alive, *dst);
    } else {
      *dst = alive;
    }
  }
}

constexpr int kChunkRows = 64;  // TMA box height: a tile arrives in up to 4 chunks
constexpr int kSlots = 2;        // chunk staging slots (double buffer)

template <bool kTma>
__global__ void __launch_bounds__(kLifeThreads, 3)
    life_kernel(const __grid_constant__ CUtensorMap map, const __grid_constant__ CUtensorMap map_dst,
                const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, int W, int H, int64_t pitch, int ring,
                int steps, int T, int TH, int LH, int tiles_x, int tiles_y, unsigned* err) {
  // dynamic shared memory, 128-byte aligned for TMA; derived pointers stay
  // in the shared window (no integer round trip), so accesses compile to
  // shared-memory instructions
  extern __shared__ __align__(128) uint8_t smem_raw[];
  uint8_t* slots = smem_raw;
  if ((smem_u32(smem_raw) & 127u) != 0) {
    if (threadIdx.x == 0) atomicOr(err, kDevErrAlign);
    return;
  }
  uint32_t* bitsA = reinterpret_cast<uint32_t*>(slots + kSlots * kChunkRows * kLifeLW);
  uint32_t* bitsB = bitsA + kBitPlaneWords;
  uint64_t* bars = reinterpret_cast<uint64_t*>(bitsB + kBitPlaneWords);

  const int tid = threadIdx.x;
  // zero both planes once: the padding rows/words are never written again and
  // rows at or beyond LH stay zero until the first tile's steps run over them
  for (int i = tid; i < 2 * kBitPlaneWords; i += kLifeThreads) bitsA[i] = 0u;
  if (kTma && tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_barrier_init();
    prefetch_tensormap(&map);
    prefetch_tensormap(&map_dst);
  }
  __syncthreads();

  const int ntiles = tiles_x * tiles_y;
  const int nchunks = (LH + kChunkRows - 1) / kChunkRows;
  const int j = tid & (kWords - 1);
  const int y0 = (tid >> 3) * kRowsPerStrip;  // 32 strips of 8 rows
  bool bad_value = false;

  // Ring cells (outside r <= h < H-r, r <= w < W-r) are never written, so
  // each global buffer keeps its own ring and step k reads the ring of the
  // buffer it reads from. Tiles that reach the ring therefore also stage the
  // destination buffer: its ring is what the odd steps of the pass read.
  auto touches_ring = [&](int t) {
    const int gy0 = (t / tiles_x) * TH - T;
    const int gx0 = (t % tiles_x) * kLifeTW - kLifeHX;
    return (gy0 < ring) || (gy0 + LH > H - ring) || (gx0 < ring) || (gx0 + kLifeLW > W - ring);
  };
  auto chunks_of = [&](int t) { return (touches_ring(t) && steps >= 2) ? 2 * nchunks : nchunks; };

  // Producer (thread 0): chunk loads run two ahead of the packing, across tile
  // boundaries, so the next tile streams in while this one steps.
  int p_tile = blockIdx.x, p_idx = 0, p_len = 0;
  uint32_t p_slot = 0;
  auto produce = [&]() {
    if (p_tile >= ntiles) return;
    if (p_idx == 0) p_len = chunks_of(p_tile);
    const int gy0 = (p_tile / tiles_x) * TH - T;
    const int gx0 = (p_tile % tiles_x) * kLifeTW - kLifeHX;
    const bool from_dst = p_idx >= nchunks;
    const int c = from_dst ? p_idx - nchunks : p_idx;
    fence_proxy_async();
    mbar_arrive_expect_tx(&bars[p_slot], static_cast<uint32_t>(kChunkRows * kLifeLW));
    tma_load_2d(slots + p_slot * kChunkRows * kLifeLW, from_dst ? &map_dst : &map, gx0, gy0 + c * kChunkRows,
                &bars[p_slot]);
    p_slot ^= 1u;
    if (++p_idx == p_len) {
      p_idx = 0;
      p_tile += gridDim.x;
    }
  };
  if (kTma && tid == 0) {
    produce();
    produce();
  }

  uint32_t c_slot = 0;
  uint32_t phase[kSlots] = {0u, 0u};
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int ty = tile / tiles_x;
    const int tx = tile - ty * tiles_x;
    const int gy0 = ty * TH - T;          // global row of local row 0
    const int gx0 = tx * kLifeTW - kLifeHX;  // global column of local column 0
    const bool ring_tile = touches_ring(tile);
    const int nstage = (ring_tile && steps >= 2) ? 2 : 1;

    for (int k = 0; k < nstage; ++k) {
      uint32_t* plane = (k == 0) ? bitsA : bitsB;
      for (int c = 0; c < nchunks; ++c) {
        uint8_t* slot = slots + c_slot * kChunkRows * kLifeLW;
        if (kTma) {
          // one thread waits; the block barrier publishes the chunk
          int ok = 1;
          if (tid == 0) ok = mbar_wait_bounded(&bars[c_slot], phase[c_slot], err) ? 1 : 0;
          phase[c_slot] ^= 1u;
          if (!__syncthreads_and(ok)) return;
        } else {
          const uint8_t* from = (k == 0) ? src : dst;
          for (int i = tid; i < kChunkRows * 16; i += kLifeThreads) {
            const int row = i >> 4, cc = i & 15;
            const int gy = gy0 + c * kChunkRows + row, gx = gx0 + cc * 16;
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
            *reinterpret_cast<uint4*>(slot + row * kLifeLW + cc * 16) = v;
          }
          __syncthreads();
        }
        // bytes -> bit words (chunk row counts are even, so each warp's trip
        // count is uniform and the pair shuffle sees both halves)
        const int rows = min(kChunkRows, LH - c * kChunkRows);
        for (int i = tid; i < rows * 16; i += kLifeThreads) {
          const int row = i >> 4, cc = i & 15;
          uint4 v = *reinterpret_cast<const uint4*>(slot + row * kLifeLW + cc * 16);
          if ((v.x | v.y | v.z | v.w) & 0xFEFEFEFEu) {
            if (k == 0) {
              bad_value = true;  // every source cell is state
            } else {
              // only the destination's ring is read; its interior may hold anything
              const int gy = gy0 + c * kChunkRows + row, gx = gx0 + cc * 16;
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
          if ((cc & 1) == 0) plane[bit_index(c * kChunkRows + row, cc >> 1)] = half | (other << 16);
        }
        __syncthreads();  // the slot is free again
        if (kTma && tid == 0) produce();
        c_slot ^= 1u;
      }
      // rows [LH, 256) of the plane restart from zero for every tile
      for (int i = LH * kWords + tid; i < kBitRows * kWords; i += kLifeThreads)
        plane[bit_index(i >> 3, i & 7)] = 0u;
    }
    __syncthreads();

    // ---- the steps, on bit planes. Rows at or beyond LH are computed too
    // (from zeros); like the tile edges they only feed the halo.
    const uint32_t colmask = bit_range(ring - (gx0 + 32 * j), (W - ring) - (gx0 + 32 * j));
    for (int s = 0; s < steps; ++s) {
      const uint32_t* in = (s & 1) ? bitsB : bitsA;
      uint32_t* out = (s & 1) ? bitsA : bitsB;
      if (ring_tile) {
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
  (void)LH;
  return 128 + static_cast<size_t>(kSlots) * kChunkRows * kLifeLW + 2 * static_cast<size_t>(kBitPlaneWords) * 4 +
         kSlots * 8;
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
