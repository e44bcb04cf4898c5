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
// P: the bit plane's row pitch in words (a zero row above row 0 and a zero
// word left of word 0, so word (row, j) sits at (row + 1) * P + j + 1).
template <bool kMasked, int P = kBitPitch>
__device__ __forceinline__ void life_strip(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, int y0, int j,
                                           uint32_t colmask, int gy0, int ring, int H) {
  uint32_t c[kRowsPerStrip + 2], t0[kRowsPerStrip + 2], t1[kRowsPerStrip + 2];
  uint32_t p0[kRowsPerStrip + 2], p1[kRowsPerStrip + 2];
  const uint32_t* base = in + (y0 * P + j + 1);  // row y0 - 1
#pragma unroll
  for (int k = 0; k < kRowsPerStrip + 2; ++k) {
    const uint32_t* r = base + k * P;
    const uint32_t l = r[-1], cc = r[0], e = r[1];
    const uint32_t we = __funnelshift_l(l, cc, 1);  // bit b = cell b-1
    const uint32_t ea = __funnelshift_r(cc, e, 1);  // bit b = cell b+1
    c[k] = cc;
    t0[k] = lop3<kXor3>(we, cc, ea);
    t1[k] = lop3<kMaj>(we, cc, ea);
    p0[k] = we ^ ea;
    p1[k] = we & ea;
  }
  uint32_t* o = out + ((y0 + 1) * P + j + 1);
#pragma unroll
  for (int k = 1; k <= kRowsPerStrip; ++k) {
    const uint32_t s0 = lop3<kXor3>(t0[k - 1], p0[k], t0[k + 1]);
    const uint32_t k0 = lop3<kMaj>(t0[k - 1], p0[k], t0[k + 1]);
    const uint32_t x1 = lop3<kXor3>(t1[k - 1], p1[k], t1[k + 1]);
    const uint32_t y1 = lop3<kMaj>(t1[k - 1], p1[k], t1[k + 1]);
    const uint32_t two_or_three = lop3<kNotAAndBxC>(y1, x1, k0);
    const uint32_t alive = lop3<kAAndBorC>(two_or_three, s0, c[k]);
    uint32_t* dst = o + (k - 1) * P;
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

// ---------------------------------------------------------------------------
// Bit-plane passes. A run packs the source and destination grids once into
// two global bit planes (one bit per cell, rows of PW words), runs every pass
// between the planes -- 16 MB for an 8192^2 grid, resident in L2 -- and
// unpacks the final plane into the result buffer's interior once. A pass
// tile is 16 words (512 cells) x LH rows with one word (32 cells) and T rows
// of halo on each side, staged by cp.async into a shared bit plane.
constexpr int kBW = 16;                          // words per loaded tile row
constexpr int kBCore = kBW - 2;                  // core words
constexpr int kBP = kBW + 2;                     // shared plane pitch (zero word each side)
constexpr int kBRows = 256;
constexpr int kBPlane = (kBRows + 2) * kBP;      // words per shared plane
constexpr int kBThreads = kBW * (kBRows / kRowsPerStrip);  // 512: a word column x an 8-row strip each

// packs rows of `src` (bytes 0/1) into a bit plane; check: 0 = every cell must
// be 0/1, 1 = only the ring (the interior of a destination is overwritten
// before it is read)
__global__ void __launch_bounds__(256) life_pack_kernel(const uint8_t* __restrict__ src, int64_t pitch, int W, int H,
                                                        uint32_t* __restrict__ plane, int PW, int ring, int check,
                                                        unsigned* err) {
  bool bad = false;
  const int64_t n = static_cast<int64_t>(H) * PW;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int row = static_cast<int>(i / PW), wd = static_cast<int>(i - static_cast<int64_t>(row) * PW);
    const int c0 = wd * 32;
    const uint8_t* r = src + static_cast<int64_t>(row) * pitch;
    const bool row_ring = row < ring || row >= H - ring;
    uint32_t bits = 0;
    if (c0 + 32 <= W && (reinterpret_cast<uintptr_t>(r + c0) & 15) == 0) {
      const uint4 a = *reinterpret_cast<const uint4*>(r + c0);
      const uint4 b = *reinterpret_cast<const uint4*>(r + c0 + 16);
      const uint32_t any = a.x | a.y | a.z | a.w | b.x | b.y | b.z | b.w;
      if (any & 0xFEFEFEFEu) {
        for (int k = 0; k < 32; ++k) {
          const uint8_t v = r[c0 + k];
          const bool in_ring = row_ring || c0 + k < ring || c0 + k >= W - ring;
          if (v > 1 && (check == 0 || in_ring)) bad = true;
        }
      }
      const uint4 am = make_uint4(a.x & 0x01010101u, a.y & 0x01010101u, a.z & 0x01010101u, a.w & 0x01010101u);
      const uint4 bm = make_uint4(b.x & 0x01010101u, b.y & 0x01010101u, b.z & 0x01010101u, b.w & 0x01010101u);
      bits = pack16(am) | (pack16(bm) << 16);
    } else {
      for (int k = 0; k < 32 && c0 + k < W; ++k) {
        const uint8_t v = r[c0 + k];
        const bool in_ring = row_ring || c0 + k < ring || c0 + k >= W - ring;
        if (v > 1 && (check == 0 || in_ring)) bad = true;
        bits |= static_cast<uint32_t>(v & 1u) << k;
      }
    }
    plane[i] = bits;
  }
  if (bad) atomicOr(err, kDevErrValue);
}

// writes the interior cells (ring <= h < H-ring, ring <= w < W-ring) of a bit
// plane into `dst` as bytes; ring cells of `dst` are left as they are
__global__ void __launch_bounds__(256) life_unpack_kernel(const uint32_t* __restrict__ plane, int PW, uint8_t* dst,
                                                          int64_t pitch, int W, int H, int ring) {
  const int rows = H - 2 * ring;
  if (rows <= 0) return;
  const int64_t n = static_cast<int64_t>(rows) * PW;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int row = ring + static_cast<int>(i / PW), wd = static_cast<int>(i % PW);
    const int c0 = wd * 32;
    if (c0 >= W - ring || c0 + 32 <= ring) continue;
    const uint32_t bits = plane[static_cast<int64_t>(row) * PW + wd];
    uint8_t* r = dst + static_cast<int64_t>(row) * pitch;
    if (c0 >= ring && c0 + 32 <= W - ring && (reinterpret_cast<uintptr_t>(r + c0) & 15) == 0) {
      *reinterpret_cast<uint4*>(r + c0) = unpack16(bits & 0xFFFFu);
      *reinterpret_cast<uint4*>(r + c0 + 16) = unpack16(bits >> 16);
    } else {
      for (int k = 0; k < 32; ++k) {
        const int c = c0 + k;
        if (c >= ring && c < W - ring) r[c] = static_cast<uint8_t>((bits >> k) & 1u);
      }
    }
  }
}

__device__ __forceinline__ void cp_async4(uint32_t* dst, const uint32_t* src, bool valid) {
  const int n = valid ? 4 : 0;  // zero-fill when the source word lies outside the plane
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// One pass of `steps` (<= T) generations from plane `src` to plane `dst`.
__global__ void __launch_bounds__(kBThreads, 2)
    life_bits_kernel(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, int PW, int W, int H, int ring,
                     int steps, int T, int TH, int LH, int tiles_x, int tiles_y) {
  extern __shared__ __align__(128) uint32_t bsm[];
  uint32_t* planeA = bsm;
  uint32_t* planeB = bsm + kBPlane;
  const int tid = threadIdx.x;
  // the zero borders (row -1, row LH.., word -1, word 16) are never written
  for (int i = tid; i < 2 * kBPlane; i += kBThreads) bsm[i] = 0u;
  __syncthreads();
  const int j = tid & (kBW - 1);
  const int y0 = (tid / kBW) * kRowsPerStrip;
  const int ntiles = tiles_x * tiles_y;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
    const int gy0 = ty * TH - T;
    const int gw0 = tx * kBCore - 1;
    const int gx0 = gw0 * 32;
    const bool ring_tile = (gy0 < ring) || (gy0 + LH > H - ring) || (gx0 < ring) || (gx0 + kBW * 32 > W - ring);
    // ring tiles also stage the destination's tile: its ring bits are read by
    // the odd steps and written back unchanged with the core words
    const int nstage = ring_tile ? 2 : 1;
    // stage the source tile (and, for ring tiles, the destination's) by cp.async
    for (int k = 0; k < nstage; ++k) {
      const uint32_t* g = (k == 0) ? src : dst;
      uint32_t* pl = (k == 0) ? planeA : planeB;
      for (int i = tid; i < LH * kBW; i += kBThreads) {
        const int row = i / kBW, wd = i - row * kBW;
        const int gy = gy0 + row, gw = gw0 + wd;
        const bool ok = gy >= 0 && gy < H && gw >= 0 && gw < PW;
        cp_async4(pl + (row + 1) * kBP + wd + 1, ok ? g + static_cast<int64_t>(gy) * PW + gw : g, ok);
      }
    }
    cp_async_wait_all();
    __syncthreads();
    // rows at or beyond LH stay zero from the last tile only if LH is the
    // same; clear them (they feed only the halo, but keep them defined)
    for (int i = LH * kBW + tid; i < kBRows * kBW; i += kBThreads) {
      const int row = i / kBW, wd = i - row * kBW;
      planeA[(row + 1) * kBP + wd + 1] = 0u;
      planeB[(row + 1) * kBP + wd + 1] = 0u;
    }
    __syncthreads();
    const uint32_t colmask = bit_range(ring - (gx0 + 32 * j), (W - ring) - (gx0 + 32 * j));
    // strips wholly below the loaded rows stay zero and are skipped: a tile
    // costs its loaded height, not the plane's 256 rows
    const bool active = y0 < LH;
    for (int s = 0; s < steps; ++s) {
      const uint32_t* in = (s & 1) ? planeB : planeA;
      uint32_t* out = (s & 1) ? planeA : planeB;
      if (active) {
        if (ring_tile) {
          life_strip<true, kBP>(in, out, y0, j, colmask, gy0, ring, H);
        } else {
          life_strip<false, kBP>(in, out, y0, j, colmask, gy0, ring, H);
        }
      }
      __syncthreads();
    }
    // core words -> destination plane
    const uint32_t* fin = (steps & 1) ? planeB : planeA;
    for (int i = tid; i < TH * kBCore; i += kBThreads) {
      const int r = i / kBCore, wd = 1 + (i - r * kBCore);
      const int row = T + r;
      const int gy = gy0 + row, gw = gw0 + wd;
      if (gy < 0 || gy >= H || gw >= PW) continue;
      dst[static_cast<int64_t>(gy) * PW + gw] = fin[(row + 1) * kBP + wd + 1];
    }
    __syncthreads();
  }
}

}  // namespace

int life_bits_words(int W) { return ((W + 31) / 32 + 3) & ~3; }

int life_bits_tiles(int W, int H, int TH) {
  return ((life_bits_words(W) + kBCore - 1) / kBCore) * ((H + TH - 1) / TH);
}

size_t life_bits_smem_bytes() { return 2 * static_cast<size_t>(kBPlane) * sizeof(uint32_t); }

int life_bits_ctas_per_sm() {
  int n = 0;
  const size_t smem = life_bits_smem_bytes();
  cudaFuncSetAttribute(life_bits_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, life_bits_kernel, kBThreads, smem) != cudaSuccess) return 1;
  return n > 0 ? n : 1;
}

cudaError_t life_bits_pack(const uint8_t* src, int64_t pitch, int W, int H, uint32_t* plane, int ring, bool ring_only,
                           unsigned* err, int sms, cudaStream_t s) {
  const int PW = life_bits_words(W);
  life_pack_kernel<<<4 * sms, 256, 0, s>>>(src, pitch, W, H, plane, PW, ring, ring_only ? 1 : 0, err);
  return cudaGetLastError();
}

cudaError_t life_bits_unpack(const uint32_t* plane, uint8_t* dst, int64_t pitch, int W, int H, int ring, int sms,
                             cudaStream_t s) {
  life_unpack_kernel<<<4 * sms, 256, 0, s>>>(plane, life_bits_words(W), dst, pitch, W, H, ring);
  return cudaGetLastError();
}

cudaError_t life_bits_pass(const uint32_t* src, uint32_t* dst, int W, int H, int ring, int steps, int T, int TH,
                           int ctas, cudaStream_t s) {
  const int LH = TH + 2 * T;
  const int tiles_x = (life_bits_words(W) + kBCore - 1) / kBCore;
  const int tiles_y = (H + TH - 1) / TH;
  life_bits_kernel<<<ctas, kBThreads, life_bits_smem_bytes(), s>>>(src, dst, life_bits_words(W), W, H, ring, steps,
                                                                     T, TH, LH, tiles_x, tiles_y);
  return cudaGetLastError();
}

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
