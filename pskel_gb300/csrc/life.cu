// Game of Life, temporally blocked and bit-sliced, on bit planes.
//
// A run packs the source and destination grids (one 0/1 byte per cell, the
// reference's layout) once into two global bit planes -- one bit per cell,
// 16 MB for an 8192^2 grid, so the planes stay in L2 -- runs every pass
// between the planes and unpacks the final plane's interior into the result
// buffer once. A pass advances the grid by up to 31 steps: each persistent
// CTA walks tiles of 14 x 32 core columns and TH core rows, stages the
// 16-word x (TH + 2T)-row halo tile into a shared bit plane with cp.async,
// runs the steps there (neighbour counts with bit-sliced full adders: 32
// cells per word and about a dozen LOP3/funnel-shift operations per word and
// step) and writes the core words back. Ring cells (outside r <= h < H-r,
// r <= w < W-r) are never updated, the semantics of Stencil2D::runOpenMP
// (PSkelStencil.hpp:2197-2257): tiles that reach the ring also stage the
// destination plane's tile, whose ring bits the odd steps read and the
// write-back keeps.
//
// Redundant halo work: the tile carries T rows and 32 columns of halo on each
// side; garbage entering from the tile edge advances one cell per step, so
// the core is exact after T <= 31 steps.
#include "common.cuh"
#include "kernels.h"

namespace pskel {
namespace {

constexpr int kRowsPerStrip = 8;  // rows of one word column a thread steps

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
template <bool kMasked, int P>
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
                                                        unsigned* err, int row0, int row1) {
  bool bad = false;
  const int64_t n = static_cast<int64_t>(row1 - row0) * PW;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int rr = static_cast<int>(i / PW), wd = static_cast<int>(i - static_cast<int64_t>(rr) * PW);
    const int row = row0 + rr;
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
    plane[static_cast<int64_t>(row) * PW + wd] = bits;
  }
  if (bad) atomicOr(err, kDevErrValue);
}

// writes the interior cells (ring <= h < H-ring, ring <= w < W-ring) of a bit
// plane into `dst` as bytes; ring cells of `dst` are left as they are
__global__ void __launch_bounds__(256) life_unpack_kernel(const uint32_t* __restrict__ plane, int PW, uint8_t* dst,
                                                          int64_t pitch, int W, int H, int ring, int row0,
                                                          int row1) {
  // interior rows of [row0, row1)
  const int lo = max(ring, row0), hi = min(H - ring, row1);
  const int rows = hi - lo;
  if (rows <= 0) return;
  const int64_t n = static_cast<int64_t>(rows) * PW;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int row = lo + static_cast<int>(i / PW), wd = static_cast<int>(i % PW);
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

constexpr unsigned kLifeSpinLimit = 1u << 24;  // polls of a neighbour's completion count (each with a sleep)

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_cg(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.global.cg.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Every pass of a run in one launch. Work items (pass, tile) are handed out
// in order by an atomic counter; before tile t of pass p is staged, thread 0
// waits (bounded) until every tile of pass p-1 whose core the tile reads --
// rows within ceil(T/TH) tiles, one tile column either side -- has completed
// (done[] counts the passes each tile has completed). Those tiles also were
// the last readers of the region this tile writes. All CTAs are resident and
// items are taken in order, so every awaited item is held by a running CTA.
// Planes written by other SMs are read through L2 (ld.global.cg).
// Pass i has 1 + 2 * (q + (i < r)) steps (the odd-length plan of
// plan_passes).
__global__ void __launch_bounds__(kBThreads, 2)
    life_bits_persistent_kernel(uint32_t* __restrict__ planeX, uint32_t* __restrict__ planeY, int PW, int W, int H,
                                int ring, int npasses, int q, int r, int T, int TH, int LH, int tiles_x, int tiles_y,
                                unsigned long long* next_item, unsigned* done, unsigned* err,
                                const __grid_constant__ LifeWindow win) {
  extern __shared__ __align__(128) uint32_t bsm[];
  uint32_t* planeA = bsm;
  uint32_t* planeB = bsm + kBPlane;
  __shared__ long long s_item;
  __shared__ int s_pass, s_tile;
  (void)npasses;
  const int tid = threadIdx.x;
  for (int i = tid; i < 2 * kBPlane; i += kBThreads) bsm[i] = 0u;
  __syncthreads();
  const int j = tid & (kBW - 1);
  const int y0 = (tid / kBW) * kRowsPerStrip;
  const int ntiles = tiles_x * tiles_y;
  // this launch's items: passes win.pass0 .. + win.np, each over all tiles or
  // (windowed) over tile rows [win.lo[j], ...) holding win.start[j+1] -
  // win.start[j] items; completion counts persist between the launches of a run
  const long long nitems = win.windowed ? win.start[win.np] : static_cast<long long>(win.np) * ntiles;
  const int dy = (T + TH - 1) / TH;
  for (;;) {
    if (tid == 0) {
      const long long it = static_cast<long long>(atomicAdd(next_item, 1ull));
      s_item = it;
      if (it < nitems) {
        if (win.windowed) {
          int j = 0;
          while (j + 1 < win.np && win.start[j + 1] <= it) ++j;
          const long long k = it - win.start[j];
          s_pass = win.pass0 + j;
          s_tile = static_cast<int>((win.lo[j] + k / tiles_x) * tiles_x + k % tiles_x);
        } else {
          s_pass = win.pass0 + static_cast<int>(it / ntiles);
          s_tile = static_cast<int>(it % ntiles);
        }
      }
    }
    __syncthreads();
    const long long item = s_item;
    if (item >= nitems) break;
    const int pass = s_pass;
    const int tile = s_tile;
    const int steps = 1 + 2 * (q + (pass < r ? 1 : 0));
    const uint32_t* src = (pass & 1) ? planeY : planeX;
    uint32_t* dst = (pass & 1) ? planeX : planeY;
    const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
    int ok = 1;
    if (tid == 0 && pass > 0) {
      for (int yy = max(0, ty - dy); yy <= min(tiles_y - 1, ty + dy) && ok; ++yy) {
        for (int xx = max(0, tx - 1); xx <= min(tiles_x - 1, tx + 1) && ok; ++xx) {
          const unsigned* d = &done[yy * tiles_x + xx];
          unsigned polls = 0;
          while (ld_acquire_u32(d) < static_cast<unsigned>(pass)) {
            if (++polls >= kLifeSpinLimit) {
              atomicOr(err, kDevErrBarrier);
              ok = 0;
              break;
            }
            __nanosleep(32);
          }
        }
      }
    }
    if (!__syncthreads_and(ok)) break;
    __threadfence();
    const int gy0 = ty * TH - T;
    const int gw0 = tx * kBCore - 1;
    const int gx0 = gw0 * 32;
    const bool ring_tile = (gy0 < ring) || (gy0 + LH > H - ring) || (gx0 < ring) || (gx0 + kBW * 32 > W - ring);
    const int nstage = ring_tile ? 2 : 1;
    for (int k = 0; k < nstage; ++k) {
      const uint32_t* g = (k == 0) ? src : dst;
      uint32_t* pl = (k == 0) ? planeA : planeB;
#pragma unroll 8
      for (int i = tid; i < LH * kBW; i += kBThreads) {
        const int row = i / kBW, wd = i - row * kBW;
        const int gy = gy0 + row, gw = gw0 + wd;
        const bool in = gy >= 0 && gy < H && gw >= 0 && gw < PW;
        pl[(row + 1) * kBP + wd + 1] = in ? ld_cg(g + static_cast<int64_t>(gy) * PW + gw) : 0u;
      }
    }
    for (int i = LH * kBW + tid; i < kBRows * kBW; i += kBThreads) {
      const int row = i / kBW, wd = i - row * kBW;
      planeA[(row + 1) * kBP + wd + 1] = 0u;
      planeB[(row + 1) * kBP + wd + 1] = 0u;
    }
    __syncthreads();
    const uint32_t colmask = bit_range(ring - (gx0 + 32 * j), (W - ring) - (gx0 + 32 * j));
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
    const uint32_t* fin = (steps & 1) ? planeB : planeA;
    for (int i = tid; i < TH * kBCore; i += kBThreads) {
      const int rr = i / kBCore, wd = 1 + (i - rr * kBCore);
      const int row = T + rr;
      const int gy = gy0 + row, gw = gw0 + wd;
      if (gy < 0 || gy >= H || gw >= PW) continue;
      dst[static_cast<int64_t>(gy) * PW + gw] = fin[(row + 1) * kBP + wd + 1];
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) atomicAdd(&done[tile], 1u);
  }
}

}  // namespace

int life_bits_words(int W) { return ((W + 31) / 32 + 3) & ~3; }

int life_bits_tiles(int W, int H, int TH) {
  return ((life_bits_words(W) + kBCore - 1) / kBCore) * ((H + TH - 1) / TH);
}

size_t life_bits_smem_bytes() { return 2 * static_cast<size_t>(kBPlane) * sizeof(uint32_t); }


cudaError_t life_bits_pack(const uint8_t* src, int64_t pitch, int W, int H, uint32_t* plane, int ring, bool ring_only,
                           unsigned* err, int sms, cudaStream_t s) {
  const int PW = life_bits_words(W);
  life_pack_kernel<<<4 * sms, 256, 0, s>>>(src, pitch, W, H, plane, PW, ring, ring_only ? 1 : 0, err, 0, H);
  return cudaGetLastError();
}

cudaError_t life_bits_pack_rows(const uint8_t* src, int64_t pitch, int W, int H, uint32_t* plane, int ring,
                                int row0, int row1, unsigned* err, int sms, cudaStream_t s) {
  if (row1 <= row0) return cudaSuccess;
  const int PW = life_bits_words(W);
  life_pack_kernel<<<4 * sms, 256, 0, s>>>(src, pitch, W, H, plane, PW, ring, 0, err, row0, row1);
  return cudaGetLastError();
}

cudaError_t life_bits_unpack(const uint32_t* plane, uint8_t* dst, int64_t pitch, int W, int H, int ring, int sms,
                             cudaStream_t s) {
  life_unpack_kernel<<<4 * sms, 256, 0, s>>>(plane, life_bits_words(W), dst, pitch, W, H, ring, 0, H);
  return cudaGetLastError();
}

cudaError_t life_bits_unpack_rows(const uint32_t* plane, uint8_t* dst, int64_t pitch, int W, int H, int ring,
                                  int row0, int row1, int sms, cudaStream_t s) {
  if (row1 <= row0) return cudaSuccess;
  life_unpack_kernel<<<4 * sms, 256, 0, s>>>(plane, life_bits_words(W), dst, pitch, W, H, ring, row0, row1);
  return cudaGetLastError();
}


size_t life_bits_sync_bytes(int W, int H, int TH) {
  return 16 + sizeof(unsigned) * static_cast<size_t>(life_bits_tiles(W, H, TH));
}

int life_bits_persistent_ctas_per_sm() {
  int n = 0;
  const size_t smem = life_bits_smem_bytes();
  cudaFuncSetAttribute(life_bits_persistent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       static_cast<int>(smem));
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, life_bits_persistent_kernel, kBThreads, smem) != cudaSuccess)
    return 1;
  return n > 0 ? n : 1;
}

cudaError_t life_bits_run_persistent(uint32_t* X, uint32_t* Y, int W, int H, int ring, int npasses, int q, int r,
                                     int T, int TH, int ctas, void* sync, unsigned* err, cudaStream_t s) {
  const int LH = TH + 2 * T;
  const int PW = life_bits_words(W);
  const int tiles_x = (PW + kBCore - 1) / kBCore;
  const int tiles_y = (H + TH - 1) / TH;
  cudaError_t e = cudaMemsetAsync(sync, 0, life_bits_sync_bytes(W, H, TH), s);
  if (e != cudaSuccess) return e;
  unsigned long long* next = static_cast<unsigned long long*>(sync);
  unsigned* done = reinterpret_cast<unsigned*>(static_cast<char*>(sync) + 16);
  LifeWindow win;
  memset(&win, 0, sizeof(win));
  win.np = npasses;
  life_bits_persistent_kernel<<<ctas, kBThreads, life_bits_smem_bytes(), s>>>(
      X, Y, PW, W, H, ring, npasses, q, r, T, TH, LH, tiles_x, tiles_y, next, done, err, win);
  return cudaGetLastError();
}

cudaError_t life_bits_clear_sync(void* sync, int W, int H, int TH, cudaStream_t s) {
  return cudaMemsetAsync(sync, 0, life_bits_sync_bytes(W, H, TH), s);
}

cudaError_t life_bits_run_window(uint32_t* X, uint32_t* Y, int W, int H, int ring, const LifeWindow& win, int q,
                                 int r, int T, int TH, int ctas, void* sync, unsigned* err, cudaStream_t s) {
  const int LH = TH + 2 * T;
  const int PW = life_bits_words(W);
  const int tiles_x = (PW + kBCore - 1) / kBCore;
  const int tiles_y = (H + TH - 1) / TH;
  // the item counter restarts; the per-tile completion counts carry over
  cudaError_t e = cudaMemsetAsync(sync, 0, 16, s);
  if (e != cudaSuccess) return e;
  unsigned long long* next = static_cast<unsigned long long*>(sync);
  unsigned* done = reinterpret_cast<unsigned*>(static_cast<char*>(sync) + 16);
  life_bits_persistent_kernel<<<ctas, kBThreads, life_bits_smem_bytes(), s>>>(
      X, Y, PW, W, H, ring, win.pass0 + win.np, q, r, T, TH, LH, tiles_x, tiles_y, next, done, err, win);
  return cudaGetLastError();
}

}  // namespace pskel
