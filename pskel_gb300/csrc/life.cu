// Game of Life, temporally blocked and bit-sliced, on bit planes.
//
// A run packs the source and destination grids (one 0/1 byte per cell, the
// reference's layout) once into two global bit planes -- one bit per cell,
// 16 MB for an 8192^2 grid, so the planes stay in L2 -- runs every pass
// between the planes in one persistent launch and unpacks the final plane's
// interior into the result buffer once.
//
// A pass advances a tile by up to 31 steps with the tile held in registers:
// one warp spans 32 words (1024 cells) of a tile row, lane l holding word
// 30*tx - 1 + l (lanes 1..30 are the tile's core, lanes 0 and 31 its one-word
// halo), and each lane holds a column of R words of its warp's rows (R = 24
// for passes of 15 steps or more, 16 for shorter ones) plus a copy of the
// row above and below. West/east neighbour words come
// from the adjacent lanes by warp shuffles, rows above/below from the
// lane's own registers; after each step the warps of a block exchange their
// first and last rows through shared memory, each warp meeting only its two
// neighbours (pairwise named barriers). A step costs per 32-cell word 2
// shuffles, 2 funnel shifts and 10 LOP3s (row sums shared by the three rows
// that use them, bit-sliced full adders). Work items (pass, tile) come from an
// atomic counter; a producer warp takes the next item, waits (bounded) until
// the tiles of the previous pass its window reads are done, and loads the
// window from L2 into shared memory by 2D TMA (boxes of at most 256 rows)
// while the consumer warps step the current tile; they then copy it into
// their registers.
//
// Ring cells (outside r <= h < H-r, r <= w < W-r) are never updated, the
// semantics of Stencil2D::runOpenMP (PSkelStencil.hpp:2197-2257): in the
// step-by-step run a ring cell holds the source buffer's value after even
// steps and the destination buffer's after odd ones. Tiles that reach the
// ring therefore keep, per word, the interior mask M and the flip
// D = (src ^ dst) outside M in shared memory, and a step writes
// M ? rule : old ^ D.
//
// Redundant halo work: garbage enters a tile at its outermost rows (never
// refreshed) and at lanes 0 and 31 (no neighbour lane) and advances one cell
// per step, so after T <= 31 steps rows T .. T + TH - 1 of the window and
// lanes 1..30 are exact.
#include "common.cuh"
#include "kernels.h"

namespace pskel {
namespace {

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

// Register-resident tile geometry (kernels.h: life_bits_rows, kLifeWarps,
// kLifeCoreWords): with R rows per lane, consumer warp w of a block holds
// rows w*R .. w*R + R + 1 of the tile's window of kLifeWarps*R + 2 rows.
static_assert(kLifeCoreWords == 30, "a tile is one warp of words with one halo word each side");

// Row sums of one row for the bit-sliced neighbour count: with we / ea the
// west / east neighbour of every cell (the adjacent lanes' words by shuffles,
// bit b of `we` = cell b-1), (t0, t1) = we + c + ea and (p0, p1) = we + ea as
// 2-bit bit-sliced numbers.
__device__ __forceinline__ void row_sums(uint32_t c, uint32_t& t0, uint32_t& t1, uint32_t& p0, uint32_t& p1) {
  const uint32_t l = __shfl_up_sync(0xFFFFFFFFu, c, 1);    // lane 0 gets its own word: halo lane
  const uint32_t e = __shfl_down_sync(0xFFFFFFFFu, c, 1);  // lane 31 likewise
  const uint32_t we = __funnelshift_l(l, c, 1);            // (c << 1) | (l >> 31)
  const uint32_t ea = __funnelshift_r(c, e, 1);            // (c >> 1) | (e << 31)
  t0 = lop3<kXor3>(we, c, ea);
  t1 = lop3<kMaj>(we, c, ea);
  p0 = we ^ ea;
  p1 = we & ea;
}

// One step of a warp's rows 1..R from rows 0..R+1, in place.
// The neighbour count of a cell is (row above: t) + (its row: p) + (row
// below: t); the three 2-bit numbers are added with full adders: s0 = low
// bit, k0 = its carry, x1/y1 = sum/carry of the twos. With k0 folded in,
// count in {2, 3} <=> ~y1 & (x1 ^ k0), and the cell lives iff that holds and
// (s0 | alive): count 3, or count 2 and alive. A count of 8 leaves y1 set,
// so it is dead as it must be. kRing: cells outside the interior mask M of
// the row take old ^ D instead (M, D per row and lane in shared memory).
template <bool kRing, int R>
__device__ __forceinline__ void life_reg_step(uint32_t (&x)[R + 2], const uint32_t* __restrict__ Mw,
                                              const uint32_t* __restrict__ Dw, int lane) {
  uint32_t a0, a1, u0, u1, b0, b1, q0, q1;
  row_sums(x[0], a0, a1, u0, u1);
  row_sums(x[1], b0, b1, q0, q1);
#pragma unroll
  for (int i = 1; i <= R; ++i) {
    uint32_t c0, c1, r0, r1;
    row_sums(x[i + 1], c0, c1, r0, r1);  // row i+1 still holds the previous step
    const uint32_t s0 = lop3<kXor3>(a0, q0, c0);
    const uint32_t k0 = lop3<kMaj>(a0, q0, c0);
    const uint32_t x1 = lop3<kXor3>(a1, q1, c1);
    const uint32_t y1 = lop3<kMaj>(a1, q1, c1);
    const uint32_t two_or_three = lop3<kNotAAndBxC>(y1, x1, k0);
    const uint32_t alive = lop3<kAAndBorC>(two_or_three, s0, x[i]);
    if (kRing) {
      const uint32_t m = Mw[(i - 1) * 32 + lane];
      const uint32_t d = Dw[(i - 1) * 32 + lane];
      x[i] = lop3<kSelect>(m, alive, x[i] ^ d);
    } else {
      x[i] = alive;
    }
    a0 = b0;
    a1 = b1;
    b0 = c0;
    b1 = c1;
    q0 = r0;
    q1 = r1;
  }
  (void)u0;
  (void)u1;
}

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

// A block is NW consumer warps, which hold and step the tile (R rows per
// lane), and one producer warp, which fetches the next work item, waits for
// its dependencies and loads its window by TMA into shared memory while the
// consumers step the current one.
// The TMA box: the window's 32 words start at word 30 tx - 1, which is not
// 16-byte aligned; the box starts at the aligned word below it (x & ~3) and
// is 36 words wide, and lanes read from the offset (0..3).
constexpr int kLifeBoxWords = 36;
template <int R, int NW>
struct LifeGeo {
  static constexpr int kWindowRows = NW * R + 2;
  // the window arrives as kBoxes TMA boxes of kBoxRows rows (a box has at
  // most 256 rows; several boxes have a multiple of 8 rows, so that each
  // lands 128-byte aligned, and may fetch a few rows past the window)
  static constexpr int kBoxes = (kWindowRows + 255) / 256;
  static constexpr int kBoxRows = kBoxes == 1 ? kWindowRows : ((kWindowRows + kBoxes - 1) / kBoxes + 7) / 8 * 8;
  static constexpr int kThreads = (NW + 1) * 32;
  static constexpr int kConsumerThreads = NW * 32;
  static constexpr uint32_t kBoxBytes = kBoxes * kBoxRows * kLifeBoxWords * 4;  // one window's boxes
  static constexpr int kBoxStride = (kBoxBytes + 127) / 128 * 128;
  // shared memory (bytes): source window, destination window (ring tiles),
  // the exchange rows (two parities x warps x {first, last} row x 32 lanes),
  // M and D of ring tiles (R rows x 32 lanes per warp each), two mbarriers
  // and the item slot
  static constexpr int kXchWords = 2 * NW * 2 * 32;
  static constexpr int kRingWords = NW * R * 32;
  static constexpr int kSmemWords = 2 * kBoxStride / 4 + kXchWords + 2 * kRingWords;
  static constexpr size_t kSmemBytes = static_cast<size_t>(kSmemWords) * 4 + 64;
  static_assert(kBoxBytes % 16 == 0, "TMA transaction bytes");
  static_assert(kBoxRows * kBoxes >= kWindowRows && kBoxRows <= 256, "TMA box rows");
  static_assert((kBoxRows * kLifeBoxWords * 4) % 128 == 0 || kBoxes == 1, "box destinations 128-byte aligned");
  static_assert(NW <= 15, "one named barrier per neighbouring pair, ids 1..14, and 15 for all consumers");
};

struct LifeSlot {
  int valid;  // 0: no more items (or an error): consumers leave
  int pass, tile;
};

// All consumer warps (named barrier 15; the producer warp takes no part).
template <int NW>
__device__ __forceinline__ void consumers_barrier() {
  asm volatile("bar.sync 15, %0;" ::"n"(NW * 32) : "memory");
}

// Consumer warp w and w+1 share named barrier 1 + w (ids 1..14). A warp
// synchronises with its two neighbours only, in two rounds -- even warps
// first with the warp below, odd warps first with the warp above -- so the
// pairs (0,1), (2,3), ... meet first and (1,2), (3,4), ... second, and no
// chain of waits runs through the block.
__device__ __forceinline__ void pair_barrier(int id) { asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory"); }
template <int NW>
__device__ __forceinline__ void neighbours_barrier(int w) {
  if ((w & 1) == 0) {
    if (w + 1 < NW) pair_barrier(1 + w);
    if (w > 0) pair_barrier(w);
  } else {
    pair_barrier(w);
    if (w + 1 < NW) pair_barrier(1 + w);
  }
}

// Every pass of a run in one launch. Work items (pass, tile) are handed out
// in order by an atomic counter. The producer warp of a block takes an item,
// waits (bounded) until every tile of pass p-1 whose core the item's window
// reads -- rows within ceil(T/TH) tiles, one tile column either side -- has
// completed (done[] counts the consumer warps that finished each tile, so a
// pass is kLifeWarps counts), waits for the window buffer to be free and
// loads the window (and, for ring tiles, the destination plane's) by TMA.
// Those tiles were also the last readers of the region the item writes. All
// blocks are resident and items are taken in order, so every awaited item is
// held by a running block (possibly this one: its consumers finish the
// current item without the producer). A latched error word stops the
// producers at their next poll or item; the consumers then leave. Pass i has
// 1 + 2 * (q + (i < r)) steps (the odd-length plan of plan_passes).
template <int R, int NW, int kMinBlocks>
__global__ void __launch_bounds__(LifeGeo<R, NW>::kThreads, kMinBlocks)
    life_bits_persistent_kernel(const __grid_constant__ CUtensorMap mapX, const __grid_constant__ CUtensorMap mapY,
                                uint32_t* __restrict__ planeX, uint32_t* __restrict__ planeY, int PW, int W, int H,
                                int ring, int q, int r, int T, int TH, int tiles_x, int tiles_y,
                                unsigned long long* next_item, unsigned* done, unsigned* err,
                                const __grid_constant__ LifeWindow win, unsigned spin_limit) {
  using G = LifeGeo<R, NW>;
  extern __shared__ __align__(128) uint8_t lsm_raw[];
  uint32_t* win_src = reinterpret_cast<uint32_t*>(lsm_raw);
  uint32_t* win_dst = reinterpret_cast<uint32_t*>(lsm_raw + G::kBoxStride);
  uint32_t* xch = reinterpret_cast<uint32_t*>(lsm_raw + 2 * G::kBoxStride);
  uint32_t* Ms = xch + G::kXchWords;
  uint32_t* Ds = Ms + G::kRingWords;
  uint64_t* bars = reinterpret_cast<uint64_t*>(lsm_raw + static_cast<size_t>(G::kSmemWords) * 4);
  uint64_t* full = &bars[0];
  uint64_t* empty = &bars[1];
  LifeSlot* slot = reinterpret_cast<LifeSlot*>(&bars[2]);
  __shared__ int s_ok;
  const int tid = threadIdx.x;
  const int lane = tid & 31, w = tid >> 5;
  if ((smem_u32(lsm_raw) & 127u) != 0) {  // TMA needs the aligned base; uniform across the block
    if (tid == 0) atomicOr(err, kDevErrAlign);
    return;
  }
  if (tid == 0) {
    mbar_init(full, 1);
    mbar_init(empty, NW);
    fence_barrier_init();
    prefetch_tensormap(&mapX);
    prefetch_tensormap(&mapY);
  }
  __syncthreads();
  const int ntiles = tiles_x * tiles_y;
  // this launch's items: passes win.pass0 .. + win.np, each over all tiles or
  // (windowed) over tile rows [win.lo[j], ...) holding win.start[j+1] -
  // win.start[j] items; completion counts persist between the launches of a run
  const long long nitems = win.windowed ? win.start[win.np] : static_cast<long long>(win.np) * ntiles;

  if (w == NW) {
    // ---------------------------------------------------------- producer
    if (lane != 0) return;
    const int dy = (T + TH - 1) / TH;
    uint32_t empty_phase = 0;
    for (long long k = 0;; ++k) {
      const long long it = error_latched(err) ? nitems : static_cast<long long>(atomicAdd(next_item, 1ull));
      int valid = it < nitems ? 1 : 0;
      int pass = 0, tile = 0;
      if (valid) {
        if (win.windowed) {
          int j = 0;
          while (j + 1 < win.np && win.start[j + 1] <= it) ++j;
          const long long kk = it - win.start[j];
          pass = win.pass0 + j;
          tile = static_cast<int>((win.lo[j] + kk / tiles_x) * tiles_x + kk % tiles_x);
        } else {
          pass = win.pass0 + static_cast<int>(it / ntiles);
          tile = static_cast<int>(it % ntiles);
        }
      }
      const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
      if (valid && pass > 0) {
        const unsigned need = static_cast<unsigned>(pass) * NW;
        for (int yy = max(0, ty - dy); yy <= min(tiles_y - 1, ty + dy) && valid; ++yy) {
          for (int xx = max(0, tx - 1); xx <= min(tiles_x - 1, tx + 1) && valid; ++xx) {
            const unsigned* d = &done[yy * tiles_x + xx];
            unsigned polls = 0;
            while (ld_acquire_u32(d) < need) {
              if (error_latched(err)) {  // another block gave up: stop, it reported why
                valid = 0;
                break;
              }
              if (++polls >= spin_limit) {
                atomicOr(err, kDevErrBarrier);
                valid = 0;
                break;
              }
              __nanosleep(32);
            }
          }
        }
      }
      // the consumers have copied the previous window (and read its slot)
      if (k > 0) {
        if (!mbar_wait_bounded(empty, empty_phase, err)) valid = 0;
        empty_phase ^= 1u;
      }
      slot->valid = valid;
      slot->pass = pass;
      slot->tile = tile;
      if (!valid) {
        mbar_arrive(full);  // releases the consumers with valid = 0
        return;
      }
      const int wy0 = ty * TH - T;
      const int gx = tx * kLifeCoreWords - 1;
      const bool ring_tile = wy0 < ring || wy0 + G::kWindowRows > H - ring || gx * 32 < ring ||
                             (gx + 32) * 32 > W - ring;
      const CUtensorMap* msrc = (pass & 1) ? &mapY : &mapX;
      const CUtensorMap* mdst = (pass & 1) ? &mapX : &mapY;
      // the tiles awaited above wrote through the generic proxy; TMA reads
      // through the async proxy
      fence_proxy_async_global();
      mbar_arrive_expect_tx(full, G::kBoxBytes * (ring_tile ? 2u : 1u));
#pragma unroll
      for (int b = 0; b < G::kBoxes; ++b) {
        const int off = b * G::kBoxRows * kLifeBoxWords;
        tma_load_2d(win_src + off, msrc, gx & ~3, wy0 + b * G::kBoxRows, full);
        if (ring_tile) tma_load_2d(win_dst + off, mdst, gx & ~3, wy0 + b * G::kBoxRows, full);
      }
    }
  }

  // ------------------------------------------------------------ consumers
  uint32_t* Mw = Ms + w * R * 32;
  uint32_t* Dw = Ds + w * R * 32;
  uint32_t full_phase = 0;
  for (;;) {
    // one thread waits (bounded) and the decision is shared, so every
    // consumer warp takes the same path through the named barriers below
    if (tid == 0) s_ok = mbar_wait_bounded(full, full_phase, err) ? 1 : 0;
    consumers_barrier<NW>();
    if (!s_ok) break;
    mbar_try_wait(full, full_phase);  // completed: the TMA data is visible to this thread too
    full_phase ^= 1u;
    const volatile LifeSlot* vs = slot;
    if (!vs->valid) break;
    const int pass = vs->pass, tile = vs->tile;
    const int steps = 1 + 2 * (q + (pass < r ? 1 : 0));
    uint32_t* dst = (pass & 1) ? planeX : planeY;
    const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
    const int wy0 = ty * TH - T;
    const int gx = tx * kLifeCoreWords - 1;
    const int gw = gx + lane;
    const int col = (gx - (gx & ~3)) + lane;  // this lane's word in the box
    const int gyw = wy0 + w * R;      // this warp's row 0
    const bool ring_tile = wy0 < ring || wy0 + G::kWindowRows > H - ring || gx * 32 < ring ||
                           (gx + 32) * 32 > W - ring;
    uint32_t x[R + 2];
#pragma unroll
    for (int i = 0; i < R + 2; ++i) x[i] = win_src[(w * R + i) * kLifeBoxWords + col];
    if (ring_tile) {
      // interior mask and ring flip of the rows this warp steps (only it reads them)
      const bool gw_in = gw >= 0 && gw < PW;
      const uint32_t colmask = gw_in ? bit_range(ring - 32 * gw, (W - ring) - 32 * gw) : 0u;
#pragma unroll
      for (int i = 1; i <= R; ++i) {
        const int gy = gyw + i;
        const uint32_t m = (gw_in && gy >= ring && gy < H - ring) ? colmask : 0u;
        const uint32_t b = win_dst[(w * R + i) * kLifeBoxWords + col];
        Mw[(i - 1) * 32 + lane] = m;
        Dw[(i - 1) * 32 + lane] = (x[i] ^ b) & ~m;
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(empty);  // this warp is done with the window and the slot
    int par = 0;
    for (int s = 0; s < steps; ++s) {
      if (ring_tile) {
        life_reg_step<true, R>(x, Mw, Dw, lane);
      } else {
        life_reg_step<false, R>(x, Mw, Dw, lane);
      }
      if (s + 1 < steps) {
        // exchange the first and last rows with the warps above and below;
        // two parities, so one meeting per step suffices: a warp rewrites its
        // slot of a parity two steps later, after meeting its neighbours
        // again, which they do only once they have read the slot
        uint32_t* xb = xch + par * (2 * NW * 32);
        xb[(2 * w) * 32 + lane] = x[1];
        xb[(2 * w + 1) * 32 + lane] = x[R];
        neighbours_barrier<NW>(w);
        if (w > 0) x[0] = xb[(2 * (w - 1) + 1) * 32 + lane];
        if (w < NW - 1) x[R + 1] = xb[(2 * (w + 1)) * 32 + lane];
        par ^= 1;
      }
    }
    // write back the core: rows [ty*TH, ty*TH + TH) of the grid, lanes 1..30
    const int gc0 = ty * TH;
    const int gc1 = min(H, gc0 + TH);
    if (lane >= 1 && lane <= kLifeCoreWords && gw < PW) {
#pragma unroll
      for (int i = 1; i <= R; ++i) {
        const int gy = gyw + i;
        if (gy >= gc0 && gy < gc1) dst[static_cast<int64_t>(gy) * PW + gw] = x[i];
      }
    }
    __threadfence();
    __syncwarp();
    if (lane == 0) atomicAdd(&done[tile], 1u);
  }
}

}  // namespace

namespace {

// The kernels as launched: life_bits_rows(T) rows per lane, kLifeWarps
// consumer warps, one block per SM. Measured on GB300 (8192^2, 1000
// generations): 24 rows x 15 warps (128 registers: the register file
// exactly; a 362-row window in two TMA boxes) 27.7 T updates/s at T = 17;
// 16 rows x 15 warps (242 rows, one box) 27.4 T at T = 13, 27.3 T at T = 15,
// and at one step per pass 9.1 T against 7.6 T for the 24-row window; 8 rows
// x 15 warps at two blocks per SM 21.5 T (T = 7, the best T for it; its
// windows are half as tall, so the halo rows and the per-step exchange cost
// twice as much per row); 16 rows x 7 warps at two blocks per SM 22.5 T. The
// row shifts as integer multiply-adds on the idle FMA pipe (by 2 and 2^31
// from a kernel argument) instead of funnel shifts on the ALU pipe: 23.3 T.
constexpr int kLifeMinBlocks = 1;
static_assert(life_bits_rows(kLifeBitsMaxT) == kLifeRowsTall && life_bits_rows(1) == kLifeRowsShort, "geometries");

template <int R>
struct LifeKernel {
  using G = LifeGeo<R, kLifeWarps>;
  static constexpr auto fn = life_bits_persistent_kernel<R, kLifeWarps, kLifeMinBlocks>;
  static cudaError_t allow_smem() {
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(G::kSmemBytes));
  }
};

}  // namespace

int life_bits_words(int W) { return ((W + 31) / 32 + 3) & ~3; }

int life_bits_tiles_x(int W) { return (life_bits_words(W) + kLifeCoreWords - 1) / kLifeCoreWords; }

int life_bits_max_tile_h(int T) { return life_bits_window_rows(T) - 2 * T; }

int life_bits_tiles(int W, int H, int TH) { return life_bits_tiles_x(W) * ((H + TH - 1) / TH); }

size_t life_bits_smem_bytes(int T) {
  return life_bits_rows(T) == kLifeRowsTall ? LifeKernel<kLifeRowsTall>::G::kSmemBytes
                                            : LifeKernel<kLifeRowsShort>::G::kSmemBytes;
}


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

namespace {
template <int R>
int life_ctas_per_sm() {
  using K = LifeKernel<R>;
  int n = 0;
  K::allow_smem();
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, K::fn, K::G::kThreads, K::G::kSmemBytes) != cudaSuccess)
    return 1;
  return n > 0 ? n : 1;
}
}  // namespace

int life_bits_persistent_ctas_per_sm(int T) {
  return life_bits_rows(T) == kLifeRowsTall ? life_ctas_per_sm<kLifeRowsTall>() : life_ctas_per_sm<kLifeRowsShort>();
}

cudaError_t life_bits_run_persistent(uint32_t* X, uint32_t* Y, int W, int H, int ring, int npasses, int q, int r,
                                     int T, int TH, int ctas, void* sync, unsigned* err, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(sync, 0, life_bits_sync_bytes(W, H, TH), s);
  if (e != cudaSuccess) return e;
  LifeWindow win;
  memset(&win, 0, sizeof(win));
  win.np = npasses;
  return life_bits_run_window(X, Y, W, H, ring, win, q, r, T, TH, ctas, sync, err, s, false);
}

cudaError_t life_bits_clear_sync(void* sync, int W, int H, int TH, cudaStream_t s) {
  return cudaMemsetAsync(sync, 0, life_bits_sync_bytes(W, H, TH), s);
}

cudaError_t life_bits_run_window(uint32_t* X, uint32_t* Y, int W, int H, int ring, const LifeWindow& win, int q,
                                 int r, int T, int TH, int ctas, void* sync, unsigned* err, cudaStream_t s,
                                 bool restart, unsigned spin_limit) {
  if (spin_limit == 0) spin_limit = kLifeSpinLimit;
  if (T < 1 || T > kLifeBitsMaxT || TH < 1 || TH > life_bits_max_tile_h(T)) return cudaErrorInvalidValue;
  const int PW = life_bits_words(W);
  const int tiles_x = life_bits_tiles_x(W);
  const int tiles_y = (H + TH - 1) / TH;
  // the item counter restarts; the per-tile completion counts carry over
  if (restart) {
    cudaError_t e = cudaMemsetAsync(sync, 0, 16, s);
    if (e != cudaSuccess) return e;
  }
  unsigned long long* next = static_cast<unsigned long long*>(sync);
  unsigned* done = reinterpret_cast<unsigned*>(static_cast<char*>(sync) + 16);
  // both planes as 2D tensors of 32-bit words (rows of PW words, 16-byte
  // aligned: PW is a multiple of 4); boxes of 36 words x the window's rows,
  // zero-filled outside the plane
  CUtensorMap mx, my;
  const uint64_t dims[2] = {static_cast<uint64_t>(PW), static_cast<uint64_t>(H)};
  const uint64_t strides[1] = {static_cast<uint64_t>(PW) * 4};
  auto launch = [&](auto kernel) -> cudaError_t {
    using K = decltype(kernel);
    const uint32_t box[2] = {static_cast<uint32_t>(kLifeBoxWords), static_cast<uint32_t>(K::G::kBoxRows)};
    cudaError_t e = encode_tmap(&mx, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, X, dims, strides, box);
    if (e == cudaSuccess) e = encode_tmap(&my, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, Y, dims, strides, box);
    if (e == cudaSuccess) e = K::allow_smem();
    if (e != cudaSuccess) return e;
    K::fn<<<ctas, K::G::kThreads, K::G::kSmemBytes, s>>>(mx, my, X, Y, PW, W, H, ring, q, r, T, TH, tiles_x, tiles_y,
                                                         next, done, err, win, spin_limit);
    return cudaGetLastError();
  };
  return life_bits_rows(T) == kLifeRowsTall ? launch(LifeKernel<kLifeRowsTall>{}) : launch(LifeKernel<kLifeRowsShort>{});
}

}  // namespace pskel
