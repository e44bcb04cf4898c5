// Internal launch interface between the C ABI (capi.cu) and the kernels.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace pskel {

// Encodes a tiled tensor map through the driver entry point (no libcuda link).
// rank 2: dims {W, H}, row stride in bytes; rank 3 adds the third dimension.
cudaError_t encode_tmap(CUtensorMap* map, CUtensorMapDataType type, int rank, void* base, const uint64_t* dims,
                        const uint64_t* strides_bytes, const uint32_t* box);

// Splits `iters` steps into passes of at most `T` steps whose count has the
// parity of `iters`, so a ping-pong over the passes ends in the buffer a
// step-by-step ping-pong would end in.
std::vector<int> plan_passes(int64_t iters, int T);

// ------------------------------------------------------------------ Life

// Bit-plane Life: pack both grids once into global bit planes (rows of
// life_bits_words(W) words), run the passes between the planes, unpack the
// final plane's interior into the result buffer. A tile is one warp of words
// wide (kLifeCoreWords core words, one halo word each side) and holds a
// window of life_bits_window_rows(T) rows in registers (kLifeWarps consumer
// warps x life_bits_rows(T) rows, plus one row above and below); after
// T <= kLifeBitsMaxT steps its core of TH <= life_bits_max_tile_h(T) =
// life_bits_window_rows(T) - 2T rows is exact. Passes of kLifeTallT steps or
// more use the taller window (its halo rows are a smaller share), shorter
// passes the shorter one (less to load per step).
constexpr int kLifeBitsMaxT = 31;
constexpr int kLifeRowsTall = 24;
constexpr int kLifeRowsShort = 16;
constexpr int kLifeTallT = 15;
constexpr int kLifeWarps = 15;
constexpr int kLifeCoreWords = 30;
constexpr int life_bits_rows(int T) { return T >= kLifeTallT ? kLifeRowsTall : kLifeRowsShort; }
constexpr int life_bits_window_rows(int T) { return kLifeWarps * life_bits_rows(T) + 2; }
int life_bits_words(int W);
int life_bits_tiles_x(int W);
int life_bits_max_tile_h(int T);
size_t life_bits_smem_bytes(int T);
int life_bits_tiles(int W, int H, int TH);
cudaError_t life_bits_pack(const uint8_t* src, int64_t pitch, int W, int H, uint32_t* plane, int ring, bool ring_only,
                           unsigned* err, int sms, cudaStream_t s);
cudaError_t life_bits_unpack(const uint32_t* plane, uint8_t* dst, int64_t pitch, int W, int H, int ring, int sms,
                             cudaStream_t s);
// Every pass in one persistent launch: pass i (of npasses) has
// 1 + 2 * (q + (i < r)) steps and reads X (even i) or Y (odd i). Tiles wait
// (bounded) for their neighbours' previous pass; `sync` holds the item
// counter and per-tile completion counts (life_bits_sync_bytes, cleared here).
// ctas must not exceed the resident CTAs (life_bits_persistent_ctas_per_sm(T)).
size_t life_bits_sync_bytes(int W, int H, int TH);
// A launch's share of the passes of a run: passes pass0 .. pass0+np-1, each
// over every tile, or (windowed) pass pass0+j over the tile rows
// lo[j] .. lo[j] + (start[j+1]-start[j]) / tiles_x - 1 (start: prefix item
// counts). Launches of one run share the completion counts, so a tile waits
// for its neighbourhood's previous pass whichever launch ran it.
constexpr int kLifeMaxWindow = 16;
struct LifeWindow {
  int pass0, np, windowed;
  int lo[kLifeMaxWindow];
  long long start[kLifeMaxWindow + 1];
};
cudaError_t life_bits_clear_sync(void* sync, int W, int H, int TH, cudaStream_t s);
// restart: clear the item counter first (the completion counts carry over);
// spin_limit: polls of a dependency wait before it latches kDevErrBarrier (0:
// the library's limit; the bounded-wait self-test passes a short one)
cudaError_t life_bits_run_window(uint32_t* X, uint32_t* Y, int W, int H, int ring, const LifeWindow& win, int q,
                                 int r, int T, int TH, int ctas, void* sync, unsigned* err, cudaStream_t s,
                                 bool restart = true, unsigned spin_limit = 0);
// Pack rows [row0, row1) (every cell checked to be 0/1) / unpack the interior
// cells of rows [row0, row1).
cudaError_t life_bits_pack_rows(const uint8_t* src, int64_t pitch, int W, int H, uint32_t* plane, int ring,
                                int row0, int row1, unsigned* err, int sms, cudaStream_t s);
cudaError_t life_bits_unpack_rows(const uint32_t* plane, uint8_t* dst, int64_t pitch, int W, int H, int ring,
                                  int row0, int row1, int sms, cudaStream_t s);
int life_bits_persistent_ctas_per_sm(int T);
cudaError_t life_bits_run_persistent(uint32_t* X, uint32_t* Y, int W, int H, int ring, int npasses, int q, int r,
                                     int T, int TH, int ctas, void* sync, unsigned* err, cudaStream_t s);

// ------------------------------------------------------- 2D float stencils

enum class Op2D { Linear, Advect };

constexpr int kMaxMask2D = 32;
constexpr int kStencil2DThreads = 256;

struct Stencil2DParams {
  int W, H;
  int64_t pitch;
  int ring;        // r: cells with r <= h < H-r, r <= w < W-r are updated
  int R;           // max |offset|: halo per step
  int steps;       // steps in this pass
  int T;           // geometry steps (halo = R*T rows)
  int TW, TH;      // core tile
  int LW, LH;      // loaded tile
  int HX, HY;      // horizontal / vertical halo
  int tiles_x, tiles_y;
  int nm;                 // linear: mask size
  int off[kMaxMask2D];    // linear: dh*LW + dw per entry
  float wt[kMaxMask2D];   // linear: weights
  float K, dt, inv_dx;    // advect
  const void* src;
  void* dst;
  const void* u;
  const void* v;
  unsigned* err;
  uint32_t fuse_guard;  // always 0: the kernels form -0.0f from it at run time (neg_zero2)
};

struct Stencil2DGeom {
  int T, TW, TH, LW, LH, HX, HY, tiles_x, tiles_y, ctas;
};

// dtype: 1 = f32, 2 = bf16 (pskel_dtype values).
size_t stencil2d_smem_bytes(Op2D op, int dtype, int LW, int LH);
int stencil2d_max_ctas_per_sm(Op2D op, int dtype, int nm, int LW, int LH);
cudaError_t stencil2d_pass(Op2D op, int dtype, bool use_tma, const CUtensorMap* map_src, const CUtensorMap* map_dst,
                           const CUtensorMap* map_u,
                           const CUtensorMap* map_v, const Stencil2DParams& p, int ctas, cudaStream_t s);

// Register-windowed 2D kernel for reach-1 masks of a known shape and for
// advection. Shapes (entries in summation order): 0 = N,S,W,E;
// 1 = C,N,S,W,E; 2 = the 3x3 box row by row. Returns -1 for other masks.
int fast2d_shape(const int* offsets, int n);
// The default steps per pass of the reach-1 kernels (measured on GB300):
// linear shapes 7 (4096^2 fp32: T=5/7 1.32/1.30 T cell updates/s, T=1 0.70),
// 13 on grids of at most 1M cells, which run every pass in one launch and
// have fewer tiles than resident CTAs (1024^2 fp32: T=7/9/11/13/15/17
// 582/638/681/712/700/690 G cell updates/s: 286 tiles at T=13 put two on
// nearly every SM; 1448^2: T=7/11 928/897);
// advection fp32 5; advection bf16 1 (the HBM-bound streaming kernel) on
// grids of 4M cells or more, else 7.
inline int fast2d_default_steps(bool advect, int dtype, int64_t W, int64_t H) {
  if (!advect) return W * H <= (int64_t(1) << 20) ? 13 : 7;
  if (dtype != 2) return 5;
  return W * H >= (int64_t(1) << 22) ? 1 : 7;
}
size_t fast2d_smem_bytes(bool advect, int dtype, int S);
int fast2d_max_ctas_per_sm(bool advect, int dtype, int S);
// opk: a shape above, or 3 for advection. Tile: 128 cells wide, 16 * S + 2
// rows high (S = 4 or 8), 512 threads.
cudaError_t fast2d_pass(int opk, int dtype, int S, const CUtensorMap* ms, const CUtensorMap* md,
                        const CUtensorMap* mu, const CUtensorMap* mv, const Stencil2DParams& p, int ctas,
                        cudaStream_t s);

// Every pass of a run in one persistent launch of the same tiles (for grids
// of few tiles per pass): items (pass, tile) in order, each tile waiting
// (bounded) for the tiles of the previous pass that its loaded tile overlaps.
// Even passes read the buffer of map_in / p.src and write p.dst, odd passes
// the reverse; pass i has 1 + 2 * (q + (i < r)) steps. `sync` (capacity
// fast2d_multipass_sync_bytes, cleared here) holds the item counter and the
// per-tile completion counts.
size_t fast2d_multipass_smem_bytes(int dtype, int S);
size_t fast2d_multipass_sync_bytes(int ntiles);
// Self-test of the multi-pass kernel's dependency waits
// (pskel_selftest_bounded_wait): while set on the calling thread, the next
// multi-pass 2D run hands out its items from pass `skip_passes` on (the
// earlier passes never run) and gives a dependency wait up after `spin_limit`
// polls. Zero (the default): no effect.
struct DepWaitTest {
  unsigned spin_limit;
  int skip_passes;
};
DepWaitTest& dep_wait_test();
cudaError_t fast2d_multipass(int opk, int dtype, int S, const CUtensorMap* map_in, const CUtensorMap* map_out,
                             const Stencil2DParams& p, int npasses, int q, int r, void* sync, int ctas,
                             cudaStream_t s);

// One step of a reach-1 2D stencil of a known shape (opk 0..2) or advection
// (opk 3), streaming (no temporal blocking), rows staged by TMA: persistent
// blocks (a producer warp and 8 consumer warps) over items of 32 16-byte
// vectors of columns x p.TH rows; `phi` maps the source as 32-bit words with
// a box of 136 words x 8 rows, `u`/`v` (advection) the winds with a box of
// 128 words x 8 rows. Buffers, winds and the row pitch 16-byte aligned.
int stream2d_tma_blocks_per_sm(int opk, int dtype);
int64_t stream2d_tma_items(int W, int H, int HC, int dtype);
cudaError_t stream2d_tma_step(int opk, int dtype, const CUtensorMap* phi, const CUtensorMap* u, const CUtensorMap* v,
                              const Stencil2DParams& p, int ctas, cudaStream_t s);

// ------------------------------------------------------- 3D float stencils

constexpr int kMaxMask3D = 32;
constexpr int kMax3DSteps = 8;  // time steps fused per pass
constexpr int kStencil3DThreads = 256;
constexpr int kPrefetch3D = 3;  // input planes in flight ahead of the march

struct Stencil3DParams {
  int W, H, D;        // h slowest, d fastest
  int R;              // max |offset|
  int NP;             // planes per level ring = 2R + 1
  int steps, T;       // steps in this pass, geometry steps
  int TW, TD;         // core tile in (w, d)
  int LW, LD;         // plane window
  int HW, HD;         // halos in w and d
  int tiles_w, tiles_d;
  int HC, hchunks;    // output planes per work item, work items along h
  int nm;
  int off_h[kMaxMask3D];      // dh per entry
  int off_plane[kMaxMask3D];  // dw * LD + dd per entry
  int off_w[kMaxMask3D];      // dw per entry
  int off_d[kMaxMask3D];      // dd per entry
  float wt[kMaxMask3D];
  float halo;
  const void* src;
  void* dst;
  unsigned* err;
  int64_t step0;       // steps completed before this pass
  int every;           // report ||u_g - u_{g-1}|| when g % every == 0 (0: never)
  double* partials;    // scratch: steps x ctas fp64 partial sums
  double* residuals;   // device: one norm per reported step
  int hbeg, hend;      // streaming 7-point kernel: planes [hbeg, hend) (hend 0: all)
  uint32_t fuse_guard;  // always 0: the kernels form -0.0f from it at run time (neg_zero2)
};

// The 7-point cross, two steps per launch (stream3d_tb.cu): the one-step
// streaming kernel's items with the second step fused behind the first in
// shared memory. Reads p.src (through `map`: the grid as 32-bit words, boxes
// of 136 words x stream3d_tb2_box_rows() rows x 1 plane), writes the state
// after two steps to p.dst. Residual partials: 2 x ctas doubles when a step of
// the pass is reported; the norms are reduced into p.residuals.
int stream3d_tb2_blocks_per_sm(int dtype);
uint32_t stream3d_tb2_box_rows();
cudaError_t stream3d_tb2_pass(int dtype, const CUtensorMap* map, const Stencil3DParams& p, int ctas,
                              cudaStream_t s);
// Sums `steps` levels of per-CTA partials (level k at (k-1) * ctas) in a fixed
// order and stores sqrt at residuals[(step0 + k) / every - 1] for reported k.
cudaError_t stream3d_reduce_residuals(const double* partials, int ctas, int steps, int64_t step0, int every,
                                      double* residuals, cudaStream_t s);

size_t stencil3d_smem_bytes(int LW, int LD, int NP, int T, size_t esize);
int stencil3d_max_ctas_per_sm(size_t smem);
// One step of the generic streaming (not temporally blocked) kernel: a block
// per 32 (d) x 8 (w) columns and h chunk of p.HC planes; residual partials,
// when the step is reported, go to p.partials[one per block].
int64_t stream3d_ctas(int W, int D, int hchunks);
cudaError_t stream3d_step(int dtype, const Stencil3DParams& p, cudaStream_t s);
// The 7-point cross in (centre, h-1, h+1, w-1, w+1, d-1, d+1) order with D a
// multiple of the 16-byte vector (4 fp32 / 8 bf16 cells).
bool stream3d_is_cross7(const int* offsets, int n, int64_t D, int esize);
// The 7-point cross with TMA-staged planes (persistent blocks over work items
// of 32 vectors of d x 16 w x p.HC planes); `map` is a 3D tensor map of the
// source viewed as 32-bit words (dims D*esize/4, W, H; box 136 words x 18
// rows x 1 plane). Residual partials: one per block.
size_t stream3d_tma_smem_bytes(int dtype);
int stream3d_tma_blocks_per_sm(int dtype);
int64_t stream3d_tma_items(int W, int D, int hchunks, int esize);
cudaError_t stream3d_tma_step(int dtype, const CUtensorMap* map, const Stencil3DParams& p, int ctas,
                              cudaStream_t s);
// One step of planes [p.hbeg, p.hend) with the streaming 7-point kernel; with
// `acc` set the step's squared difference sum is added to *acc (one block,
// fixed order) instead of written as a norm.
cudaError_t stream3d_tma_band(int dtype, const CUtensorMap* map, const Stencil3DParams& p, int ctas, double* acc,
                              cudaStream_t s);
// residuals[i] = sqrt(acc[i]) for i < n.
cudaError_t stream3d_finish_residuals(const double* acc, int n, double* residuals, cudaStream_t s);
// acc[0] += the sum of partials[0..n) (one block, fixed order).
cudaError_t stream3d_accumulate(const double* partials, int n, double* acc, cudaStream_t s);
// One two-step pass over the whole grid whose squared-difference sums of its
// first / second step are added to acc1 / acc2 (each reported when non-null;
// partials: 2 * ctas doubles).
cudaError_t stream3d_tb2_band(int dtype, const CUtensorMap* map, const Stencil3DParams& p, int ctas, double* acc1,
                              double* acc2, cudaStream_t s);
cudaError_t stencil3d_pass(int dtype, bool use_tma, const CUtensorMap* map_src, const Stencil3DParams& p, int ctas,
                           cudaStream_t s);

}  // namespace pskel
