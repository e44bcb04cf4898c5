// 2D fp32 / bf16-storage stencils of reach 1 with a known mask shape
// (weights at run time) and the advection-diffusion op: register-windowed
// temporal blocking.
//
// Same tiling and semantics as stencil2d.cu (TMA-staged halo tiles, T steps
// per pass ping-ponging between two shared buffers, the destination's ring
// staged for ring tiles, interior cells only written back), but each thread
// owns one 4-cell column vector of a strip of S rows
// and reads every shared-memory row once per step with one vector load (128
// bits fp32, 64 bits bf16) plus its two edge neighbours, keeping a
// (S + 2)-row window in registers. The tile is 128 cells wide and
// 16 * S + 2 rows high (16 warps of S rows each);
// garbage from the tile edges advances one cell per step into the halo, which
// the core never reaches in T <= halo steps; step s computes the full width
// and only the rows [s, LH - s) that are still exact.
//
// fp32 tiles clear of the ring keep their rows in registers between steps
// instead (fast2d_tile.cuh). Arithmetic is the oracle's: products and sums in
// mask order, unfused (two neighbouring cells per instruction with the paired
// fp32 forms of common.cuh), bf16 results rounded every step.
#include <atomic>

#include "fast2d_tile.cuh"

namespace pskel {
namespace {

using namespace fast2d;

// OpK: 0..2 linear shapes above, 3 = advection.
template <class TS, int OpK, int S>
__global__ void __launch_bounds__(kFastThreads, S <= 4 ? 2 : 1)
    fast2d_kernel(const __grid_constant__ CUtensorMap map_src, const __grid_constant__ CUtensorMap map_dst,
                  const __grid_constant__ CUtensorMap map_u, const __grid_constant__ CUtensorMap map_v,
                  const __grid_constant__ Stencil2DParams p) {
  constexpr int N = Vec<TS>::N;
  constexpr int LW = 32 * N;
  constexpr int LH = (kFastThreads / 32) * S + 2;
  constexpr size_t kBuf = (static_cast<size_t>(LW) * LH * sizeof(TS) + 127) & ~size_t(127);
  constexpr uint32_t kTileBytes = static_cast<uint32_t>(LW * LH * sizeof(TS));
  // dynamic shared memory, 128-byte aligned for TMA; derived pointers stay
  // in the shared window (no integer round trip), so accesses compile to
  // shared-memory instructions
  extern __shared__ __align__(128) uint8_t smem_raw[];
  uint8_t* base = smem_raw;
  if ((smem_u32(smem_raw) & 127u) != 0) {
    if (threadIdx.x == 0) atomicOr(p.err, kDevErrAlign);
    return;
  }
  auto buf = [&](int i) { return reinterpret_cast<TS*>(base + static_cast<size_t>(i) * kBuf); };
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + kFastBufs * kBuf);  // one per buffer
  (void)map_u;
  (void)map_v;

  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int i = 0; i < kFastBufs; ++i) mbar_init(&bars[i], 1);
    fence_barrier_init();
    prefetch_tensormap(&map_src);
    prefetch_tensormap(&map_dst);
  }
  __syncthreads();

  constexpr auto shp = shape_of<(OpK < 3 ? OpK : 0)>();
  float wt[9];
#pragma unroll
  for (int n = 0; n < 9; ++n) wt[n] = (n < shp.n) ? p.wt[n] : 0.0f;

  TS* dst = static_cast<TS*>(p.dst);
  uint32_t phase_bits = 0;  // bit i: parity of the next completion of bars[i]
  const int ntiles = p.tiles_x * p.tiles_y;
  auto origin = [&](int t, int& gy0, int& gx0) {
    const int ty = t / p.tiles_x;
    gy0 = ty * p.TH - p.HY;
    gx0 = (t - ty * p.tiles_x) * p.TW - p.HX;
  };
  auto load = [&](int b, const CUtensorMap* m, int gy0, int gx0) {
    fence_proxy_async();
    mbar_arrive_expect_tx(&bars[b], kTileBytes);
    tma_load_2d(buf(b), m, gx0, gy0, &bars[b]);
  };
  // one thread waits on a buffer's barrier; the block barrier that follows
  // publishes the tile to the other threads
  auto wait1 = [&](int b) -> bool { return mbar_wait_bounded(&bars[b], (phase_bits >> b) & 1u, p.err); };

  if (tid == 0 && static_cast<int>(blockIdx.x) < ntiles) {
    int gy0, gx0;
    origin(blockIdx.x, gy0, gx0);
    load(0, &map_src, gy0, gx0);
  }
  int it = 0;  // tiles processed by this CTA: buffer rotation
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int bs = it % 3, bp = (it + 2) % 3, bn = (it + 1) % 3;  // source, partner, next source
    int gy0, gx0;
    origin(tile, gy0, gx0);
    const bool ring_tile = (gy0 < p.ring) || (gy0 + LH > p.H - p.ring) || (gx0 < p.ring) || (gx0 + LW > p.W - p.ring);
    const bool stage_dst = ring_tile && p.steps >= 2;
    if (tid == 0) {
      // the partner buffer was last read by the previous tile's write-back
      if (stage_dst) load(bp, &map_dst, gy0, gx0);
      const int next = tile + static_cast<int>(gridDim.x);
      if (next < ntiles) {
        int ny0, nx0;
        origin(next, ny0, nx0);
        load(bn, &map_src, ny0, nx0);
      }
    }
    int ok = 1;
    if (tid == 0) ok = (wait1(bs) && (!stage_dst || wait1(bp))) ? 1 : 0;
    phase_bits ^= (1u << bs);
    if (stage_dst) phase_bits ^= (1u << bp);
    if (!__syncthreads_and(ok)) return;

    TileGeom g;
    g.W = p.W;
    g.H = p.H;
    g.ring = p.ring;
    g.steps = p.steps;
    g.TW = p.TW;
    g.TH = p.TH;
    g.HX = p.HX;
    g.HY = p.HY;
    g.pitch = p.pitch;
    g.K = p.K;
    g.dt = p.dt;
    g.inv_dx = p.inv_dx;
    g.u = p.u;
    g.v = p.v;
    fast2d_run_tile<TS, OpK, S>(buf(bs), buf(bp), dst, g, gy0, gx0, ring_tile, wt, neg_zero2(p.fuse_guard));
    __syncthreads();
  }
}

// One run of fast2d_multipass_kernel: the pass plan and the shared counters.
struct Fast2DRun {
  int npasses, q, r;              // pass i has 1 + 2 * (q + (i < r)) steps
  unsigned long long* next_item;  // next (pass, tile) item to hand out, counted from first_item
  unsigned* done;                 // passes completed, one count per tile
  long long first_item;           // 0 (the bounded-wait self-test starts later)
  unsigned spin_limit;            // polls of one dependency wait before it gives up
};

constexpr unsigned kFastSpinLimit = 1u << 24;  // polls of a neighbour's completion count (each with a sleep)

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* q) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(q) : "memory");
  return v;
}


// Every pass of a run in one persistent launch (grids of few tiles per pass,
// where the end of each pass would leave SMs idle and every launch adds its
// own latency). Work items (pass, tile) are handed out in order by an atomic
// counter; before tile t of pass i is staged, thread 0 waits (bounded) until
// each tile of pass i-1 whose core overlaps t's loaded tile has completed
// (done[] counts the passes each tile has completed). Those tiles are also
// the last readers of t's core in the buffer pass i writes. An awaited item
// precedes the waiting one, so a running CTA holds it or has finished it.
// A wait that runs out latches kDevErrBarrier; the other CTAs see the latched
// word at their next poll or item and stop.
// Even passes read `in` (map_in) and write `out`, odd passes the reverse;
// pass i has 1 + 2 * (q + (i < r)) steps (the odd-length plan).
template <class TS, int OpK, int S>
__global__ void __launch_bounds__(kFastThreads, S <= 4 ? 2 : 1)
    fast2d_multipass_kernel(const __grid_constant__ CUtensorMap map_in, const __grid_constant__ CUtensorMap map_out,
                            const __grid_constant__ Stencil2DParams p, const __grid_constant__ Fast2DRun run) {
  constexpr int N = Vec<TS>::N;
  constexpr int LW = 32 * N;
  constexpr int LH = (kFastThreads / 32) * S + 2;
  constexpr size_t kBuf = (static_cast<size_t>(LW) * LH * sizeof(TS) + 127) & ~size_t(127);
  constexpr uint32_t kTileBytes = static_cast<uint32_t>(LW * LH * sizeof(TS));
  extern __shared__ __align__(128) uint8_t smem_raw[];
  if ((smem_u32(smem_raw) & 127u) != 0) {
    if (threadIdx.x == 0) atomicOr(p.err, kDevErrAlign);
    return;
  }
  TS* buf0 = reinterpret_cast<TS*>(smem_raw);
  TS* buf1 = reinterpret_cast<TS*>(smem_raw + kBuf);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + 2 * kBuf);
  __shared__ long long s_item;

  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_barrier_init();
    prefetch_tensormap(&map_in);
    prefetch_tensormap(&map_out);
  }
  __syncthreads();
  constexpr auto shp = shape_of<(OpK < 3 ? OpK : 0)>();
  float wt[9];
#pragma unroll
  for (int n = 0; n < 9; ++n) wt[n] = (n < shp.n) ? p.wt[n] : 0.0f;

  const int ntiles = p.tiles_x * p.tiles_y;
  const long long nitems = static_cast<long long>(run.npasses) * ntiles;
  const int dy = (p.HY + p.TH - 1) / p.TH;  // tile rows / columns whose cores the loaded tile overlaps
  const int dx = (p.HX + p.TW - 1) / p.TW;
  uint32_t phase_bits = 0;  // bit i: parity of the next completion of bars[i]
  for (;;) {
    if (tid == 0)
      s_item = error_latched(p.err) ? nitems : run.first_item + static_cast<long long>(atomicAdd(run.next_item, 1ull));
    __syncthreads();
    const long long item = s_item;
    if (item >= nitems) break;
    const int pass = static_cast<int>(item / ntiles);
    const int tile = static_cast<int>(item - static_cast<long long>(pass) * ntiles);
    const int ty = tile / p.tiles_x, tx = tile - ty * p.tiles_x;
    const int gy0 = ty * p.TH - p.HY;
    const int gx0 = tx * p.TW - p.HX;
    const int steps = 1 + 2 * (run.q + (pass < run.r ? 1 : 0));
    const bool fwd = (pass & 1) == 0;
    const bool ring_tile = (gy0 < p.ring) || (gy0 + LH > p.H - p.ring) || (gx0 < p.ring) || (gx0 + LW > p.W - p.ring);
    const bool stage_dst = ring_tile && steps >= 2;
    int ok = 1;
    if (tid < 32) {
      if (pass > 0) {
        // the lanes of warp 0 wait for one neighbour tile each, so the
        // acquire loads' round trips overlap instead of adding up
        const int y0 = max(0, ty - dy), x0 = max(0, tx - dx);
        const int nx = min(p.tiles_x - 1, tx + dx) - x0 + 1;
        const int nn = (min(p.tiles_y - 1, ty + dy) - y0 + 1) * nx;
        for (int i = tid; i < nn && ok; i += 32) {
          const unsigned* d = &run.done[(y0 + i / nx) * p.tiles_x + x0 + i % nx];
          unsigned polls = 0;
          while (ld_acquire_gpu(d) < static_cast<unsigned>(pass)) {
            if (error_latched(p.err)) {  // another CTA gave up and reported why
              ok = 0;
              break;
            }
            if (++polls >= run.spin_limit) {
              atomicOr(p.err, kDevErrBarrier);
              ok = 0;
              break;
            }
            __nanosleep(32);
          }
        }
        ok = __all_sync(0xFFFFFFFFu, ok);
        __syncwarp();  // orders every lane's acquire before lane 0's load below
      }
      if (ok && tid == 0) {
        // the previous pass wrote through the generic proxy, TMA reads through
        // the async proxy; the buffers were last read by this CTA's threads
        fence_proxy_async_global();
        fence_proxy_async();
        mbar_arrive_expect_tx(&bars[0], kTileBytes);
        tma_load_2d(buf0, fwd ? &map_in : &map_out, gx0, gy0, &bars[0]);
        if (stage_dst) {
          mbar_arrive_expect_tx(&bars[1], kTileBytes);
          tma_load_2d(buf1, fwd ? &map_out : &map_in, gx0, gy0, &bars[1]);
        }
        ok = mbar_wait_bounded(&bars[0], phase_bits & 1u, p.err) ? 1 : 0;
        if (ok && stage_dst) ok = mbar_wait_bounded(&bars[1], (phase_bits >> 1) & 1u, p.err) ? 1 : 0;
      }
    }
    if (!__syncthreads_and(ok)) break;
    phase_bits ^= 1u;
    if (stage_dst) phase_bits ^= 2u;

    TileGeom g;
    g.W = p.W;
    g.H = p.H;
    g.ring = p.ring;
    g.steps = steps;
    g.TW = p.TW;
    g.TH = p.TH;
    g.HX = p.HX;
    g.HY = p.HY;
    g.pitch = p.pitch;
    g.K = p.K;
    g.dt = p.dt;
    g.inv_dx = p.inv_dx;
    g.u = p.u;
    g.v = p.v;
    TS* dst = static_cast<TS*>(fwd ? p.dst : const_cast<void*>(p.src));
    fast2d_run_tile<TS, OpK, S>(buf0, buf1, dst, g, gy0, gx0, ring_tile, wt, neg_zero2(p.fuse_guard));
    // the block's write-back is ordered before thread 0's release by the
    // barrier; one gpu-scope fence then publishes all of it
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      fence_proxy_async_global();
      atomicAdd(&run.done[tile], 1u);
    }
  }
}

// CTAs of `kern` that fit on the current device at once; cached per device
// in `cache` (one array per kernel instantiation; threads that race both
// compute the same value).
constexpr int kMaxCachedDevices = 64;
template <class Kern>
int resident_ctas(Kern kern, size_t smem, std::atomic<int>* cache) {
  int dev = 0;
  cudaGetDevice(&dev);
  const bool cached = dev >= 0 && dev < kMaxCachedDevices;
  if (cached) {
    const int v = cache[dev].load(std::memory_order_relaxed);
    if (v > 0) return v;
  }
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFastThreads, smem);
  const int v = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  if (cached) cache[dev].store(v, std::memory_order_relaxed);
  return v;
}

template <class TS, int OpK, int S>
cudaError_t launch_multipass(const CUtensorMap* mi, const CUtensorMap* mo, const Stencil2DParams& p,
                             const Fast2DRun& run, int ctas, cudaStream_t s) {
  const size_t smem = fast2d_multipass_smem_bytes(sizeof(TS) == 2 ? 2 : 1, S);
  auto kern = fast2d_multipass_kernel<TS, OpK, S>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  // every CTA resident (items are taken only by running CTAs, so this is for
  // speed, not for progress)
  static std::atomic<int> resident_by_device[kMaxCachedDevices];
  const int resident = resident_ctas(kern, smem, resident_by_device);
  if (ctas > resident) ctas = resident;
  kern<<<ctas, kFastThreads, smem, s>>>(*mi, *mo, p, run);
  return cudaGetLastError();
}

template <class TS, int S>
cudaError_t dispatch_multipass(int opk, const CUtensorMap* mi, const CUtensorMap* mo, const Stencil2DParams& p,
                               const Fast2DRun& run, int ctas, cudaStream_t s) {
  switch (opk) {
    case 0: return launch_multipass<TS, 0, S>(mi, mo, p, run, ctas, s);
    case 1: return launch_multipass<TS, 1, S>(mi, mo, p, run, ctas, s);
    case 2: return launch_multipass<TS, 2, S>(mi, mo, p, run, ctas, s);
    default: return launch_multipass<TS, 3, S>(mi, mo, p, run, ctas, s);
  }
}

template <class TS, int OpK, int S>
cudaError_t launch_fast(const CUtensorMap* ms, const CUtensorMap* md, const CUtensorMap* mu, const CUtensorMap* mv,
                        const Stencil2DParams& p, int ctas, cudaStream_t s) {
  const size_t smem = fast2d_smem_bytes(OpK == 3, sizeof(TS) == 2 ? 2 : 1, S);
  auto kern = fast2d_kernel<TS, OpK, S>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  // persistent CTAs: no more than can be resident (registers or shared memory)
  static std::atomic<int> resident_by_device[kMaxCachedDevices];
  const int resident = resident_ctas(kern, smem, resident_by_device);
  if (ctas > resident) ctas = resident;
  kern<<<ctas, kFastThreads, smem, s>>>(*ms, *md, *mu, *mv, p);
  return cudaGetLastError();
}

template <class TS, int S>
cudaError_t dispatch_op(int opk, const CUtensorMap* ms, const CUtensorMap* md, const CUtensorMap* mu,
                        const CUtensorMap* mv, const Stencil2DParams& p, int ctas, cudaStream_t s) {
  switch (opk) {
    case 0: return launch_fast<TS, 0, S>(ms, md, mu, mv, p, ctas, s);
    case 1: return launch_fast<TS, 1, S>(ms, md, mu, mv, p, ctas, s);
    case 2: return launch_fast<TS, 2, S>(ms, md, mu, mv, p, ctas, s);
    default: return launch_fast<TS, 3, S>(ms, md, mu, mv, p, ctas, s);
  }
}

}  // namespace

int fast2d_shape(const int* offsets, int n) {
  for (int k = 0; k < 3; ++k) {
    int sn = 0;
    const int* dh = nullptr;
    const int* dw = nullptr;
    static const int j_dh[4] = {-1, 1, 0, 0}, j_dw[4] = {0, 0, -1, 1};
    static const int c_dh[5] = {0, -1, 1, 0, 0}, c_dw[5] = {0, 0, 0, -1, 1};
    static const int b_dh[9] = {-1, -1, -1, 0, 0, 0, 1, 1, 1}, b_dw[9] = {-1, 0, 1, -1, 0, 1, -1, 0, 1};
    if (k == 0) { sn = 4; dh = j_dh; dw = j_dw; }
    if (k == 1) { sn = 5; dh = c_dh; dw = c_dw; }
    if (k == 2) { sn = 9; dh = b_dh; dw = b_dw; }
    if (sn != n) continue;
    bool same = true;
    for (int i = 0; i < n && same; ++i) same = offsets[2 * i] == dh[i] && offsets[2 * i + 1] == dw[i];
    if (same) return k;
  }
  return -1;
}

size_t fast2d_smem_bytes(bool advect, int dtype, int S) {
  (void)advect;
  const size_t esz = (dtype == 2) ? 2 : 4;
  const size_t lw = 128;
  const size_t lh = 16 * S + 2;
  const size_t buf = (lw * lh * esz + 127) & ~size_t(127);
  return 128 + kFastBufs * buf + 8 * kFastBufs;
}

int fast2d_max_ctas_per_sm(bool advect, int dtype, int S) {
  const size_t smem = fast2d_smem_bytes(advect, dtype, S);
  int dev = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  const int by_smem = static_cast<int>(per_sm / (smem + 1024));
  return by_smem < 8 ? by_smem : 8;
}

size_t fast2d_multipass_smem_bytes(int dtype, int S) {
  const size_t esz = (dtype == 2) ? 2 : 4;
  const size_t buf = (static_cast<size_t>(128) * (16 * S + 2) * esz + 127) & ~size_t(127);
  return 128 + 2 * buf + 16;
}

size_t fast2d_multipass_sync_bytes(int ntiles) { return 16 + 4 * static_cast<size_t>(ntiles); }

DepWaitTest& dep_wait_test() {
  thread_local DepWaitTest t{0u, 0};
  return t;
}

cudaError_t fast2d_multipass(int opk, int dtype, int S, const CUtensorMap* map_in, const CUtensorMap* map_out,
                             const Stencil2DParams& p, int npasses, int q, int r, void* sync, int ctas,
                             cudaStream_t s) {
  const int ntiles = p.tiles_x * p.tiles_y;
  cudaError_t e = cudaMemsetAsync(sync, 0, fast2d_multipass_sync_bytes(ntiles), s);
  if (e != cudaSuccess) return e;
  Fast2DRun run;
  run.npasses = npasses;
  run.q = q;
  run.r = r;
  run.next_item = static_cast<unsigned long long*>(sync);
  run.done = reinterpret_cast<unsigned*>(static_cast<char*>(sync) + 16);
  const DepWaitTest& t = dep_wait_test();
  run.first_item = static_cast<long long>(t.skip_passes) * ntiles;
  run.spin_limit = t.spin_limit ? t.spin_limit : kFastSpinLimit;
  if (dtype == 2)
    return S == 8 ? dispatch_multipass<__nv_bfloat16, 8>(opk, map_in, map_out, p, run, ctas, s)
                  : dispatch_multipass<__nv_bfloat16, 4>(opk, map_in, map_out, p, run, ctas, s);
  return S == 8 ? dispatch_multipass<float, 8>(opk, map_in, map_out, p, run, ctas, s)
                : dispatch_multipass<float, 4>(opk, map_in, map_out, p, run, ctas, s);
}

cudaError_t fast2d_pass(int opk, int dtype, int S, const CUtensorMap* ms, const CUtensorMap* md,
                        const CUtensorMap* mu, const CUtensorMap* mv, const Stencil2DParams& p, int ctas,
                        cudaStream_t s) {
  if (dtype == 2)
    return S == 8 ? dispatch_op<__nv_bfloat16, 8>(opk, ms, md, mu, mv, p, ctas, s)
                  : dispatch_op<__nv_bfloat16, 4>(opk, ms, md, mu, mv, p, ctas, s);
  return S == 8 ? dispatch_op<float, 8>(opk, ms, md, mu, mv, p, ctas, s)
                : dispatch_op<float, 4>(opk, ms, md, mu, mv, p, ctas, s);
}

}  // namespace pskel
