// Batched iterative 2D stencils: many grids of different sizes, iteration
// counts and temporal blocks in ONE persistent launch, captured once in a
// CUDA graph and replayed.
//
// Work items are (grid, pass, tile). They are enumerated in rounds: round r
// holds every tile of pass r of every grid that has a pass r, grids in input
// order. Resident CTAs (never more than can be co-resident) take items in
// that order from a global counter. Before working on a tile of pass r > 0 a
// CTA waits until all tiles of pass r-1 of the same grid have been written
// (a per-grid completion counter); every such tile was taken earlier by a
// resident CTA, so the wait always ends. It is still bounded: after
// kBatchSpinLimit polls the CTA latches kDevErrBarrier and stops, and every
// other CTA stops at its next poll or item once it sees the latched word.
//
// Each tile is processed by the register-windowed tile routine of the
// single-grid kernel (fast2d_tile.cuh): TMA-staged source tile, destination
// tile for ring tiles, T steps in shared memory (in registers for fp32 tiles
// clear of the ring), interior cells written back.
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/pskel_gb300.h"
#include "capi_internal.h"
#include "fast2d_tile.cuh"

namespace pskel {
namespace {

using namespace fast2d;

struct BatchGridDev {
  void* in;
  void* out;
  int64_t pitch;
  int W, H, ring, TW, TH, HX, HY, tiles_x, ntiles;
  int pass_off;  // this grid's pass lengths start at passes[pass_off]
};

struct BatchSeg {
  int64_t start;  // first item of the segment
  int g;          // grid
  int pass;       // pass index within the grid
};

struct BatchParams {
  float wt[9];
  unsigned* err;
  uint32_t fuse_guard;  // always 0: the kernel forms -0.0f from it at run time (neg_zero2)
};

constexpr unsigned kBatchSpinLimit = 1u << 24;  // polls of a completion counter (with a short sleep each)

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}


template <class TS, int OpK, int S>
__global__ void __launch_bounds__(kFastThreads, S <= 4 ? 2 : 1)
    batch2d_kernel(const BatchGridDev* __restrict__ grids, const CUtensorMap* __restrict__ maps,
                   const int* __restrict__ passes, const BatchSeg* __restrict__ segs, int nsegs, int64_t nitems,
                   unsigned long long* next_item, unsigned* done, const __grid_constant__ BatchParams bp) {
  constexpr int N = Vec<TS>::N;
  constexpr int LW = 32 * N;
  constexpr int LH = (kFastThreads / 32) * S + 2;
  constexpr size_t kBuf = (static_cast<size_t>(LW) * LH * sizeof(TS) + 127) & ~size_t(127);
  constexpr uint32_t kTileBytes = static_cast<uint32_t>(LW * LH * sizeof(TS));
  extern __shared__ __align__(128) uint8_t smem_raw[];
  if ((smem_u32(smem_raw) & 127u) != 0) {
    if (threadIdx.x == 0) atomicOr(bp.err, kDevErrAlign);
    return;
  }
  TS* buf0 = reinterpret_cast<TS*>(smem_raw);
  TS* buf1 = reinterpret_cast<TS*>(smem_raw + kBuf);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + 2 * kBuf);
  __shared__ int64_t s_item;
  __shared__ int s_seg;

  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_barrier_init();
  }
  __syncthreads();
  float wt[9];
#pragma unroll
  for (int n = 0; n < 9; ++n) wt[n] = bp.wt[n];
  uint32_t phase_bits = 0;

  for (;;) {
    if (tid == 0) {
      const int64_t item = error_latched(bp.err) ? nitems : static_cast<int64_t>(atomicAdd(next_item, 1ull));
      s_item = item;
      if (item < nitems) {
        int lo = 0, hi = nsegs - 1;  // last segment with start <= item
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (segs[mid].start <= item) lo = mid; else hi = mid - 1;
        }
        s_seg = lo;
      }
    }
    __syncthreads();
    const int64_t item = s_item;
    if (item >= nitems) break;
    const BatchSeg seg = segs[s_seg];
    const BatchGridDev G = grids[seg.g];
    const int tile = static_cast<int>(item - seg.start);
    const int ty = tile / G.tiles_x;
    const int gy0 = ty * G.TH - G.HY;
    const int gx0 = (tile - ty * G.tiles_x) * G.TW - G.HX;
    const int steps = passes[G.pass_off + seg.pass];
    const bool ring_tile = (gy0 < G.ring) || (gy0 + LH > G.H - G.ring) || (gx0 < G.ring) || (gx0 + LW > G.W - G.ring);
    const bool stage_dst = ring_tile && steps >= 2;
    const bool fwd = (seg.pass % 2) == 0;  // even passes read `in`
    int ok = 1;
    if (tid == 0) {
      // every tile of the previous pass of this grid must be written
      if (seg.pass > 0) {
        const unsigned target = static_cast<unsigned>(seg.pass) * static_cast<unsigned>(G.ntiles);
        unsigned polls = 0;
        while (ld_acquire(&done[seg.g]) < target) {
          if (error_latched(bp.err)) {  // another CTA gave up and reported why
            ok = 0;
            break;
          }
          if (++polls >= kBatchSpinLimit) {
            atomicOr(bp.err, kDevErrBarrier);
            ok = 0;
            break;
          }
          __nanosleep(64);
        }
      }
      if (ok) {
        // the previous pass wrote through the generic proxy; TMA reads through the async proxy
        fence_proxy_async_global();
        fence_proxy_async();
        const CUtensorMap* msrc = &maps[2 * seg.g + (fwd ? 0 : 1)];
        const CUtensorMap* mdst = &maps[2 * seg.g + (fwd ? 1 : 0)];
        mbar_arrive_expect_tx(&bars[0], kTileBytes);
        tma_load_2d(buf0, msrc, gx0, gy0, &bars[0]);
        if (stage_dst) {
          mbar_arrive_expect_tx(&bars[1], kTileBytes);
          tma_load_2d(buf1, mdst, gx0, gy0, &bars[1]);
        }
        ok = mbar_wait_bounded(&bars[0], phase_bits & 1u, bp.err) ? 1 : 0;
        if (ok && stage_dst) ok = mbar_wait_bounded(&bars[1], (phase_bits >> 1) & 1u, bp.err) ? 1 : 0;
      }
    }
    if (!__syncthreads_and(ok)) break;
    phase_bits ^= 1u;
    if (stage_dst) phase_bits ^= 2u;

    TileGeom g;
    g.W = G.W;
    g.H = G.H;
    g.ring = G.ring;
    g.steps = steps;
    g.TW = G.TW;
    g.TH = G.TH;
    g.HX = G.HX;
    g.HY = G.HY;
    g.pitch = G.pitch;
    g.K = g.dt = g.inv_dx = 0.0f;
    g.u = g.v = nullptr;
    TS* dst = static_cast<TS*>(fwd ? G.out : G.in);
    fast2d_run_tile<TS, OpK, S>(buf0, buf1, dst, g, gy0, gx0, ring_tile, wt, neg_zero2(bp.fuse_guard));
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      fence_proxy_async_global();
      atomicAdd(&done[seg.g], 1u);
    }
  }
}

constexpr int kBatchS = 4;

template <class TS, int OpK>
void* batch_kernel_ptr() {
  return reinterpret_cast<void*>(batch2d_kernel<TS, OpK, kBatchS>);
}

void* batch_kernel(int dtype, int opk) {
  if (dtype == PSKEL_BF16) {
    switch (opk) {
      case 0: return batch_kernel_ptr<__nv_bfloat16, 0>();
      case 1: return batch_kernel_ptr<__nv_bfloat16, 1>();
      default: return batch_kernel_ptr<__nv_bfloat16, 2>();
    }
  }
  switch (opk) {
    case 0: return batch_kernel_ptr<float, 0>();
    case 1: return batch_kernel_ptr<float, 1>();
    default: return batch_kernel_ptr<float, 2>();
  }
}

}  // namespace
}  // namespace pskel

using namespace pskel;

struct pskel_batch {
  int device = 0;
  int n = 0;
  int ctas = 0;
  size_t smem = 0;
  void* kernel = nullptr;
  BatchGridDev* d_grids = nullptr;
  CUtensorMap* d_maps = nullptr;
  int* d_passes = nullptr;
  BatchSeg* d_segs = nullptr;
  int nsegs = 0;
  int64_t nitems = 0;
  unsigned long long* d_next = nullptr;
  unsigned* d_done = nullptr;
  BatchParams params;
  cudaStream_t capture = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t cell_updates = 0;
};

static void batch_free(pskel_batch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->capture) cudaStreamDestroy(b->capture);
  cudaFree(b->d_grids);
  cudaFree(b->d_maps);
  cudaFree(b->d_passes);
  cudaFree(b->d_segs);
  cudaFree(b->d_next);
  cudaFree(b->d_done);
  delete b;
}

extern "C" {

pskel_status pskel_batch_create(const pskel_stencil* st, const pskel_batch_grid* grids, int32_t n,
                                pskel_batch** out) {
  clear_error();
  if (!st || !grids || !out || n <= 0) return fail(PSKEL_ERR_INVALID, "batch: NULL argument or no grids");
  *out = nullptr;
  if (st->op != PSKEL_OP_LINEAR) return fail(PSKEL_ERR_UNSUPPORTED, "batch: linear mask stencils only");
  if (st->dtype != PSKEL_F32 && st->dtype != PSKEL_BF16)
    return fail(PSKEL_ERR_UNSUPPORTED, "batch: f32 and bf16 storage only");
  int R = 0, ring = 0;
  if (pskel_status s = check_mask(st->mask, 2, true, &R, &ring)) return s;
  const int opk = (R == 1) ? fast2d_shape(st->mask.offsets, st->mask.size) : -1;
  if (opk < 0)
    return fail(PSKEL_ERR_UNSUPPORTED, "batch: the mask must be the N,S,W,E cross, the C,N,S,W,E cross or the 3x3 box");
  DeviceContext* c = nullptr;
  if (pskel_status s = get_context(&c)) return s;
  const int dtype = static_cast<int>(st->dtype);
  const int esz = dtype == PSKEL_BF16 ? 2 : 4;
  const int vec = 16 / esz;
  const int LW = 128, LH = 16 * kBatchS + 2;

  std::vector<BatchGridDev> gd(n);
  std::vector<CUtensorMap> maps(2 * static_cast<size_t>(n));
  std::vector<int> pass_len;
  std::vector<std::vector<int>> plans(n);
  int64_t updates = 0;
  for (int i = 0; i < n; ++i) {
    const pskel_batch_grid& G = grids[i];
    const int64_t pitch = G.pitch ? G.pitch : G.width;
    if (!G.in || !G.out || G.in == G.out) return fail(PSKEL_ERR_INVALID, "batch grid %d: bad buffers", i);
    if (G.width <= 0 || G.height <= 0 || G.width >= (1 << 30) || G.height >= (1 << 30) || pitch < G.width)
      return fail(PSKEL_ERR_INVALID, "batch grid %d: bad shape", i);
    if (G.iterations < 0) return fail(PSKEL_ERR_INVALID, "batch grid %d: negative iterations", i);
    if (G.height < ring || G.width < ring) return fail(PSKEL_ERR_INVALID, "batch grid %d smaller than the mask range", i);
    const int64_t pb = pitch * esz;
    if ((reinterpret_cast<uintptr_t>(G.in) & 15) || (reinterpret_cast<uintptr_t>(G.out) & 15) || (pb & 15))
      return fail(PSKEL_ERR_UNSUPPORTED, "batch grid %d: buffers and row pitch must be 16-byte aligned", i);
    int T = G.schedule.time_steps > 0 ? G.schedule.time_steps : 7;  // the linear shapes' default
    T = static_cast<int>(std::min<int64_t>(T, std::max<int64_t>(G.iterations, 1)));
    if (T > 1 && (T & 1) == 0) --T;
    int HX = 0;
    for (;;) {
      HX = ((T + vec - 1) / vec) * vec;
      if ((LW - 2 * HX >= 4 && LH - 2 * T >= 2) || T == 1) break;
      T -= 2;
    }
    BatchGridDev& d = gd[i];
    d.in = G.in;
    d.out = G.out;
    d.pitch = pitch;
    d.W = static_cast<int>(G.width);
    d.H = static_cast<int>(G.height);
    d.ring = ring;
    d.HX = HX;
    d.HY = T;
    d.TW = LW - 2 * HX;
    d.TH = LH - 2 * T;
    d.tiles_x = (d.W + d.TW - 1) / d.TW;
    d.ntiles = d.tiles_x * ((d.H + d.TH - 1) / d.TH);
    d.pass_off = static_cast<int>(pass_len.size());
    plans[i] = plan_passes(G.iterations, T);
    for (int v : plans[i]) pass_len.push_back(v);
    updates += G.width * G.height * G.iterations;
    const CUtensorMapDataType tt = dtype == PSKEL_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const uint64_t dims[2] = {static_cast<uint64_t>(G.width), static_cast<uint64_t>(G.height)};
    const uint64_t strides[1] = {static_cast<uint64_t>(pb)};
    const uint32_t box[2] = {static_cast<uint32_t>(LW), static_cast<uint32_t>(LH)};
    cudaError_t e = encode_tmap(&maps[2 * i], tt, 2, G.in, dims, strides, box);
    if (e == cudaSuccess) e = encode_tmap(&maps[2 * i + 1], tt, 2, G.out, dims, strides, box);
    if (e != cudaSuccess) return cuda_fail(e, "cuTensorMapEncodeTiled (batch)");
  }
  // rounds: every grid's pass r, in grid order
  std::vector<BatchSeg> segs;
  int64_t start = 0;
  size_t max_passes = 0;
  for (auto& p : plans) max_passes = std::max(max_passes, p.size());
  for (size_t r = 0; r < max_passes; ++r) {
    for (int i = 0; i < n; ++i) {
      if (r >= plans[i].size()) continue;
      BatchSeg sg;
      sg.start = start;
      sg.g = i;
      sg.pass = static_cast<int>(r);
      segs.push_back(sg);
      start += gd[i].ntiles;
    }
  }
  pskel_batch* b = new pskel_batch();
  b->device = c->device;
  b->n = n;
  b->nsegs = static_cast<int>(segs.size());
  b->nitems = start;
  b->cell_updates = updates;
  memset(&b->params, 0, sizeof(b->params));
  for (int k = 0; k < st->mask.size && k < 9; ++k) b->params.wt[k] = st->mask.weights[k];
  b->params.err = c->err;
  b->kernel = batch_kernel(dtype, opk);
  b->smem = 2 * ((static_cast<size_t>(LW) * LH * esz + 127) & ~size_t(127)) + 16;
  cudaError_t e = cudaFuncSetAttribute(b->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(b->smem));
  int per_sm = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, b->kernel, kFastThreads, b->smem);
  // co-residency of every CTA is what makes the dependency waits safe
  b->ctas = std::max(1, per_sm) * c->sms;
  if (b->nitems > 0 && b->ctas > b->nitems) b->ctas = static_cast<int>(b->nitems);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_grids, sizeof(BatchGridDev) * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_maps, sizeof(CUtensorMap) * 2 * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_passes, sizeof(int) * std::max<size_t>(1, pass_len.size()));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_segs, sizeof(BatchSeg) * std::max<size_t>(1, segs.size()));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_next, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_done, sizeof(unsigned) * n);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_grids, gd.data(), sizeof(BatchGridDev) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_maps, maps.data(), sizeof(CUtensorMap) * 2 * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !pass_len.empty())
    e = cudaMemcpy(b->d_passes, pass_len.data(), sizeof(int) * pass_len.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !segs.empty())
    e = cudaMemcpy(b->d_segs, segs.data(), sizeof(BatchSeg) * segs.size(), cudaMemcpyHostToDevice);
  // the whole run is one graph: reset the counters, one persistent launch
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaMemsetAsync(b->d_next, 0, sizeof(unsigned long long), b->capture);
    cudaMemsetAsync(b->d_done, 0, sizeof(unsigned) * n, b->capture);
    if (b->nitems > 0) {
      const BatchGridDev* a0 = b->d_grids;
      const CUtensorMap* a1 = b->d_maps;
      const int* a2 = b->d_passes;
      const BatchSeg* a3 = b->d_segs;
      int a4 = b->nsegs;
      int64_t a5 = b->nitems;
      unsigned long long* a6 = b->d_next;
      unsigned* a7 = b->d_done;
      BatchParams a8 = b->params;
      void* args[] = {&a0, &a1, &a2, &a3, &a4, &a5, &a6, &a7, &a8};
      cudaLaunchKernel(b->kernel, dim3(b->ctas), dim3(kFastThreads), args, b->smem, b->capture);
    }
    e = cudaStreamEndCapture(b->capture, &b->graph);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  if (e != cudaSuccess) {
    batch_free(b);
    return cuda_fail(e, "batch set-up");
  }
  *out = b;
  return PSKEL_OK;
}

pskel_status pskel_batch_run(pskel_batch* b, void* stream) {
  clear_error();
  if (!b) return fail(PSKEL_ERR_INVALID, "batch is NULL");
  cudaError_t e = cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "batch graph launch");
  return PSKEL_OK;
}

int64_t pskel_batch_cell_updates(const pskel_batch* b) { return b ? b->cell_updates : 0; }

pskel_status pskel_batch_destroy(pskel_batch* b) {
  clear_error();
  batch_free(b);
  return PSKEL_OK;
}

}  // extern "C"
