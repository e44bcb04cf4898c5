// Out-of-core iterative stencils: grids that live in host memory (Grace
// LPDDR behind NVLink-C2C) and are streamed through the GPU in slabs.
//
// Replaces the host tiling of StencilBase::runIterativeTilingGPU /
// runTilingGPU / runAutoGPU (PSkelStencil.hpp:766-861, 1663-1760 of the
// reference, tile geometry in PSkelStencilTiling.h:75-140): the grid is cut
// into tiles, each tile is copied to the device with a halo wide enough for
// `innerIterations` steps, iterated there, and its core copied back; the
// outer loop ping-pongs between two host arrays.
//
// Here the tiles are full-width row slabs (whole h-planes in 3D): one slab is
// one contiguous host range, so every copy is a single large DMA over C2C.
// Three device slots rotate through H2D copy, compute and D2H copy on three
// streams, so the copy engines (both directions) and the SMs work on three
// consecutive slabs at once. A slab of the next pass waits only for the
// write-backs of the slabs its rows come from.
//
// Each visit runs `T` steps on a sub-grid of the slab's rows plus a halo.
// The sub-grid's edge rows that are not grid edges hold stale values (2D: the
// sub-grid's ring is never written; 3D: the sub-grid's outside reads the mask
// halo value), and the error spreads by the mask reach R per step, so after T
// steps it covers ring + (T-1)·R rows in 2D and T·R planes in 3D: those are
// the halo widths, and the core rows come back exact.
//
// 2D ring semantics (each array keeps its own ring, the result sits in the
// output array for odd iteration counts and in the input array for even ones)
// are kept by giving every pass an odd length (pskel_plan_passes) and by
// mapping the two logical arrays of the step-by-step run onto two physical
// host arrays so that the last pass writes `out_host`: the physical array
// standing for a logical one carries that array's ring. The ring columns of
// both logical arrays are kept on the device for the whole run and scattered
// into each slab's destination buffer by device copies.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "capi_internal.h"

namespace pskel {

pskel_status validate2d(const pskel_stencil* st, const void* in, const void* out, int64_t W, int64_t H, int64_t pitch,
                        int64_t iters, int* R, int* ring);

namespace {

constexpr int kSlots = 3;
constexpr int32_t kDefaultInner = 15;

size_t dtype_bytes(pskel_dtype t) { return t == PSKEL_U8 ? 1 : (t == PSKEL_BF16 ? 2 : 4); }

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// A host range pinned for the duration of a call when the caller passed
// pageable memory; a range that cannot be registered (overlapping an already
// registered range, read-only mapping) is copied through the driver's staging
// path instead, which is slower but gives the same bytes.
struct HostPin {
  void* ptr = nullptr;
  bool registered = false;
  void pin(const void* p, size_t bytes) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) == cudaSuccess && a.type != cudaMemoryTypeUnregistered) return;
    cudaGetLastError();
    if (cudaHostRegister(const_cast<void*>(p), bytes, cudaHostRegisterDefault) == cudaSuccess) {
      ptr = const_cast<void*>(p);
      registered = true;
    } else {
      cudaGetLastError();
    }
  }
  ~HostPin() {
    if (registered) cudaHostUnregister(ptr);
  }
};

struct Streams {
  cudaStream_t s[3] = {nullptr, nullptr, nullptr};  // H2D, compute, D2H
  std::vector<cudaEvent_t> ev;
  cudaError_t create() {
    for (auto& x : s) {
      cudaError_t e = cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  cudaError_t event(cudaEvent_t* out) {
    cudaError_t e = cudaEventCreateWithFlags(out, cudaEventDisableTiming);
    if (e == cudaSuccess) ev.push_back(*out);
    return e;
  }
  ~Streams() {
    for (auto& x : s)
      if (x) cudaStreamSynchronize(x);
    for (auto e : ev) cudaEventDestroy(e);
    for (auto& x : s)
      if (x) cudaStreamDestroy(x);
  }
};

struct DeviceAlloc {
  void* ptr = nullptr;
  ~DeviceAlloc() {
    if (ptr) cudaFree(ptr);
  }
};

struct PinnedAlloc {
  void* ptr = nullptr;
  ~PinnedAlloc() {
    if (ptr) cudaFreeHost(ptr);
  }
};

// One run's geometry: rows are h-rows (2D) or h-planes (3D).
struct Plan {
  int dims = 2;
  int64_t W = 0, H = 0, D = 1;
  size_t esz = 0;
  size_t host_row = 0;  // bytes of one row on the host (contiguous)
  size_t dev_row = 0;   // bytes of one row on the device (2D: 128-byte pitch)
  int ring = 0, R = 0;  // 2D ring (mask range) and reach
  int fields = 2;       // device buffers per slot: grid pair, plus winds
  std::vector<int> passes;
  int64_t halo = 0;     // widest halo (rows), from the longest pass
  int64_t slab = 0;     // core rows per slab
  int64_t slabs = 0;
  size_t slot_bytes = 0;
  size_t ringcol_bytes = 0;  // 2D: ring columns of one logical array
  size_t device_bytes = 0;
};

int64_t halo_rows(const Plan& p, int T) {
  return p.dims == 2 ? p.ring + static_cast<int64_t>(T - 1) * p.R : static_cast<int64_t>(T) * p.R;
}

pskel_status make_plan(Plan& p, int64_t iterations, int64_t slab_rows, int32_t inner, int64_t device_bytes) {
  if (inner < 0) return fail(PSKEL_ERR_INVALID, "negative inner iteration count");
  if (slab_rows < 0) return fail(PSKEL_ERR_INVALID, "negative slab height");
  if (device_bytes < 0) return fail(PSKEL_ERR_INVALID, "negative device budget");
  const int T = inner > 0 ? inner : kDefaultInner;
  if (iterations > 0) {
    const int n = pskel_plan_passes(iterations, T, nullptr, 0);
    p.passes.resize(static_cast<size_t>(n));
    pskel_plan_passes(iterations, T, p.passes.data(), n);
  }
  int Tmax = 1;
  for (int t : p.passes) Tmax = std::max(Tmax, t);
  p.halo = halo_rows(p, Tmax);
  p.ringcol_bytes = (p.dims == 2) ? static_cast<size_t>(p.H) * 2 * p.ring * p.esz : 0;
  // Device memory besides the slots: ring columns of both logical arrays, and
  // for Life the two bit planes and the pass counters of one sub-grid (about
  // a quarter byte per cell).
  const size_t fixed = 2 * p.ringcol_bytes + (1 << 20);
  const size_t per_row = static_cast<size_t>(kSlots) * p.fields * p.dev_row + (p.dims == 2 ? p.W / 4 + 64 : 0);
  int64_t S = slab_rows;
  if (S == 0) {
    size_t budget = static_cast<size_t>(device_bytes);
    if (budget == 0) {
      size_t fr = 0, tot = 0;
      cudaError_t e = cudaMemGetInfo(&fr, &tot);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemGetInfo");
      budget = fr / 10 * 9;
    }
    if (budget <= fixed) return fail(PSKEL_ERR_NOMEM, "device budget %zu bytes is below the fixed need", budget);
    const int64_t rows = static_cast<int64_t>((budget - fixed) / per_row);
    S = rows - 2 * p.halo;
    if (S < 1)
      return fail(PSKEL_ERR_NOMEM,
                  "device budget %zu bytes holds %lld rows per slot, fewer than a halo of %lld rows on each side",
                  budget, (long long)rows, (long long)p.halo);
  }
  S = std::min<int64_t>(S, p.H);
  p.slab = S;
  p.slabs = (p.H + S - 1) / S;
  const int64_t sub_max = std::min<int64_t>(p.H, S + 2 * p.halo);
  p.slot_bytes = align_up(static_cast<size_t>(sub_max) * p.dev_row, 256);
  p.device_bytes = static_cast<size_t>(kSlots) * p.fields * p.slot_bytes + 2 * p.ringcol_bytes;
  return PSKEL_OK;
}

// Copies `rows` rows of `row_bytes` from a host range into device rows of
// pitch `dpitch` (or back).
cudaError_t rows_h2d(void* d, size_t dpitch, const void* h, size_t row_bytes, int64_t rows, cudaStream_t s) {
  if (rows <= 0) return cudaSuccess;
  if (dpitch == row_bytes)
    return cudaMemcpyAsync(d, h, row_bytes * static_cast<size_t>(rows), cudaMemcpyHostToDevice, s);
  return cudaMemcpy2DAsync(d, dpitch, h, row_bytes, row_bytes, static_cast<size_t>(rows), cudaMemcpyHostToDevice, s);
}

cudaError_t rows_d2h(void* h, size_t row_bytes, const void* d, size_t dpitch, int64_t rows, cudaStream_t s) {
  if (rows <= 0) return cudaSuccess;
  if (dpitch == row_bytes)
    return cudaMemcpyAsync(h, d, row_bytes * static_cast<size_t>(rows), cudaMemcpyDeviceToHost, s);
  return cudaMemcpy2DAsync(h, row_bytes, d, dpitch, row_bytes, static_cast<size_t>(rows), cudaMemcpyDeviceToHost, s);
}

// Host copy of the 2D ring cells (rows [0,r) and [H-r,H), columns [0,r) and
// [W-r,W) of the rows between) from `src` to `dst`.
void copy_ring_host(uint8_t* dst, const uint8_t* src, const Plan& p) {
  const int64_t r = p.ring;
  if (r == 0) return;
  const size_t row = p.host_row;
  const int64_t top = std::min<int64_t>(r, p.H);
  std::memcpy(dst, src, row * static_cast<size_t>(top));
  const int64_t bot0 = std::max<int64_t>(p.H - r, top);
  std::memcpy(dst + row * bot0, src + row * bot0, row * static_cast<size_t>(p.H - bot0));
  const size_t cw = static_cast<size_t>(std::min<int64_t>(r, p.W)) * p.esz;
  const size_t off = static_cast<size_t>(p.W - std::min<int64_t>(r, p.W)) * p.esz;
  for (int64_t y = top; y < bot0; ++y) {
    std::memcpy(dst + row * y, src + row * y, cw);
    std::memcpy(dst + row * y + off, src + row * y + off, cw);
  }
}

struct Run {
  Plan p;
  pskel_stencil st;
  const pskel_schedule* sched = nullptr;
  const uint8_t* in = nullptr;  // in_host
  uint8_t* out = nullptr;       // out_host
  uint8_t* scratch = nullptr;   // second physical array (pinned)
  uint8_t* dev = nullptr;       // slots, then ring columns
  DeviceContext* c = nullptr;
};

uint8_t* slot_buf(const Run& r, int slot, int field) {
  return r.dev + (static_cast<size_t>(slot) * r.p.fields + field) * r.p.slot_bytes;
}

uint8_t* ringcols(const Run& r, int logical) {
  return r.dev + static_cast<size_t>(kSlots) * r.p.fields * r.p.slot_bytes + logical * r.p.ringcol_bytes;
}

pskel_status run_slabs(Run& r) {
  const Plan& p = r.p;
  const int P = static_cast<int>(p.passes.size());
  Streams ss;
  cudaError_t e = ss.create();
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
  cudaStream_t s_in = ss.s[0], s_comp = ss.s[1], s_out = ss.s[2];
  cudaEvent_t ev_in[kSlots], ev_comp[kSlots], ev_free[kSlots];
  for (int i = 0; i < kSlots; ++i) {
    if ((e = ss.event(&ev_in[i])) != cudaSuccess || (e = ss.event(&ev_comp[i])) != cudaSuccess ||
        (e = ss.event(&ev_free[i])) != cudaSuccess)
      return cuda_fail(e, "cudaEventCreate");
  }
  // ev_done[j % 2][k]: slab k of pass j written back to the host
  std::vector<cudaEvent_t> ev_done[2];
  for (auto& v : ev_done) {
    v.resize(static_cast<size_t>(p.slabs));
    for (auto& x : v)
      if ((e = ss.event(&x)) != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
  }
  std::vector<bool> slot_used(kSlots, false);

  // Ring columns of both logical arrays on the device (2D): logical 0 is the
  // input array, 1 the output array.
  if (p.dims == 2 && p.ring > 0) {
    const size_t cw = static_cast<size_t>(p.ring) * p.esz;
    for (int L = 0; L < 2; ++L) {
      const uint8_t* src = (L == 0) ? r.in : r.out;
      uint8_t* d = ringcols(r, L);
      e = cudaMemcpy2DAsync(d, 2 * cw, src, p.host_row, cw, static_cast<size_t>(p.H), cudaMemcpyHostToDevice, s_in);
      if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(d + cw, 2 * cw, src + (p.W - p.ring) * p.esz, p.host_row, cw,
                              static_cast<size_t>(p.H), cudaMemcpyHostToDevice, s_in);
      if (e != cudaSuccess) return cuda_fail(e, "copy ring columns to device");
    }
    // The physical arrays take the rings of the logical arrays they stand for:
    // out_host stands for the array holding the result (the output array for
    // an odd count), the scratch array for the other one.
    if (cudaStreamSynchronize(s_in) != cudaSuccess) return cuda_fail(cudaGetLastError(), "ring column copy");
    const bool final_is_out = (P % 2 == 1);
    if (P >= 2) copy_ring_host(r.scratch, final_is_out ? r.in : r.out, p);
    if (!final_is_out) copy_ring_host(r.out, r.in, p);
  }

  int64_t visit = 0;
  for (int j = 0; j < P; ++j) {
    const int T = p.passes[static_cast<size_t>(j)];
    const int64_t halo = halo_rows(p, T);
    const bool dst_is_out = ((P - 1 - j) % 2 == 0);
    uint8_t* dst = dst_is_out ? r.out : r.scratch;
    const uint8_t* src = (j == 0) ? r.in : (dst_is_out ? r.scratch : r.out);
    const int logical_dst = (j % 2 == 0) ? 1 : 0;
    for (int64_t k = 0; k < p.slabs; ++k, ++visit) {
      const int slot = static_cast<int>(visit % kSlots);
      const int64_t y0 = k * p.slab, y1 = std::min(p.H, y0 + p.slab);
      const int64_t a = std::max<int64_t>(0, y0 - halo), b = std::min<int64_t>(p.H, y1 + halo);
      const int64_t hs = b - a;
      uint8_t* dA = slot_buf(r, slot, 0);
      uint8_t* dB = slot_buf(r, slot, 1);
      // H2D: the slot is free once its previous slab was written back, and the
      // source rows are final once the previous pass wrote them back.
      if (slot_used[slot] && (e = cudaStreamWaitEvent(s_in, ev_free[slot], 0)) != cudaSuccess)
        return cuda_fail(e, "cudaStreamWaitEvent");
      if (j > 0) {
        const int64_t klast = std::min<int64_t>(p.slabs - 1, (b - 1) / p.slab);
        if ((e = cudaStreamWaitEvent(s_in, ev_done[(j - 1) % 2][klast], 0)) != cudaSuccess)
          return cuda_fail(e, "cudaStreamWaitEvent");
      }
      e = rows_h2d(dA, p.dev_row, src + p.host_row * a, p.host_row, hs, s_in);
      if (e == cudaSuccess && p.dims == 2 && p.ring > 0) {
        const int64_t rr = std::min<int64_t>(p.ring, hs);
        // sub-grid ring rows: the destination array's own ring rows at a grid
        // edge, any valid state (the source rows) elsewhere
        e = rows_h2d(dB, p.dev_row, (a == 0 ? dst : src) + p.host_row * a, p.host_row, rr, s_in);
        if (e == cudaSuccess)
          e = rows_h2d(dB + p.dev_row * (hs - rr), p.dev_row, (b == p.H ? dst : src) + p.host_row * (b - rr),
                       p.host_row, rr, s_in);
        const int64_t mid = hs - 2 * p.ring;
        if (e == cudaSuccess && mid > 0) {
          const size_t cw = static_cast<size_t>(p.ring) * p.esz;
          const uint8_t* rc = ringcols(r, logical_dst) + static_cast<size_t>(a + p.ring) * 2 * cw;
          e = cudaMemcpy2DAsync(dB + p.dev_row * p.ring, p.dev_row, rc, 2 * cw, cw, static_cast<size_t>(mid),
                                cudaMemcpyDeviceToDevice, s_in);
          if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(dB + p.dev_row * p.ring + (p.W - p.ring) * p.esz, p.dev_row, rc + cw, 2 * cw, cw,
                                  static_cast<size_t>(mid), cudaMemcpyDeviceToDevice, s_in);
        }
      }
      pskel_stencil sub = r.st;
      if (e == cudaSuccess && p.dims == 2 && r.st.op == PSKEL_OP_ADVECT) {
        uint8_t* dU = slot_buf(r, slot, 2);
        uint8_t* dV = slot_buf(r, slot, 3);
        e = rows_h2d(dU, p.dev_row, static_cast<const uint8_t*>(r.st.wind_u) + p.host_row * a, p.host_row, hs, s_in);
        if (e == cudaSuccess)
          e = rows_h2d(dV, p.dev_row, static_cast<const uint8_t*>(r.st.wind_v) + p.host_row * a, p.host_row, hs,
                       s_in);
        sub.wind_u = dU;
        sub.wind_v = dV;
      }
      if (e != cudaSuccess) return cuda_fail(e, "copy slab to device");
      if ((e = cudaEventRecord(ev_in[slot], s_in)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");

      // compute
      if ((e = cudaStreamWaitEvent(s_comp, ev_in[slot], 0)) != cudaSuccess) return cuda_fail(e, "cudaStreamWaitEvent");
      pskel_status q;
      if (p.dims == 2)
        q = pskel_iterate2d(&sub, dA, dB, p.W, hs, static_cast<int64_t>(p.dev_row / p.esz), T, r.sched, s_comp);
      else
        q = pskel_iterate3d(&sub, dA, dB, p.W, hs, p.D, T, r.sched, 0, nullptr, s_comp);
      if (q != PSKEL_OK) return q;
      if ((e = cudaEventRecord(ev_comp[slot], s_comp)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");

      // D2H of the core rows
      if ((e = cudaStreamWaitEvent(s_out, ev_comp[slot], 0)) != cudaSuccess)
        return cuda_fail(e, "cudaStreamWaitEvent");
      const uint8_t* res = (T % 2 == 1) ? dB : dA;
      e = rows_d2h(dst + p.host_row * y0, p.host_row, res + p.dev_row * (y0 - a), p.dev_row, y1 - y0, s_out);
      if (e != cudaSuccess) return cuda_fail(e, "copy slab to host");
      if ((e = cudaEventRecord(ev_free[slot], s_out)) != cudaSuccess ||
          (e = cudaEventRecord(ev_done[j % 2][k], s_out)) != cudaSuccess)
        return cuda_fail(e, "cudaEventRecord");
      slot_used[slot] = true;
    }
  }
  return device_sync_check(r.c, s_out);
}

pskel_status run_tiled(Run& r, int64_t iterations, int64_t slab_rows, int32_t inner, int64_t device_bytes) {
  Plan& p = r.p;
  if (pskel_status s = get_context(&r.c)) return s;
  if (iterations == 0) {
    std::memcpy(r.out, r.in, p.host_row * static_cast<size_t>(p.H));
    return PSKEL_OK;
  }
  if (pskel_status s = make_plan(p, iterations, slab_rows, inner, device_bytes)) return s;
  const size_t grid_bytes = p.host_row * static_cast<size_t>(p.H);
  HostPin pin_in, pin_out, pin_u, pin_v;
  pin_in.pin(r.in, grid_bytes);
  pin_out.pin(r.out, grid_bytes);
  if (p.fields == 4) {
    pin_u.pin(r.st.wind_u, grid_bytes);
    pin_v.pin(r.st.wind_v, grid_bytes);
  }
  PinnedAlloc scratch;
  if (p.passes.size() >= 2) {
    cudaError_t e = cudaMallocHost(&scratch.ptr, grid_bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMallocHost(out-of-core scratch array)");
    r.scratch = static_cast<uint8_t*>(scratch.ptr);
  }
  DeviceAlloc dev;
  cudaError_t e = cudaMalloc(&dev.ptr, p.device_bytes);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(out-of-core slots)");
  r.dev = static_cast<uint8_t*>(dev.ptr);
  pskel_status s = run_slabs(r);
  cudaDeviceSynchronize();  // nothing in flight may touch the buffers freed below
  return s;
}

pskel_status fill_plan2d(const pskel_stencil* st, int64_t W, int64_t H, Plan& p) {
  int R = 0, ring = 0;
  // validate2d wants distinct non-null pointers; the host arrays are checked
  // by the callers
  static const char dummy[2] = {0, 0};
  if (pskel_status s = validate2d(st, &dummy[0], &dummy[1], W, H, W, 0, &R, &ring)) return s;
  p.dims = 2;
  p.W = W;
  p.H = H;
  p.D = 1;
  p.esz = dtype_bytes(st->dtype);
  p.host_row = static_cast<size_t>(W) * p.esz;
  p.dev_row = align_up(p.host_row, 128);
  p.ring = ring;
  p.R = R;
  p.fields = (st->op == PSKEL_OP_ADVECT) ? 4 : 2;
  return PSKEL_OK;
}

pskel_status fill_plan3d(const pskel_stencil* st, int64_t W, int64_t H, int64_t D, Plan& p) {
  int R = 0;
  static const char dummy[2] = {0, 0};
  if (pskel_status s = validate3d(st, &dummy[0], &dummy[1], W, H, D, 0, 0, &R)) return s;
  p.dims = 3;
  p.W = W;
  p.H = H;
  p.D = D;
  p.esz = dtype_bytes(st->dtype);
  p.host_row = static_cast<size_t>(W) * D * p.esz;
  p.dev_row = p.host_row;
  p.ring = 0;
  p.R = R;
  p.fields = 2;
  return PSKEL_OK;
}

}  // namespace
}  // namespace pskel

using namespace pskel;

extern "C" {

pskel_status pskel_run2d_host_tiled(const pskel_stencil* st, const void* in_host, void* out_host, int64_t width,
                                    int64_t height, int64_t iterations, int64_t slab_rows, int32_t inner_iterations,
                                    int64_t device_bytes, const pskel_schedule* sched) {
  clear_error();
  if (!in_host || !out_host) return fail(PSKEL_ERR_INVALID, "host array pointer is NULL");
  if (in_host == out_host) return fail(PSKEL_ERR_INVALID, "input and output must be distinct arrays");
  if (iterations < 0) return fail(PSKEL_ERR_INVALID, "negative iteration count");
  Run r;
  if (pskel_status s = fill_plan2d(st, width, height, r.p)) return s;
  r.st = *st;
  r.sched = sched;
  r.in = static_cast<const uint8_t*>(in_host);
  r.out = static_cast<uint8_t*>(out_host);
  return run_tiled(r, iterations, slab_rows, inner_iterations, device_bytes);
}

pskel_status pskel_run3d_host_tiled(const pskel_stencil* st, const void* in_host, void* out_host, int64_t width,
                                    int64_t height, int64_t depth, int64_t iterations, int64_t slab_planes,
                                    int32_t inner_iterations, int64_t device_bytes, const pskel_schedule* sched) {
  clear_error();
  if (!in_host || !out_host) return fail(PSKEL_ERR_INVALID, "host array pointer is NULL");
  if (in_host == out_host) return fail(PSKEL_ERR_INVALID, "input and output must be distinct arrays");
  if (iterations < 0) return fail(PSKEL_ERR_INVALID, "negative iteration count");
  Run r;
  if (pskel_status s = fill_plan3d(st, width, height, depth, r.p)) return s;
  r.st = *st;
  r.sched = sched;
  r.in = static_cast<const uint8_t*>(in_host);
  r.out = static_cast<uint8_t*>(out_host);
  return run_tiled(r, iterations, slab_planes, inner_iterations, device_bytes);
}

pskel_status pskel_tiled_plan(const pskel_stencil* st, int64_t width, int64_t height, int64_t depth,
                              int64_t iterations, int64_t slab_rows, int32_t inner_iterations, int64_t device_bytes,
                              int64_t plan[4]) {
  clear_error();
  if (!plan) return fail(PSKEL_ERR_INVALID, "plan output pointer is NULL");
  if (iterations < 0) return fail(PSKEL_ERR_INVALID, "negative iteration count");
  if (!st) return fail(PSKEL_ERR_INVALID, "stencil descriptor is NULL");
  Plan p;
  pskel_status s = (st->mask.dimension == 3) ? fill_plan3d(st, width, height, depth, p)
                                             : fill_plan2d(st, width, height, p);
  if (s != PSKEL_OK) return s;
  if (pskel_status q = make_plan(p, iterations > 0 ? iterations : 1, slab_rows, inner_iterations, device_bytes))
    return q;
  plan[0] = p.slab;
  plan[1] = p.halo;
  plan[2] = p.slabs;
  plan[3] = static_cast<int64_t>(p.device_bytes);
  return PSKEL_OK;
}

}  // extern "C"
