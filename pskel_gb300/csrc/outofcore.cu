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
// Device slots rotate through H2D copy, compute and D2H copy on three streams,
// so both copy directions and the SMs work on consecutive slabs at once.
//
// Each visit runs `T` steps on a sub-grid of the slab's rows plus a halo.
// The sub-grid's edge rows that are not grid edges hold stale values (2D: the
// sub-grid's ring is never written; 3D: the sub-grid's outside reads the mask
// halo value), and the error spreads by the mask reach R per step, so after T
// steps it covers ring + (T-1)·R rows in 2D and T·R planes in 3D: those are
// the halo widths, and the core rows come back exact.
//
// One host array holds the state: the first pass reads `in_host` and writes
// `out_host`, every later pass updates `out_host` in place. A slab's core is
// written back only after every slab whose halo reads those rows has been
// copied in (its "last reader"), so no pass reads a row that it already
// advanced. 2D ring semantics (each array keeps its own ring; the result sits
// in the output array for odd iteration counts and in the input array for
// even ones) are kept by giving every pass an odd length (pskel_plan_passes)
// and by keeping both arrays' rings on the device: each slab's destination
// buffer gets the ring of the array the step-by-step run writes in that pass,
// and the rows written back carry it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <deque>
#include <vector>

#include "capi_internal.h"

namespace pskel {

pskel_status validate2d(const pskel_stencil* st, const void* in, const void* out, int64_t W, int64_t H, int64_t pitch,
                        int64_t iters, int* R, int* ring);

namespace {

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
  int slots = 3;        // device slots: 2 + the slabs a halo can span
  size_t slot_bytes = 0;
  size_t ringcol_bytes = 0;  // 2D: ring columns of one array (H rows x 2 ring)
  size_t ringrow_bytes = 0;  // 2D: top and bottom ring rows of one array
  size_t device_bytes = 0;
};

int64_t halo_rows(const Plan& p, int T) {
  return p.dims == 2 ? p.ring + static_cast<int64_t>(T - 1) * p.R : static_cast<int64_t>(T) * p.R;
}

void size_plan(Plan& p, int64_t S) {
  S = std::max<int64_t>(1, std::min<int64_t>(S, p.H));
  p.slab = S;
  p.slabs = (p.H + S - 1) / S;
  p.slots = 2 + static_cast<int>(std::min<int64_t>(p.slabs, (p.halo + S - 1) / S));
  p.slots = std::max(p.slots, 3);
  const int64_t sub_max = std::min<int64_t>(p.H, S + 2 * p.halo);
  p.slot_bytes = align_up(static_cast<size_t>(sub_max) * p.dev_row, 256);
  p.device_bytes = static_cast<size_t>(p.slots) * p.fields * p.slot_bytes + 2 * (p.ringcol_bytes + p.ringrow_bytes);
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
  if (p.dims == 2) {
    p.ringcol_bytes = align_up(static_cast<size_t>(p.H) * 2 * p.ring * p.esz, 256);
    p.ringrow_bytes = align_up(2 * static_cast<size_t>(p.ring) * p.dev_row, 256);
  }
  if (slab_rows > 0) {
    size_plan(p, slab_rows);
    return PSKEL_OK;
  }
  size_t budget = static_cast<size_t>(device_bytes);
  if (budget == 0) {
    size_t fr = 0, tot = 0;
    cudaError_t e = cudaMemGetInfo(&fr, &tot);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemGetInfo");
    budget = fr / 10 * 9;
  }
  // Device memory besides the slots: both arrays' rings, and for Life the two
  // bit planes and pass counters of one sub-grid (a quarter byte per cell).
  const size_t fixed = 2 * (p.ringcol_bytes + p.ringrow_bytes) + (1 << 20);
  const size_t per_row = static_cast<size_t>(3) * p.fields * p.dev_row + (p.dims == 2 ? p.W / 4 + 64 : 0);
  const int64_t rows = budget > fixed ? static_cast<int64_t>((budget - fixed) / per_row) : 0;
  // three slots of slab + 2 halo rows, the slab no thinner than the halo
  int64_t S = rows - 2 * p.halo;
  if (S >= p.H) S = p.H;
  if (S < std::min<int64_t>(p.halo, p.H) || S < 1)
    return fail(PSKEL_ERR_NOMEM,
                "device budget %zu bytes holds %lld rows per slot, too few for slabs of at least the halo (%lld rows) "
                "with a halo on each side",
                budget, (long long)rows, (long long)p.halo);
  size_plan(p, S);
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

cudaError_t rows_d2d(void* d, const void* src, size_t pitch, size_t row_bytes, int64_t rows, cudaStream_t s) {
  if (rows <= 0) return cudaSuccess;
  return cudaMemcpy2DAsync(d, pitch, src, pitch, row_bytes, static_cast<size_t>(rows), cudaMemcpyDeviceToDevice, s);
}

struct Run {
  Plan p;
  pskel_stencil st;
  const pskel_schedule* sched = nullptr;
  const uint8_t* in = nullptr;  // in_host
  uint8_t* out = nullptr;       // out_host
  uint8_t* dev = nullptr;       // slots, then ring columns and rows of both arrays
  DeviceContext* c = nullptr;
};

uint8_t* slot_buf(const Run& r, int slot, int field) {
  return r.dev + (static_cast<size_t>(slot) * r.p.fields + field) * r.p.slot_bytes;
}

// Ring columns (H rows x [left ring | right ring]) and ring rows (top ring
// rows, then bottom ring rows, device pitch) of array L: 0 input, 1 output.
uint8_t* ringcols(const Run& r, int L) {
  return r.dev + static_cast<size_t>(r.p.slots) * r.p.fields * r.p.slot_bytes + L * r.p.ringcol_bytes;
}
uint8_t* ringrows(const Run& r, int L) {
  return r.dev + static_cast<size_t>(r.p.slots) * r.p.fields * r.p.slot_bytes + 2 * r.p.ringcol_bytes +
         L * r.p.ringrow_bytes;
}

// Copies both arrays' rings to the device (2D).
cudaError_t stage_rings(const Run& r, cudaStream_t s) {
  const Plan& p = r.p;
  const size_t cw = static_cast<size_t>(p.ring) * p.esz;
  const int64_t rr = std::min<int64_t>(p.ring, p.H);
  for (int L = 0; L < 2; ++L) {
    const uint8_t* src = (L == 0) ? r.in : r.out;
    uint8_t* d = ringcols(r, L);
    cudaError_t e =
        cudaMemcpy2DAsync(d, 2 * cw, src, p.host_row, cw, static_cast<size_t>(p.H), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(d + cw, 2 * cw, src + (p.W - p.ring) * p.esz, p.host_row, cw, static_cast<size_t>(p.H),
                            cudaMemcpyHostToDevice, s);
    uint8_t* rw = ringrows(r, L);
    if (e == cudaSuccess) e = rows_h2d(rw, p.dev_row, src, p.host_row, rr, s);
    if (e == cudaSuccess)
      e = rows_h2d(rw + p.dev_row * p.ring, p.dev_row, src + p.host_row * (p.H - rr), p.host_row, rr, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

struct Visit {
  int64_t k;      // slab index within the pass
  int slot;
  int64_t y0, y1;  // core rows
  int64_t a;       // first sub-grid row
  int T;
  int64_t last_reader;  // last slab of the pass whose sub-grid holds a core row
};

pskel_status run_slabs(Run& r) {
  const Plan& p = r.p;
  const int P = static_cast<int>(p.passes.size());
  const int NS = p.slots;
  Streams ss;
  cudaError_t e = ss.create();
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
  cudaStream_t s_in = ss.s[0], s_comp = ss.s[1], s_out = ss.s[2];
  std::vector<cudaEvent_t> ev_in(NS), ev_comp(NS), ev_free(NS);
  cudaEvent_t ev_loaded;  // recorded on s_in after each slab's copies in
  for (int i = 0; i < NS; ++i)
    if ((e = ss.event(&ev_in[i])) != cudaSuccess || (e = ss.event(&ev_comp[i])) != cudaSuccess ||
        (e = ss.event(&ev_free[i])) != cudaSuccess)
      return cuda_fail(e, "cudaEventCreate");
  if ((e = ss.event(&ev_loaded)) != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
  // ev_done[j % 2][k]: slab k of pass j written back to the host
  std::vector<cudaEvent_t> ev_done[2];
  for (auto& v : ev_done) {
    v.resize(static_cast<size_t>(p.slabs));
    for (auto& x : v)
      if ((e = ss.event(&x)) != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
  }
  std::vector<bool> slot_used(static_cast<size_t>(NS), false);
  if (p.dims == 2 && p.ring > 0 && (e = stage_rings(r, s_in)) != cudaSuccess)
    return cuda_fail(e, "copy rings to device");

  std::deque<Visit> pending;  // computed, not yet written back
  auto write_back = [&](const Visit& v, int j) -> pskel_status {
    cudaError_t x = cudaStreamWaitEvent(s_out, ev_comp[v.slot], 0);
    if (x == cudaSuccess) x = cudaStreamWaitEvent(s_out, ev_loaded, 0);
    const uint8_t* res = (v.T % 2 == 1) ? slot_buf(r, v.slot, 1) : slot_buf(r, v.slot, 0);
    if (x == cudaSuccess)
      x = rows_d2h(r.out + p.host_row * v.y0, p.host_row, res + p.dev_row * (v.y0 - v.a), p.dev_row, v.y1 - v.y0,
                   s_out);
    if (x == cudaSuccess) x = cudaEventRecord(ev_free[v.slot], s_out);
    if (x == cudaSuccess) x = cudaEventRecord(ev_done[j % 2][v.k], s_out);
    return x == cudaSuccess ? PSKEL_OK : cuda_fail(x, "copy slab to host");
  };

  int64_t visit = 0;
  for (int j = 0; j < P; ++j) {
    const int T = p.passes[static_cast<size_t>(j)];
    const int64_t halo = halo_rows(p, T);
    const uint8_t* src = (j == 0) ? r.in : r.out;
    const int Ldst = (j % 2 == 0) ? 1 : 0;  // the array step-by-step writes in this pass
    for (int64_t k = 0; k < p.slabs; ++k, ++visit) {
      Visit v;
      v.k = k;
      v.slot = static_cast<int>(visit % NS);
      v.y0 = k * p.slab;
      v.y1 = std::min(p.H, v.y0 + p.slab);
      v.a = std::max<int64_t>(0, v.y0 - halo);
      v.T = T;
      v.last_reader = std::min<int64_t>(p.slabs - 1, (v.y1 - 1 + halo) / p.slab);
      const int64_t b = std::min<int64_t>(p.H, v.y1 + halo);
      const int64_t hs = b - v.a;
      uint8_t* dA = slot_buf(r, v.slot, 0);
      uint8_t* dB = slot_buf(r, v.slot, 1);
      // copies in: the slot is free once its previous slab was written back;
      // the source rows are final once the previous pass wrote them back
      if (slot_used[v.slot] && (e = cudaStreamWaitEvent(s_in, ev_free[v.slot], 0)) != cudaSuccess)
        return cuda_fail(e, "cudaStreamWaitEvent");
      if (j > 0) {
        const int64_t klast = std::min<int64_t>(p.slabs - 1, (b - 1) / p.slab);
        if ((e = cudaStreamWaitEvent(s_in, ev_done[(j - 1) % 2][klast], 0)) != cudaSuccess)
          return cuda_fail(e, "cudaStreamWaitEvent");
      }
      e = rows_h2d(dA, p.dev_row, src + p.host_row * v.a, p.host_row, hs, s_in);
      if (e == cudaSuccess && p.dims == 2 && p.ring > 0) {
        // sub-grid ring: the destination array's own ring rows at a grid
        // edge, the source rows elsewhere (any state works there), and the
        // destination array's ring columns in between
        const int64_t rr = std::min<int64_t>(p.ring, hs);
        const size_t row = p.W * p.esz;
        e = rows_d2d(dB, v.a == 0 ? ringrows(r, Ldst) : dA, p.dev_row, row, rr, s_in);
        if (e == cudaSuccess)
          e = rows_d2d(dB + p.dev_row * (hs - rr),
                       b == p.H ? ringrows(r, Ldst) + p.dev_row * (p.ring - rr) + p.dev_row * p.ring
                                : dA + p.dev_row * (hs - rr),
                       p.dev_row, row, rr, s_in);
        const int64_t mid = hs - 2 * p.ring;
        if (e == cudaSuccess && mid > 0) {
          const size_t cw = static_cast<size_t>(p.ring) * p.esz;
          const uint8_t* rc = ringcols(r, Ldst) + static_cast<size_t>(v.a + p.ring) * 2 * cw;
          e = cudaMemcpy2DAsync(dB + p.dev_row * p.ring, p.dev_row, rc, 2 * cw, cw, static_cast<size_t>(mid),
                                cudaMemcpyDeviceToDevice, s_in);
          if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(dB + p.dev_row * p.ring + (p.W - p.ring) * p.esz, p.dev_row, rc + cw, 2 * cw, cw,
                                  static_cast<size_t>(mid), cudaMemcpyDeviceToDevice, s_in);
        }
      }
      pskel_stencil sub = r.st;
      if (e == cudaSuccess && p.fields == 4) {
        uint8_t* dU = slot_buf(r, v.slot, 2);
        uint8_t* dV = slot_buf(r, v.slot, 3);
        e = rows_h2d(dU, p.dev_row, static_cast<const uint8_t*>(r.st.wind_u) + p.host_row * v.a, p.host_row, hs,
                     s_in);
        if (e == cudaSuccess)
          e = rows_h2d(dV, p.dev_row, static_cast<const uint8_t*>(r.st.wind_v) + p.host_row * v.a, p.host_row, hs,
                       s_in);
        sub.wind_u = dU;
        sub.wind_v = dV;
      }
      if (e == cudaSuccess) e = cudaEventRecord(ev_in[v.slot], s_in);
      if (e == cudaSuccess) e = cudaEventRecord(ev_loaded, s_in);
      if (e != cudaSuccess) return cuda_fail(e, "copy slab to device");

      // compute
      if ((e = cudaStreamWaitEvent(s_comp, ev_in[v.slot], 0)) != cudaSuccess)
        return cuda_fail(e, "cudaStreamWaitEvent");
      pskel_status q;
      if (p.dims == 2)
        q = pskel_iterate2d(&sub, dA, dB, p.W, hs, static_cast<int64_t>(p.dev_row / p.esz), T, r.sched, s_comp);
      else
        q = pskel_iterate3d(&sub, dA, dB, p.W, hs, p.D, T, r.sched, 0, nullptr, s_comp);
      if (q != PSKEL_OK) return q;
      if ((e = cudaEventRecord(ev_comp[v.slot], s_comp)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
      slot_used[v.slot] = true;

      // write back every pending core whose last reader is now loaded
      pending.push_back(v);
      while (!pending.empty() && (pending.front().last_reader <= k || k == p.slabs - 1)) {
        if (pskel_status w = write_back(pending.front(), j)) return w;
        pending.pop_front();
      }
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
  if (pskel_status s = ensure_buffer(r.c->tiles, p.device_bytes)) return s;
  r.dev = static_cast<uint8_t*>(r.c->tiles.ptr);
  return run_slabs(r);
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
