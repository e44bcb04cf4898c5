// C ABI entry points (include/pskel_gb300.h): argument checks, schedule
// geometry, tensor maps, the pass loop and the host-array round trip.
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pskel_gb300.h"
#include "capi_internal.h"
#include "common.cuh"
#include "kernels.h"

namespace pskel {

// ----------------------------------------------------------- error reporting

static thread_local std::string g_last_error;
static thread_local int64_t g_last_launches2d = 0;  // kernel launches of the last pskel_iterate2d

pskel_status fail(pskel_status code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

pskel_status cuda_fail(cudaError_t e, const char* what) {
  return fail(e == cudaErrorMemoryAllocation ? PSKEL_ERR_NOMEM : PSKEL_ERR_CUDA, "%s: %s", what,
              cudaGetErrorString(e));
}

void clear_error() { g_last_error.clear(); }

// ---------------------------------------------------------- device context

static std::mutex g_ctx_mu;
static std::map<int, DeviceContext*> g_ctx;

pskel_status get_context(DeviceContext** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  auto it = g_ctx.find(dev);
  if (it != g_ctx.end()) {
    *out = it->second;
    return PSKEL_OK;
  }
  DeviceContext* c = new DeviceContext();
  c->device = dev;
  e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
  cudaDeviceGetAttribute(&c->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  e = cudaMalloc(&c->err, 64);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(error word)");
  e = cudaMemset(c->err, 0, 64);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemset(error word)");
  e = cudaHostAlloc(reinterpret_cast<void**>(&c->err_host), 64, cudaHostAllocDefault);
  if (e != cudaSuccess) return cuda_fail(e, "cudaHostAlloc(error word copy)");
  *c->err_host = 0;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy_in, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy_out, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
  g_ctx[dev] = c;
  *out = c;
  return PSKEL_OK;
}

pskel_status ensure_buffer(DeviceBuffer& b, size_t bytes) {
  if (b.bytes >= bytes && b.ptr) return PSKEL_OK;
  if (b.ptr) cudaFree(b.ptr);
  b.ptr = nullptr;
  b.bytes = 0;
  cudaError_t e = cudaMalloc(&b.ptr, bytes ? bytes : 16);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(staging buffer)");
  b.bytes = bytes;
  return PSKEL_OK;
}

pskel_status device_sync_check(DeviceContext* c, cudaStream_t s) {
  // the error word follows the stream's work in a copy to pinned host memory,
  // so one synchronisation covers both
  cudaError_t e = cudaMemcpyAsync(c->err_host, c->err, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  const cudaError_t es = cudaStreamSynchronize(s);
  if (es != cudaSuccess) return cuda_fail(es, "kernel execution");
  if (e != cudaSuccess) return cuda_fail(e, "reading the device error word");
  const unsigned word = *static_cast<volatile unsigned*>(c->err_host);
  if (word) {
    cudaMemset(c->err, 0, sizeof(unsigned));
    std::string msg = "device error:";
    if (word & kDevErrTimeout) msg += " a TMA/mbarrier wait timed out;";
    if (word & kDevErrValue) msg += " a Life cell outside {0,1};";
    if (word & kDevErrBarrier) msg += " a dependency wait between tiles or passes timed out;";
    if (word & kDevErrAlign) msg += " dynamic shared memory was not 128-byte aligned;";
    return fail(PSKEL_ERR_DEVICE, "%s", msg.c_str());
  }
  return PSKEL_OK;
}

// ------------------------------------------------------------ tensor maps

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

cudaError_t encode_tmap(CUtensorMap* map, CUtensorMapDataType type, int rank, void* base, const uint64_t* dims,
                        const uint64_t* strides_bytes, const uint32_t* box) {
  if (!g_encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess) return e;
    if (q != cudaDriverEntryPointSuccess || !fn) return cudaErrorNotSupported;
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  cuuint64_t gd[3];
  cuuint64_t gs[2];
  cuuint32_t bx[3];
  cuuint32_t es[3] = {1, 1, 1};
  for (int i = 0; i < rank; ++i) {
    gd[i] = dims[i];
    bx[i] = box[i];
  }
  for (int i = 0; i + 1 < rank; ++i) gs[i] = strides_bytes[i];
  CUresult r = g_encode(map, type, static_cast<cuuint32_t>(rank), base, gd, gs, bx, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

std::vector<int> plan_passes(int64_t iters, int T) {
  // Every pass has an odd number of steps. Ring cells are never written, so
  // the reference's state after k steps sits in `out` (k odd) or `in` (k even)
  // together with that buffer's ring. A pass that reads one buffer and writes
  // the other therefore has to advance an odd number of steps for the ring it
  // sees at every step, and the buffer it ends in, to match the reference's.
  std::vector<int> p;
  if (iters <= 0) return p;
  const int To = (T <= 1) ? 1 : ((T & 1) ? T : T - 1);
  int64_t L = (iters + To - 1) / To;
  if ((L & 1) != (iters & 1)) ++L;  // a sum of L odd numbers has the parity of L
  const int64_t extra_pairs = (iters - L) / 2;  // each pass: 1 + 2 * (its share of pairs)
  const int64_t q = extra_pairs / L, r = extra_pairs % L;
  for (int64_t i = 0; i < L; ++i) p.push_back(static_cast<int>(1 + 2 * (q + (i < r ? 1 : 0))));
  return p;
}

std::vector<int> plan_passes_any(int64_t iters, int T) {
  // Passes of at most T steps (any length) whose count has the parity of
  // `iters`, so a ping-pong over the passes ends in the buffer a step-by-step
  // ping-pong ends in. For grids where every cell is written each step.
  std::vector<int> p;
  if (iters <= 0) return p;
  if (T < 1) T = 1;
  for (int64_t k = 0; k < iters / T; ++k) p.push_back(T);
  if (iters % T) p.push_back(static_cast<int>(iters % T));
  if ((static_cast<int64_t>(p.size()) & 1) != (iters & 1)) {
    for (size_t i = 0; i < p.size(); ++i) {
      if (p[i] >= 2) {
        const int a = p[i] / 2, b = p[i] - a;
        p[i] = a;
        p.insert(p.begin() + static_cast<long>(i) + 1, b);
        break;
      }
    }
  }
  return p;
}

// --------------------------------------------------------------- validation

static size_t dtype_size(pskel_dtype d) { return d == PSKEL_U8 ? 1 : (d == PSKEL_F32 ? 4 : 2); }

pskel_status check_mask(const pskel_mask& m, int dim, bool need_weights, int* max_off, int* ring) {
  if (m.dimension != dim) return fail(PSKEL_ERR_INVALID, "mask dimension %d, expected %d", m.dimension, dim);
  if (m.size < 1) return fail(PSKEL_ERR_INVALID, "mask has no entries");
  if (!m.offsets) return fail(PSKEL_ERR_INVALID, "mask offsets pointer is NULL");
  if (need_weights && !m.weights) return fail(PSKEL_ERR_INVALID, "mask weights pointer is NULL");
  if (m.range < 0) return fail(PSKEL_ERR_INVALID, "negative mask range");
  int R = 0;
  for (int i = 0; i < m.size * dim; ++i) R = std::max(R, std::abs(m.offsets[i]));
  int r = m.range > 0 ? m.range : R;
  if (r < R)
    return fail(PSKEL_ERR_INVALID,
                "mask range %d is smaller than its largest offset %d: updated cells would read outside the grid", r, R);
  *max_off = R;
  *ring = r;
  return PSKEL_OK;
}

static pskel_status check_life_mask(const pskel_mask& m) {
  if (m.size != 8) return fail(PSKEL_ERR_UNSUPPORTED, "Life kernel needs the 8-entry Moore mask, got %d entries", m.size);
  int seen = 0;
  for (int n = 0; n < 8; ++n) {
    const int dh = m.offsets[2 * n], dw = m.offsets[2 * n + 1];
    if (dh < -1 || dh > 1 || dw < -1 || dw > 1 || (dh == 0 && dw == 0))
      return fail(PSKEL_ERR_UNSUPPORTED, "Life kernel needs the Moore mask; entry %d is (%d,%d)", n, dh, dw);
    const int bit = 1 << ((dh + 1) * 3 + (dw + 1));
    if (seen & bit) return fail(PSKEL_ERR_UNSUPPORTED, "Life mask repeats offset (%d,%d)", dh, dw);
    seen |= bit;
  }
  return PSKEL_OK;
}

static bool tma_ok(const void* p, int64_t pitch_bytes) {
  return (reinterpret_cast<uintptr_t>(p) & 15) == 0 && (pitch_bytes & 15) == 0 && pitch_bytes < (int64_t(1) << 40);
}

// ------------------------------------------------------------- 2D iterate

// Game of Life on bit planes: both grids are packed once into two global bit
// planes (L2-resident for grids up to ~16k x 16k), the passes run between the
// planes, and the final plane's interior is unpacked into the result buffer.
// The other buffer is not written; ring cells of the result keep their bytes.
// Generations per pass of the Life kernel by default (measured on GB300,
// 8192^2, 24 rows per lane: T = 13/15/17/19/21/25 26.9/27.3/27.7/27.2/27.4/27.0
// T updates/s; at T = 17 its 328-row cores tile the 8192 rows 25 times).
constexpr int kLifeDefaultSteps = 17;

static pskel_status iterate_life(const pskel_stencil& st, void* in, void* out, int64_t W, int64_t H, int64_t pitch,
                                 int64_t iters, int ring, const pskel_schedule* sched, DeviceContext* c,
                                 cudaStream_t s) {
  (void)st;
  if (iters <= 0) return PSKEL_OK;
  const int64_t it1 = std::max<int64_t>(iters, 1);
  struct Geo {
    int T, TH;
  };
  auto geom_for = [&](int T, Geo& g) -> bool {
    T = static_cast<int>(std::min<int64_t>(std::min(T, kLifeBitsMaxT), it1));
    if (T > 1 && (T & 1) == 0) --T;  // passes have odd lengths (plan_passes)
    int TH = (sched && sched->tile_h > 0) ? sched->tile_h : life_bits_max_tile_h(T);
    TH = std::min(TH, life_bits_max_tile_h(T));
    if (TH < 1) return false;
    g.T = T;
    g.TH = TH;
    return true;
  };
  Geo g{1, 254};
  if (sched && sched->time_steps > 0) {
    if (!geom_for(sched->time_steps, g))
      return fail(PSKEL_ERR_INVALID, "Life tile height too small for %d steps per pass", sched->time_steps);
  } else {
    // Default: kLifeDefaultSteps generations per pass on full-height tiles
    if (!geom_for(kLifeDefaultSteps, g) && !geom_for(1, g)) return fail(PSKEL_ERR_INVALID, "no Life geometry fits");
  }
  const int64_t tiles = life_bits_tiles(static_cast<int>(W), static_cast<int>(H), g.TH);
  // every pass in one persistent launch: no more CTAs than can be resident
  const int64_t resident = static_cast<int64_t>(life_bits_persistent_ctas_per_sm(g.T)) * c->sms;
  int ctas = (sched && sched->ctas > 0) ? sched->ctas : static_cast<int>(resident);
  ctas = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(ctas, resident), tiles)));
  const size_t plane = static_cast<size_t>(life_bits_words(static_cast<int>(W))) * static_cast<size_t>(H);
  if (pskel_status q = ensure_buffer(c->life_bits, 2 * plane * sizeof(uint32_t))) return q;
  uint32_t* A = static_cast<uint32_t*>(c->life_bits.ptr);
  uint32_t* B = A + plane;
  cudaError_t e = life_bits_pack(static_cast<const uint8_t*>(in), pitch, static_cast<int>(W), static_cast<int>(H), A,
                                 ring, false, c->err, c->sms, s);
  if (e == cudaSuccess)
    e = life_bits_pack(static_cast<const uint8_t*>(out), pitch, static_cast<int>(W), static_cast<int>(H), B, ring,
                       true, c->err, c->sms, s);
  if (e != cudaSuccess) return cuda_fail(e, "Life pack launch");
  const std::vector<int> passes = plan_passes(iters, g.T);
  // plan_passes: the first r passes have 2 more steps than the others (1 + 2q)
  const int q = (passes.back() - 1) / 2;
  int r = 0;
  while (r < static_cast<int>(passes.size()) && passes[r] > passes.back()) ++r;
  if (pskel_status qs = ensure_buffer(c->life_sync, life_bits_sync_bytes(static_cast<int>(W), static_cast<int>(H), g.TH)))
    return qs;
  e = life_bits_run_persistent(A, B, static_cast<int>(W), static_cast<int>(H), ring, static_cast<int>(passes.size()), q,
                               r, g.T, g.TH, ctas, c->life_sync.ptr, c->err, s);
  if (e != cudaSuccess) return cuda_fail(e, "Life kernel launch");
  // an odd number of passes (odd iterations) ends in B, whose result goes to `out`
  const bool odd = (passes.size() % 2) == 1;
  e = life_bits_unpack(odd ? B : A, static_cast<uint8_t*>(odd ? out : in), pitch, static_cast<int>(W),
                       static_cast<int>(H), ring, c->sms, s);
  if (e != cudaSuccess) return cuda_fail(e, "Life unpack launch");
  g_last_launches2d = 4;  // two packs, the persistent run, the unpack
  return PSKEL_OK;
}

static bool tma_ok(const void* p, int64_t pitch_bytes);

// The register-windowed kernel (stencil2d_fast.cu) for reach-1 masks of a
// known shape and for advection, when every buffer can be staged by TMA.
static pskel_status iterate_fast2d(const pskel_stencil& st, int opk, void* in, void* out, int64_t W, int64_t H,
                                   int64_t pitch, int64_t iters, int ring, const pskel_schedule* sched,
                                   DeviceContext* c, cudaStream_t s, bool* used) {
  *used = false;
  const bool advect = st.op == PSKEL_OP_ADVECT;
  const int dtype = static_cast<int>(st.dtype);
  const int N = 4;                 // cells per thread vector
  const int vec = (dtype == PSKEL_BF16) ? 8 : 4;  // TMA x alignment (16 bytes) in cells
  const int LW = 128;
  const int S = (sched && sched->tile_h > 64) ? 8 : 4;
  const int LH = 16 * S + 2;
  int T = (sched && sched->time_steps > 0) ? sched->time_steps : fast2d_default_steps(advect, dtype, W, H);
  T = static_cast<int>(std::min<int64_t>(T, std::max<int64_t>(iters, 1)));
  if (T > 1 && (T & 1) == 0) --T;  // passes have odd lengths (plan_passes)
  int HX = 0, HY = 0;
  for (;;) {
    HY = T;
    HX = ((T + vec - 1) / vec) * vec;
    if ((LW - 2 * HX >= N && LH - 2 * HY >= 2) || T == 1) break;
    T -= 2;
  }
  const size_t smem = fast2d_smem_bytes(advect, dtype, S);
  if (smem > static_cast<size_t>(c->smem_optin)) return PSKEL_OK;
  const int64_t pb = pitch * static_cast<int64_t>(dtype == PSKEL_BF16 ? 2 : 4);
  bool ok = tma_ok(in, pb) && tma_ok(out, pb);
  if (advect) ok = ok && tma_ok(st.wind_u, pb) && tma_ok(st.wind_v, pb);  // vector loads of the winds
  if (!ok) return PSKEL_OK;
  Stencil2DParams p;
  memset(&p, 0, sizeof(p));
  p.W = static_cast<int>(W);
  p.H = static_cast<int>(H);
  p.pitch = pitch;
  p.ring = ring;
  p.R = 1;
  p.err = c->err;
  if (advect) {
    p.K = st.diffusivity;
    p.dt = st.dt;
    p.inv_dx = st.inv_dx;
    p.u = st.wind_u;
    p.v = st.wind_v;
  } else {
    p.nm = st.mask.size;
    for (int n = 0; n < p.nm; ++n) p.wt[n] = st.mask.weights[n];
  }
  if (T == 1) {
    // one step per pass: the streaming kernel with rows staged by TMA,
    // persistent blocks over items of 32 vectors of columns x HC rows
    // (tile_h; by default a multiple of 8 rows, at least 32, chosen like the
    // 3D h chunks: block b takes items b, b + ctas, ..., so the busiest block
    // streams ceil(items / ctas) items of about HC + 8 rows (its 8-row boxes);
    // the HC minimising that, then the rows loaded in all, wins)
    const int esz = dtype == PSKEL_BF16 ? 2 : 4;
    const int64_t resident = static_cast<int64_t>(stream2d_tma_blocks_per_sm(opk, dtype)) * c->sms;
    const int64_t strips = stream2d_tma_items(static_cast<int>(W), static_cast<int>(H), static_cast<int>(H), dtype);
    int HC = 32;
    double best = 0.0;
    for (int64_t hc = 32; hc < H + 8; hc += 8) {
      const int64_t items = strips * ((H + hc - 1) / hc), used = std::min<int64_t>(items, resident);
      const double cost = static_cast<double>((items + used - 1) / used) * static_cast<double>(hc + 8) +
                          1e-3 * static_cast<double>(items * (hc + 8)) / static_cast<double>(resident);
      if (hc == 32 || cost < best) {
        best = cost;
        HC = static_cast<int>(hc);
      }
    }
    if (sched && sched->tile_h > 0) HC = static_cast<int>(std::min<int64_t>(sched->tile_h, H));
    p.TH = HC;
    p.tiles_y = static_cast<int>((H + HC - 1) / HC);
    const int64_t items = stream2d_tma_items(static_cast<int>(W), static_cast<int>(H), HC, dtype);
    int ctas = static_cast<int>(std::min<int64_t>(items, resident));
    if (sched && sched->ctas > 0) ctas = std::min(ctas, sched->ctas);
    ctas = std::max(ctas, 1);
    const uint64_t dims[2] = {static_cast<uint64_t>((W * esz + 3) / 4), static_cast<uint64_t>(H)};
    const uint64_t strides[1] = {static_cast<uint64_t>(pb)};
    const uint32_t box_phi[2] = {136u, 8u};
    const uint32_t box_w[2] = {128u, 8u};
    CUtensorMap m_in, m_out, m_u, m_v;
    memset(&m_u, 0, sizeof(m_u));
    memset(&m_v, 0, sizeof(m_v));
    cudaError_t e = encode_tmap(&m_in, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, in, dims, strides, box_phi);
    if (e == cudaSuccess) e = encode_tmap(&m_out, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, out, dims, strides, box_phi);
    if (advect && e == cudaSuccess)
      e = encode_tmap(&m_u, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<void*>(st.wind_u), dims, strides, box_w);
    if (advect && e == cudaSuccess)
      e = encode_tmap(&m_v, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<void*>(st.wind_v), dims, strides, box_w);
    if (e != cudaSuccess) return cuda_fail(e, "cuTensorMapEncodeTiled (2D rows)");
    *used = true;
    for (int64_t k = 0; k < iters; ++k) {
      const bool fwd = (k % 2 == 0);
      p.src = fwd ? in : out;
      p.dst = fwd ? out : in;
      p.steps = 1;
      e = stream2d_tma_step(opk, dtype, fwd ? &m_in : &m_out, &m_u, &m_v, p, ctas, s);
      if (e != cudaSuccess) return cuda_fail(e, "2D streaming kernel launch");
    }
    g_last_launches2d = iters;
    return PSKEL_OK;
  }
  p.T = T;
  p.TW = LW - 2 * HX;
  p.TH = LH - 2 * HY;
  p.LW = LW;
  p.LH = LH;
  p.HX = HX;
  p.HY = HY;
  p.tiles_x = static_cast<int>((W + p.TW - 1) / p.TW);
  p.tiles_y = static_cast<int>((H + p.TH - 1) / p.TH);
  const int ntiles = p.tiles_x * p.tiles_y;
  const int per_sm = std::max(1, fast2d_max_ctas_per_sm(advect, dtype, S));
  int ctas = (sched && sched->ctas > 0) ? sched->ctas : per_sm * c->sms;
  ctas = std::max(1, std::min(ctas, ntiles));
  const CUtensorMapDataType tt = (dtype == PSKEL_BF16) ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  const uint64_t dims[2] = {static_cast<uint64_t>(W), static_cast<uint64_t>(H)};
  const uint64_t strides[1] = {static_cast<uint64_t>(pb)};
  const uint32_t box[2] = {static_cast<uint32_t>(LW), static_cast<uint32_t>(LH)};
  CUtensorMap m_in, m_out, m_u, m_v;
  memset(&m_u, 0, sizeof(m_u));
  memset(&m_v, 0, sizeof(m_v));
  cudaError_t e = encode_tmap(&m_in, tt, 2, in, dims, strides, box);
  if (e == cudaSuccess) e = encode_tmap(&m_out, tt, 2, out, dims, strides, box);
  if (e != cudaSuccess) return cuda_fail(e, "cuTensorMapEncodeTiled");
  *used = true;
  const std::vector<int> passes = plan_passes(iters, T);
  // Grids of at most three waves of tiles per pass (two resident CTAs per SM
  // for 4-row strips, one for 8-row strips) run every pass in one persistent
  // launch: tiles of pass i start as soon as their neighbourhood of pass i-1
  // is done, so neither the tail of a pass nor a launch boundary leaves SMs
  // idle. Larger grids keep one launch per pass, whose tiles prefetch the
  // next tile's source while they compute. Measured on GB300 (Jacobi f32,
  // T = 7, GCells/s, one launch per pass vs one launch): 1448^2 (364 tiles)
  // 692 vs 928, 2048^2 (760) 800 vs 954, 2896^2 (1456) 1265 vs 1017; advection
  // f32 2048^2 T = 5: 272 vs 422; advection f32 4096^2 (2738 tiles) 432 vs 425.
  const int mp_per_sm = (S <= 4) ? 2 : 1;
  bool multipass = passes.size() >= 2 && ntiles <= 3 * mp_per_sm * c->sms;
  if (const char* ev = getenv("PSKEL_FAST2D_MULTIPASS")) multipass = passes.size() >= 2 && ev[0] == '1';
  if (dep_wait_test().spin_limit) multipass = passes.size() >= 2;  // the bounded-wait self-test
  if (multipass) {
    const size_t sync_bytes = fast2d_multipass_sync_bytes(ntiles);
    if (pskel_status q = ensure_buffer(c->fast2d_sync, sync_bytes)) return q;
    const int q = (passes.back() - 1) / 2;
    int r = 0;
    while (r < static_cast<int>(passes.size()) && passes[r] > passes.back()) ++r;
    const int64_t items = static_cast<int64_t>(passes.size()) * ntiles;
    int mctas = (sched && sched->ctas > 0) ? sched->ctas : per_sm * c->sms;
    mctas = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(mctas, items)));
    p.src = in;
    p.dst = out;
    p.steps = passes[0];
    e = fast2d_multipass(opk, dtype, S, &m_in, &m_out, p, static_cast<int>(passes.size()), q, r, c->fast2d_sync.ptr,
                         mctas, s);
    if (e != cudaSuccess) return cuda_fail(e, "2D multi-pass stencil kernel launch");
    g_last_launches2d = 1;
    return PSKEL_OK;
  }
  for (size_t i = 0; i < passes.size(); ++i) {
    const bool fwd = (i % 2 == 0);
    p.src = fwd ? in : out;
    p.dst = fwd ? out : in;
    p.steps = passes[i];
    e = fast2d_pass(opk, dtype, S, fwd ? &m_in : &m_out, fwd ? &m_out : &m_in, &m_u, &m_v, p, ctas, s);
    if (e != cudaSuccess) return cuda_fail(e, "2D stencil kernel launch");
  }
  g_last_launches2d = static_cast<int64_t>(passes.size());
  return PSKEL_OK;
}

static pskel_status iterate_float2d(const pskel_stencil& st, void* in, void* out, int64_t W, int64_t H, int64_t pitch,
                                    int64_t iters, int R, int ring, const pskel_schedule* sched, DeviceContext* c,
                                    cudaStream_t s) {
  const Op2D op = (st.op == PSKEL_OP_ADVECT) ? Op2D::Advect : Op2D::Linear;
  const int opk = (op == Op2D::Advect) ? 3 : (R == 1 ? fast2d_shape(st.mask.offsets, st.mask.size) : -1);
  const bool generic_requested = sched && sched->tile_w > 0;  // explicit tile widths select the generic kernel
  if (opk >= 0 && !generic_requested) {
    bool used = false;
    if (pskel_status q = iterate_fast2d(st, opk, in, out, W, H, pitch, iters, ring, sched, c, s, &used)) return q;
    if (used) return PSKEL_OK;
  }
  const int dtype = static_cast<int>(st.dtype);
  const size_t esz = dtype_size(st.dtype);
  const int vec = static_cast<int>(16 / esz);
  int T = (sched && sched->time_steps > 0) ? sched->time_steps : (op == Op2D::Advect ? 4 : 8);
  T = static_cast<int>(std::min<int64_t>(T, std::max<int64_t>(iters, 1)));
  if (T > 1 && (T & 1) == 0) --T;  // passes have odd lengths (plan_passes)
  if (R == 0) T = 1;  // a mask reaching no neighbour needs no halo
  int TW = (sched && sched->tile_w > 0) ? sched->tile_w : (op == Op2D::Advect ? 64 : 128);
  int TH = (sched && sched->tile_h > 0) ? sched->tile_h : 64;
  TW = std::max(vec, (TW / vec) * vec);
  // shrink the temporal block until the halo tile fits a TMA box (<= 256 per side)
  int HY = 0, HX = 0;
  for (;;) {
    HY = R * T;
    HX = ((R * T + vec - 1) / vec) * vec;
    if ((TW + 2 * HX <= 256 && TH + 2 * HY <= 256) || T == 1) break;
    T = std::max(1, T - 2);
  }
  if (TW + 2 * HX > 256) TW = std::max(vec, ((256 - 2 * HX) / vec) * vec);
  if (TH + 2 * HY > 256) TH = 256 - 2 * HY;
  if (TW < vec || TH < 1 || TW + 2 * HX > 256 || TH + 2 * HY > 256)
    return fail(PSKEL_ERR_UNSUPPORTED, "mask reach %d too large for the 2D tile kernel", R);
  int LW = TW + 2 * HX, LH = TH + 2 * HY;
  while (stencil2d_smem_bytes(op, dtype, LW, LH) > static_cast<size_t>(c->smem_optin) && TH > 8) {
    TH /= 2;
    LH = TH + 2 * HY;
  }
  if (stencil2d_smem_bytes(op, dtype, LW, LH) > static_cast<size_t>(c->smem_optin))
    return fail(PSKEL_ERR_UNSUPPORTED, "2D tile does not fit in shared memory");

  Stencil2DParams p;
  memset(&p, 0, sizeof(p));
  p.W = static_cast<int>(W);
  p.H = static_cast<int>(H);
  p.pitch = pitch;
  p.ring = ring;
  p.R = R;
  p.T = T;
  p.TW = TW;
  p.TH = TH;
  p.LW = LW;
  p.LH = LH;
  p.HX = HX;
  p.HY = HY;
  p.tiles_x = static_cast<int>((W + TW - 1) / TW);
  p.tiles_y = static_cast<int>((H + TH - 1) / TH);
  p.err = c->err;
  if (op == Op2D::Linear) {
    p.nm = st.mask.size;
    for (int n = 0; n < p.nm; ++n) {
      p.off[n] = st.mask.offsets[2 * n] * LW + st.mask.offsets[2 * n + 1];
      p.wt[n] = st.mask.weights[n];
    }
  } else {
    p.K = st.diffusivity;
    p.dt = st.dt;
    p.inv_dx = st.inv_dx;
    p.u = st.wind_u;
    p.v = st.wind_v;
  }
  const int ntiles = p.tiles_x * p.tiles_y;
  const int per_sm = std::max(1, stencil2d_max_ctas_per_sm(op, dtype, p.nm, LW, LH));
  int ctas = (sched && sched->ctas > 0) ? sched->ctas : per_sm * c->sms;
  ctas = std::max(1, std::min(ctas, ntiles));

  const int64_t pitch_bytes = pitch * static_cast<int64_t>(esz);
  bool use_tma = tma_ok(in, pitch_bytes) && tma_ok(out, pitch_bytes);
  if (op == Op2D::Advect) use_tma = use_tma && tma_ok(st.wind_u, pitch_bytes) && tma_ok(st.wind_v, pitch_bytes);
  CUtensorMap m_in, m_out, m_u, m_v;
  memset(&m_in, 0, sizeof(m_in));
  memset(&m_out, 0, sizeof(m_out));
  memset(&m_u, 0, sizeof(m_u));
  memset(&m_v, 0, sizeof(m_v));
  if (use_tma) {
    const CUtensorMapDataType tt = (dtype == PSKEL_BF16) ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const uint64_t dims[2] = {static_cast<uint64_t>(W), static_cast<uint64_t>(H)};
    const uint64_t strides[1] = {static_cast<uint64_t>(pitch_bytes)};
    const uint32_t box[2] = {static_cast<uint32_t>(LW), static_cast<uint32_t>(LH)};
    cudaError_t e = encode_tmap(&m_in, tt, 2, in, dims, strides, box);
    if (e == cudaSuccess) e = encode_tmap(&m_out, tt, 2, out, dims, strides, box);
    if (e == cudaSuccess && op == Op2D::Advect) {
      e = encode_tmap(&m_u, tt, 2, const_cast<void*>(st.wind_u), dims, strides, box);
      if (e == cudaSuccess) e = encode_tmap(&m_v, tt, 2, const_cast<void*>(st.wind_v), dims, strides, box);
    }
    if (e != cudaSuccess) return cuda_fail(e, "cuTensorMapEncodeTiled");
  }
  const std::vector<int> passes = plan_passes(iters, T);
  for (size_t i = 0; i < passes.size(); ++i) {
    const bool fwd = (i % 2 == 0);
    p.src = fwd ? in : out;
    p.dst = fwd ? out : in;
    p.steps = passes[i];
    cudaError_t e = stencil2d_pass(op, dtype, use_tma, fwd ? &m_in : &m_out, fwd ? &m_out : &m_in, &m_u, &m_v, p,
                                   ctas, s);
    if (e != cudaSuccess) return cuda_fail(e, "2D stencil kernel launch");
  }
  g_last_launches2d = static_cast<int64_t>(passes.size());
  return PSKEL_OK;
}

pskel_status validate2d(const pskel_stencil* st, const void* in, const void* out, int64_t W, int64_t H, int64_t pitch,
                        int64_t iters, int* R, int* ring) {
  if (!st) return fail(PSKEL_ERR_INVALID, "stencil descriptor is NULL");
  if (!in || !out) return fail(PSKEL_ERR_INVALID, "grid buffer pointer is NULL");
  if (in == out) return fail(PSKEL_ERR_INVALID, "input and output must be distinct buffers");
  if (W <= 0 || H <= 0) return fail(PSKEL_ERR_INVALID, "grid %lld x %lld is empty", (long long)W, (long long)H);
  if (W >= (int64_t(1) << 31) || H >= (int64_t(1) << 31)) return fail(PSKEL_ERR_UNSUPPORTED, "grid side >= 2^31");
  if (pitch < W) return fail(PSKEL_ERR_INVALID, "row pitch %lld is smaller than the width", (long long)pitch);
  if (iters < 0) return fail(PSKEL_ERR_INVALID, "negative iteration count");
  switch (st->op) {
    case PSKEL_OP_LINEAR:
      if (st->dtype != PSKEL_F32 && st->dtype != PSKEL_BF16)
        return fail(PSKEL_ERR_UNSUPPORTED, "linear 2D stencil supports f32 and bf16 storage");
      if (st->mask.size > kMaxMask2D) return fail(PSKEL_ERR_UNSUPPORTED, "2D mask larger than %d entries", kMaxMask2D);
      if (pskel_status s = check_mask(st->mask, 2, true, R, ring)) return s;
      break;
    case PSKEL_OP_LIFE:
      if (st->dtype != PSKEL_U8) return fail(PSKEL_ERR_UNSUPPORTED, "Life runs on uint8 cells");
      if (pskel_status s = check_mask(st->mask, 2, false, R, ring)) return s;
      if (pskel_status s = check_life_mask(st->mask)) return s;
      break;
    case PSKEL_OP_ADVECT:
      if (st->dtype != PSKEL_F32 && st->dtype != PSKEL_BF16)
        return fail(PSKEL_ERR_UNSUPPORTED, "advection supports f32 and bf16 storage");
      if (!st->wind_u || !st->wind_v) return fail(PSKEL_ERR_INVALID, "advection wind field pointer is NULL");
      if (st->mask.size > 0) {
        if (pskel_status s = check_mask(st->mask, 2, false, R, ring)) return s;
        if (*ring < 1) return fail(PSKEL_ERR_INVALID, "advection needs a ring of at least 1");
      } else {
        *ring = 1;
      }
      *R = 1;
      break;
    default:
      return fail(PSKEL_ERR_INVALID, "unknown stencil op %d", static_cast<int>(st->op));
  }
  if (*R > 16) return fail(PSKEL_ERR_UNSUPPORTED, "mask reach %d > 16", *R);
  if (H < *ring || W < *ring) return fail(PSKEL_ERR_INVALID, "grid smaller than the mask range");
  return PSKEL_OK;
}

// ------------------------------------------------------------- 3D iterate

pskel_status validate3d(const pskel_stencil* st, const void* in, const void* out, int64_t W, int64_t H, int64_t D,
                        int64_t iters, int64_t every, int* R) {
  if (!st) return fail(PSKEL_ERR_INVALID, "stencil descriptor is NULL");
  if (!in || !out) return fail(PSKEL_ERR_INVALID, "grid buffer pointer is NULL");
  if (in == out) return fail(PSKEL_ERR_INVALID, "input and output must be distinct buffers");
  if (W <= 0 || H <= 0 || D <= 0) return fail(PSKEL_ERR_INVALID, "3D grid is empty");
  if (W >= (int64_t(1) << 31) || H >= (int64_t(1) << 31) || D >= (int64_t(1) << 31))
    return fail(PSKEL_ERR_UNSUPPORTED, "grid side >= 2^31");
  if (iters < 0) return fail(PSKEL_ERR_INVALID, "negative iteration count");
  if (every < 0) return fail(PSKEL_ERR_INVALID, "negative residual interval");
  if (st->op != PSKEL_OP_LINEAR) return fail(PSKEL_ERR_UNSUPPORTED, "3D grids support the linear mask stencil");
  if (st->dtype != PSKEL_F32 && st->dtype != PSKEL_BF16)
    return fail(PSKEL_ERR_UNSUPPORTED, "3D stencil supports f32 and bf16 storage");
  if (st->mask.size > kMaxMask3D) return fail(PSKEL_ERR_UNSUPPORTED, "3D mask larger than %d entries", kMaxMask3D);
  int ring = 0;
  if (pskel_status s = check_mask(st->mask, 3, true, R, &ring)) return s;
  if (*R > 3) return fail(PSKEL_ERR_UNSUPPORTED, "3D mask reach %d > 3", *R);
  return PSKEL_OK;
}

// The streaming 7-point kernels apply: the mask is the 7-point cross, D fills
// whole 16-byte vectors, the buffers are 16-byte aligned, and (bf16) the halo
// value is a bf16 value (the kernels hold halos in storage format).
static bool cross7_ok(const pskel_stencil& st, const void* in, const void* out, int64_t D) {
  const size_t esz = dtype_size(st.dtype);
  uint32_t hb;
  std::memcpy(&hb, &st.mask.halo_value, sizeof(hb));
  const bool halo_exact = st.dtype != PSKEL_BF16 || (hb & 0xFFFFu) == 0u;
  return stream3d_is_cross7(st.mask.offsets, st.mask.size, D, static_cast<int>(esz)) && halo_exact &&
         (reinterpret_cast<uintptr_t>(in) % 16) == 0 && (reinterpret_cast<uintptr_t>(out) % 16) == 0;
}

// Steps per pass of the 7-point cross by default, measured on GB300 (512^3,
// 50 steps): fp32 two (one HBM round trip per two steps: 844 against 787
// GCells/s at one step per launch); bf16 one (the one-step kernel is bound by
// HBM at half the bytes and runs 1179 against 1048 for two steps).
static int cross7_default_steps(pskel_dtype dt) { return dt == PSKEL_F32 ? 2 : 1; }

// Per-pass lengths of a two-step run: an even number of two-step passes and
// the rest one-step passes, so that the pass count has the parity of `iters`
// and the state ends in the buffer the step-by-step ping-pong ends in.
static std::vector<int> plan_tb2(int64_t iters) {
  std::vector<int> p;
  const int64_t twos = (iters / 2) & ~int64_t(1);
  for (int64_t i = 0; i < twos; ++i) p.push_back(2);
  for (int64_t i = 0; i < iters - 2 * twos; ++i) p.push_back(1);
  return p;
}

// h chunks of a streaming 3D launch (items of at least `min_planes` planes,
// or tile_h planes): block b takes items b, b + ctas, ..., so a launch lasts
// as long as its busiest block, which streams ceil(items / ctas) items of
// HC + `halo` planes each (the planes an item loads). The count minimising
// that, then the planes loaded in all (halo re-reads), wins. Measured on
// 512^3 heat against about four (one step) or two (two steps) items per
// block: bf16 one step 29 -> 7 chunks 1277 -> 1301 GCells/s, bf16 two steps
// 15 -> 7 chunks 1157 -> 1207, fp32 two steps 8 -> 7 chunks 1038 -> 1052
// (fp32 one step keeps 19).
static void configure_hchunks(Stencil3DParams& q, int64_t W, int64_t H, int64_t D, int esz, int64_t resident,
                              int halo, int64_t min_planes, const pskel_schedule* sched, int64_t& ctas) {
  const int64_t cols = stream3d_tma_items(static_cast<int>(W), static_cast<int>(D), 1, esz);
  int64_t chunks = 1;
  double best = 0.0;
  for (int64_t k = 1; k <= std::max<int64_t>(1, H / min_planes); ++k) {
    const int64_t hc = (H + k - 1) / k, hk = (H + hc - 1) / hc;
    const int64_t items = cols * hk, used = std::min<int64_t>(items, resident);
    const double cost = static_cast<double>((items + used - 1) / used) * static_cast<double>(hc + halo) +
                        1e-3 * static_cast<double>(items * (hc + halo)) / static_cast<double>(resident);
    if (k == 1 || cost < best) {
      best = cost;
      chunks = k;
    }
  }
  if (sched && sched->tile_h > 0) chunks = std::max<int64_t>(1, (H + sched->tile_h - 1) / sched->tile_h);
  q.HC = static_cast<int>((H + chunks - 1) / chunks);
  q.hchunks = static_cast<int>((H + q.HC - 1) / q.HC);
  const int64_t items = stream3d_tma_items(static_cast<int>(W), static_cast<int>(D), q.hchunks, esz);
  ctas = std::min<int64_t>(items, resident);
  if (sched && sched->ctas > 0) ctas = std::min<int64_t>(ctas, sched->ctas);
}

// The 7-point cross, one step per launch, planes staged by TMA: persistent
// blocks over work items of (32 vectors of d) x 16 w x HC planes, about four
// items per resident block.
static pskel_status stream3d_cross7(const pskel_stencil& st, Stencil3DParams& p, void* in, void* out, int64_t W,
                                    int64_t H, int64_t D, int64_t iters, const pskel_schedule* sched, int64_t every,
                                    double* partials_override, int64_t partials_cap, DeviceContext* c,
                                    cudaStream_t s, int steps) {
  const int dtype = static_cast<int>(st.dtype);
  const int esz = static_cast<int>(dtype_size(st.dtype));
  const std::vector<int> passes = steps == 2 ? plan_tb2(iters) : std::vector<int>(static_cast<size_t>(iters), 1);
  const bool any2 = !passes.empty() && passes.front() == 2;
  const bool any1 = !passes.empty() && passes.back() == 1;
  auto configure = [&](Stencil3DParams& q, int per_sm, int halo, int64_t min_planes, int64_t& ctas) {
    configure_hchunks(q, W, H, D, esz, static_cast<int64_t>(per_sm) * c->sms, halo, min_planes, sched, ctas);
  };
  Stencil3DParams p2 = p;
  int64_t ctas1 = 0, ctas2 = 0;
  configure(p, stream3d_tma_blocks_per_sm(dtype), 2, 8, ctas1);     // planes h0-1 .. h1
  if (any2) configure(p2, stream3d_tb2_blocks_per_sm(dtype), 4, 16, ctas2);  // h0-2 .. h1+1
  if (every > 0) {
    const int64_t need = std::max<int64_t>(any1 ? ctas1 : 0, any2 ? 2 * ctas2 : 0);
    double* part = nullptr;
    if (partials_override) {
      if (need > partials_cap)
        return fail(PSKEL_ERR_UNSUPPORTED, "residual scratch of %lld partials exceeds the fixed capacity %lld",
                    (long long)need, (long long)partials_cap);
      part = partials_override;
    } else {
      if (pskel_status q = ensure_buffer(c->partials, static_cast<size_t>(need) * sizeof(double))) return q;
      part = static_cast<double*>(c->partials.ptr);
    }
    p.partials = p2.partials = part;
  }
  // the grid as 32-bit words: a 16-byte vector is 4 words for either dtype;
  // boxes of 136 words x (16 w rows + the halo rows of the kernel) x 1 plane
  CUtensorMap maps1[2], maps2[2];
  const uint64_t dims[3] = {static_cast<uint64_t>(D) * esz / 4, static_cast<uint64_t>(W), static_cast<uint64_t>(H)};
  const uint64_t strides[2] = {static_cast<uint64_t>(D) * esz, static_cast<uint64_t>(D) * esz * W};
  const uint32_t box1[3] = {136, 18, 1};
  const uint32_t box2[3] = {136, stream3d_tb2_box_rows(), 1};
  cudaError_t e = cudaSuccess;
  if (any1) {
    e = encode_tmap(&maps1[0], CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, in, dims, strides, box1);
    if (e == cudaSuccess) e = encode_tmap(&maps1[1], CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, out, dims, strides, box1);
  }
  if (any2 && e == cudaSuccess) {
    e = encode_tmap(&maps2[0], CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, in, dims, strides, box2);
    if (e == cudaSuccess) e = encode_tmap(&maps2[1], CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, out, dims, strides, box2);
  }
  if (e != cudaSuccess) return cuda_fail(e, "cuTensorMapEncodeTiled (3D planes)");
  int64_t k = 0;
  for (size_t i = 0; i < passes.size(); ++i) {
    const bool fwd = (i % 2 == 0);
    Stencil3DParams& q = passes[i] == 2 ? p2 : p;
    q.src = fwd ? in : out;
    q.dst = fwd ? out : in;
    q.steps = passes[i];
    q.step0 = k;
    if (passes[i] == 2)
      e = stream3d_tb2_pass(dtype, &maps2[fwd ? 0 : 1], q, static_cast<int>(ctas2), s);
    else
      e = stream3d_tma_step(dtype, &maps1[fwd ? 0 : 1], q, static_cast<int>(ctas1), s);
    if (e != cudaSuccess) return cuda_fail(e, "3D stencil kernel launch");
    k += passes[i];
  }
  return PSKEL_OK;
}

// One step per launch with the streaming kernel (no temporal blocking).
// steps: 1, or 2 for the two-step 7-point kernel (the 7-point cross only).
static pskel_status stream3d(const pskel_stencil& st, void* in, void* out, int64_t W, int64_t H, int64_t D,
                             int64_t iters, int R, const pskel_schedule* sched, int64_t every, double* residuals,
                             double* partials_override, int64_t partials_cap, DeviceContext* c, cudaStream_t s,
                             int steps = 1) {
  Stencil3DParams p;
  memset(&p, 0, sizeof(p));
  p.W = static_cast<int>(W);
  p.H = static_cast<int>(H);
  p.D = static_cast<int>(D);
  p.R = R;
  p.nm = st.mask.size;
  for (int n = 0; n < p.nm; ++n) {
    p.off_h[n] = st.mask.offsets[3 * n];
    p.off_w[n] = st.mask.offsets[3 * n + 1];
    p.off_d[n] = st.mask.offsets[3 * n + 2];
    p.wt[n] = st.mask.weights[n];
  }
  p.halo = st.mask.halo_value;
  p.err = c->err;
  p.every = static_cast<int>(every);
  p.residuals = residuals;
  if (cross7_ok(st, in, out, D))
    return stream3d_cross7(st, p, in, out, W, H, D, iters, sched, every, partials_override, partials_cap, c, s, steps);
  // h chunks: a few blocks per SM slot, each marching at least 16 planes
  const int64_t cols = stream3d_ctas(static_cast<int>(W), static_cast<int>(D), 1);
  int64_t chunks = std::max<int64_t>(1, (static_cast<int64_t>(32) * c->sms + cols - 1) / cols);
  chunks = std::min<int64_t>(chunks, std::max<int64_t>(1, H / 16));
  if (sched && sched->tile_h > 0) chunks = std::max<int64_t>(1, (H + sched->tile_h - 1) / sched->tile_h);
  p.HC = static_cast<int>((H + chunks - 1) / chunks);
  p.hchunks = static_cast<int>((H + p.HC - 1) / p.HC);
  if (every > 0) {
    const int64_t need = stream3d_ctas(p.W, p.D, p.hchunks);
    if (partials_override) {
      if (need > partials_cap)
        return fail(PSKEL_ERR_UNSUPPORTED, "residual scratch of %lld partials exceeds the fixed capacity %lld",
                    (long long)need, (long long)partials_cap);
      p.partials = partials_override;
    } else {
      if (pskel_status q = ensure_buffer(c->partials, static_cast<size_t>(need) * sizeof(double))) return q;
      p.partials = static_cast<double*>(c->partials.ptr);
    }
  }
  for (int64_t k = 0; k < iters; ++k) {
    const bool fwd = (k % 2 == 0);
    p.src = fwd ? in : out;
    p.dst = fwd ? out : in;
    p.steps = 1;
    p.step0 = k;
    cudaError_t e = stream3d_step(static_cast<int>(st.dtype), p, s);
    if (e != cudaSuccess) return cuda_fail(e, "3D stencil kernel launch");
  }
  return PSKEL_OK;
}

pskel_status iterate3d(const pskel_stencil& st, void* in, void* out, int64_t W, int64_t H, int64_t D,
                              int64_t iters, int R, const pskel_schedule* sched, int64_t every, double* residuals,
                              double* partials_override, int64_t partials_cap, DeviceContext* c, cudaStream_t s) {
  const int dtype = static_cast<int>(st.dtype);
  const size_t esz = dtype_size(st.dtype);
  const int vec = static_cast<int>(16 / esz);
  const bool cross7 = cross7_ok(st, in, out, D);
  int T = (sched && sched->time_steps > 0) ? sched->time_steps : (cross7 ? cross7_default_steps(st.dtype) : 1);
  T = static_cast<int>(std::min<int64_t>(std::min(T, kMax3DSteps), std::max<int64_t>(iters, 1)));
  if (R == 0) T = 1;
  if (T == 1 || (T == 2 && cross7))
    return stream3d(st, in, out, W, H, D, iters, R, sched, every, residuals, partials_override, partials_cap, c, s,
                    T);
  int TW = (sched && sched->tile_w > 0) ? sched->tile_w : 32;
  int TD = (sched && sched->tile_d > 0) ? sched->tile_d : 64;
  TD = std::max(vec, (TD / vec) * vec);
  Stencil3DParams p;
  memset(&p, 0, sizeof(p));
  int LW = 0, LD = 0, HW = 0, HD = 0;
  size_t smem = 0;
  for (;;) {
    HW = R * T;
    HD = ((R * T + vec - 1) / vec) * vec;
    LW = TW + 2 * HW;
    LD = TD + 2 * HD;
    smem = stencil3d_smem_bytes(LW, LD, 2 * R + 1, T, esz);
    if ((smem <= static_cast<size_t>(c->smem_optin) && LD <= 256 && LW <= 256) || (T == 1 && TW <= 8)) break;
    if (T > 1) --T; else TW = std::max(1, TW / 2);
  }
  if (smem > static_cast<size_t>(c->smem_optin) || LD > 256 || LW > 256)
    return fail(PSKEL_ERR_UNSUPPORTED, "3D tile does not fit in shared memory");
  p.W = static_cast<int>(W);
  p.H = static_cast<int>(H);
  p.D = static_cast<int>(D);
  p.R = R;
  p.NP = 2 * R + 1;
  p.T = T;
  p.TW = TW;
  p.TD = TD;
  p.LW = LW;
  p.LD = LD;
  p.HW = HW;
  p.HD = HD;
  p.tiles_w = static_cast<int>((W + TW - 1) / TW);
  p.tiles_d = static_cast<int>((D + TD - 1) / TD);
  // chunks of h: enough work items for every resident CTA, each long enough
  // that the warm-up planes (steps * R per chunk) stay a small fraction
  {
    const int cols = p.tiles_w * p.tiles_d;
    const int per_sm0 = std::max(1, stencil3d_max_ctas_per_sm(smem));
    const int want = 2 * per_sm0 * c->sms;
    int chunks = std::max(1, (want + cols - 1) / cols);
    const int min_planes = std::max(16, 8 * R * T);
    chunks = static_cast<int>(std::min<int64_t>(chunks, std::max<int64_t>(1, H / min_planes)));
    if (sched && sched->tile_h > 0) chunks = static_cast<int>(std::max<int64_t>(1, (H + sched->tile_h - 1) / sched->tile_h));
    p.HC = static_cast<int>((H + chunks - 1) / chunks);
    p.hchunks = static_cast<int>((H + p.HC - 1) / p.HC);
  }
  p.nm = st.mask.size;
  for (int n = 0; n < p.nm; ++n) {
    p.off_h[n] = st.mask.offsets[3 * n];
    p.off_w[n] = st.mask.offsets[3 * n + 1];
    p.off_d[n] = st.mask.offsets[3 * n + 2];
    p.off_plane[n] = st.mask.offsets[3 * n + 1] * LD + st.mask.offsets[3 * n + 2];
    p.wt[n] = st.mask.weights[n];
  }
  p.halo = st.mask.halo_value;
  p.err = c->err;
  p.every = static_cast<int>(every);
  p.residuals = residuals;
  const int ntiles = p.tiles_w * p.tiles_d * p.hchunks;
  const int per_sm = std::max(1, stencil3d_max_ctas_per_sm(smem));
  int ctas = (sched && sched->ctas > 0) ? sched->ctas : per_sm * c->sms;
  ctas = std::max(1, std::min(ctas, ntiles));
  if (every > 0) {
    const size_t need = static_cast<size_t>(T) * ctas;
    if (partials_override) {
      if (static_cast<int64_t>(need) > partials_cap)
        return fail(PSKEL_ERR_UNSUPPORTED, "residual scratch of %zu partials exceeds the fixed capacity %lld", need,
                    (long long)partials_cap);
      p.partials = partials_override;
    } else {
      if (pskel_status q = ensure_buffer(c->partials, need * sizeof(double))) return q;
      p.partials = static_cast<double*>(c->partials.ptr);
    }
  }
  const int64_t Db = D * static_cast<int64_t>(esz);
  const bool use_tma = (reinterpret_cast<uintptr_t>(in) & 15) == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0 &&
                       (Db & 15) == 0;
  CUtensorMap m_in, m_out;
  memset(&m_in, 0, sizeof(m_in));
  memset(&m_out, 0, sizeof(m_out));
  if (use_tma) {
    const CUtensorMapDataType tt = (dtype == PSKEL_BF16) ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const uint64_t dims[3] = {static_cast<uint64_t>(D), static_cast<uint64_t>(W), static_cast<uint64_t>(H)};
    const uint64_t strides[2] = {static_cast<uint64_t>(Db), static_cast<uint64_t>(Db * W)};
    const uint32_t box[3] = {static_cast<uint32_t>(LD), static_cast<uint32_t>(LW), 1u};
    cudaError_t e = encode_tmap(&m_in, tt, 3, in, dims, strides, box);
    if (e == cudaSuccess) e = encode_tmap(&m_out, tt, 3, out, dims, strides, box);
    if (e != cudaSuccess) return cuda_fail(e, "cuTensorMapEncodeTiled (3D)");
  }
  const std::vector<int> passes = plan_passes_any(iters, T);
  int64_t done = 0;
  for (size_t i = 0; i < passes.size(); ++i) {
    const bool fwd = (i % 2 == 0);
    p.src = fwd ? in : out;
    p.dst = fwd ? out : in;
    p.steps = passes[i];
    p.step0 = done;
    cudaError_t e = stencil3d_pass(dtype, use_tma, fwd ? &m_in : &m_out, p, ctas, s);
    if (e != cudaSuccess) return cuda_fail(e, "3D stencil kernel launch");
    done += passes[i];
  }
  return PSKEL_OK;
}

}  // namespace pskel

using namespace pskel;

extern "C" {

int32_t pskel_version(void) { return 100; }

const char* pskel_last_error(void) { return g_last_error.c_str(); }

int64_t pskel_last_launches2d(void) { return g_last_launches2d; }

int32_t pskel_plan_passes(int64_t iterations, int32_t time_steps, int32_t* passes, int32_t cap) {
  const std::vector<int> p = plan_passes(iterations, time_steps);
  for (int32_t i = 0; i < cap && i < static_cast<int32_t>(p.size()); ++i) passes[i] = p[i];
  return static_cast<int32_t>(p.size());
}

pskel_status pskel_sync(void* stream) {
  clear_error();
  DeviceContext* c = nullptr;
  if (pskel_status s = get_context(&c)) return s;
  return device_sync_check(c, static_cast<cudaStream_t>(stream));
}

pskel_status pskel_iterate2d(const pskel_stencil* st, void* in, void* out, int64_t width, int64_t height,
                             int64_t pitch, int64_t iterations, const pskel_schedule* sched, void* stream) {
  clear_error();
  g_last_launches2d = 0;
  if (pitch == 0) pitch = width;
  int R = 0, ring = 0;
  if (pskel_status s = validate2d(st, in, out, width, height, pitch, iterations, &R, &ring)) return s;
  if (iterations == 0) return PSKEL_OK;
  DeviceContext* c = nullptr;
  if (pskel_status s = get_context(&c)) return s;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (st->op == PSKEL_OP_LIFE) return iterate_life(*st, in, out, width, height, pitch, iterations, ring, sched, c, s);
  return iterate_float2d(*st, in, out, width, height, pitch, iterations, R, ring, sched, c, s);
}

// Waits for a host call's copy streams on every return path, so that no copy
// touches the caller's arrays after the call has returned.
struct StreamDrain {
  cudaStream_t a, b;  // b may be null (one stream)
  ~StreamDrain() {
    cudaStreamSynchronize(a);
    if (b) cudaStreamSynchronize(b);
  }
};

// Events of one host call, destroyed when it returns.
struct EventSet {
  std::vector<cudaEvent_t> ev;
  cudaError_t make(size_t n) {
    ev.resize(n, nullptr);
    for (auto& e : ev) {
      cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
      if (r != cudaSuccess) return r;
    }
    return cudaSuccess;
  }
  ~EventSet() {
    for (auto e : ev)
      if (e) cudaEventDestroy(e);
  }
};

// The output array's ring (rows [0,r), [H-r,H), columns [0,r), [W-r,W) of the
// rows between) from host to device: read by every second step.
static cudaError_t copy_ring_h2d(const uint8_t* oh, uint8_t* od, size_t row, size_t pitch_bytes, int64_t W,
                                 int64_t H, int ring, size_t esz, cudaStream_t s) {
  if (ring <= 0) return cudaSuccess;
  const size_t r = static_cast<size_t>(std::min<int64_t>(ring, H));
  cudaError_t e = cudaMemcpy2DAsync(od, pitch_bytes, oh, row, row, r, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && H > ring) {
    const size_t top = static_cast<size_t>(H - r);
    e = cudaMemcpy2DAsync(od + top * pitch_bytes, pitch_bytes, oh + top * row, row, row, r, cudaMemcpyHostToDevice, s);
  }
  if (e == cudaSuccess && H > 2 * ring) {
    const size_t mid = static_cast<size_t>(H - 2 * ring);
    const size_t cw = std::min<size_t>(static_cast<size_t>(ring), static_cast<size_t>(W)) * esz;
    e = cudaMemcpy2DAsync(od + r * pitch_bytes, pitch_bytes, oh + r * row, row, cw, mid, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && W > ring) {
      const size_t off = static_cast<size_t>(W - ring) * esz;
      e = cudaMemcpy2DAsync(od + r * pitch_bytes + off, pitch_bytes, oh + r * row + off, row, cw, mid,
                            cudaMemcpyHostToDevice, s);
    }
  }
  return e;
}

// Host-staged Game of Life with the copies overlapped by the compute. The
// grid's rows arrive in kLifeChunks chunks (one copy stream); after chunk k
// has arrived and been packed, one persistent launch advances the first Pw
// passes over the tile rows whose inputs are there: pass p over tile rows
// below edge(p, k), edge(0, k) = the tiles whose staged rows (core + T) lie
// in the chunks so far, edge(p, k) = edge(p-1, k) - ceil(T/TH) (the
// neighbourhood a tile waits for). The middle passes run in one launch over
// every tile; the last Pw passes run as a second wavefront over chunks of
// tile rows, after each launch of which the rows it left final are unpacked
// and copied to the host (another stream) while the next launch computes.
// The launches of a run share the per-tile completion counts, so every wait
// between tiles is the single-launch kernel's; results are bit-identical.
// Measured on 8192^2, 1000 generations (copies 0.34 + 0.36 ms, compute
// 3.05 ms): 2 chunks, 4 passes per wavefront 3.55 ms per host call against
// 3.72 ms without overlap; 4 chunks 3.75 ms (the thinner bands of a round form
// a 4-pass dependency chain over few tiles and leave the GPU underused).
constexpr int kLifeChunks = 2;
constexpr int kLifeWavePasses = 4;

static pskel_status run_life_host_wavefront(const uint8_t* in_host, uint8_t* out_host, int64_t W, int64_t H,
                                            int64_t iters, int ring, int steps, DeviceContext* c, bool* used) {
  *used = false;
  int T = static_cast<int>(std::min<int64_t>(std::min(steps > 0 ? steps : kLifeDefaultSteps, kLifeBitsMaxT), iters));
  if (T > 1 && (T & 1) == 0) --T;
  const int TH = life_bits_max_tile_h(T);
  const std::vector<int> passes = plan_passes(iters, T);
  const int P = static_cast<int>(passes.size());
  const int tiles_y = static_cast<int>((H + TH - 1) / TH);
  const int tiles_x = life_bits_tiles_x(static_cast<int>(W));
  if (P < 2 || tiles_y < 4 * kLifeChunks || H >= (int64_t(1) << 30)) return PSKEL_OK;
  *used = true;
  const int q = (passes.back() - 1) / 2;
  int r = 0;
  while (r < P && passes[r] > passes.back()) ++r;
  const int dy = (T + TH - 1) / TH;
  const int Pw = std::min(kLifeWavePasses, P / 2);
  const size_t row = static_cast<size_t>(W);
  const size_t pitch_bytes = (row + 127) & ~size_t(127);
  const size_t bytes = pitch_bytes * static_cast<size_t>(H);
  if (pskel_status q2 = ensure_buffer(c->host_in, bytes)) return q2;
  if (pskel_status q2 = ensure_buffer(c->host_out, bytes)) return q2;
  const size_t plane = static_cast<size_t>(life_bits_words(static_cast<int>(W))) * static_cast<size_t>(H);
  if (pskel_status q2 = ensure_buffer(c->life_bits, 2 * plane * sizeof(uint32_t))) return q2;
  if (pskel_status q2 = ensure_buffer(c->life_sync, life_bits_sync_bytes(static_cast<int>(W), static_cast<int>(H), TH)))
    return q2;
  uint8_t* din = static_cast<uint8_t*>(c->host_in.ptr);
  uint8_t* dout = static_cast<uint8_t*>(c->host_out.ptr);
  uint32_t* X = static_cast<uint32_t*>(c->life_bits.ptr);
  uint32_t* Y = X + plane;
  const int Wi = static_cast<int>(W), Hi = static_cast<int>(H);
  const int64_t pitch = static_cast<int64_t>(pitch_bytes);
  const int64_t resident = static_cast<int64_t>(life_bits_persistent_ctas_per_sm(T)) * c->sms;
  cudaStream_t s = c->stream, s_in = c->copy_in, s_out = c->copy_out;
  StreamDrain drain{s_in, s_out};
  const int CT = (tiles_y + kLifeChunks - 1) / kLifeChunks;  // tile rows per chunk
  const int C = (tiles_y + CT - 1) / CT;
  EventSet ev;
  cudaError_t e = ev.make(2 * static_cast<size_t>(C));
  if (e != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
  auto chunk_rows = [&](int k, int64_t& r0, int64_t& r1) {
    r0 = std::min<int64_t>(H, static_cast<int64_t>(k) * CT * TH);
    r1 = (k == C - 1) ? H : std::min<int64_t>(H, static_cast<int64_t>(k + 1) * CT * TH);
  };
  // the output array's ring first: copies into the device share the copy
  // engine, and everything on the compute stream waits for this one
  e = copy_ring_h2d(out_host, dout, row, pitch_bytes, W, H, ring, 1, s);
  if (e != cudaSuccess) return cuda_fail(e, "copy output ring to device");
  for (int k = 0; k < C; ++k) {
    int64_t r0, r1;
    chunk_rows(k, r0, r1);
    e = cudaMemcpy2DAsync(din + r0 * pitch_bytes, pitch_bytes, in_host + r0 * row, row, row,
                          static_cast<size_t>(r1 - r0), cudaMemcpyHostToDevice, s_in);
    if (e == cudaSuccess) e = cudaEventRecord(ev.ev[k], s_in);
    if (e != cudaSuccess) return cuda_fail(e, "copy input rows to device");
  }
  e = life_bits_clear_sync(c->life_sync.ptr, Wi, Hi, TH, s);
  if (e == cudaSuccess) e = life_bits_pack(dout, pitch, Wi, Hi, Y, ring, true, c->err, c->sms, s);
  if (e != cudaSuccess) return cuda_fail(e, "Life set-up");
  auto launch = [&](const LifeWindow& w, int64_t items) -> cudaError_t {
    if (items <= 0) return cudaSuccess;
    const int ctas = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(resident, items)));
    return life_bits_run_window(X, Y, Wi, Hi, ring, w, q, r, T, TH, ctas, c->life_sync.ptr, c->err, s);
  };
  auto windowed = [&](int pass0, const std::vector<int>& lo, const std::vector<int>& hi, LifeWindow& w) -> int64_t {
    memset(&w, 0, sizeof(w));
    w.pass0 = pass0;
    w.np = static_cast<int>(lo.size());
    w.windowed = 1;
    for (int j = 0; j < w.np; ++j) {
      w.lo[j] = lo[j];
      w.start[j + 1] = w.start[j] + static_cast<long long>(std::max(0, hi[j] - lo[j])) * tiles_x;
    }
    return w.start[w.np];
  };
  // phase 1: the first Pw passes as the rows arrive
  std::vector<int> prev(Pw, 0);
  for (int k = 0; k < C; ++k) {
    int64_t r0, r1;
    chunk_rows(k, r0, r1);
    if ((e = cudaStreamWaitEvent(s, ev.ev[k], 0)) != cudaSuccess) return cuda_fail(e, "cudaStreamWaitEvent");
    if ((e = life_bits_pack_rows(din, pitch, Wi, Hi, X, ring, static_cast<int>(r0), static_cast<int>(r1), c->err,
                                 c->sms, s)) != cudaSuccess)
      return cuda_fail(e, "Life pack launch");
    std::vector<int> lo(Pw), hi(Pw);
    for (int p = 0; p < Pw; ++p) {
      int h;
      if (k == C - 1) {
        h = tiles_y;
      } else if (p == 0) {
        h = static_cast<int>(std::max<int64_t>(0, (r1 - T) / TH));
      } else {
        h = std::max(0, hi[p - 1] - dy);
      }
      lo[p] = prev[p];
      hi[p] = std::max(h, lo[p]);
    }
    LifeWindow w;
    const int64_t items = windowed(0, lo, hi, w);
    if ((e = launch(w, items)) != cudaSuccess) return cuda_fail(e, "Life kernel launch");
    prev = hi;
  }
  // phase 2: the middle passes over every tile
  if (P - Pw > Pw) {
    LifeWindow w;
    memset(&w, 0, sizeof(w));
    w.pass0 = Pw;
    w.np = P - 2 * Pw;
    if ((e = launch(w, static_cast<int64_t>(w.np) * tiles_x * tiles_y)) != cudaSuccess)
      return cuda_fail(e, "Life kernel launch");
  }
  // phase 3: the last Pw passes as a wavefront; final rows go back as they are done
  const int p0 = P - Pw;
  const uint32_t* fin = ((P - 1) & 1) ? X : Y;
  uint8_t* res = (P % 2 == 1) ? dout : din;  // the result buffer keeps its own ring
  std::fill(prev.begin(), prev.end(), 0);
  for (int k = 0; k < C; ++k) {
    std::vector<int> lo(Pw), hi(Pw);
    for (int p = 0; p < Pw; ++p) {
      int h;
      if (k == C - 1)
        h = tiles_y;
      else if (p == 0)
        h = std::min(tiles_y, (k + 1) * CT);
      else
        h = std::max(0, hi[p - 1] - dy);
      lo[p] = prev[p];
      hi[p] = std::max(h, lo[p]);
    }
    LifeWindow w;
    const int64_t items = windowed(p0, lo, hi, w);
    if ((e = launch(w, items)) != cudaSuccess) return cuda_fail(e, "Life kernel launch");
    const int64_t f0 = std::min<int64_t>(H, static_cast<int64_t>(lo[Pw - 1]) * TH);
    const int64_t f1 = (k == C - 1) ? H : std::min<int64_t>(H, static_cast<int64_t>(hi[Pw - 1]) * TH);
    if (f1 > f0) {
      e = life_bits_unpack_rows(fin, res, pitch, Wi, Hi, ring, static_cast<int>(f0), static_cast<int>(f1), c->sms, s);
      if (e == cudaSuccess) e = cudaEventRecord(ev.ev[C + k], s);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s_out, ev.ev[C + k], 0);
      if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(out_host + f0 * row, row, res + f0 * pitch_bytes, pitch_bytes, row,
                              static_cast<size_t>(f1 - f0), cudaMemcpyDeviceToHost, s_out);
      if (e != cudaSuccess) return cuda_fail(e, "copy result rows to host");
    }
    prev = hi;
  }
  if ((e = cudaStreamSynchronize(s_out)) != cudaSuccess) return cuda_fail(e, "kernel execution");
  return device_sync_check(c, s);
}

pskel_status pskel_run2d_host(const pskel_stencil* st, const void* in_host, void* out_host, int64_t width,
                              int64_t height, int64_t iterations, const pskel_schedule* sched) {
  clear_error();
  int R = 0, ring = 0;
  if (!in_host || !out_host) return fail(PSKEL_ERR_INVALID, "host array pointer is NULL");
  if (pskel_status s = validate2d(st, in_host, out_host, width, height, width, iterations, &R, &ring)) return s;
  if (st->op == PSKEL_OP_ADVECT && (!st->wind_u || !st->wind_v))
    return fail(PSKEL_ERR_INVALID, "advection wind field pointer is NULL");
  DeviceContext* c = nullptr;
  if (pskel_status s = get_context(&c)) return s;
  const bool default_tiles = !sched || (sched->tile_h == 0 && sched->ctas == 0);
  if (st->op == PSKEL_OP_LIFE && default_tiles && iterations > 0) {
    bool used = false;
    pskel_status q = run_life_host_wavefront(static_cast<const uint8_t*>(in_host), static_cast<uint8_t*>(out_host),
                                             width, height, iterations, ring, sched ? sched->time_steps : 0, c,
                                             &used);
    if (used || q != PSKEL_OK) return q;
  }
  const size_t esz = dtype_size(st->dtype);
  const size_t row = static_cast<size_t>(width) * esz;
  const size_t pitch_bytes = (row + 127) & ~size_t(127);
  const size_t bytes = pitch_bytes * static_cast<size_t>(height);
  const int64_t pitch = static_cast<int64_t>(pitch_bytes / esz);
  if (pskel_status s = ensure_buffer(c->host_in, bytes)) return s;
  if (pskel_status s = ensure_buffer(c->host_out, bytes)) return s;
  if (st->op == PSKEL_OP_ADVECT) {
    if (pskel_status q = ensure_buffer(c->host_u, bytes)) return q;
    if (pskel_status q = ensure_buffer(c->host_v, bytes)) return q;
  }
  // The input goes over on the compute stream; the output array's ring (many
  // short rows: its columns) and the winds go over on the copy stream at the
  // same time, and the compute stream waits for them.
  cudaStream_t s = c->stream, s_in = c->copy_in;
  StreamDrain drain{s_in, nullptr};
  EventSet ev;
  cudaError_t e = ev.make(1);
  if (e != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
  e = cudaMemcpy2DAsync(c->host_in.ptr, pitch_bytes, in_host, row, row, height, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "copy input to device");
  if (iterations >= 1 && ring > 0) {
    // The output array's ring is read by every second step and is part of the
    // result when the iteration count is odd; its interior is never read.
    e = copy_ring_h2d(static_cast<const uint8_t*>(out_host), static_cast<uint8_t*>(c->host_out.ptr), row,
                      pitch_bytes, width, height, ring, esz, s_in);
    if (e != cudaSuccess) return cuda_fail(e, "copy output ring to device");
  }
  pskel_stencil dev = *st;
  if (st->op == PSKEL_OP_ADVECT) {
    e = cudaMemcpy2DAsync(c->host_u.ptr, pitch_bytes, st->wind_u, row, row, height, cudaMemcpyHostToDevice, s_in);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(c->host_v.ptr, pitch_bytes, st->wind_v, row, row, height, cudaMemcpyHostToDevice, s_in);
    if (e != cudaSuccess) return cuda_fail(e, "copy wind fields to device");
    dev.wind_u = c->host_u.ptr;
    dev.wind_v = c->host_v.ptr;
  }
  if ((e = cudaEventRecord(ev.ev[0], s_in)) != cudaSuccess || (e = cudaStreamWaitEvent(s, ev.ev[0], 0)) != cudaSuccess)
    return cuda_fail(e, "ordering the copies before the run");
  if (pskel_status q = pskel_iterate2d(&dev, c->host_in.ptr, c->host_out.ptr, width, height, pitch, iterations, sched, s))
    return q;
  const void* result = (iterations % 2 == 1) ? c->host_out.ptr : c->host_in.ptr;
  e = cudaMemcpy2DAsync(out_host, row, result, pitch_bytes, row, height, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail(e, "copy result to host");
  return device_sync_check(c, s);
}

pskel_status pskel_iterate3d(const pskel_stencil* st, void* in, void* out, int64_t width, int64_t height, int64_t depth,
                             int64_t iterations, const pskel_schedule* sched, int64_t residual_every,
                             double* residuals, void* stream) {
  clear_error();
  int R = 0;
  if (pskel_status s = validate3d(st, in, out, width, height, depth, iterations, residual_every, &R)) return s;
  if (residual_every > 0 && iterations >= residual_every && !residuals)
    return fail(PSKEL_ERR_INVALID, "residual output pointer is NULL");
  if (iterations == 0) return PSKEL_OK;
  DeviceContext* c = nullptr;
  if (pskel_status s = get_context(&c)) return s;
  return iterate3d(*st, in, out, width, height, depth, iterations, R, sched, residual_every, residuals, nullptr, 0, c,
                   static_cast<cudaStream_t>(stream));
}

// Host-staged 3D run of the 7-point cross at one step per launch, with the
// copies overlapped by the compute. Chunk k of S planes is copied in on its
// own stream. The first Tw steps run as a wavefront over the chunks: round k
// runs, for each step t, the band of planes whose inputs are final,
// [edge(t,k-1), edge(t,k)) with edge(t,k) = (k+1)S - t (all planes for the
// last chunk). A band of step t reads step t-1 planes that this or an
// earlier round computed, and never overwrites a step t-2 plane that a later
// band still reads. The middle steps run over the whole grid; the last Tw
// steps run as a second wavefront from the complete state, and the planes
// each of its rounds leaves final go back to the host on a third stream while
// the next rounds compute. With two steps per pass (the fp32 default), the
// middle steps run as pairs of two-step passes (a pair leaves the state in
// the buffer the step-by-step run has it in). Residual steps add each band's squared-difference
// sum to the step's accumulator in launch order (deterministic), square roots
// at the end. Results equal pskel_iterate3d's bit for bit (the norms up to
// the grouping of the fp64 sums).

static bool wavefront3d_applies(const pskel_stencil& st, int64_t H, int64_t D, int64_t iters, int64_t every,
                                const pskel_schedule* sched) {
  const size_t esz = dtype_size(st.dtype);
  uint32_t hb;
  std::memcpy(&hb, &st.mask.halo_value, sizeof(hb));
  const bool halo_exact = st.dtype != PSKEL_BF16 || (hb & 0xFFFFu) == 0u;
  const bool plain = !sched || (sched->time_steps <= 2 && sched->tile_h == 0 && sched->ctas == 0);
  return plain && halo_exact && iters >= 2 && iters <= 256 && H >= 128 && (every == 0 || iters / every <= 4096) &&
         stream3d_is_cross7(st.mask.offsets, st.mask.size, D, static_cast<int>(esz));
}

static pskel_status run3d_wavefront(const pskel_stencil& st, int64_t W, int64_t H, int64_t D, int64_t iters,
                                    int64_t every, const void* in_host, void* out_host, double* residuals_host,
                                    const pskel_schedule* sched, DeviceContext* c) {
  const int dtype = static_cast<int>(st.dtype);
  const int esz = static_cast<int>(dtype_size(st.dtype));
  const size_t plane = static_cast<size_t>(W) * D * esz;
  const size_t bytes = plane * static_cast<size_t>(H);
  const int64_t nres = every > 0 ? iters / every : 0;
  if (pskel_status q = ensure_buffer(c->host_in, bytes)) return q;
  if (pskel_status q = ensure_buffer(c->host_out, bytes)) return q;
  uint8_t* A = static_cast<uint8_t*>(c->host_in.ptr);
  uint8_t* B = static_cast<uint8_t*>(c->host_out.ptr);
  const int per_sm = stream3d_tma_blocks_per_sm(dtype);
  const int64_t resident = static_cast<int64_t>(per_sm) * c->sms;
  Stencil3DParams p;
  memset(&p, 0, sizeof(p));
  p.W = static_cast<int>(W);
  p.H = static_cast<int>(H);
  p.D = static_cast<int>(D);
  p.R = 1;
  p.nm = st.mask.size;
  for (int n = 0; n < p.nm; ++n) {
    p.off_h[n] = st.mask.offsets[3 * n];
    p.off_w[n] = st.mask.offsets[3 * n + 1];
    p.off_d[n] = st.mask.offsets[3 * n + 2];
    p.wt[n] = st.mask.weights[n];
  }
  p.halo = st.mask.halo_value;
  p.err = c->err;
  double* acc = nullptr;
  // the middle steps two per pass when that is the schedule (fp32's default)
  const int ts = sched ? sched->time_steps : 0;
  const bool two = ts == 2 || (ts == 0 && cross7_default_steps(st.dtype) == 2);
  Stencil3DParams p2 = p;
  int64_t ctas2 = 0;
  if (two)
    configure_hchunks(p2, W, H, D, esz, static_cast<int64_t>(stream3d_tb2_blocks_per_sm(dtype)) * c->sms, 4, 16,
                      nullptr, ctas2);
  if (nres > 0) {
    if (pskel_status q = ensure_buffer(c->residuals, static_cast<size_t>(nres) * sizeof(double))) return q;
    if (pskel_status q = ensure_buffer(c->res_acc, static_cast<size_t>(nres) * sizeof(double))) return q;
    const int64_t need = std::max<int64_t>(resident, 2 * ctas2);
    if (pskel_status q = ensure_buffer(c->partials, static_cast<size_t>(need) * sizeof(double))) return q;
    acc = static_cast<double*>(c->res_acc.ptr);
    p.partials = p2.partials = static_cast<double*>(c->partials.ptr);
  }
  CUtensorMap maps[2], maps2[2];
  const uint64_t dims[3] = {static_cast<uint64_t>(D) * esz / 4, static_cast<uint64_t>(W), static_cast<uint64_t>(H)};
  const uint64_t strides[2] = {static_cast<uint64_t>(D) * esz, static_cast<uint64_t>(D) * esz * W};
  const uint32_t box[3] = {136, 18, 1};
  const uint32_t box2[3] = {136, stream3d_tb2_box_rows(), 1};
  cudaError_t e = encode_tmap(&maps[0], CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, A, dims, strides, box);
  if (e == cudaSuccess) e = encode_tmap(&maps[1], CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, B, dims, strides, box);
  if (two && e == cudaSuccess) e = encode_tmap(&maps2[0], CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, A, dims, strides, box2);
  if (two && e == cudaSuccess) e = encode_tmap(&maps2[1], CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, B, dims, strides, box2);
  if (e != cudaSuccess) return cuda_fail(e, "cuTensorMapEncodeTiled (3D planes)");
  const int64_t C0 = std::min<int64_t>(16, H / 64);
  const int64_t S = (H + C0 - 1) / C0;
  const int64_t C = (H + S - 1) / S;
  EventSet ev;
  if ((e = ev.make(2 * static_cast<size_t>(C) + 1)) != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
  cudaStream_t s = c->stream, s_in = c->copy_in, s_out = c->copy_out;
  StreamDrain drain{s_in, s_out};
  const uint8_t* hin = static_cast<const uint8_t*>(in_host);
  uint8_t* hout = static_cast<uint8_t*>(out_host);
  for (int64_t k = 0; k < C; ++k) {
    const int64_t h0 = k * S, h1 = std::min(H, h0 + S);
    e = cudaMemcpyAsync(A + h0 * plane, hin + h0 * plane, static_cast<size_t>(h1 - h0) * plane,
                        cudaMemcpyHostToDevice, s_in);
    if (e == cudaSuccess) e = cudaEventRecord(ev.ev[k], s_in);
    if (e != cudaSuccess) return cuda_fail(e, "copy input planes to device");
  }
  if (nres > 0 && (e = cudaMemsetAsync(acc, 0, static_cast<size_t>(nres) * sizeof(double), s)) != cudaSuccess)
    return cuda_fail(e, "cudaMemsetAsync");
  const int64_t cols = stream3d_tma_items(p.W, p.D, 1, esz);
  const uint8_t* result = (iters % 2 == 1) ? B : A;
  // one step t over planes [lo, up)
  auto step = [&](int64_t t, int64_t lo, int64_t up) -> cudaError_t {
    const int64_t band = up - lo;
    int64_t chunks = std::max<int64_t>(1, (4 * resident + cols - 1) / cols);
    chunks = std::min<int64_t>(chunks, std::max<int64_t>(1, band / 8));
    p.HC = static_cast<int>((band + chunks - 1) / chunks);
    p.hchunks = static_cast<int>((band + p.HC - 1) / p.HC);
    const int64_t ctas = std::min<int64_t>(stream3d_tma_items(p.W, p.D, p.hchunks, esz), resident);
    p.hbeg = static_cast<int>(lo);
    p.hend = static_cast<int>(up);
    const bool fwd = ((t - 1) % 2 == 0);
    p.src = fwd ? A : B;
    p.dst = fwd ? B : A;
    p.steps = 1;
    p.step0 = t - 1;
    double* slot = (nres > 0 && t % every == 0) ? acc + (t / every - 1) : nullptr;
    return stream3d_tma_band(dtype, &maps[fwd ? 0 : 1], p, static_cast<int>(ctas), slot, s);
  };
  // Band limits of a wavefront that starts from a complete state at step t0:
  // after round k, step t holds planes [0, edge(t, k)).
  auto edge = [&](int64_t t, int64_t t0, int64_t k) -> int64_t {
    if (k < 0) return 0;
    if (k == C - 1) return H;
    return std::max<int64_t>(0, std::min<int64_t>(H, (k + 1) * S - (t - t0)));
  };
  // Only the first and the last Tw steps run as (less efficient) thin bands:
  // enough steps to cover the copies, the rest as whole-grid steps. Measured
  // on 512^3 heat, 50 steps: Tw 8, 12, 16 -> 11.5, 10.6, 10.9 ms (13.8 ms with
  // no overlap).
  const int64_t Tw = std::min<int64_t>(iters / 2, 12);
  const int64_t t_last = iters - Tw;  // the closing wavefront starts from step t_last
  for (int64_t k = 0; k < C; ++k) {
    if ((e = cudaStreamWaitEvent(s, ev.ev[k], 0)) != cudaSuccess) return cuda_fail(e, "cudaStreamWaitEvent");
    for (int64_t t = 1; t <= Tw; ++t) {
      const int64_t lo = edge(t, 0, k - 1), up = edge(t, 0, k);
      if (lo < up && (e = step(t, lo, up)) != cudaSuccess) return cuda_fail(e, "3D stencil kernel launch");
    }
  }
  int64_t tm = Tw;  // steps done by the middle phase so far
  // two-step passes in pairs: the first leaves step tm+2 in the other buffer,
  // the second brings step tm+4 back to the buffer of step tm
  auto rep = [&](int64_t t) -> double* { return (nres > 0 && t % every == 0) ? acc + (t / every - 1) : nullptr; };
  for (; two && tm + 4 <= t_last; tm += 4) {
    uint8_t* X = (tm % 2 == 0) ? A : B;
    uint8_t* Y = (X == A) ? B : A;
    for (int h = 0; h < 2; ++h) {
      p2.src = h == 0 ? X : Y;
      p2.dst = h == 0 ? Y : X;
      p2.steps = 2;
      p2.step0 = tm + 2 * h;
      if ((e = stream3d_tb2_band(dtype, &maps2[p2.src == A ? 0 : 1], p2, static_cast<int>(ctas2), rep(tm + 2 * h + 1),
                                 rep(tm + 2 * h + 2), s)) != cudaSuccess)
        return cuda_fail(e, "3D stencil kernel launch");
    }
  }
  for (int64_t t = tm + 1; t <= t_last; ++t)
    if ((e = step(t, 0, H)) != cudaSuccess) return cuda_fail(e, "3D stencil kernel launch");
  for (int64_t k = 0; k < C; ++k) {
    for (int64_t t = t_last + 1; t <= iters; ++t) {
      const int64_t lo = edge(t, t_last, k - 1), up = edge(t, t_last, k);
      if (lo < up && (e = step(t, lo, up)) != cudaSuccess) return cuda_fail(e, "3D stencil kernel launch");
    }
    // planes this round left final go back while the next rounds compute
    const int64_t f0 = edge(iters, t_last, k - 1), f1 = edge(iters, t_last, k);
    if (f1 > f0) {
      if ((e = cudaEventRecord(ev.ev[C + k], s)) != cudaSuccess ||
          (e = cudaStreamWaitEvent(s_out, ev.ev[C + k], 0)) != cudaSuccess ||
          (e = cudaMemcpyAsync(hout + f0 * plane, result + f0 * plane, static_cast<size_t>(f1 - f0) * plane,
                               cudaMemcpyDeviceToHost, s_out)) != cudaSuccess)
        return cuda_fail(e, "copy result planes to host");
    }
  }
  if (nres > 0) {
    e = stream3d_finish_residuals(acc, static_cast<int>(nres), static_cast<double*>(c->residuals.ptr), s);
    if (e == cudaSuccess) e = cudaEventRecord(ev.ev[2 * C], s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s_out, ev.ev[2 * C], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(residuals_host, c->residuals.ptr, static_cast<size_t>(nres) * sizeof(double),
                          cudaMemcpyDeviceToHost, s_out);
    if (e != cudaSuccess) return cuda_fail(e, "copy residual norms to host");
  }
  if ((e = cudaStreamSynchronize(s_out)) != cudaSuccess) return cuda_fail(e, "kernel execution");
  return device_sync_check(c, s);
}

pskel_status pskel_run3d_host(const pskel_stencil* st, const void* in_host, void* out_host, int64_t width,
                              int64_t height, int64_t depth, int64_t iterations, const pskel_schedule* sched,
                              int64_t residual_every, double* residuals_host) {
  clear_error();
  int R = 0;
  if (!in_host || !out_host) return fail(PSKEL_ERR_INVALID, "host array pointer is NULL");
  if (pskel_status s = validate3d(st, in_host, out_host, width, height, depth, iterations, residual_every, &R)) return s;
  const int64_t nres = residual_every > 0 ? iterations / residual_every : 0;
  if (nres > 0 && !residuals_host) return fail(PSKEL_ERR_INVALID, "residual output pointer is NULL");
  DeviceContext* c = nullptr;
  if (pskel_status s = get_context(&c)) return s;
  if (wavefront3d_applies(*st, height, depth, iterations, residual_every, sched))
    return run3d_wavefront(*st, width, height, depth, iterations, residual_every, in_host, out_host, residuals_host,
                           sched, c);
  const size_t bytes = static_cast<size_t>(width) * height * depth * dtype_size(st->dtype);
  if (pskel_status s = ensure_buffer(c->host_in, bytes)) return s;
  if (pskel_status s = ensure_buffer(c->host_out, bytes)) return s;
  if (nres > 0)
    if (pskel_status s = ensure_buffer(c->residuals, static_cast<size_t>(nres) * sizeof(double))) return s;
  cudaStream_t s = c->stream;
  cudaError_t e = cudaMemcpyAsync(c->host_in.ptr, in_host, bytes, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "copy input to device");
  if (pskel_status q = iterate3d(*st, c->host_in.ptr, c->host_out.ptr, width, height, depth, iterations, R, sched,
                                 residual_every, static_cast<double*>(c->residuals.ptr), nullptr, 0, c, s))
    return q;
  // every cell is written each step, so the result is whole in one buffer
  const void* result = (iterations % 2 == 1) ? c->host_out.ptr : c->host_in.ptr;
  e = cudaMemcpyAsync(out_host, result, bytes, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && nres > 0)
    e = cudaMemcpyAsync(residuals_host, c->residuals.ptr, static_cast<size_t>(nres) * sizeof(double),
                        cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail(e, "copy result to host");
  return device_sync_check(c, s);
}

}  // extern "C"
