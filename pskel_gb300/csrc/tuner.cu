// Schedule search for the 2D stencils: the candidate space, measured timings
// (the exhaustive tuner), the reference's genetic search restated (the
// analytic objective of PSkelStencil.hpp:1883-1941), schedule features for the
// MLP cost model, and the cost-model registry used by pskel_auto_schedule2d
// (runIterativeAutoGPU).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/pskel_gb300.h"
#include "capi_internal.h"
#include "kernels.h"

namespace pskel {
namespace {

bool fast_path(const pskel_stencil& st) {
  if (st.op == PSKEL_OP_ADVECT) return true;
  if (st.op != PSKEL_OP_LINEAR || st.mask.size <= 0 || !st.mask.offsets) return false;
  int R = 0;
  for (int i = 0; i < 2 * st.mask.size; ++i) R = std::max(R, std::abs(st.mask.offsets[i]));
  return R == 1 && fast2d_shape(st.mask.offsets, st.mask.size) >= 0;
}

pskel_schedule sched(int tw, int th, int T) {
  pskel_schedule s;
  s.tile_w = tw;
  s.tile_h = th;
  s.tile_d = 0;
  s.time_steps = T;
  s.ctas = 0;
  return s;
}

// SplitMix64 stream for the genetic search
struct Rng {
  uint64_t z;
  explicit Rng(uint64_t seed) : z(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
  uint64_t next() {
    z += 0x9E3779B97F4A7C15ull;
    uint64_t x = z;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
  }
  double uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
};

constexpr int kFeatures = 11;

// Tile geometry a schedule gets (the selection rules of the Life, register-
// windowed and generic 2D paths in capi.cu), for the cost-model features.
struct TileEstimate {
  int T;           // steps per pass after clamping
  int TW, TH;      // core tile
  int LW, LH;      // loaded tile (core + redundant halo)
  bool tall;       // the taller tile variant
  int64_t passes;
};

TileEstimate estimate_tiles(const pskel_stencil& st, int64_t W, int64_t H, int64_t iters, const pskel_schedule& s) {
  TileEstimate g{};
  const int64_t it = std::max<int64_t>(iters, 1);
  auto clamp_odd = [&](int T, int tmax) {
    T = static_cast<int>(std::min<int64_t>(std::min(T, tmax), it));
    if (T > 1 && (T & 1) == 0) --T;
    return std::max(T, 1);
  };
  if (st.op == PSKEL_OP_LIFE) {
    g.T = clamp_odd(s.time_steps > 0 ? s.time_steps : 15, kLifeBitsMaxT);
    const int th_max = life_bits_max_tile_h(g.T);
    g.TH = std::max(1, s.tile_h > 0 ? std::min(s.tile_h, th_max) : th_max);
    g.LH = g.TH + 2 * g.T;
    g.TW = 32 * kLifeCoreWords;  // the core words of a one-warp-wide bit-plane tile
    g.LW = 32 * (kLifeCoreWords + 2);
    g.tall = false;
  } else if (fast_path(st)) {
    const int vec = st.dtype == PSKEL_BF16 ? 8 : 4;
    const int S = s.tile_h > 64 ? 8 : 4;
    g.LW = 128;
    g.LH = 16 * S + 2;
    int T = clamp_odd(
        s.time_steps > 0 ? s.time_steps : fast2d_default_steps(st.op == PSKEL_OP_ADVECT, st.dtype, W, H), 1 << 20);
    int HX = 0;
    for (;;) {
      HX = ((T + vec - 1) / vec) * vec;
      if ((g.LW - 2 * HX >= 4 && g.LH - 2 * T >= 2) || T == 1) break;
      T -= 2;
    }
    g.T = T;
    g.TW = g.LW - 2 * HX;
    g.TH = g.LH - 2 * T;
    g.tall = S == 8;
  } else {
    int R = 1;
    if (st.mask.size > 0 && st.mask.offsets) {
      R = 0;
      for (int i = 0; i < 2 * st.mask.size; ++i) R = std::max(R, std::abs(st.mask.offsets[i]));
    }
    g.T = clamp_odd(s.time_steps > 0 ? s.time_steps : (st.op == PSKEL_OP_ADVECT ? 4 : 8), 1 << 20);
    if (R == 0) g.T = 1;
    g.TW = s.tile_w > 0 ? s.tile_w : 128;
    g.TH = s.tile_h > 0 ? s.tile_h : 64;
    g.LW = g.TW + 2 * R * g.T;
    g.LH = g.TH + 2 * R * g.T;
    g.tall = g.TH > 64;
  }
  g.TW = std::max(g.TW, 1);
  g.TH = std::max(g.TH, 1);
  g.passes = static_cast<int64_t>(plan_passes(it, g.T).size());
  return g;
}

pskel_mlp* g_model = nullptr;
bool g_model_env_tried = false;

}  // namespace
}  // namespace pskel

using namespace pskel;

extern "C" {

int32_t pskel_candidates2d(const pskel_stencil* st, int64_t width, int64_t height, int64_t iterations,
                           pskel_schedule* out, int32_t cap) {
  if (!st || width <= 0 || height <= 0) return 0;
  (void)width;
  (void)height;
  std::vector<pskel_schedule> c;
  const int64_t it = std::max<int64_t>(iterations, 1);
  if (st->op == PSKEL_OP_LIFE) {
    for (int T = 1; T <= kLifeBitsMaxT && T <= it; T += 2) c.push_back(sched(0, 0, T));
  } else if (fast_path(*st)) {
    for (int T = 1; T <= 15 && T <= it; T += 2)
      for (int th : {0, 130}) c.push_back(sched(0, th, T));
  } else {
    for (int T = 1; T <= 7 && T <= it; T += 2)
      for (int tw : {64, 128})
        for (int th : {32, 64}) c.push_back(sched(tw, th, T));
  }
  const int32_t n = static_cast<int32_t>(c.size());
  for (int32_t i = 0; i < n && i < cap && out; ++i) out[i] = c[i];
  return n;
}

pskel_status pskel_time2d(const pskel_stencil* st, void* in, void* out, int64_t width, int64_t height, int64_t pitch,
                          int64_t iterations, const pskel_schedule* scheds, int32_t n, int32_t reps, double* ms,
                          void* stream) {
  clear_error();
  if (!scheds || !ms || n <= 0 || reps <= 0) return fail(PSKEL_ERR_INVALID, "time2d: bad arguments");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  std::vector<float> t(reps);
  for (int32_t i = 0; i < n; ++i) {
    // one untimed run (first-use set-up), then `reps` timed runs; median
    if (pskel_status q = pskel_iterate2d(st, in, out, width, height, pitch, iterations, &scheds[i], stream)) {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      return q;
    }
    for (int32_t r = 0; r < reps; ++r) {
      cudaEventRecord(a, s);
      pskel_status q = pskel_iterate2d(st, in, out, width, height, pitch, iterations, &scheds[i], stream);
      cudaEventRecord(b, s);
      if (q) {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return q;
      }
      cudaEventSynchronize(b);
      cudaEventElapsedTime(&t[r], a, b);
    }
    std::sort(t.begin(), t.end());
    ms[i] = t[reps / 2];
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return pskel_sync(stream);
}

pskel_status pskel_time_batch2d(const pskel_stencil* st, void* pool, int64_t pool_bytes, int64_t width,
                                int64_t height, int64_t iterations, const pskel_schedule* scheds, int32_t n,
                                int32_t reps, double* ms, int32_t* copies_used, void* stream) {
  clear_error();
  if (!st || !pool || pool_bytes <= 0 || !scheds || !ms || n <= 0 || reps <= 0 || width <= 0 || height <= 0)
    return fail(PSKEL_ERR_INVALID, "time_batch2d: bad arguments");
  const int64_t esz = st->dtype == PSKEL_BF16 ? 2 : 4;
  const int64_t pitch = ((width * esz + 15) / 16) * 16 / esz;
  const int64_t buf = ((pitch * height * esz + 255) / 256) * 256;
  const int64_t fit = pool_bytes / (2 * buf);
  if (fit < 1) return fail(PSKEL_ERR_INVALID, "time_batch2d: the pool holds no copy of the grid");
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(pool, 0, static_cast<size_t>(std::min<int64_t>(pool_bytes, 2 * buf * fit)), s);
  if (e != cudaSuccess) return cuda_fail(e, "time_batch2d pool clear");
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  std::vector<float> t(reps);
  pskel_status q = PSKEL_OK;
  for (int32_t i = 0; i < n && q == PSKEL_OK; ++i) {
    // enough copies for two waves of tiles of the batched kernel (two CTAs
    // per SM), as many as the pool holds
    const TileEstimate g = estimate_tiles(*st, width, height, iterations, scheds[i]);
    const int64_t tiles = ((width + g.TW - 1) / g.TW) * ((height + g.TH - 1) / g.TH);
    const int64_t want = std::max<int64_t>(1, (4 * static_cast<int64_t>(sms) + tiles - 1) / tiles);
    const int64_t copies = std::min<int64_t>(want, fit);
    std::vector<pskel_batch_grid> grids(static_cast<size_t>(copies));
    for (int64_t k = 0; k < copies; ++k) {
      pskel_batch_grid& G = grids[static_cast<size_t>(k)];
      G.in = static_cast<char*>(pool) + (2 * k) * buf;
      G.out = static_cast<char*>(pool) + (2 * k + 1) * buf;
      G.width = width;
      G.height = height;
      G.pitch = pitch;
      G.iterations = iterations;
      G.schedule = scheds[i];
    }
    pskel_batch* bt = nullptr;
    q = pskel_batch_create(st, grids.data(), static_cast<int32_t>(copies), &bt);
    if (q != PSKEL_OK) break;
    q = pskel_batch_run(bt, stream);  // untimed first run
    for (int32_t r = 0; r < reps && q == PSKEL_OK; ++r) {
      cudaEventRecord(a, s);
      q = pskel_batch_run(bt, stream);
      cudaEventRecord(b, s);
      cudaEventSynchronize(b);
      cudaEventElapsedTime(&t[r], a, b);
    }
    if (q == PSKEL_OK) q = pskel_sync(stream);
    pskel_batch_destroy(bt);
    std::sort(t.begin(), t.end());
    ms[i] = t[reps / 2] / static_cast<double>(copies);
    if (copies_used) copies_used[i] = static_cast<int32_t>(copies);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return q;
}

// The reference's genetic search (solve2D/objective2D, PSkelStencil.hpp:
// 1883-1941) restated: a simple GA (GAlib 2.4.7's GASimpleGA, absent from the
// reference tree) over two 16-bit binary-to-decimal genes, tile height h in
// [1, maxHeight] and steps per tile it in [1, iterations]; sigma-truncation
// scaling, roulette-wheel selection, one-point crossover, bit-flip mutation,
// the best individual carried over. The objective is the reference's analytic
// one, (h / tileHeight) * (it * h) / (height * iterations) with
// tileHeight = min(height, 2 * it * range + h), zero when two tiles of
// width x tileHeight do not fit the memory budget -- here one CTA's shared
// memory for the 128-cell wide on-chip tile. No timing is measured.
pskel_status pskel_ga_schedule2d(const pskel_stencil* st, int64_t width, int64_t height, int64_t iterations,
                                 uint64_t seed, int32_t popsize, int32_t ngen, pskel_schedule* out, double* score) {
  clear_error();
  if (!st || !out || width <= 0 || height <= 0 || iterations <= 0 || popsize < 2 || ngen < 1)
    return fail(PSKEL_ERR_INVALID, "ga_schedule2d: bad arguments");
  int R = 1;
  if (st->mask.size > 0 && st->mask.offsets) {
    R = 0;
    for (int i = 0; i < 2 * st->mask.size; ++i) R = std::max(R, std::abs(st->mask.offsets[i]));
    R = std::max(R, 1);
  }
  const double type_size = st->dtype == PSKEL_U8 ? 1.0 : (st->dtype == PSKEL_BF16 ? 2.0 : 4.0);
  const double tile_w = st->op == PSKEL_OP_LIFE ? 256.0 : 128.0;
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || optin <= 0)
    optin = 227 * 1024;
  const double mem_free = static_cast<double>(optin);
  const double H = static_cast<double>(height), I = static_cast<double>(iterations);
  const double div = (2.0 * tile_w * H * type_size) / (mem_free * 1.1);
  const double max_h = std::max(1.0, std::ceil(H / std::max(div, 1e-12)));
  auto objective = [&](double h, double it) {
    const double tile_h = std::floor(std::min(H, 2.0 * it * R + h));  // a size_t in the reference
    if (2.0 * tile_w * tile_h * type_size > mem_free) return 0.0;
    return (h / tile_h) * ((it * h) / (H * I));
  };
  constexpr int kBits = 16;
  const uint32_t kMaxCode = (1u << kBits) - 1;
  auto decode = [&](uint32_t code, double lo, double hi) { return lo + (hi - lo) * code / kMaxCode; };
  struct Ind {
    uint32_t g[2];
    double f;
  };
  Rng rng(seed);
  std::vector<Ind> pop(popsize), nxt(popsize);
  auto eval = [&](Ind& x) { x.f = objective(decode(x.g[0], 1.0, max_h), decode(x.g[1], 1.0, I)); };
  for (auto& x : pop) {
    x.g[0] = static_cast<uint32_t>(rng.next() & kMaxCode);
    x.g[1] = static_cast<uint32_t>(rng.next() & kMaxCode);
    eval(x);
  }
  std::vector<double> fit(popsize);
  for (int gen = 0; gen < ngen; ++gen) {
    // sigma-truncation scaling: f' = max(0, f - (mean - 2 sigma))
    double mean = 0, var = 0;
    for (auto& x : pop) mean += x.f;
    mean /= popsize;
    for (auto& x : pop) var += (x.f - mean) * (x.f - mean);
    const double sigma = std::sqrt(var / std::max(1, popsize - 1));
    double total = 0;
    for (int i = 0; i < popsize; ++i) {
      fit[i] = std::max(0.0, pop[i].f - (mean - 2.0 * sigma));
      total += fit[i];
    }
    auto pick = [&]() -> const Ind& {
      if (total <= 0) return pop[rng.next() % popsize];
      double r = rng.uniform() * total;
      for (int i = 0; i < popsize; ++i) {
        r -= fit[i];
        if (r <= 0) return pop[i];
      }
      return pop[popsize - 1];
    };
    const Ind* best = &pop[0];
    for (auto& x : pop)
      if (x.f > best->f) best = &x;
    for (int i = 0; i < popsize; i += 2) {
      Ind a = pick(), b = pick();
      if (rng.uniform() < 0.6) {  // pcross
        const int cut = 1 + static_cast<int>(rng.next() % (2 * kBits - 1));
        const uint64_t mask = (cut >= 2 * kBits) ? ~0ull : ((1ull << cut) - 1);
        const uint64_t ca = (uint64_t(a.g[1]) << kBits) | a.g[0];
        const uint64_t cb = (uint64_t(b.g[1]) << kBits) | b.g[0];
        const uint64_t na = (ca & mask) | (cb & ~mask), nb = (cb & mask) | (ca & ~mask);
        a.g[0] = static_cast<uint32_t>(na & kMaxCode);
        a.g[1] = static_cast<uint32_t>((na >> kBits) & kMaxCode);
        b.g[0] = static_cast<uint32_t>(nb & kMaxCode);
        b.g[1] = static_cast<uint32_t>((nb >> kBits) & kMaxCode);
      }
      for (Ind* x : {&a, &b})
        for (int v = 0; v < 2; ++v)
          for (int bit = 0; bit < kBits; ++bit)
            if (rng.uniform() < 0.01) x->g[v] ^= (1u << bit);  // pmut
      eval(a);
      eval(b);
      nxt[i] = a;
      if (i + 1 < popsize) nxt[i + 1] = b;
    }
    // the previous generation's best replaces the new generation's worst
    int worst = 0;
    for (int i = 1; i < popsize; ++i)
      if (nxt[i].f < nxt[worst].f) worst = i;
    nxt[worst] = *best;
    pop.swap(nxt);
  }
  const Ind* best = &pop[0];
  for (auto& x : pop)
    if (x.f > best->f) best = &x;
  const double h = decode(best->g[0], 1.0, max_h), it = decode(best->g[1], 1.0, I);
  // map the reference's (tile height, steps per tile) onto this library's schedule
  int T = static_cast<int>(it);
  T = std::max(1, std::min(T, 15));
  if ((T & 1) == 0) --T;
  *out = sched(0, static_cast<int>(h), T);
  if (score) *score = best->f;
  return PSKEL_OK;
}

int32_t pskel_schedule_features2d(const pskel_stencil* st, int64_t width, int64_t height, int64_t iterations,
                                  const pskel_schedule* s, float* out) {
  // The MLP input for one candidate (kFeatures values):
  //  [log2 W, log2 H, log2 iterations, steps per pass / 8, tall-tile flag,
  //   bytes per cell / 4, op, log2 passes, log2 redundant-halo factor,
  //   log2 tiles per pass, log2 cell updates including redundant ones]
  if (!st || !s || !out) return 0;
  const TileEstimate g = estimate_tiles(*st, width, height, iterations, *s);
  const double it = static_cast<double>(std::max<int64_t>(iterations, 1));
  const double esz = st->dtype == PSKEL_U8 ? 1.0 : (st->dtype == PSKEL_BF16 ? 2.0 : 4.0);
  const double redundancy = (static_cast<double>(g.LW) * g.LH) / (static_cast<double>(g.TW) * g.TH);
  const double tiles = std::ceil(static_cast<double>(width) / g.TW) * std::ceil(static_cast<double>(height) / g.TH);
  out[0] = static_cast<float>(std::log2(static_cast<double>(width)));
  out[1] = static_cast<float>(std::log2(static_cast<double>(height)));
  out[2] = static_cast<float>(std::log2(it));
  out[3] = static_cast<float>(g.T) / 8.0f;
  out[4] = g.tall ? 1.0f : 0.0f;
  out[5] = static_cast<float>(esz) / 4.0f;
  out[6] = static_cast<float>(st->op);
  out[7] = static_cast<float>(std::log2(std::max(1.0, static_cast<double>(g.passes))));
  out[8] = static_cast<float>(std::log2(redundancy));
  out[9] = static_cast<float>(std::log2(tiles));
  out[10] = static_cast<float>(std::log2(static_cast<double>(width) * height * it * redundancy));
  return kFeatures;
}

pskel_status pskel_set_cost_model(pskel_mlp* m) {
  clear_error();
  g_model = m;
  g_model_env_tried = true;
  return PSKEL_OK;
}

pskel_status pskel_mlp_save(const pskel_mlp* m, const char* path) {
  clear_error();
  if (!m || !path) return fail(PSKEL_ERR_INVALID, "mlp_save: NULL argument");
  const int64_t n = pskel_mlp_num_params(m);
  std::vector<float> p(static_cast<size_t>(n));
  if (pskel_status q = pskel_mlp_get_params(m, p.data())) return q;
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(PSKEL_ERR_INVALID, "mlp_save: cannot open %s", path);
  int32_t hdr[4] = {0x4C504D50 /* "PMLP" */, 0, 0, 0};
  // shape is recovered from the parameter count and the stored dims
  pskel_mlp_shape(m, &hdr[1], &hdr[2], &hdr[3]);
  std::fwrite(hdr, sizeof(hdr), 1, f);
  std::fwrite(p.data(), sizeof(float), p.size(), f);
  std::fclose(f);
  return PSKEL_OK;
}

pskel_status pskel_mlp_load(const char* path, pskel_mlp** out) {
  clear_error();
  if (!path || !out) return fail(PSKEL_ERR_INVALID, "mlp_load: NULL argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(PSKEL_ERR_INVALID, "mlp_load: cannot open %s", path);
  int32_t hdr[4];
  if (std::fread(hdr, sizeof(hdr), 1, f) != 1 || hdr[0] != 0x4C504D50) {
    std::fclose(f);
    return fail(PSKEL_ERR_INVALID, "mlp_load: %s is not a cost-model file", path);
  }
  pskel_mlp* m = nullptr;
  if (pskel_status q = pskel_mlp_create(hdr[1], hdr[2], hdr[3], 0, &m)) {
    std::fclose(f);
    return q;
  }
  std::vector<float> p(static_cast<size_t>(pskel_mlp_num_params(m)));
  const size_t got = std::fread(p.data(), sizeof(float), p.size(), f);
  std::fclose(f);
  if (got != p.size()) {
    pskel_mlp_destroy(m);
    return fail(PSKEL_ERR_INVALID, "mlp_load: %s is truncated", path);
  }
  if (pskel_status q = pskel_mlp_set_params(m, p.data())) {
    pskel_mlp_destroy(m);
    return q;
  }
  *out = m;
  return PSKEL_OK;
}

pskel_status pskel_auto_schedule2d(const pskel_stencil* st, int64_t width, int64_t height, int64_t iterations,
                                   pskel_schedule* out) {
  clear_error();
  if (!st || !out) return fail(PSKEL_ERR_INVALID, "auto_schedule2d: NULL argument");
  *out = sched(0, 0, 0);
  if (!g_model_env_tried) {
    g_model_env_tried = true;
    if (const char* path = std::getenv("PSKEL_COST_MODEL")) {
      pskel_mlp* m = nullptr;
      if (pskel_mlp_load(path, &m) == PSKEL_OK) g_model = m;
      clear_error();
    }
  }
  if (!g_model) return PSKEL_OK;  // the library's default schedule
  pskel_schedule cand[64];
  const int32_t n = std::min<int32_t>(64, pskel_candidates2d(st, width, height, iterations, cand, 64));
  if (n <= 0) return PSKEL_OK;
  std::vector<float> x(static_cast<size_t>(n) * kFeatures), y(n);
  for (int32_t i = 0; i < n; ++i)
    pskel_schedule_features2d(st, width, height, iterations, &cand[i], &x[static_cast<size_t>(kFeatures) * i]);
  if (pskel_status q = pskel_mlp_predict(g_model, x.data(), n, y.data())) return q;
  int32_t best = 0;
  for (int32_t i = 1; i < n; ++i)
    if (y[i] < y[best]) best = i;
  *out = cand[best];
  return PSKEL_OK;
}

}  // extern "C"
