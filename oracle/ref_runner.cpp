// Reference runner: drives the reference's own Stencil2D/Stencil3D::runIterativeCPU
// (PSkelStencil.hpp:880-938, OpenMP drivers :2197-2257 and :2104-2113) on raw
// binary inputs, with the stencil functors this project defines for its
// workloads written against the reference's user API (PSkelStencil.h:139-156).
//
// Test infrastructure only: compiled by oracle/make_ref.py against a copy of the
// reference headers into oracle/_ref/pskel_ref. The product never runs it.
//
// Usage (all arrays raw little-endian, row-major, the reference's layouts:
// 2D [h][w], 3D [h][w][d] with d fastest, PSkelArray.hpp:349-352,658-677):
//   pskel_ref lin2d  f32|f64|bf16 W H ITERS THREADS MASKFILE IN OUTINIT RESULT
//   pskel_ref life   W H ITERS THREADS IN OUTINIT RESULT
//   pskel_ref advect f32|f64|bf16 W H ITERS THREADS K DT INVDX IN OUTINIT U V RESULT
//   pskel_ref lin3d  f32|f64|bf16 W H D ITERS THREADS MASKFILE HALO IN OUTINIT RESULT [EVERY RESFILE]
// f64 reads and writes doubles; bf16 reads and writes 16-bit bfloat patterns.
// MASKFILE: "size dim" then per entry "dh dw [dd] weight" (weight may be hex-float).
// lin3d with EVERY>0 also writes the FP64 residual norms ||u_k - u_{k-1}||_2 at
// k = EVERY, 2*EVERY, ... (one double each) to RESFILE.
#include "PSkel.h"

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace PSkel;

// bfloat16 storage type: conversions round to nearest even (NaN kept quiet).
struct bf16 {
  uint16_t bits;
  bf16() : bits(0) {}
  template <class V> explicit bf16(V v) { bits = from_float(static_cast<float>(v)); }
  operator float() const {
    uint32_t u = static_cast<uint32_t>(bits) << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
  }
  static uint16_t from_float(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7f800000u) == 0x7f800000u && (u & 0x007fffffu)) return static_cast<uint16_t>((u >> 16) | 0x40);
    u += 0x7fffu + ((u >> 16) & 1u);
    return static_cast<uint16_t>(u >> 16);
  }
};

template <class T> struct Compute { typedef float type; };
template <> struct Compute<double> { typedef double type; };

struct LinArgs { int unused; };
struct LifeArgs { int unused; };
template <class T> struct AdvArgs {
  Array2D<T> wind_x, wind_y;
  typename Compute<T>::type K, dt, inv_dx;
};

namespace PSkel {
// Weighted linear mask: out = w0*v0 + w1*v1 + ... in mask order, no FMA.
template <class T, class M>
__parallel__ void stencilKernel(Array2D<T> in, Array2D<T> out, Mask2D<M> mask, LinArgs args, size_t h, size_t w) {
  typedef typename Compute<T>::type C;
  C acc = static_cast<C>(mask.getWeight(0)) * static_cast<C>(mask.get(0, in, h, w));
  for (size_t n = 1; n < mask.size; ++n)
    acc = acc + static_cast<C>(mask.getWeight(n)) * static_cast<C>(mask.get(n, in, h, w));
  out(h, w) = static_cast<T>(acc);
}

// Game of Life on the mask's neighbourhood (the rule of PSkelStencil.hpp:389-440).
__parallel__ void stencilKernel(Array2D<uint8_t> in, Array2D<uint8_t> out, Mask2D<uint8_t> mask, LifeArgs args,
                                size_t h, size_t w) {
  int s = 0;
  for (size_t n = 0; n < mask.size; ++n) s += mask.get(n, in, h, w);
  uint8_t c = in(h, w);
  out(h, w) = (s == 3 || (s == 2 && c == 1)) ? 1 : 0;
}

// Upwind advection + diffusion, the arithmetic of PSkelStencil.hpp:347-387 with
// the diffusivity, time step and 1/dx as parameters and per-cell winds.
template <class T, class M>
__parallel__ void stencilKernel(Array2D<T> in, Array2D<T> out, Mask2D<M> mask, AdvArgs<T> args, size_t h, size_t w) {
  typedef typename Compute<T>::type C;
  C c = static_cast<C>(in(h, w));
  C n = static_cast<C>(in(h - 1, w));
  C e = static_cast<C>(in(h, w + 1));
  C wv = static_cast<C>(in(h, w - 1));
  C s = static_cast<C>(in(h + 1, w));
  C sum = C(4) * c - (((n + e) + wv) + s);
  C xw = static_cast<C>(args.wind_x(h, w));
  C yw = static_cast<C>(args.wind_y(h, w));
  int xf = (xw > 0) ? 1 : -1;
  int yf = (yw > 0) ? 1 : -1;
  C cvy = static_cast<C>(yf) * yw;
  C cvx = static_cast<C>(xf) * xw;
  C nbx = static_cast<C>(in(h, w + xf));
  C nby = static_cast<C>(in(h + yf, w));
  C temp_wind = (-cvx * ((c - nbx) * args.inv_dx)) - (cvy * ((c - nby) * args.inv_dx));
  C cond = ((-args.K) * (sum * C(0.25))) * args.dt;
  C result = c + cond;
  out(h, w) = static_cast<T>(result + temp_wind * args.dt);
}

// Weighted linear 3D mask; out-of-range neighbours read the mask halo value
// through Mask3D::get (PSkelMask.hpp:186-199).
template <class T, class M>
__parallel__ void stencilKernel(Array3D<T> in, Array3D<T> out, Mask3D<M> mask, LinArgs args, size_t h, size_t w,
                                size_t d) {
  typedef typename Compute<T>::type C;
  C acc = static_cast<C>(mask.getWeight(0)) * static_cast<C>(mask.get(0, in, h, w, d));
  for (size_t n = 1; n < mask.size; ++n)
    acc = acc + static_cast<C>(mask.getWeight(n)) * static_cast<C>(mask.get(n, in, h, w, d));
  out(h, w, d) = static_cast<T>(acc);
}
}  // namespace PSkel

namespace {

struct MaskSpec {
  int size = 0, dim = 0;
  std::vector<int> off;
  std::vector<double> wt;
};

MaskSpec read_mask(const char* path) {
  MaskSpec m;
  FILE* f = std::fopen(path, "r");
  if (!f) { std::perror(path); std::exit(2); }
  if (std::fscanf(f, "%d %d", &m.size, &m.dim) != 2) { std::fprintf(stderr, "bad mask header\n"); std::exit(2); }
  for (int n = 0; n < m.size; ++n) {
    for (int k = 0; k < m.dim; ++k) {
      int o;
      if (std::fscanf(f, "%d", &o) != 1) { std::fprintf(stderr, "bad mask offset\n"); std::exit(2); }
      m.off.push_back(o);
    }
    char buf[128];
    if (std::fscanf(f, "%127s", buf) != 1) { std::fprintf(stderr, "bad mask weight\n"); std::exit(2); }
    m.wt.push_back(std::strtod(buf, nullptr));
  }
  std::fclose(f);
  return m;
}

template <class T> void read_into(const char* path, T* dst, size_t n) {
  FILE* f = std::fopen(path, "rb");
  if (!f) { std::perror(path); std::exit(2); }
  if (std::fread(dst, sizeof(T), n, f) != n) { std::fprintf(stderr, "short read %s\n", path); std::exit(2); }
  std::fclose(f);
}

template <class T> void write_from(const char* path, const T* src, size_t n) {
  FILE* f = std::fopen(path, "wb");
  if (!f) { std::perror(path); std::exit(2); }
  if (std::fwrite(src, sizeof(T), n, f) != n) { std::fprintf(stderr, "short write %s\n", path); std::exit(2); }
  std::fclose(f);
}

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void report(double t0, double t1, size_t cells, size_t iters) {
  std::printf("{\"wall_s\": %.9g, \"cell_updates\": %zu}\n", t1 - t0, cells * iters);
}

template <class T, class M> int run_lin2d(char** a) {
  size_t W = std::strtoull(a[0], 0, 10), H = std::strtoull(a[1], 0, 10);
  size_t it = std::strtoull(a[2], 0, 10), th = std::strtoull(a[3], 0, 10);
  MaskSpec ms = read_mask(a[4]);
  Array2D<T> in(W, H), out(W, H);
  read_into(a[5], in.hostArray, W * H);
  read_into(a[6], out.hostArray, W * H);
  Mask2D<M> mask(ms.size);
  for (int n = 0; n < ms.size; ++n) mask.set(n, ms.off[2 * n], ms.off[2 * n + 1], M(ms.wt[n]));
  Stencil2D<Array2D<T>, Mask2D<M>, LinArgs> st(in, out, mask, LinArgs{0});
  double t0 = now();
  st.runIterativeCPU(it, th);
  report(t0, now(), W * H, it);
  write_from(a[7], out.hostArray, W * H);
  return 0;
}

int run_life(char** a) {
  size_t W = std::strtoull(a[0], 0, 10), H = std::strtoull(a[1], 0, 10);
  size_t it = std::strtoull(a[2], 0, 10), th = std::strtoull(a[3], 0, 10);
  Array2D<uint8_t> in(W, H), out(W, H);
  read_into(a[4], in.hostArray, W * H);
  read_into(a[5], out.hostArray, W * H);
  int moore[8][2] = {{-1, -1}, {-1, 0}, {-1, 1}, {0, -1}, {0, 1}, {1, -1}, {1, 0}, {1, 1}};
  Mask2D<uint8_t> mask(8, moore);
  Stencil2D<Array2D<uint8_t>, Mask2D<uint8_t>, LifeArgs> st(in, out, mask, LifeArgs{0});
  double t0 = now();
  st.runIterativeCPU(it, th);
  report(t0, now(), W * H, it);
  write_from(a[6], out.hostArray, W * H);
  return 0;
}

template <class T, class M> int run_advect(char** a) {
  typedef typename Compute<T>::type C;
  size_t W = std::strtoull(a[0], 0, 10), H = std::strtoull(a[1], 0, 10);
  size_t it = std::strtoull(a[2], 0, 10), th = std::strtoull(a[3], 0, 10);
  float K = std::strtof(a[4], 0), dt = std::strtof(a[5], 0), inv_dx = std::strtof(a[6], 0);
  Array2D<T> in(W, H), out(W, H);
  AdvArgs<T> args;
  args.wind_x = Array2D<T>(W, H);
  args.wind_y = Array2D<T>(W, H);
  args.K = static_cast<C>(K);
  args.dt = static_cast<C>(dt);
  args.inv_dx = static_cast<C>(inv_dx);
  read_into(a[7], in.hostArray, W * H);
  read_into(a[8], out.hostArray, W * H);
  read_into(a[9], args.wind_x.hostArray, W * H);
  read_into(a[10], args.wind_y.hostArray, W * H);
  Mask2D<M> mask(4);
  mask.set(0, -1, 0, M(1)); mask.set(1, 0, 1, M(1)); mask.set(2, 0, -1, M(1)); mask.set(3, 1, 0, M(1));
  Stencil2D<Array2D<T>, Mask2D<M>, AdvArgs<T> > st(in, out, mask, args);
  double t0 = now();
  st.runIterativeCPU(it, th);
  report(t0, now(), W * H, it);
  write_from(a[11], out.hostArray, W * H);
  return 0;
}

template <class T> double diff_norm(const T* a, const T* b, size_t n) {
  double s = 0.0;
  for (size_t i = 0; i < n; ++i) {
    double d = static_cast<double>(static_cast<typename Compute<T>::type>(a[i])) -
               static_cast<double>(static_cast<typename Compute<T>::type>(b[i]));
    s += d * d;
  }
  return std::sqrt(s);
}

template <class T, class M> int run_lin3d(int argc, char** a) {
  size_t W = std::strtoull(a[0], 0, 10), H = std::strtoull(a[1], 0, 10), D = std::strtoull(a[2], 0, 10);
  size_t it = std::strtoull(a[3], 0, 10), th = std::strtoull(a[4], 0, 10);
  MaskSpec ms = read_mask(a[5]);
  double halo = std::strtod(a[6], 0);
  size_t every = argc > 11 ? std::strtoull(a[10], 0, 10) : 0;
  size_t N = W * H * D;
  Array3D<T> A(W, H, D), B(W, H, D);
  read_into(a[7], A.hostArray, N);
  read_into(a[8], B.hostArray, N);
  Mask3D<M> mask(ms.size, M(halo));
  for (int n = 0; n < ms.size; ++n)
    mask.set(n, ms.off[3 * n], ms.off[3 * n + 1], ms.off[3 * n + 2], M(ms.wt[n]));
  std::vector<double> norms;
  double t0 = now();
  if (every == 0) {
    Stencil3D<Array3D<T>, Mask3D<M>, LinArgs> st(A, B, mask, LinArgs{0});
    st.runIterativeCPU(it, th);
  } else {
    // Run in chunks so the state before each reporting step is observable. The
    // ping-pong of runIterativeCPU is reproduced by swapping the array roles.
    Array3D<T> cur = A, nxt = B;  // cur holds the current state
    size_t done = 0;
    while (done < it) {
      size_t k = it - done;
      size_t next_report = (done / every + 1) * every;
      if (next_report <= it && next_report - done < k) k = next_report - done;
      if (k > 1) {
        Stencil3D<Array3D<T>, Mask3D<M>, LinArgs> st(cur, nxt, mask, LinArgs{0});
        st.runIterativeCPU(k - 1, th);
        if ((k - 1) % 2 == 1) std::swap(cur, nxt);  // odd: result in nxt
      }
      Stencil3D<Array3D<T>, Mask3D<M>, LinArgs> st1(cur, nxt, mask, LinArgs{0});
      st1.runIterativeCPU(1, th);
      std::swap(cur, nxt);
      done += k;
      if (done % every == 0) norms.push_back(diff_norm(cur.hostArray, nxt.hostArray, N));
    }
    if (cur.hostArray != B.hostArray) std::memcpy(B.hostArray, cur.hostArray, N * sizeof(T));
  }
  report(t0, now(), N, it);
  write_from(a[9], B.hostArray, N);
  if (every) write_from(a[11], norms.data(), norms.size());
  return 0;
}

void usage() {
  std::fprintf(stderr, "usage: pskel_ref lin2d|life|advect|lin3d ... (see source header)\n");
  std::exit(2);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) usage();
  std::string cmd = argv[1];
  if (cmd == "life") {
    if (argc != 9) usage();
    return run_life(argv + 2);
  }
  if (argc < 3) usage();
  std::string dt = argv[2];
  char** a = argv + 3;
  int na = argc - 3;
  if (cmd == "lin2d") {
    if (na != 8) usage();
    if (dt == "f32") return run_lin2d<float, float>(a);
    if (dt == "f64") return run_lin2d<double, double>(a);
    if (dt == "bf16") return run_lin2d<bf16, bf16>(a);
  } else if (cmd == "advect") {
    if (na != 12) usage();
    if (dt == "f32") return run_advect<float, float>(a);
    if (dt == "f64") return run_advect<double, double>(a);
    if (dt == "bf16") return run_advect<bf16, bf16>(a);
  } else if (cmd == "lin3d") {
    if (na != 10 && na != 12) usage();
    if (dt == "f32") return run_lin3d<float, float>(na + 1, a);
    if (dt == "f64") return run_lin3d<double, double>(na + 1, a);
    if (dt == "bf16") return run_lin3d<bf16, float>(na + 1, a);
  }
  usage();
  return 2;
}
