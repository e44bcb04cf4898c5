// Reference GPU runner: drives the reference's own Stencil2D::runIterativeGPU
// (PSkelStencil.hpp:1046-1097: one stencilTilingCU launch per time step,
// :572-652 with the launch of runCUDA :1764-1792, each step followed by a
// device synchronisation) on raw binary inputs, with the Game of Life and the
// weighted 2D mask written against the reference's user API
// (PSkelStencil.h:139-156), as in oracle/ref_runner.cpp.
//
// Test infrastructure only: compiled by oracle/make_ref.py with nvcc against the
// oracle's copy of the reference headers (PSKEL_CUDA) into
// oracle/_ref/pskel_ref_gpu. It measures the reference's GPU path beside the
// library; the product never runs it.
//
// Usage (raw little-endian arrays, [h][w] row-major):
//   pskel_ref_gpu life  W H ITERS BX BY IN OUTINIT RESULT
//   pskel_ref_gpu lin2d W H ITERS BX BY MASKFILE IN OUTINIT RESULT   (float32)
// BX x BY is the thread block (the reference's test scripts use 32 x 4). One
// untimed call of two steps warms the context and the module first (it reads
// only the input array, which runIterativeGPU never writes on the host). The
// timed call prints the reference's own "GPU_time" line (copies in and out and
// the step loop) and then {"wall_s": ..., "cell_updates": ...} (the whole call,
// device allocation and release included).
#include "PSkel.h"

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace PSkel;

struct LinArgs { int unused; };
struct LifeArgs { int unused; };

namespace PSkel {
// Weighted linear mask: out = w0*v0 + w1*v1 + ... in mask order (the
// reference's GPU build contracts these into FMAs where nvcc chooses to).
__parallel__ void stencilKernel(Array2D<float> in, Array2D<float> out, Mask2D<float> mask, LinArgs args, size_t h,
                                size_t w) {
  float acc = mask.getWeight(0) * mask.get(0, in, h, w);
  for (size_t n = 1; n < mask.size; ++n) acc = acc + mask.getWeight(n) * mask.get(n, in, h, w);
  out(h, w) = acc;
}

// Game of Life on the mask's neighbourhood (the rule of PSkelStencil.hpp:389-440).
__parallel__ void stencilKernel(Array2D<uint8_t> in, Array2D<uint8_t> out, Mask2D<uint8_t> mask, LifeArgs args,
                                size_t h, size_t w) {
  int s = 0;
  for (size_t n = 0; n < mask.size; ++n) s += mask.get(n, in, h, w);
  uint8_t c = in(h, w);
  out(h, w) = (s == 3 || (s == 2 && c == 1)) ? 1 : 0;
}
}  // namespace PSkel

namespace {

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

template <class S> void timed(S& st, size_t W, size_t H, size_t it, size_t bx, size_t by) {
  st.runIterativeGPU(2, bx, by);  // warm-up: context, module, first allocations
  std::fflush(stdout);
  const double t0 = now();
  st.runIterativeGPU(it, bx, by);
  const double t1 = now();
  std::fflush(stdout);
  std::printf("{\"wall_s\": %.9g, \"cell_updates\": %zu}\n", t1 - t0, W * H * it);
}

int run_life(char** a) {
  const size_t W = std::strtoull(a[0], 0, 10), H = std::strtoull(a[1], 0, 10), it = std::strtoull(a[2], 0, 10);
  const size_t bx = std::strtoull(a[3], 0, 10), by = std::strtoull(a[4], 0, 10);
  Array2D<uint8_t> in(W, H), out(W, H);
  read_into(a[5], in.hostArray, W * H);
  read_into(a[6], out.hostArray, W * H);
  int moore[8][2] = {{-1, -1}, {-1, 0}, {-1, 1}, {0, -1}, {0, 1}, {1, -1}, {1, 0}, {1, 1}};
  Mask2D<uint8_t> mask(8, moore);
  Stencil2D<Array2D<uint8_t>, Mask2D<uint8_t>, LifeArgs> st(in, out, mask, LifeArgs{0});
  timed(st, W, H, it, bx, by);
  write_from(a[7], out.hostArray, W * H);
  return 0;
}

int run_lin2d(char** a) {
  const size_t W = std::strtoull(a[0], 0, 10), H = std::strtoull(a[1], 0, 10), it = std::strtoull(a[2], 0, 10);
  const size_t bx = std::strtoull(a[3], 0, 10), by = std::strtoull(a[4], 0, 10);
  FILE* f = std::fopen(a[5], "r");
  if (!f) { std::perror(a[5]); std::exit(2); }
  int size = 0, dim = 0;
  if (std::fscanf(f, "%d %d", &size, &dim) != 2 || dim != 2 || size < 1) { std::fprintf(stderr, "bad mask\n"); std::exit(2); }
  Mask2D<float> mask(size);
  for (int n = 0; n < size; ++n) {
    int dh = 0, dw = 0;
    char buf[128];
    if (std::fscanf(f, "%d %d %127s", &dh, &dw, buf) != 3) { std::fprintf(stderr, "bad mask entry\n"); std::exit(2); }
    mask.set(n, dh, dw, static_cast<float>(std::strtod(buf, nullptr)));
  }
  std::fclose(f);
  Array2D<float> in(W, H), out(W, H);
  read_into(a[6], in.hostArray, W * H);
  read_into(a[7], out.hostArray, W * H);
  Stencil2D<Array2D<float>, Mask2D<float>, LinArgs> st(in, out, mask, LinArgs{0});
  timed(st, W, H, it, bx, by);
  write_from(a[8], out.hostArray, W * H);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  const std::string cmd = argc > 1 ? argv[1] : "";
  if (cmd == "life" && argc == 10) return run_life(argv + 2);
  if (cmd == "lin2d" && argc == 11) return run_lin2d(argv + 2);
  std::fprintf(stderr, "usage: pskel_ref_gpu life|lin2d ... (see source header)\n");
  return 2;
}
