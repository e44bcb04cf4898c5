// A PSkel application written against the reference's API, built on the
// GB300 drop-in headers. Used by tests/test_dropin_gpu.py.
//
//   dropin_app SCENARIO W H D ITERS IN OUTINIT RESULT [RESIDUALS]
//
// Grids are raw files in the reference's layouts; D is 1 for 2D scenarios.
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "PSkel.h"
#include "PSkelMap.h"

using namespace PSkel;

struct JacobiLib : LinearStencil {};
struct JacobiUser {
  int unused;
};
struct LifeLib : LifeStencil {};
struct LifeUser {
  int unused;
};
struct HeatLib : LinearStencil {};
struct HeatUser {
  int unused;
};

namespace PSkel {
// weighted sum in mask order (the linear stencil's definition)
__parallel__ void stencilKernel(Array2D<float> in, Array2D<float> out, Mask2D<float> mask, JacobiLib, size_t h,
                                size_t w) {
  float acc = mask.getWeight(0) * mask.get(0, in, h, w);
  for (size_t n = 1; n < mask.size; ++n) acc = acc + mask.getWeight(n) * mask.get(n, in, h, w);
  out(h, w) = acc;
}
__parallel__ void stencilKernel(Array2D<float> in, Array2D<float> out, Mask2D<float> mask, JacobiUser, size_t h,
                                size_t w) {
  float acc = mask.getWeight(0) * mask.get(0, in, h, w);
  for (size_t n = 1; n < mask.size; ++n) acc = acc + mask.getWeight(n) * mask.get(n, in, h, w);
  out(h, w) = acc;
}
__parallel__ void stencilKernel(Array2D<uint8_t> in, Array2D<uint8_t> out, Mask2D<uint8_t> mask, LifeUser, size_t h,
                                size_t w) {
  int s = 0;
  for (size_t n = 0; n < mask.size; ++n) s += mask.get(n, in, h, w);
  const uint8_t c = in(h, w);
  out(h, w) = (s == 3 || (s == 2 && c == 1)) ? 1 : 0;
}
__parallel__ void stencilKernel(Array2D<uint8_t> in, Array2D<uint8_t> out, Mask2D<uint8_t> mask, LifeLib, size_t h,
                                size_t w) {
  stencilKernel(in, out, mask, LifeUser{0}, h, w);
}
__parallel__ void stencilKernel(Array3D<float> in, Array3D<float> out, Mask3D<float> mask, HeatUser, size_t h,
                                size_t w, size_t d) {
  float acc = mask.getWeight(0) * mask.get(0, in, h, w, d);
  for (size_t n = 1; n < mask.size; ++n) acc = acc + mask.getWeight(n) * mask.get(n, in, h, w, d);
  out(h, w, d) = acc;
}
__parallel__ void stencilKernel(Array3D<float> in, Array3D<float> out, Mask3D<float> mask, HeatLib, size_t h, size_t w,
                                size_t d) {
  stencilKernel(in, out, mask, HeatUser{0}, h, w, d);
}
// 2D functor reading a per-cell coefficient from an Args2D field (pinned host
// memory mapped into the device): out = c + k * (((n + s) + (w + e)) - 4c)
struct CoefArgs {
  Args2D<float> coef;
};
__parallel__ void stencilKernel(Array2D<float> in, Array2D<float> out, Mask2D<float> mask, CoefArgs a, size_t h,
                                size_t w) {
  const float c = in(h, w);
  const float sum = (mask.get(0, in, h, w) + mask.get(1, in, h, w)) + (mask.get(2, in, h, w) + mask.get(3, in, h, w));
  out(h, w) = c + a.coef(static_cast<int>(w), static_cast<int>(h)) * (sum - 4.0f * c);
}
// 1D stencil: weighted sum over a 1D mask, halo value outside the array
struct Smooth1D {
  int unused;
};
__parallel__ void stencilKernel(Array<float> in, Array<float> out, Mask<float> mask, Smooth1D, size_t i) {
  float acc = mask.getWeight(0) * mask.get(0, in, i);
  for (size_t n = 1; n < mask.size; ++n) acc = acc + mask.getWeight(n) * mask.get(n, in, i);
  out(i) = acc;
}
// Map skeleton: an affine map out = a * in + b (product then sum, rounded each)
struct Affine {
  float a, b;
};
__parallel__ void mapKernel(Array<float> in, Array<float> out, Affine g, size_t i) { out(i) = g.a * in(i) + g.b; }
__parallel__ void mapKernel(Array2D<float> in, Array2D<float> out, Affine g, size_t h, size_t w) {
  out(h, w) = g.a * in(h, w) + g.b;
}
__parallel__ void mapKernel(Array3D<float> in, Array3D<float> out, Affine g, size_t h, size_t w, size_t d) {
  out(h, w, d) = g.a * in(h, w, d) + g.b;
}
}  // namespace PSkel

template <class T>
static void read_raw(const char* path, T* dst, size_t n) {
  FILE* f = std::fopen(path, "rb");
  if (!f || std::fread(dst, sizeof(T), n, f) != n) {
    std::fprintf(stderr, "cannot read %s\n", path);
    std::exit(2);
  }
  std::fclose(f);
}
template <class T>
static void write_raw(const char* path, const T* src, size_t n) {
  FILE* f = std::fopen(path, "wb");
  if (!f || std::fwrite(src, sizeof(T), n, f) != n) {
    std::fprintf(stderr, "cannot write %s\n", path);
    std::exit(2);
  }
  std::fclose(f);
}

static Mask2D<float> jacobi_mask() {
  Mask2D<float> m(4);
  m.set(0, -1, 0, 0.25f);
  m.set(1, 1, 0, 0.25f);
  m.set(2, 0, -1, 0.25f);
  m.set(3, 0, 1, 0.25f);
  return m;
}

static Mask3D<float> heat_mask(float halo) {
  Mask3D<float> m(7, halo);
  const int off[7][3] = {{0, 0, 0}, {-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
  for (int n = 0; n < 7; ++n) m.set(n, off[n][0], off[n][1], off[n][2], n == 0 ? 0.25f : 0.125f);
  return m;
}

int main(int argc, char** argv) {
  if (argc < 9) {
    std::fprintf(stderr, "usage: dropin_app SCENARIO W H D ITERS IN OUTINIT RESULT [RESIDUALS]\n");
    return 2;
  }
  const std::string sc = argv[1];
  const size_t W = std::strtoull(argv[2], 0, 10), H = std::strtoull(argv[3], 0, 10), D = std::strtoull(argv[4], 0, 10);
  const size_t it = std::strtoull(argv[5], 0, 10);
  const char *fin = argv[6], *fout = argv[7], *fres = argv[8];

  if (sc == "map1d_time" || sc == "stencil1d_time") {
    // Throughput through the public API: W cells, runIterativeGPU(it / 100)
    // and runIterativeGPU(it) timed on the host (each call copies the array in
    // and the result out); the difference of the two, divided by the
    // difference of the iteration counts, is the time of one iteration on the
    // device. Prints one JSON line: microseconds and GB/s per iteration (8
    // bytes per cell: one read, one write).
    Array<float> in(W), out(W);
    for (size_t i = 0; i < W; ++i) {
      in.hostArray[i] = static_cast<float>(i % 1000) * 0.001f;
      out.hostArray[i] = 0.5f;
    }
    Mask<float> mask(5, 0.5f);
    const int off[5] = {-2, -1, 0, 1, 3};
    const float wt[5] = {0.125f, 0.25f, 0.3f, 0.2f, 0.125f};
    for (int n = 0; n < 5; ++n) mask.set(n, off[n], wt[n]);
    Map<Array<float>, Affine> m(in, out, Affine{0.75f, 0.125f});
    Stencil<Array<float>, Mask<float>, Smooth1D> st(in, out, mask, Smooth1D{0});
    const bool is_map = sc == "map1d_time";
    auto run = [&](size_t n) -> double {
      const auto t0 = std::chrono::steady_clock::now();
      if (is_map)
        m.runIterativeGPU(n, 0);
      else
        st.runIterativeGPU(n, 0, 0);
      return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    };
    const size_t it1 = it / 100 > 0 ? it / 100 : 1;
    run(2);  // warm-up
    const double t1 = run(it1), t2 = run(it);
    const double us = (t2 - t1) / static_cast<double>(it - it1) * 1e6;
    std::printf("{\"scenario\": \"%s\", \"cells\": %zu, \"iterations\": [%zu, %zu], \"seconds\": [%.6f, %.6f], "
                "\"us_per_iteration\": %.3f, \"GBps\": %.1f}\n",
                is_map ? "map1d" : "stencil1d", W, it1, it, t1, t2, us, 8.0 * static_cast<double>(W) / us * 1e-3);
    return it > it1 ? 0 : 3;
  }
  if (sc == "coef_time") {
    // The Args2D functor (a coefficient per cell read from mapped pinned host
    // memory, as the reference keeps Args fields) on W x H cells, timed like
    // the scenarios above; bytes per cell: 4 (in) + 4 (out) from HBM and 4
    // (the coefficient) over the host link.
    Array2D<float> in(W, H), out(W, H);
    for (size_t i = 0; i < W * H; ++i) {
      in.hostArray[i] = static_cast<float>(i % 1000) * 0.001f;
      out.hostArray[i] = 0.5f;
    }
    CoefArgs args{Args2D<float>(static_cast<int>(W), static_cast<int>(H))};
    for (size_t h = 0; h < H; ++h)
      for (size_t w = 0; w < W; ++w) args.coef(static_cast<int>(w), static_cast<int>(h)) = 0.05f;
    Mask2D<float> mask = jacobi_mask();
    Stencil2D<Array2D<float>, Mask2D<float>, CoefArgs> st(in, out, mask, args);
    auto run = [&](size_t n) -> double {
      const auto t0 = std::chrono::steady_clock::now();
      st.runIterativeGPU(n, 0, 0);
      return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    };
    const size_t it1 = it / 10 > 0 ? it / 10 : 1;
    run(2);
    const double t1 = run(it1), t2 = run(it);
    const double us = (t2 - t1) / static_cast<double>(it - it1) * 1e6;
    const double cells = static_cast<double>(W) * static_cast<double>(H);
    std::printf("{\"scenario\": \"coef2d\", \"cells\": %.0f, \"iterations\": [%zu, %zu], \"seconds\": [%.6f, %.6f], "
                "\"us_per_iteration\": %.3f, \"GCells_per_s\": %.1f, \"host_link_GBps\": %.1f}\n",
                cells, it1, it, t1, t2, us, cells / us * 1e-3, 4.0 * cells / us * 1e-3);
    return it > it1 ? 0 : 3;
  }

  if (sc.rfind("jacobi", 0) == 0) {
    Array2D<float> in(W, H), out(W, H);
    read_raw(fin, in.hostArray, W * H);
    read_raw(fout, out.hostArray, W * H);
    Mask2D<float> mask = jacobi_mask();
    if (sc == "jacobi_lib") {
      Stencil2D<Array2D<float>, Mask2D<float>, JacobiLib> st(in, out, mask, JacobiLib());
      st.runIterativeGPU(it, 32, 4);
    } else if (sc == "jacobi_pyramid") {
      Stencil2D<Array2D<float>, Mask2D<float>, JacobiLib> st(in, out, mask, JacobiLib());
      st.runIterativeGPU(it, 3, 32, 4);
    } else if (sc == "jacobi_tiling") {
      Stencil2D<Array2D<float>, Mask2D<float>, JacobiLib> st(in, out, mask, JacobiLib());
      st.runIterativeTilingGPU(it, 64, 32, 1, 5);
      if (st.ranOutOfCore()) std::printf("out of core\n");
    } else if (sc == "jacobi_auto") {
      Stencil2D<Array2D<float>, Mask2D<float>, JacobiLib> st(in, out, mask, JacobiLib());
      st.runIterativeAutoGPU(it);
      if (st.ranOutOfCore()) std::printf("out of core\n");
    } else if (sc == "jacobi_user") {
      Stencil2D<Array2D<float>, Mask2D<float>, JacobiUser> st(in, out, mask, JacobiUser{0});
      st.runIterativeGPU(it, 0, 0);
    } else if (sc == "jacobi_user_tiling") {
      Stencil2D<Array2D<float>, Mask2D<float>, JacobiUser> st(in, out, mask, JacobiUser{0});
      st.runIterativeTilingGPU(it, 64, 24, 1, 5);
      if (st.ranOutOfCore()) std::printf("out of core\n");
    } else if (sc == "jacobi_user_auto") {
      Stencil2D<Array2D<float>, Mask2D<float>, JacobiUser> st(in, out, mask, JacobiUser{0});
      st.runIterativeAutoGPU(it);
      if (st.ranOutOfCore()) std::printf("out of core\n");
    } else if (sc == "jacobi_cpu") {
      Stencil2D<Array2D<float>, Mask2D<float>, JacobiUser> st(in, out, mask, JacobiUser{0});
      st.runIterativeCPU(it, 4);
    } else {
      return 3;
    }
    write_raw(fres, out.hostArray, W * H);
  } else if (sc.rfind("life", 0) == 0) {
    Array2D<uint8_t> in(W, H), out(W, H);
    read_raw(fin, in.hostArray, W * H);
    read_raw(fout, out.hostArray, W * H);
    int moore[8][2] = {{-1, -1}, {-1, 0}, {-1, 1}, {0, -1}, {0, 1}, {1, -1}, {1, 0}, {1, 1}};
    Mask2D<uint8_t> mask(8, moore);
    if (sc == "life_lib") {
      Stencil2D<Array2D<uint8_t>, Mask2D<uint8_t>, LifeLib> st(in, out, mask, LifeLib());
      st.runIterativeGPU(it, 32, 4);
    } else if (sc == "life_tiling") {
      Stencil2D<Array2D<uint8_t>, Mask2D<uint8_t>, LifeLib> st(in, out, mask, LifeLib());
      st.runIterativeTilingGPU(it, 0, 16, 1, 7);
      if (st.ranOutOfCore()) std::printf("out of core\n");
    } else if (sc == "life_user") {
      Stencil2D<Array2D<uint8_t>, Mask2D<uint8_t>, LifeUser> st(in, out, mask, LifeUser{0});
      st.runIterativeGPU(it, 7, 32, 4);
    } else {
      return 3;
    }
    write_raw(fres, out.hostArray, W * H);
  } else if (sc.rfind("coef", 0) == 0) {
    // the coefficient field k(h, w) = 0.05 + 0.2 * ((h * 7 + w * 3) % 11) / 10
    Array2D<float> in(W, H), out(W, H);
    read_raw(fin, in.hostArray, W * H);
    read_raw(fout, out.hostArray, W * H);
    CoefArgs args{Args2D<float>(static_cast<int>(W), static_cast<int>(H))};
    for (size_t h = 0; h < H; ++h)
      for (size_t w = 0; w < W; ++w)
        args.coef(static_cast<int>(w), static_cast<int>(h)) = 0.05f + 0.2f * static_cast<float>((h * 7 + w * 3) % 11) / 10.0f;
    Mask2D<float> mask = jacobi_mask();
    Stencil2D<Array2D<float>, Mask2D<float>, CoefArgs> st(in, out, mask, args);
    if (sc == "coef_gpu") {
      st.runIterativeGPU(it, 0, 0);
    } else if (sc == "coef_tiling") {
      st.runIterativeTilingGPU(it, 64, 16, 1, 3);
      if (st.ranOutOfCore()) std::printf("out of core\n");
    } else if (sc == "coef_cpu") {
      st.runIterativeCPU(it, 4);
    } else {
      return 3;
    }
    write_raw(fres, out.hostArray, W * H);
  } else if (sc.rfind("stencil1d", 0) == 0) {
    // 1D: W cells; mask offsets -2, -1, 0, 1, 3 with halo value 0.5
    Array<float> in(W), out(W);
    read_raw(fin, in.hostArray, W);
    read_raw(fout, out.hostArray, W);
    Mask<float> mask(5, 0.5f);
    const int off[5] = {-2, -1, 0, 1, 3};
    const float wt[5] = {0.125f, 0.25f, 0.3f, 0.2f, 0.125f};
    for (int n = 0; n < 5; ++n) mask.set(n, off[n], wt[n]);
    Stencil<Array<float>, Mask<float>, Smooth1D> st(in, out, mask, Smooth1D{0});
    if (sc == "stencil1d_gpu")
      st.runIterativeGPU(it, 0, 0);
    else if (sc == "stencil1d_cpu")
      st.runIterativeCPU(it, 4);
    else
      return 3;
    write_raw(fres, out.hostArray, W);
  } else if (sc.rfind("map", 0) == 0) {
    const Affine g{0.75f, 0.125f};
    const size_t n = W * H * D;
    if (sc == "map1d_gpu" || sc == "map1d_seq") {
      Array<float> in(n), out(n);
      read_raw(fin, in.hostArray, n);
      read_raw(fout, out.hostArray, n);
      Map<Array<float>, Affine> m(in, out, g);
      if (sc == "map1d_gpu") m.runIterativeGPU(it, 0); else m.runIterativeSequential(it);
      write_raw(fres, out.hostArray, n);
    } else if (sc == "map2d_gpu" || sc == "map2d_cpu") {
      Array2D<float> in(W, H), out(W, H);
      read_raw(fin, in.hostArray, n);
      read_raw(fout, out.hostArray, n);
      Map2D<Array2D<float>, Affine> m(in, out, g);
      if (sc == "map2d_gpu") m.runIterativeGPU(it, 32); else m.runIterativeCPU(it, 4);
      write_raw(fres, out.hostArray, n);
    } else if (sc == "map3d_gpu") {
      Array3D<float> in(W, H, D), out(W, H, D);
      read_raw(fin, in.hostArray, n);
      read_raw(fout, out.hostArray, n);
      Map3D<Array3D<float>, Affine> m(in, out, g);
      if (it == 1) m.runGPU(); else m.runIterativeGPU(it);
      write_raw(fres, out.hostArray, n);
    } else {
      return 3;
    }
  } else if (sc.rfind("heat", 0) == 0) {
    Array3D<float> in(W, H, D), out(W, H, D);
    read_raw(fin, in.hostArray, W * H * D);
    read_raw(fout, out.hostArray, W * H * D);
    Mask3D<float> mask = heat_mask(0.5f);
    if (sc == "heat_lib") {
      Stencil3D<Array3D<float>, Mask3D<float>, HeatLib> st(in, out, mask, HeatLib());
      st.setResidualInterval(2);
      st.runIterativeGPU(it, 0, 0);
      if (argc > 9) write_raw(argv[9], st.residuals().data(), st.residuals().size());
    } else if (sc == "heat_tiling") {
      Stencil3D<Array3D<float>, Mask3D<float>, HeatLib> st(in, out, mask, HeatLib());
      st.runIterativeTilingGPU(it, W, 8, D, 3);
      if (st.ranOutOfCore()) std::printf("out of core\n");
    } else if (sc == "heat_user") {
      Stencil3D<Array3D<float>, Mask3D<float>, HeatUser> st(in, out, mask, HeatUser{0});
      st.runIterativeGPU(it, 0, 0);
    } else if (sc == "heat_user_tiling") {
      Stencil3D<Array3D<float>, Mask3D<float>, HeatUser> st(in, out, mask, HeatUser{0});
      st.runIterativeTilingGPU(it, W, 6, D, 3);
      if (st.ranOutOfCore()) std::printf("out of core\n");
    } else {
      return 3;
    }
    write_raw(fres, out.hostArray, W * H * D);
  } else {
    return 3;
  }
  std::printf("ok %s\n", sc.c_str());
  return 0;
}
