// A PSkel application that uses only the reference's API: user stencilKernel
// functors, Array2D/3D, Mask2D/3D, Stencil2D/3D and their run methods. The
// same source is built against the reference's own headers (the oracle's
// copy, with g++ for the host scenarios and nvcc for the GPU ones) and
// against this repository's include/ (tests/test_user_app.py), so "a user
// functor compiles unchanged" is shown rather than asserted.
//
//   user_app SCENARIO W H D ITERS IN OUTINIT RESULT
//
// Scenarios: jacobi_gpu, jacobi_cpu, life_gpu, life_cpu, heat_cpu. The GPU
// scenarios exist when the build defines PSKEL_CUDA (the reference's switch),
// the host ones when it defines PSKEL_OMP. 3D runs on the host only: the
// reference's 3D GPU path does not compile.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "PSkel.h"

using namespace PSkel;

struct JacobiUser {
  int unused;
};
struct LifeUser {
  int unused;
};
struct HeatUser {
  int unused;
};

namespace PSkel {
__parallel__ void stencilKernel(Array2D<float> in, Array2D<float> out, Mask2D<float> mask, JacobiUser, size_t h,
                                size_t w) {
  float acc = mask.getWeight(0) * mask.get(0, in, h, w);
  for (size_t n = 1; n < mask.size; ++n) acc = acc + mask.getWeight(n) * mask.get(n, in, h, w);
  out(h, w) = acc;
}
__parallel__ void stencilKernel(Array2D<unsigned char> in, Array2D<unsigned char> out, Mask2D<unsigned char> mask,
                                LifeUser, size_t h, size_t w) {
  int s = 0;
  for (size_t n = 0; n < mask.size; ++n) s += mask.get(n, in, h, w);
  const unsigned char c = in(h, w);
  out(h, w) = (s == 3 || (s == 2 && c == 1)) ? 1 : 0;
}
__parallel__ void stencilKernel(Array3D<float> in, Array3D<float> out, Mask3D<float> mask, HeatUser, size_t h,
                                size_t w, size_t d) {
  float acc = mask.getWeight(0) * mask.get(0, in, h, w, d);
  for (size_t n = 1; n < mask.size; ++n) acc = acc + mask.getWeight(n) * mask.get(n, in, h, w, d);
  out(h, w, d) = acc;
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

int main(int argc, char** argv) {
  if (argc < 9) {
    std::fprintf(stderr, "usage: user_app SCENARIO W H D ITERS IN OUTINIT RESULT\n");
    return 2;
  }
  const std::string sc = argv[1];
  const size_t W = std::strtoull(argv[2], 0, 10), H = std::strtoull(argv[3], 0, 10), D = std::strtoull(argv[4], 0, 10);
  const size_t it = std::strtoull(argv[5], 0, 10);
  const char *fin = argv[6], *fout = argv[7], *fres = argv[8];
  if (sc == "jacobi_gpu" || sc == "jacobi_cpu") {
    Array2D<float> in(W, H), out(W, H);
    read_raw(fin, in.hostArray, W * H);
    read_raw(fout, out.hostArray, W * H);
    Mask2D<float> mask(4);
    mask.set(0, -1, 0, 0.25f);
    mask.set(1, 1, 0, 0.25f);
    mask.set(2, 0, -1, 0.25f);
    mask.set(3, 0, 1, 0.25f);
    JacobiUser args;
    Stencil2D<Array2D<float>, Mask2D<float>, JacobiUser> st(in, out, mask, args);
    if (sc == "jacobi_gpu") {
#ifdef PSKEL_CUDA
      st.runIterativeGPU(it, 32, 4);
#else
      return 4;
#endif
    } else {
#ifdef PSKEL_OMP
      st.runIterativeCPU(it, 4);
#else
      return 4;
#endif
    }
    write_raw(fres, out.hostArray, W * H);
  } else if (sc == "life_gpu" || sc == "life_cpu") {
    Array2D<unsigned char> in(W, H), out(W, H);
    read_raw(fin, in.hostArray, W * H);
    read_raw(fout, out.hostArray, W * H);
    int moore[8][2] = {{-1, -1}, {-1, 0}, {-1, 1}, {0, -1}, {0, 1}, {1, -1}, {1, 0}, {1, 1}};
    Mask2D<unsigned char> mask(8, moore);
    LifeUser args;
    Stencil2D<Array2D<unsigned char>, Mask2D<unsigned char>, LifeUser> st(in, out, mask, args);
    if (sc == "life_gpu") {
#ifdef PSKEL_CUDA
      st.runIterativeGPU(it, 32, 4);
#else
      return 4;
#endif
    } else {
#ifdef PSKEL_OMP
      st.runIterativeCPU(it, 4);
#else
      return 4;
#endif
    }
    write_raw(fres, out.hostArray, W * H);
  } else if (sc == "heat_cpu") {
    Array3D<float> in(W, H, D), out(W, H, D);
    read_raw(fin, in.hostArray, W * H * D);
    read_raw(fout, out.hostArray, W * H * D);
    Mask3D<float> mask(7, 0.5f);
    const int off[7][3] = {{0, 0, 0}, {-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
    for (int n = 0; n < 7; ++n) mask.set(n, off[n][0], off[n][1], off[n][2], n == 0 ? 0.25f : 0.125f);
    HeatUser args;
    Stencil3D<Array3D<float>, Mask3D<float>, HeatUser> st(in, out, mask, args);
#ifdef PSKEL_OMP
    st.runIterativeCPU(it, 4);
#else
    return 4;
#endif
    write_raw(fres, out.hostArray, W * H * D);
  } else {
    return 3;
  }
  std::printf("ok %s\n", sc.c_str());
  return 0;
}
