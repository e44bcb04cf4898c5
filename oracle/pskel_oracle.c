/*
 * CPU restatement of PSkel's iterative stencil path, the oracle for this project.
 *
 * TEST INFRASTRUCTURE ONLY. Tests, __graft_entry__.smoke() and the cpu_baseline
 * leg of bench.py load it as the checker; the product never links or calls it.
 *
 * Parity is pinned: tests/golden/ holds outputs of the reference's own
 * Stencil2D/Stencil3D::runIterativeCPU (built by oracle/make_ref.py) and
 * tests/test_oracle.py checks every function here against them bit for bit.
 *
 * Semantics restated (all file:line in the reference tree):
 *  - StencilBase::runIterativeCPU, PSkelStencil.hpp:880-938: ping-pong between
 *    the two host arrays, `in`->`out` on even steps and `out`->`in` on odd
 *    steps; when the number of iterations is even the input array is copied
 *    into the output array at the end (:932). The input array is clobbered.
 *  - Stencil2D::runOpenMP, PSkelStencil.hpp:2197-2257: only cells with
 *    r <= h < H-r and r <= w < W-r are visited (r = mask range), so ring cells
 *    are never written in either array.
 *  - Stencil3D::runOpenMP, PSkelStencil.hpp:2104-2113: every cell is visited;
 *    Mask3D::get (PSkelMask.hpp:186-199) returns the mask halo value for
 *    neighbours outside the array.
 *  - Mask2D::get (PSkelMask.hpp:292-305): in(h+dh, w+dw), no bounds check.
 *  - MaskBase::getRange (PSkelMask.hpp:201-229, 307-334): max |offset| unless
 *    a range was given.
 *  - Array layouts (PSkelArray.hpp:349-352, 658-677): 2D [h][w], 3D [h][w][d].
 * The per-cell functors are this project's workloads, written identically in
 * oracle/ref_runner.cpp against the reference API.
 *
 * Floating point: products and sums in mask order, no contraction (build with
 * -ffp-contract=off). bf16 storage: each step computes in fp32 and rounds the
 * stored value to nearest even.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define EXPORT __attribute__((visibility("default")))

static inline float bf16_to_f32(uint16_t b) {
  uint32_t u = (uint32_t)b << 16;
  float f;
  memcpy(&f, &u, 4);
  return f;
}

static inline uint16_t f32_to_bf16(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u && (u & 0x007fffffu)) return (uint16_t)((u >> 16) | 0x40);
  u += 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

EXPORT uint16_t oracle_f32_to_bf16(float f) { return f32_to_bf16(f); }

EXPORT long oracle_mask_range(int nm, int dim, const int* off) {
  long r = 0;
  for (int i = 0; i < nm * dim; ++i) {
    long a = labs((long)off[i]);
    if (a > r) r = a;
  }
  return r;
}

/* ---------------------------------------------------------------- 2D linear */

#define LIN2D_STEP(T, C, LOAD, STORE)                                                    \
  for (long h = r; h < H - r; ++h) {                                                     \
    for (long w = r; w < W - r; ++w) {                                                   \
      C acc = (C)wt[0] * (C)LOAD(src[(h + off[0]) * W + (w + off[1])]);                  \
      for (int n = 1; n < nm; ++n)                                                       \
        acc = acc + (C)wt[n] * (C)LOAD(src[(h + off[2 * n]) * W + (w + off[2 * n + 1])]); \
      dst[h * W + w] = STORE(acc);                                                       \
    }                                                                                    \
  }

#define ID(x) (x)

#define LIN2D_BODY(T, C, WT, LOAD, STORE)                                     \
  if (r <= 0) r = oracle_mask_range(nm, 2, off);                              \
  if (H < r || W < r) return -1;                                              \
  for (long it = 0; it < iters; ++it) {                                       \
    T* src = (it % 2 == 0) ? in : out;                                        \
    T* dst = (it % 2 == 0) ? out : in;                                        \
    _Pragma("omp parallel for schedule(static)") LIN2D_STEP(T, C, LOAD, STORE) \
  }                                                                           \
  if (iters % 2 == 0) memcpy(out, in, (size_t)W * (size_t)H * sizeof(T));      \
  return 0;

/* Stencil2D::runIterativeCPU with out(h,w) = sum_n wt[n] * in(h+dh_n, w+dw_n). */
EXPORT int oracle_lin2d_f32(float* in, float* out, long W, long H, int nm, const int* off, const float* wt, long r,
                            long iters) {
  LIN2D_BODY(float, float, float, ID, ID)
}

EXPORT int oracle_lin2d_f64(double* in, double* out, long W, long H, int nm, const int* off, const double* wt, long r,
                            long iters) {
  LIN2D_BODY(double, double, double, ID, ID)
}

EXPORT int oracle_lin2d_bf16(uint16_t* in, uint16_t* out, long W, long H, int nm, const int* off, const float* wt,
                             long r, long iters) {
  LIN2D_BODY(uint16_t, float, float, bf16_to_f32, f32_to_bf16)
}

/* ------------------------------------------------------------- Game of Life */

/* Stencil2D::runIterativeCPU with the Life rule over the mask neighbourhood:
 * s = sum of neighbours, out = (s==3 || (s==2 && c==1)). */
EXPORT int oracle_life(uint8_t* in, uint8_t* out, long W, long H, int nm, const int* off, long r, long iters) {
  if (r <= 0) r = oracle_mask_range(nm, 2, off);
  if (H < r || W < r) return -1;
  for (long it = 0; it < iters; ++it) {
    uint8_t* src = (it % 2 == 0) ? in : out;
    uint8_t* dst = (it % 2 == 0) ? out : in;
#pragma omp parallel for schedule(static)
    for (long h = r; h < H - r; ++h) {
      for (long w = r; w < W - r; ++w) {
        int s = 0;
        for (int n = 0; n < nm; ++n) s += src[(h + off[2 * n]) * W + (w + off[2 * n + 1])];
        uint8_t c = src[h * W + w];
        dst[h * W + w] = (s == 3 || (s == 2 && c == 1)) ? 1 : 0;
      }
    }
  }
  if (iters % 2 == 0) memcpy(out, in, (size_t)W * (size_t)H);
  return 0;
}

/* ------------------------------------------------- advection + diffusion 2D */

#define ADV_BODY(T, C, LOAD, STORE)                                                                 \
  const long r = 1;                                                                                 \
  if (H < r || W < r) return -1;                                                                    \
  for (long it = 0; it < iters; ++it) {                                                             \
    T* src = (it % 2 == 0) ? in : out;                                                              \
    T* dst = (it % 2 == 0) ? out : in;                                                              \
    _Pragma("omp parallel for schedule(static)") for (long h = r; h < H - r; ++h) {                 \
      for (long w = r; w < W - r; ++w) {                                                            \
        C c = (C)LOAD(src[h * W + w]);                                                              \
        C n = (C)LOAD(src[(h - 1) * W + w]);                                                        \
        C e = (C)LOAD(src[h * W + w + 1]);                                                          \
        C wv = (C)LOAD(src[h * W + w - 1]);                                                         \
        C s = (C)LOAD(src[(h + 1) * W + w]);                                                        \
        C sum = (C)4 * c - (((n + e) + wv) + s);                                                    \
        C xw = (C)LOAD(u[h * W + w]);                                                               \
        C yw = (C)LOAD(v[h * W + w]);                                                               \
        int xf = (xw > 0) ? 1 : -1;                                                                 \
        int yf = (yw > 0) ? 1 : -1;                                                                 \
        C cvy = (C)yf * yw;                                                                         \
        C cvx = (C)xf * xw;                                                                         \
        C nbx = (C)LOAD(src[h * W + (w + xf)]);                                                     \
        C nby = (C)LOAD(src[(h + yf) * W + w]);                                                     \
        C temp_wind = (-cvx * ((c - nbx) * idx)) - (cvy * ((c - nby) * idx));                       \
        C cond = ((-k) * (sum * (C)0.25)) * tdt;                                                    \
        C result = c + cond;                                                                        \
        dst[h * W + w] = STORE(result + temp_wind * tdt);                                           \
      }                                                                                             \
    }                                                                                               \
  }                                                                                                 \
  if (iters % 2 == 0) memcpy(out, in, (size_t)W * (size_t)H * sizeof(T));                           \
  return 0;

/* Upwind advection-diffusion (the arithmetic of PSkelStencil.hpp:347-387 with
 * diffusivity K, time step dt and 1/dx as parameters, winds u,v per cell). */
EXPORT int oracle_advect_f32(float* in, float* out, const float* u, const float* v, long W, long H, float K, float dt,
                             float inv_dx, long iters) {
  const float k = K, tdt = dt, idx = inv_dx;
  ADV_BODY(float, float, ID, ID)
}

EXPORT int oracle_advect_f64(double* in, double* out, const double* u, const double* v, long W, long H, float K,
                             float dt, float inv_dx, long iters) {
  const double k = K, tdt = dt, idx = inv_dx;
  ADV_BODY(double, double, ID, ID)
}

EXPORT int oracle_advect_bf16(uint16_t* in, uint16_t* out, const uint16_t* u, const uint16_t* v, long W, long H,
                              float K, float dt, float inv_dx, long iters) {
  const float k = K, tdt = dt, idx = inv_dx;
  ADV_BODY(uint16_t, float, bf16_to_f32, f32_to_bf16)
}

/* --------------------------------------------------------------- 3D linear */

#define LIN3D_STEP(T, C, LOAD, STORE)                                                        \
  _Pragma("omp parallel for schedule(static)") for (long h = 0; h < H; ++h) {                \
    for (long w = 0; w < W; ++w) {                                                           \
      for (long d = 0; d < D; ++d) {                                                         \
        C acc = 0;                                                                           \
        for (int n = 0; n < nm; ++n) {                                                       \
          unsigned long hh = (unsigned long)(h + off[3 * n]);                                \
          unsigned long ww = (unsigned long)(w + off[3 * n + 1]);                            \
          unsigned long dd = (unsigned long)(d + off[3 * n + 2]);                            \
          C val = (ww < (unsigned long)W && hh < (unsigned long)H && dd < (unsigned long)D)  \
                      ? (C)LOAD(src[((long)hh * W + (long)ww) * D + (long)dd])               \
                      : (C)halo;                                                             \
          C term = (C)wt[n] * val;                                                           \
          acc = (n == 0) ? term : acc + term;                                                \
        }                                                                                    \
        dst[(h * W + w) * D + d] = STORE(acc);                                               \
      }                                                                                      \
    }                                                                                        \
  }

#define NORM(T, C, LOAD)                                                        \
  {                                                                             \
    double s = 0.0;                                                             \
    for (long i = 0; i < N; ++i) {                                              \
      double dlt = (double)(C)LOAD(dst[i]) - (double)(C)LOAD(src[i]);           \
      s += dlt * dlt;                                                           \
    }                                                                           \
    norms[nnorm++] = sqrt(s);                                                   \
  }

#define LIN3D_BODY(T, C, LOAD, STORE)                                   \
  const long N = W * H * D;                                             \
  long nnorm = 0;                                                       \
  for (long it = 0; it < iters; ++it) {                                 \
    T* src = (it % 2 == 0) ? in : out;                                  \
    T* dst = (it % 2 == 0) ? out : in;                                  \
    LIN3D_STEP(T, C, LOAD, STORE)                                       \
    if (every > 0 && norms && (it + 1) % every == 0) NORM(T, C, LOAD)   \
  }                                                                     \
  if (iters % 2 == 0) memcpy(out, in, (size_t)N * sizeof(T));           \
  return (int)nnorm;

/* Stencil3D::runIterativeCPU with out(h,w,d) = sum_n wt[n] * get(n), where get
 * returns `halo` outside the array. When every > 0, norms[k/every - 1] receives
 * ||u_k - u_{k-1}||_2 in fp64 for k = every, 2*every, ...; returns their count. */
EXPORT int oracle_lin3d_f32(float* in, float* out, long W, long H, long D, int nm, const int* off, const float* wt,
                            float halo, long iters, long every, double* norms) {
  LIN3D_BODY(float, float, ID, ID)
}

EXPORT int oracle_lin3d_f64(double* in, double* out, long W, long H, long D, int nm, const int* off,
                            const double* wt, double halo, long iters, long every, double* norms) {
  LIN3D_BODY(double, double, ID, ID)
}

EXPORT int oracle_lin3d_bf16(uint16_t* in, uint16_t* out, long W, long H, long D, int nm, const int* off,
                             const float* wt, float halo, long iters, long every, double* norms) {
  LIN3D_BODY(uint16_t, float, bf16_to_f32, f32_to_bf16)
}
