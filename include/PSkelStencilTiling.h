// PSkel drop-in for GB300: StencilTiling, the geometry of a tile with its
// redundant halo for `iterations` steps.
//
// Same computation as the reference (PSkelStencilTiling.h:85-148): clamp the
// logical tile to the array, grow it by range * iterations on every side
// (clamped at the array border, with the reference's arithmetic at the low
// border), and record where the core sits inside the grown tile. The GPU kernels of this library apply the same trapezoid
// on-chip; this class is kept for applications that use it directly.
#ifndef PSKEL_STENCIL_TILING_H
#define PSKEL_STENCIL_TILING_H

#include <cstddef>

namespace PSkel {

template <class Array, class Mask>
class StencilTiling {
 public:
  Mask mask;
  Array input;
  Array output;
  size_t iterations = 0;
  size_t widthOffset = 0, heightOffset = 0, depthOffset = 0;
  size_t width = 0, height = 0, depth = 0;
  size_t coreWidthOffset = 0, coreHeightOffset = 0, coreDepthOffset = 0;
  size_t coreWidth = 0, coreHeight = 0, coreDepth = 0;

  StencilTiling(Array in, Array out, Mask m) : mask(m), input(in), output(out) {}

  void tile(size_t iters, size_t wOff, size_t hOff, size_t dOff, size_t w, size_t h, size_t d) {
    iterations = iters;
    grow(input.getWidth(), wOff, w, widthOffset, width, coreWidthOffset, coreWidth, iters);
    grow(input.getHeight(), hOff, h, heightOffset, height, coreHeightOffset, coreHeight, iters);
    grow(input.getDepth(), dOff, d, depthOffset, depth, coreDepthOffset, coreDepth, iters);
  }

 private:
  // One axis, as PSkelStencilTiling.h:102-136 computes it: the core
  // [off, off + len) is clamped to the array, then grown by range * iters on
  // both sides. When the grown tile would start before 0 it starts at 0 and
  // its length is len + range * iters (the reference subtracts the full halo
  // as "extra" once the offset has been set to 0), clamped to the array.
  void grow(size_t extent, size_t off, size_t len, size_t& out_off, size_t& out_len, size_t& core_off,
            size_t& core_len, size_t iters) {
    if (off + len > extent) len = extent - off;
    core_len = len;
    const size_t halo = mask.getRange() * iters;
    size_t lo, extra;
    if (off >= halo) {
      lo = off - halo;
      extra = 0;
    } else {
      lo = 0;
      extra = halo;
    }
    size_t grown = len + 2 * halo - extra;
    if (lo + grown > extent) grown = extent - lo;
    out_off = lo;
    out_len = grown;
    core_off = off - lo;
  }
};

}  // namespace PSkel

#endif  // PSKEL_STENCIL_TILING_H
