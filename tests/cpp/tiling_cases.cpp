// Prints StencilTiling::tile's geometry for a grid of cases, one line each.
// Built twice by tests/test_stencil_tiling.py: against the reference's
// PSkelStencilTiling.h (the oracle copy of the reference headers) and against
// this repository's include/PSkelStencilTiling.h; the outputs must be equal.
#include <cstddef>
#include <cstdio>

#include "PSkelStencilTiling.h"

struct FakeArray {  // the members StencilTiling reads
  size_t w = 0, h = 0, d = 0;
  size_t getWidth() const { return w; }
  size_t getHeight() const { return h; }
  size_t getDepth() const { return d; }
};
struct FakeMask {
  int range = 1;
  int getRange() const { return range; }
};

int main() {
  const size_t dims[][3] = {{64, 48, 1}, {100, 37, 9}, {7, 5, 3}, {1024, 1024, 1}, {33, 1, 1}};
  const int ranges[] = {1, 2, 3};
  const size_t iters[] = {1, 2, 5, 16};
  const size_t tiles[] = {1, 4, 16, 50, 2000};
  for (const auto& dm : dims)
    for (int r : ranges)
      for (size_t it : iters)
        for (size_t t : tiles)
          for (size_t off = 0; off < dm[0] + 3; off += (dm[0] > 40 ? 9 : 1)) {
            FakeArray a;
            a.w = dm[0];
            a.h = dm[1];
            a.d = dm[2];
            FakeMask m;
            m.range = r;
            PSkel::StencilTiling<FakeArray, FakeMask> st(a, a, m);
            const size_t ho = off % (dm[1] + 1), dof = off % (dm[2] + 1);
            if (off > dm[0] || ho > dm[1] || dof > dm[2]) continue;  // offsets inside the array (or at its end)
            st.tile(it, off, ho, dof, t, t / 2 + 1, t % 7 + 1);
            std::printf("%zu %zu %zu r%d it%zu t%zu off%zu: %zu %zu %zu %zu %zu %zu | %zu %zu %zu %zu %zu %zu\n", dm[0],
                        dm[1], dm[2], r, it, t, off, st.widthOffset, st.heightOffset, st.depthOffset, st.width,
                        st.height, st.depth, st.coreWidthOffset, st.coreHeightOffset, st.coreDepthOffset,
                        st.coreWidth, st.coreHeight, st.coreDepth);
          }
  return 0;
}
