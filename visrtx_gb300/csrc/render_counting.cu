// The counting build (traversal statistics) of the per-pixel kernels for
// worlds with surfaces, in its own translation unit so it compiles beside
// render.cu.
#include "render_impl.cuh"

namespace vrtx {

void dispatchSurfaceCounting(
    const FrameParams &P, int type, int *occ, int grid, cudaStream_t s)
{
  dispatchSurface<true>(P, type, occ, grid, s);
}

} // namespace vrtx
