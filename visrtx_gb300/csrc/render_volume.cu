// Per-pixel integrator launches for worlds without surfaces (volume-only
// frames): compiled for more resident blocks per SM, with the NanoVDB field
// path compiled in only where the world holds a NanoVDB field (NV), so the
// structured-regular march keeps its register budget.
#include "render_impl.cuh"

namespace vrtx {

namespace {

template <int RT, bool STATS, bool NV>
void launchVolume(const FrameParams &P, int *occ, int grid, cudaStream_t s)
{
  if (occ)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, k_render<RT, STATS, false, NV>, 128, 0);
  else
    k_render<RT, STATS, false, NV><<<grid, 128, 0, s>>>(P);
}

template <bool STATS, bool NV>
void dispatchVolume(const FrameParams &P, int type, int *occ, int grid, cudaStream_t s)
{
  switch (type) {
  case RENDERER_RAYCAST:
    launchVolume<RENDERER_RAYCAST, STATS, NV>(P, occ, grid, s);
    break;
  case RENDERER_AO:
    launchVolume<RENDERER_AO, STATS, NV>(P, occ, grid, s);
    break;
  case RENDERER_DPT:
    launchVolume<RENDERER_DPT, STATS, NV>(P, occ, grid, s);
    break;
  default:
    launchVolume<RENDERER_DIRECT_LIGHT, STATS, NV>(P, occ, grid, s);
    break;
  }
}

} // namespace

void dispatchVolumeOnly(const FrameParams &P,
    int type,
    bool stats,
    bool nanovdb,
    int *occ,
    int grid,
    cudaStream_t s)
{
  if (stats) {
    if (nanovdb)
      dispatchVolume<true, true>(P, type, occ, grid, s);
    else
      dispatchVolume<true, false>(P, type, occ, grid, s);
  } else {
    if (nanovdb)
      dispatchVolume<false, true>(P, type, occ, grid, s);
    else
      dispatchVolume<false, false>(P, type, occ, grid, s);
  }
}

} // namespace vrtx
