// Per-pixel integrator launches for worlds with surfaces (and volumes), the
// frame clear, and the dispatch of every render launch; the kernels and
// device code are in render_impl.cuh.
#include "render_impl.cuh"

namespace vrtx {

namespace {

__global__ void k_clearFrame(FramebufferGPU fb)
{
  const size_t n = (size_t)fb.w * fb.h;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    fb.accum[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (fb.depth)
      fb.depth[i] = kFltMax;
    if (fb.primID)
      fb.primID[i] = 0u;
    if (fb.objID)
      fb.objID[i] = 0u;
    if (fb.instID)
      fb.instID[i] = 0u;
    if (fb.albedo)
      fb.albedo[i] = mk3(0.f, 0.f, 0.f);
    if (fb.normal)
      fb.normal[i] = mk3(0.f, 0.f, 0.f);
  }
}

} // namespace

static void dispatchAll(const FrameParams &P,
    int type,
    bool stats,
    bool surfaces,
    bool nanovdb,
    int *occ,
    int grid,
    cudaStream_t s)
{
  if (!surfaces)
    dispatchVolumeOnly(P, type, stats, nanovdb, occ, grid, s);
  else if (stats)
    dispatchSurfaceCounting(P, type, occ, grid, s);
  else
    dispatchSurface<false>(P, type, occ, grid, s);
}

int renderOccupancyBlocks(int rendererType, bool stats, bool surfaces, bool nanovdb)
{
  int blocks = 0;
  FrameParams dummy{};
  dispatchAll(dummy, rendererType, stats, surfaces, nanovdb, &blocks, 0, 0);
  return blocks > 0 ? blocks : 1;
}

cudaError_t launchRender(
    const FrameParams &P, int gridBlocks, bool stats, cudaStream_t s)
{
  dispatchAll(P,
      P.renderer.type,
      stats,
      P.world.numInstances > 0,
      P.world.hasNanovdb != 0,
      nullptr,
      gridBlocks,
      s);
  return cudaGetLastError();
}

__global__ void k_scale3(const f3 *in, f3 *out, size_t n, float scale)
{
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n)
    out[i] = in[i] * scale;
}

cudaError_t launchScale3(const f3 *in, f3 *out, size_t n, float scale, cudaStream_t s)
{
  if (n)
    k_scale3<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, out, n, scale);
  return cudaGetLastError();
}

// The frame's colour write (writeOutputColor, the function every render
// kernel ends with) applied to n given accumulations, for checking the
// output encoding on its own
__global__ void k_writeColors(FramebufferGPU fb, const float4 *accum, uint32_t n)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    writeOutputColor(fb, accum[i], i, 0);
}

cudaError_t launchWriteColors(const FramebufferGPU &fb, const float4 *accum, uint32_t n,
    cudaStream_t s)
{
  if (n)
    k_writeColors<<<(n + 255) / 256, 256, 0, s>>>(fb, accum, n);
  return cudaGetLastError();
}

cudaError_t launchClearFrame(const FramebufferGPU &fb, cudaStream_t s)
{
  k_clearFrame<<<1216, 256, 0, s>>>(fb);
  return cudaGetLastError();
}

} // namespace vrtx
