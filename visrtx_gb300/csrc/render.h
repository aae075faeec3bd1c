// Host-side declarations of the device kernels' launch wrappers.
#pragma once

#include "gpu_types.h"

namespace vrtx {

// integrators (render.cu dispatches every per-pixel launch)
int renderOccupancyBlocks(int rendererType, bool stats, bool surfaces, bool nanovdb);
// the counting build of the per-pixel kernels for worlds with surfaces
// (render_counting.cu): launches, or with occ set reports blocks per SM
void dispatchSurfaceCounting(
    const FrameParams &P, int type, int *occ, int grid, cudaStream_t s);
// the per-pixel kernels of volume-only worlds (render_volume.cu): launches,
// or with occ set reports resident blocks per SM
void dispatchVolumeOnly(const FrameParams &P,
    int type,
    bool stats,
    bool nanovdb,
    int *occ,
    int grid,
    cudaStream_t s);
// stats: the counting build (node visits, primitive tests, BLAS entries)
cudaError_t launchRender(
    const FrameParams &P, int gridBlocks, bool stats, cudaStream_t s);
cudaError_t launchClearFrame(const FramebufferGPU &fb, cudaStream_t s);
// fb.outColorU[i] (or fb.outColorF[i]) = the frame's colour write of
// accum[i] after fb.frameID + 1 samples, for i < n
cudaError_t launchWriteColors(const FramebufferGPU &fb, const float4 *accum, uint32_t n,
    cudaStream_t s);
// out[i] = in[i] * scale for n vec3 elements (albedo / normal map)
cudaError_t launchScale3(const f3 *in, f3 *out, size_t n, float scale, cudaStream_t s);

// Wavefront "ao" renderer (opaque materials, no volumes): per sample a
// primary kernel, an any-hit kernel over the compacted AO ray queue and a
// resolve kernel. scratch: aoWavefrontBytes() bytes of device memory.
// traceEvents (optional): 2 per sample, recorded around each any-hit launch.
size_t aoWavefrontBytes(uint32_t w, uint32_t h, int aoSamples);
cudaError_t launchAOWavefront(const FrameParams &P,
    int numSMs,
    bool stats,
    void *scratch,
    cudaStream_t s,
    cudaEvent_t *traceEvents);

// Wavefront "default" renderer (opaque matte materials, no volumes, no
// background image): per sample a primary kernel that queues the AO rays
// and one shadow ray per light, the AO any-hit kernel over that queue, and
// a resolve kernel. scratch: dlWavefrontBytes() bytes.
size_t dlWavefrontBytes(uint32_t w, uint32_t h, int aoSamples, uint32_t numLights);
cudaError_t launchDLWavefront(const FrameParams &P,
    int numSMs,
    bool stats,
    void *scratch,
    cudaStream_t s,
    cudaEvent_t *traceEvents);
// "raycast" over opaque surfaces without volumes: one kernel per frame
cudaError_t launchRaycastWavefront(const FrameParams &P, bool stats, cudaStream_t s);

// scene preparation (scene.cu)
cudaError_t launchTriangleBoxes(const GeometryGPU *geoms,
    const uint2 *refs, // (surface, prim) per BLAS primitive
    const SurfaceGPU *surfaces,
    uint32_t n,
    box3 *boxes,
    cudaStream_t s);
cudaError_t launchSphereBoxes(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    uint32_t n,
    box3 *boxes,
    cudaStream_t s);
cudaError_t launchGatherTriangles(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    const uint32_t *order,
    uint32_t n,
    TriRecord *out,
    cudaStream_t s);
cudaError_t launchGatherSpheres(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    const uint32_t *order,
    uint32_t n,
    SphereRecord *out,
    cudaStream_t s);
cudaError_t launchFillRefs(uint32_t surface, uint32_t count, uint2 *out,
    cudaStream_t s);
// cylinders, cones and curves
cudaError_t launchSegmentBoxes(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    uint32_t n,
    box3 *boxes,
    cudaStream_t s);
cudaError_t launchGatherSegments(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    const uint32_t *order,
    uint32_t n,
    SegRecord *out,
    cudaStream_t s);
// two triangles per quad (idx4: uvec4 per quad or NULL)
cudaError_t launchQuadIndices(
    const uint32_t *idx4, uint32_t numQuads, uint32_t *out, cudaStream_t s);

// Conservative macrocell majorants of a structured-regular field through a
// TF table (scene.cu). Cells are 16^3 voxels from the origin; a cell's value
// range covers every voxel the trilinear filter can touch for a sample inside
// it (one voxel of apron on each side), and its majorant is the largest TF
// alpha over all table entries that range can reach through linear filtering
// (one entry of apron). ranges: scratch of 2 * numCells floats.
cudaError_t launchMacrocellRanges(cudaTextureObject_t field,
    const int dims[3],
    const int mcDims[3],
    float *ranges,
    cudaStream_t s);
cudaError_t launchMacrocellMajorants(const float *ranges,
    const int mcDims[3],
    const float4 *tf,
    int tfSize,
    float valueLo,
    float valueHi,
    float uniformOpacity,
    float *majorants,
    unsigned *emptyCells, // incremented once per cell with majorant 0
    cudaStream_t s);
// The reference's delta-tracking grid (UniformGrid.cu): per-cell value ranges
// (2 floats per cell) and max TF opacities.
cudaError_t launchReferenceGridRanges(cudaTextureObject_t field,
    f3 origin,
    f3 spacing,
    f3 invSpacing,
    box3 bounds,
    const int mcDims[3],
    float *ranges,
    cudaStream_t s);
// the brick cache of a NanoVDB field: 9^3 values per leaf (origins: 3 ints
// per leaf) evaluated by the device tree walk
cudaError_t launchNanovdbBricks(
    const NvdbGPU &grid, const int32_t *origins, uint32_t leaves, float *bricks, cudaStream_t s);
// classifies the unclassified blocks of a NanoVDB brick table: kBlockConstant
// (fill written) where the block's 9^3 region holds one value, else
// kBlockNeedsBrick
cudaError_t launchNanovdbClassifyBlocks(
    const NvdbGPU &grid, uint32_t entries, int32_t *table, float *fill, cudaStream_t s);
// the same grid over a NanoVDB field
cudaError_t launchReferenceGridRangesNanovdb(
    const NvdbGPU &grid, box3 bounds, const int mcDims[3], float *ranges, cudaStream_t s);
cudaError_t launchReferenceMajorants(const float *ranges,
    const int mcDims[3],
    cudaTextureObject_t tf,
    int tfSize,
    float uniformOpacity,
    float *majorants,
    cudaStream_t s);

} // namespace vrtx
