// BVH8 construction on the GPU (replaces the reference's optixAccelBuild call
// in buildOptixBVH, devices/rtx/optix_visrtx.cpp:288-372, whose algorithm is
// closed). Pipeline: 63-bit Morton codes of primitive centroids -> radix
// sort -> Karras binary radix tree -> bottom-up box refit -> top-down greedy
// surface-area collapse into 8-wide nodes with quantised child boxes.
#pragma once

#include "gpu_types.h"

namespace vrtx {

struct BVH8Build
{
  BVH8Node *nodes = nullptr; // device
  uint32_t numNodes = 0;
  uint32_t *primOrder = nullptr; // device: leaf slot -> input primitive
  uint32_t numPrims = 0;
  box3 bounds = emptyBox();
};

// Builds over n device-resident primitive boxes. Allocations are
// stream-ordered (cudaMallocAsync) on `stream`; the call synchronises the
// stream once at the end to read back counts. maxLeafPrims in [1, 3].
cudaError_t buildBVH8(const box3 *d_boxes,
    uint32_t n,
    cudaStream_t stream,
    BVH8Build &out,
    int maxLeafPrims = 3);

void freeBVH8(BVH8Build &b, cudaStream_t stream);

} // namespace vrtx
