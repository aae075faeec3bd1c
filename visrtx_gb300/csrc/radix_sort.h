// Stable LSD radix sort of (64-bit key, 32-bit value) pairs on the GPU (the
// BVH builder's Morton sort); see radix_sort.cu.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace vrtx {

// Device scratch bytes radixSortPairs64 needs for n pairs.
size_t radixSortScratchBytes(uint32_t n);

// Sorts n pairs by the low `bits` bits of the keys, stably. (keys, vals)
// hold the input; (keysAlt, valsAlt) are buffers of the same sizes; the
// passes ping-pong between the two and *keysOut / *valsOut name the pair
// that holds the result. All work is queued on `stream`; nothing is
// allocated.
cudaError_t radixSortPairs64(uint64_t *keys,
    uint32_t *vals,
    uint64_t *keysAlt,
    uint32_t *valsAlt,
    uint32_t n,
    int bits,
    void *scratch,
    cudaStream_t stream,
    uint64_t **keysOut,
    uint32_t **valsOut);

} // namespace vrtx
