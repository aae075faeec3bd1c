// Stable LSD radix sort of (64-bit key, 32-bit value) pairs: the Morton
// sort of the BVH builder (bvh.cu), replacing the sort inside the
// reference's closed optixAccelBuild (optix_visrtx.cpp:288-372).
//
// Each pass sorts by one 8-bit digit, low digit first, in three launches:
//  1. k_digitHist: every block counts the digits of its tile of
//     kTile = 2048 keys (lanes with equal digits are grouped with
//     match.any, so one shared-memory add serves each group); the counts
//     are stored digit-major, hist[digit * numTiles + tile];
//  2. k_digitScan: one block per digit turns its row into an exclusive
//     prefix over the tiles and writes the row total;
//  3. k_digitScatter: every block rebuilds the digit starts from the row
//     totals (a 256-entry scan in shared memory), then places its tile in
//     eight rounds of 256 keys: a key's place is its digit's start, plus
//     the keys of that digit in earlier tiles (the row prefix), earlier
//     rounds and earlier warps of this round, plus its rank among the
//     lanes of its warp with the same digit.
// Keys are placed in tile order, round order, warp order and lane order,
// so equal digits keep their input order and the whole sort is stable.
// Passes ping-pong between the two buffer pairs; only the passes that
// `bits` needs run.
#include "radix_sort.h"

#include <utility>

namespace vrtx {
namespace {

constexpr int kThreads = 256;
constexpr int kRounds = 8;
constexpr int kTile = kThreads * kRounds;
constexpr int kWarps = kThreads / 32;

__device__ __forceinline__ uint32_t lanemaskLt()
{
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__global__ void __launch_bounds__(kThreads) k_digitHist(
    const uint64_t *keys,
    uint32_t n,
    int shift,
    uint32_t mask,
    uint32_t *hist,
    uint32_t numTiles)
{
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * (uint32_t)kTile;
  const int lane = threadIdx.x & 31;
  for (int r = 0; r < kRounds; r++) {
    const uint32_t i = base + (uint32_t)r * kThreads + threadIdx.x;
    const uint32_t d = i < n ? (uint32_t)(keys[i] >> shift) & mask : 256u;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    if (d < 256u && lane == __ffs(peers) - 1)
      atomicAdd(&h[d], (uint32_t)__popc(peers));
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * numTiles + blockIdx.x] = h[threadIdx.x];
}

// inclusive block scan of one value per thread (kThreads threads)
__device__ __forceinline__ uint32_t blockInclusiveScan(uint32_t v, uint32_t *warpSums)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o)
      v += t;
  }
  if (lane == 31)
    warpSums[warp] = v;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = lane < kWarps ? warpSums[lane] : 0u;
#pragma unroll
    for (int o = 1; o < kWarps; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o)
        s += t;
    }
    if (lane < kWarps)
      warpSums[lane] = s;
  }
  __syncthreads();
  if (warp > 0)
    v += warpSums[warp - 1];
  __syncthreads(); // warpSums is reused by the next call
  return v;
}

// one block per digit: exclusive prefix of its row over the tiles, in place
__global__ void __launch_bounds__(kThreads) k_digitScan(
    uint32_t *hist, uint32_t numTiles, uint32_t *totals)
{
  __shared__ uint32_t warpSums[kWarps];
  __shared__ uint32_t chunkTotal;
  uint32_t *row = hist + (size_t)blockIdx.x * numTiles;
  uint32_t carry = 0;
  for (uint32_t c = 0; c < numTiles; c += kThreads) {
    const uint32_t i = c + threadIdx.x;
    const uint32_t v = i < numTiles ? row[i] : 0u;
    const uint32_t inc = blockInclusiveScan(v, warpSums);
    if (i < numTiles)
      row[i] = carry + inc - v;
    if (threadIdx.x == kThreads - 1)
      chunkTotal = inc;
    __syncthreads();
    carry += chunkTotal;
    __syncthreads();
  }
  if (threadIdx.x == 0)
    totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(kThreads) k_digitScatter(const uint64_t *keysIn,
    const uint32_t *valsIn,
    uint64_t *keysOut,
    uint32_t *valsOut,
    uint32_t n,
    int shift,
    uint32_t mask,
    const uint32_t *hist,
    uint32_t numTiles,
    const uint32_t *totals)
{
  __shared__ uint32_t warpSums[kWarps];
  __shared__ uint32_t start[256];
  __shared__ uint32_t warpCnt[kWarps][256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  {
    const uint32_t t = totals[threadIdx.x];
    const uint32_t inc = blockInclusiveScan(t, warpSums);
    start[threadIdx.x] = inc - t + hist[(size_t)threadIdx.x * numTiles + blockIdx.x];
    for (int w = 0; w < kWarps; w++)
      warpCnt[w][threadIdx.x] = 0;
  }
  __syncthreads();
  const uint32_t base = blockIdx.x * (uint32_t)kTile;
  const uint32_t lt = lanemaskLt();
  for (int r = 0; r < kRounds; r++) {
    const uint32_t i = base + (uint32_t)r * kThreads + threadIdx.x;
    const bool valid = i < n;
    const uint64_t key = valid ? keysIn[i] : 0ull;
    const uint32_t d = valid ? (uint32_t)(key >> shift) & mask : 256u;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    if (valid && lane == __ffs(peers) - 1)
      warpCnt[warp][d] = (uint32_t)__popc(peers);
    __syncthreads();
    if (valid) {
      uint32_t pos = start[d] + (uint32_t)__popc(peers & lt);
      for (int w = 0; w < warp; w++)
        pos += warpCnt[w][d];
      keysOut[pos] = key;
      valsOut[pos] = valsIn[i];
    }
    __syncthreads();
    uint32_t sum = 0;
    for (int w = 0; w < kWarps; w++) {
      sum += warpCnt[w][threadIdx.x];
      warpCnt[w][threadIdx.x] = 0;
    }
    start[threadIdx.x] += sum;
    __syncthreads();
  }
}

} // namespace

size_t radixSortScratchBytes(uint32_t n)
{
  const size_t tiles = (n + kTile - 1) / kTile;
  return sizeof(uint32_t) * (256 * (tiles ? tiles : 1) + 256);
}

cudaError_t radixSortPairs64(uint64_t *keys,
    uint32_t *vals,
    uint64_t *keysAlt,
    uint32_t *valsAlt,
    uint32_t n,
    int bits,
    void *scratch,
    cudaStream_t stream,
    uint64_t **keysOut,
    uint32_t **valsOut)
{
  *keysOut = keys;
  *valsOut = vals;
  if (n <= 1 || bits <= 0)
    return cudaSuccess;
  const uint32_t tiles = (n + kTile - 1) / kTile;
  uint32_t *hist = (uint32_t *)scratch;
  uint32_t *totals = hist + (size_t)256 * tiles;
  uint64_t *kin = keys, *kout = keysAlt;
  uint32_t *vin = vals, *vout = valsAlt;
  bits = bits > 64 ? 64 : bits;
  for (int shift = 0; shift < bits; shift += 8) {
    // the last pass takes only the bits below `bits`
    const int width = bits - shift < 8 ? bits - shift : 8;
    const uint32_t mask = (1u << width) - 1u;
    k_digitHist<<<tiles, kThreads, 0, stream>>>(kin, n, shift, mask, hist, tiles);
    k_digitScan<<<256, kThreads, 0, stream>>>(hist, tiles, totals);
    k_digitScatter<<<tiles, kThreads, 0, stream>>>(
        kin, vin, kout, vout, n, shift, mask, hist, tiles, totals);
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  *keysOut = kin;
  *valsOut = vin;
  return cudaGetLastError();
}

} // namespace vrtx
