// NanoVDB field sampling (device code): the reference's
// SpatialFieldSampler<nanovdb::Grid<...>> (gpu/sampleSpatialField.h:80-109)
// over a grid buffer in the layout of the NanoVDB version the reference
// vendors (external/nanovdb, 32.7). The layout, read here by byte offset:
//  * RootData: index bbox (24 B), tile count (+24), background (+28); 32-byte
//    tiles from +64: key (u64), child offset from the RootData (i64, 0 = a
//    value tile), state (u32), value (f32 at +20);
//  * upper internal node (32^3 slots): child mask at +4128, 8-byte slot table
//    at +8256; lower internal node (16^3): child mask at +544, table at +1088.
//    A slot holds the child's byte offset from the node, or a tile value in
//    its low four bytes;
//  * leaf (8^3): float values from +96, or for the quantised codecs the
//    minimum (+80), the quantum (+84) and codes from +96 (Fp4 two per byte,
//    low nibble first; Fp8 bytes; Fp16 u16; FpN 2^(flags >> 5) bits per code
//    in u32 words, flags at +15), decoded as code * quantum + minimum.
// The sample is the world -> index map (the float inverse matrix applied
// through fmaf), floor, the 2x2x2 stencil, and lerps a + w (b - a) over z,
// y, x (math/SampleFromVoxels.h:200-245), written as the fused multiply-adds
// the reference's device build contracts them to.
#pragma once

#include "gpu_types.h"

namespace vrtx {
namespace nvdb {

constexpr int kRootTiles = 64, kTileBytes = 32;
constexpr int kUpperChildMask = 4128, kUpperTable = 8256;
constexpr int kLowerChildMask = 544, kLowerTable = 1088;
constexpr int kLeafMin = 80, kLeafQuantum = 84, kLeafData = 96;

__device__ __forceinline__ uint64_t ld64(const uint8_t *p)
{
  return __ldg(reinterpret_cast<const unsigned long long *>(p));
}

__device__ __forceinline__ float ldf(const uint8_t *p)
{
  return __ldg(reinterpret_cast<const float *>(p));
}

__device__ __forceinline__ bool childBit(const uint8_t *mask, uint32_t i)
{
  return (ld64(mask + 8 * (i >> 6)) >> (i & 63u)) & 1ull;
}

// LeafData<float / Fp4 / Fp8 / Fp16 / FpN>::getValue
__device__ __forceinline__ float leafValue(const uint8_t *leaf, uint32_t type, uint32_t i)
{
  if (type == 1u)
    return ldf(leaf + kLeafData + 4 * i);
  uint32_t code;
  if (type == 14u)
    code = __ldg(leaf + kLeafData + i);
  else if (type == 15u)
    code = __ldg(reinterpret_cast<const unsigned short *>(leaf + kLeafData) + i);
  else if (type == 13u)
    code = (__ldg(leaf + kLeafData + (i >> 1)) >> ((i & 1u) << 2)) & 15u;
  else {
    const uint32_t b = __ldg(leaf + 15) >> 5; // log2 of the code width, 0..4
    const uint32_t w =
        __ldg(reinterpret_cast<const unsigned int *>(leaf + kLeafData) + (i >> (5u - b)));
    code = (w >> ((i & ((32u >> b) - 1u)) << b)) & ((1u << (1u << b)) - 1u);
  }
  return fmaf(float(code), ldf(leaf + kLeafQuantum), ldf(leaf + kLeafMin));
}

// A per-thread read accessor: the last leaf and lower node visited, so the
// taps of a stencil (and of consecutive samples) inside one leaf cost one
// load each (NanoVDB's ReadAccessor caches the same levels).
struct Accessor
{
  const uint8_t *leaf = nullptr;
  const uint8_t *lower = nullptr;
  int lx = 0, ly = 0, lz = 0; // leaf origin
  int ox = 0, oy = 0, oz = 0; // lower node origin
};

// RootNode / InternalNode / LeafNode getValue (NanoVDB.h:2947, 3528)
__device__ __forceinline__ float value(const NvdbGPU &g, Accessor &a, int x, int y, int z)
{
  if (a.leaf && (x & ~7) == a.lx && (y & ~7) == a.ly && (z & ~7) == a.lz)
    return leafValue(a.leaf, g.type, uint32_t((x & 7) << 6 | (y & 7) << 3 | (z & 7)));
  const uint8_t *lower;
  if (a.lower && (x & ~127) == a.ox && (y & ~127) == a.oy && (z & ~127) == a.oz) {
    lower = a.lower;
  } else {
    const uint64_t key = uint64_t(uint32_t(z) >> 12) | (uint64_t(uint32_t(y) >> 12) << 21)
        | (uint64_t(uint32_t(x) >> 12) << 42);
    const uint8_t *tile = nullptr;
    for (uint32_t t = 0; t < g.tiles; t++) {
      const uint8_t *p = g.root + kRootTiles + kTileBytes * t;
      if (ld64(p) == key) {
        tile = p;
        break;
      }
    }
    if (!tile)
      return g.background;
    const int64_t child = (int64_t)ld64(tile + 8);
    if (!child)
      return ldf(tile + 20);
    const uint8_t *up = g.root + child;
    const uint32_t nu = uint32_t((x & 4095) >> 7) << 10 | uint32_t((y & 4095) >> 7) << 5
        | uint32_t((z & 4095) >> 7);
    if (!childBit(up + kUpperChildMask, nu))
      return ldf(up + kUpperTable + 8 * nu);
    lower = up + (int64_t)ld64(up + kUpperTable + 8 * nu);
    a.lower = lower;
    a.ox = x & ~127;
    a.oy = y & ~127;
    a.oz = z & ~127;
  }
  const uint32_t nl = uint32_t((x & 127) >> 3) << 8 | uint32_t((y & 127) >> 3) << 4
      | uint32_t((z & 127) >> 3);
  if (!childBit(lower + kLowerChildMask, nl))
    return ldf(lower + kLowerTable + 8 * nl);
  const uint8_t *leaf = lower + (int64_t)ld64(lower + kLowerTable + 8 * nl);
  a.leaf = leaf;
  a.lx = x & ~7;
  a.ly = y & ~7;
  a.lz = z & ~7;
  return leafValue(leaf, g.type, uint32_t((x & 7) << 6 | (y & 7) << 3 | (z & 7)));
}

__device__ __forceinline__ float lerp(float a, float b, float w)
{
  return fmaf(w, __fsub_rn(b, a), a);
}

// The sample at object-space location p. The reference subtracts the float
// translation from the location in double and rounds to float; for two
// float operands that equals the float subtraction (one rounding of the
// exact difference), which is what is computed here.
__device__ __forceinline__ float sample(const NvdbGPU &g, Accessor &a, f3 p)
{
  const float dx = __fsub_rn(p.x, g.vec[0]);
  const float dy = __fsub_rn(p.y, g.vec[1]);
  const float dz = __fsub_rn(p.z, g.vec[2]);
  const float ix = fmaf(dx, g.inv[0], fmaf(dy, g.inv[1], __fmul_rn(dz, g.inv[2])));
  const float iy = fmaf(dx, g.inv[3], fmaf(dy, g.inv[4], __fmul_rn(dz, g.inv[5])));
  const float iz = fmaf(dx, g.inv[6], fmaf(dy, g.inv[7], __fmul_rn(dz, g.inv[8])));
  const float fx = floorf(ix), fy = floorf(iy), fz = floorf(iz);
  const float ux = __fsub_rn(ix, fx), uy = __fsub_rn(iy, fy), uz = __fsub_rn(iz, fz);
  const int i = int(fx), j = int(fy), k = int(fz);
  // stencil order of TrilinearSampler::stencil
  const float v000 = value(g, a, i, j, k);
  const float v001 = value(g, a, i, j, k + 1);
  const float v011 = value(g, a, i, j + 1, k + 1);
  const float v010 = value(g, a, i, j + 1, k);
  const float v100 = value(g, a, i + 1, j, k);
  const float v101 = value(g, a, i + 1, j, k + 1);
  const float v111 = value(g, a, i + 1, j + 1, k + 1);
  const float v110 = value(g, a, i + 1, j + 1, k);
  return lerp(lerp(lerp(v000, v001, uz), lerp(v010, v011, uz), uy),
      lerp(lerp(v100, v101, uz), lerp(v110, v111, uz), uy),
      ux);
}

} // namespace nvdb
} // namespace vrtx
