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
// the reference's device build contracts them to. The stencil comes from the
// field's brick cache where one covers it (every leaf's values plus a
// one-voxel apron, filled by this walk when the field is built), else from
// the walk itself.
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

// A read accessor: the last leaf and lower node visited, so the taps of a
// stencil inside one leaf cost one load each (NanoVDB's ReadAccessor caches
// the same levels).
struct Accessor
{
  const uint8_t *leaf = nullptr;
  const uint8_t *lower = nullptr;
  int lx = 0, ly = 0, lz = 0; // leaf origin
  int ox = 0, oy = 0, oz = 0; // lower node origin
};

// The leaf holding voxel (x, y, z) through the accessor's cache, or nullptr
// when no leaf covers it: `fill` is then the value of the whole leaf-sized
// region (a tile value of an internal node or the root, or the background).
// the walk from the lower-node cache or the root (once per leaf a ray enters)
__device__ __forceinline__ const uint8_t *walkToLeaf(
    const NvdbGPU &g, Accessor &a, int x, int y, int z, float &fill)
{
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
    if (!tile) {
      fill = g.background;
      return nullptr;
    }
    const int64_t child = (int64_t)ld64(tile + 8);
    if (!child) {
      fill = ldf(tile + 20);
      return nullptr;
    }
    const uint8_t *up = g.root + child;
    const uint32_t nu = uint32_t((x & 4095) >> 7) << 10 | uint32_t((y & 4095) >> 7) << 5
        | uint32_t((z & 4095) >> 7);
    if (!childBit(up + kUpperChildMask, nu)) {
      fill = ldf(up + kUpperTable + 8 * nu);
      return nullptr;
    }
    lower = up + (int64_t)ld64(up + kUpperTable + 8 * nu);
    a.lower = lower;
    a.ox = x & ~127;
    a.oy = y & ~127;
    a.oz = z & ~127;
  }
  const uint32_t nl = uint32_t((x & 127) >> 3) << 8 | uint32_t((y & 127) >> 3) << 4
      | uint32_t((z & 127) >> 3);
  if (!childBit(lower + kLowerChildMask, nl)) {
    fill = ldf(lower + kLowerTable + 8 * nl);
    return nullptr;
  }
  const uint8_t *leaf = lower + (int64_t)ld64(lower + kLowerTable + 8 * nl);
  a.leaf = leaf;
  a.lx = x & ~7;
  a.ly = y & ~7;
  a.lz = z & ~7;
  return leaf;
}

__device__ __forceinline__ const uint8_t *leafAt(
    const NvdbGPU &g, Accessor &a, int x, int y, int z, float &fill)
{
  if (a.leaf && (x & ~7) == a.lx && (y & ~7) == a.ly && (z & ~7) == a.lz)
    return a.leaf;
  return walkToLeaf(g, a, x, y, z, fill);
}

// The 2x2x2 stencil at leaf offset n (x, y, z all below 7 within the leaf):
// offsets n + {0, 1, 8, 9, 64, 65, 72, 73}, decoded with the leaf's
// minimum and quantum read once.
__device__ __forceinline__ void leafStencil(
    const uint8_t *leaf, uint32_t type, uint32_t n, float v[8])
{
  const uint32_t off[8] = {0u, 1u, 8u, 9u, 64u, 65u, 72u, 73u};
  if (type == 1u) {
    const float *f = reinterpret_cast<const float *>(leaf + kLeafData) + n;
#pragma unroll
    for (int c = 0; c < 8; c++)
      v[c] = __ldg(f + off[c]);
    return;
  }
  const float mn = ldf(leaf + kLeafMin), q = ldf(leaf + kLeafQuantum);
  uint32_t code[8];
  if (type == 14u) {
    const uint8_t *b = leaf + kLeafData + n;
#pragma unroll
    for (int c = 0; c < 8; c++)
      code[c] = __ldg(b + off[c]);
  } else if (type == 15u) {
    const unsigned short *h = reinterpret_cast<const unsigned short *>(leaf + kLeafData) + n;
#pragma unroll
    for (int c = 0; c < 8; c++)
      code[c] = __ldg(h + off[c]);
  } else if (type == 13u) {
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const uint32_t i = n + off[c];
      code[c] = (__ldg(leaf + kLeafData + (i >> 1)) >> ((i & 1u) << 2)) & 15u;
    }
  } else {
    const uint32_t b = __ldg(leaf + 15) >> 5;
    const unsigned int *w = reinterpret_cast<const unsigned int *>(leaf + kLeafData);
    const uint32_t lanes = (32u >> b) - 1u, mask = (1u << (1u << b)) - 1u;
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const uint32_t i = n + off[c];
      code[c] = (__ldg(w + (i >> (5u - b))) >> ((i & lanes) << b)) & mask;
    }
  }
#pragma unroll
  for (int c = 0; c < 8; c++)
    v[c] = fmaf(float(code[c]), q, mn);
}

// RootNode / InternalNode / LeafNode getValue (NanoVDB.h:2947, 3528)
__device__ __forceinline__ float value(const NvdbGPU &g, Accessor &a, int x, int y, int z)
{
  float fill = 0.f;
  const uint8_t *leaf = leafAt(g, a, x, y, z, fill);
  return leaf ? leafValue(leaf, g.type, uint32_t((x & 7) << 6 | (y & 7) << 3 | (z & 7))) : fill;
}

__device__ __forceinline__ float lerp(float a, float b, float w)
{
  return fmaf(w, __fsub_rn(b, a), a);
}

// A stencil that straddles leaf boundaries: each tap through the accessor,
// in a loop that is not unrolled so the walk is emitted once (about a third
// of the samples of a march take this path).
__device__ __forceinline__ float stencilAcrossLeaves(
    const NvdbGPU &g, Accessor &a, int i, int j, int k, float ux, float uy, float uz)
{
  float v[8];
#pragma unroll 1
  for (int c = 0; c < 8; c++)
    v[c] = value(g, a, i + (c >> 2), j + ((c >> 1) & 1), k + (c & 1));
  // v: (0,0,0) (0,0,1) (0,1,0) (0,1,1) (1,0,0) (1,0,1) (1,1,0) (1,1,1)
  return lerp(lerp(lerp(v[0], v[1], uz), lerp(v[2], v[3], uz), uy),
      lerp(lerp(v[4], v[5], uz), lerp(v[6], v[7], uz), uy),
      ux);
}

// The stencil at index (i, j, k) by walking the tree (blocks the brick
// cache does not cover, or fields built without it).
__device__ __forceinline__ float stencilByWalk(
    const NvdbGPU &g, Accessor &a, int i, int j, int k, float ux, float uy, float uz)
{
  if ((i & 7) != 7 && (j & 7) != 7 && (k & 7) != 7) {
    // the whole stencil lies in one leaf-sized block: one lookup
    float fill = 0.f;
    const uint8_t *leaf = leafAt(g, a, i, j, k, fill);
    float v[8];
    if (leaf) {
      leafStencil(leaf, g.type, uint32_t((i & 7) << 6 | (j & 7) << 3 | (k & 7)), v);
    } else {
#pragma unroll
      for (int c = 0; c < 8; c++)
        v[c] = fill;
    }
    // v: (0,0,0) (0,0,1) (0,1,0) (0,1,1) (1,0,0) (1,0,1) (1,1,0) (1,1,1)
    return lerp(lerp(lerp(v[0], v[1], uz), lerp(v[2], v[3], uz), uy),
        lerp(lerp(v[4], v[5], uz), lerp(v[6], v[7], uz), uy),
        ux);
  }
  return stencilAcrossLeaves(g, a, i, j, k, ux, uy, uz);
}

// The same out of line with its own accessor: with the brick cache the walk
// is rare (outside the table), and keeping it out of the march leaves the
// march's registers to the brick path. (Fields too large for the cache walk
// from the root at every sample.)
static __device__ __noinline__ float stencilByWalkOutOfLine(
    const NvdbGPU *g, int i, int j, int k, float ux, float uy, float uz)
{
  Accessor a;
  return stencilByWalk(*g, a, i, j, k, ux, uy, uz);
}

// The sample at object-space location p. The reference subtracts the float
// translation from the location in double and rounds to float; for two
// float operands that equals the float subtraction (one rounding of the
// exact difference), which is what is computed here.
// The sample at object-space location p. The reference subtracts the float
// translation from the location in double and rounds to float; for two
// float operands that equals the float subtraction (one rounding of the
// exact difference), which is what is computed here.
__device__ __forceinline__ float sample(const NvdbGPU &g, f3 p)
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
  if (g.bricks) {
    // the brick cache: the block's 9^3 values hold the whole stencil
    const int bx = (i >> 3) - g.blockLo[0], by = (j >> 3) - g.blockLo[1],
              bz = (k >> 3) - g.blockLo[2];
    if ((unsigned)bx < (unsigned)g.blockDims[0] && (unsigned)by < (unsigned)g.blockDims[1]
        && (unsigned)bz < (unsigned)g.blockDims[2]) {
      const int e = (bz * g.blockDims[1] + by) * g.blockDims[0] + bx;
      const int slot = __ldg(g.brickTable + e);
      if (slot >= 0) {
        const float *b = g.bricks + size_t(slot) * 729 + ((i & 7) * 81 + (j & 7) * 9 + (k & 7));
        return lerp(lerp(lerp(__ldg(b), __ldg(b + 1), uz), lerp(__ldg(b + 9), __ldg(b + 10), uz), uy),
            lerp(lerp(__ldg(b + 81), __ldg(b + 82), uz), lerp(__ldg(b + 90), __ldg(b + 91), uz), uy),
            ux);
      }
      // a constant region: every lerp of equal values returns that value
      if (slot == kBlockConstant)
        return __ldg(g.blockFill + e);
    }
  }
  return stencilByWalkOutOfLine(&g, i, j, k, ux, uy, uz);
}

} // namespace nvdb
} // namespace vrtx
