// Scene preparation kernels: primitive boxes, leaf-record gathers and the
// conservative macrocell majorant grid.
//
// Replaces the reference's sphere AABB transform (scene/surface/geometry/
// Sphere.cu:56-115) and its UniformGrid build (scene/volume/space_skipping/
// UniformGrid.cu:44-150). The grid here is built differently on purpose:
// the reference samples 8 texture taps per macrocell at world positions
// treated as texture coordinates, which does not bound the voxels a sample
// can see; skipping cells needs a bound that does, so every voxel of the
// cell plus a one-voxel apron is read.
#include "nvdb.cuh"
#include "render.h"

namespace vrtx {
namespace {

__device__ __forceinline__ void triIndices(
    const GeometryGPU &g, uint32_t prim, uint32_t &i0, uint32_t &i1, uint32_t &i2)
{
  if (g.indices) {
    i0 = g.indices[3 * prim];
    i1 = g.indices[3 * prim + 1];
    i2 = g.indices[3 * prim + 2];
  } else {
    i0 = 3 * prim;
    i1 = i0 + 1;
    i2 = i0 + 2;
  }
}

__global__ void k_triBoxes(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    uint32_t n,
    box3 *boxes)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const uint2 r = refs[i];
  const GeometryGPU &g = geoms[surfaces[r.x].geometry];
  uint32_t i0, i1, i2;
  triIndices(g, r.y, i0, i1, i2);
  box3 b = emptyBox();
  extend(b, g.vertices[i0]);
  extend(b, g.vertices[i1]);
  extend(b, g.vertices[i2]);
  boxes[i] = b;
}

__device__ __forceinline__ void sphereOf(
    const GeometryGPU &g, uint32_t prim, f3 &c, float &r)
{
  const uint32_t idx = g.indices ? g.indices[prim] : prim;
  c = g.vertices[idx];
  r = g.radii ? g.radii[idx] : g.radius;
}

__global__ void k_sphereBoxes(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    uint32_t n,
    box3 *boxes)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const uint2 r = refs[i];
  const GeometryGPU &g = geoms[surfaces[r.x].geometry];
  f3 c;
  float rad;
  sphereOf(g, r.y, c, rad);
  const f3 e = mk3(rad, rad, rad);
  boxes[i] = box3{c - e, c + e};
}

__global__ void k_gatherTris(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    const uint32_t *order,
    uint32_t n,
    TriRecord *out)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const uint2 r = refs[order[i]];
  const GeometryGPU &g = geoms[surfaces[r.x].geometry];
  uint32_t i0, i1, i2;
  triIndices(g, r.y, i0, i1, i2);
  const f3 a = g.vertices[i0], b = g.vertices[i1], c = g.vertices[i2];
  TriRecord t;
  t.v0 = make_float4(a.x, a.y, a.z, __uint_as_float(r.y));
  t.v1 = make_float4(b.x, b.y, b.z, __uint_as_float(r.x));
  t.v2 = make_float4(c.x, c.y, c.z, __uint_as_float(g.cullBackfaces ? 1u : 0u));
  out[i] = t;
}

__global__ void k_gatherSpheres(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    const uint32_t *order,
    uint32_t n,
    SphereRecord *out)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const uint2 r = refs[order[i]];
  const GeometryGPU &g = geoms[surfaces[r.x].geometry];
  f3 c;
  float rad;
  sphereOf(g, r.y, c, rad);
  SphereRecord s;
  s.cr = make_float4(c.x, c.y, c.z, rad);
  s.primID = r.y;
  s.surface = r.x;
  s.pad[0] = s.pad[1] = 0;
  out[i] = s;
}

// The segment of a cylinder, cone or curve primitive: end points and end
// radii, indexed as the reference's intersectors and hit population read
// them (Intersectors_ptx.cu:100-246, populateHit.h:292-303): cylinders and
// cones take a uvec2 per primitive (default 2i, 2i + 1), curves the index of
// the first vertex (default i); a cylinder has one |radius| per primitive or
// the uniform one, a cone per-vertex radii, a curve per-vertex radii or the
// uniform one (Curve.cpp:101-113).
__device__ __forceinline__ void segmentOf(
    const GeometryGPU &g, uint32_t prim, f3 &p0, float &r0, f3 &p1, float &r1)
{
  uint32_t i0, i1;
  if (g.kind == KIND_CURVE) {
    i0 = g.indices ? g.indices[prim] : prim;
    i1 = i0 + 1;
  } else {
    i0 = g.indices ? g.indices[2 * prim] : 2 * prim;
    i1 = g.indices ? g.indices[2 * prim + 1] : 2 * prim + 1;
  }
  p0 = g.vertices[i0];
  p1 = g.vertices[i1];
  if (g.kind == KIND_CYLINDER) {
    r0 = r1 = fabsf(g.radii ? g.radii[prim] : g.radius);
  } else if (g.kind == KIND_CONE) {
    r0 = g.radii[i0];
    r1 = g.radii[i1];
  } else {
    r0 = g.radii ? g.radii[i0] : g.radius;
    r1 = g.radii ? g.radii[i1] : g.radius;
  }
}

// Boxes as Cylinder.cpp:91-98 and Cone.cpp:95-103 build them; a curve
// segment's box encloses its two end spheres.
__global__ void k_segBoxes(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    uint32_t n,
    box3 *boxes)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const uint2 r = refs[i];
  const GeometryGPU &g = geoms[surfaces[r.x].geometry];
  f3 p0, p1;
  float r0, r1;
  segmentOf(g, r.y, p0, r0, p1, r1);
  box3 b;
  if (g.kind == KIND_CURVE) {
    const f3 e0 = mk3(r0, r0, r0), e1 = mk3(r1, r1, r1);
    b.lo = fmin3(p0 - e0, p1 - e1);
    b.hi = fmax3(p0 + e0, p1 + e1);
  } else {
    const float m = fmaxf(r0, r1);
    const f3 e = mk3(m, m, m);
    b.lo = fmin3(p0, p1) - e;
    b.hi = fmax3(p0, p1) + e;
  }
  boxes[i] = b;
}

__global__ void k_gatherSegs(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    const uint32_t *order,
    uint32_t n,
    SegRecord *out)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const uint2 r = refs[order[i]];
  const GeometryGPU &g = geoms[surfaces[r.x].geometry];
  f3 p0, p1;
  float r0, r1;
  segmentOf(g, r.y, p0, r0, p1, r1);
  SegRecord rec;
  rec.a = make_float4(p0.x, p0.y, p0.z, r0);
  rec.b = make_float4(p1.x, p1.y, p1.z, r1);
  rec.primID = r.y;
  rec.surface = r.x;
  rec.caps = g.caps;
  rec.pad = 0;
  out[i] = rec;
}

// Quad.cpp:115-141: quad (x, y, z, w) -> triangles (x, y, w), (z, w, y);
// without an index, quad i uses vertices 4i .. 4i + 3
__global__ void k_quadIndices(const uint32_t *idx4, uint32_t numQuads, uint32_t *out)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= numQuads)
    return;
  uint32_t x, y, z, w;
  if (idx4) {
    x = idx4[4 * i];
    y = idx4[4 * i + 1];
    z = idx4[4 * i + 2];
    w = idx4[4 * i + 3];
  } else {
    x = 4 * i;
    y = x + 1;
    z = x + 2;
    w = x + 3;
  }
  uint32_t *o = out + 6 * (size_t)i;
  o[0] = x;
  o[1] = y;
  o[2] = w;
  o[3] = z;
  o[4] = w;
  o[5] = y;
}

__global__ void k_fillRefs(uint32_t surface, uint32_t count, uint2 *out)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count)
    out[i] = make_uint2(surface, i);
}

// One block per macrocell: min/max over voxels [16c - 1, 16c + 17) per axis
// (clamped), read with point sampling at unnormalised voxel centres.
__global__ void __launch_bounds__(256) k_mcRanges(cudaTextureObject_t pointTex,
    int dx,
    int dy,
    int dz,
    int mx,
    int my,
    int mz,
    float *ranges)
{
  const int cell = blockIdx.x;
  const int cx = cell % mx, cy = (cell / mx) % my, cz = cell / (mx * my);
  const int x0 = max(16 * cx - 1, 0), x1 = min(16 * cx + 17, dx - 1);
  const int y0 = max(16 * cy - 1, 0), y1 = min(16 * cy + 17, dy - 1);
  const int z0 = max(16 * cz - 1, 0), z1 = min(16 * cz + 17, dz - 1);
  const int nx = x1 - x0 + 1, ny = y1 - y0 + 1, nz = z1 - z0 + 1;
  const int total = nx * ny * nz;
  float lo = 3.0e38f, hi = -3.0e38f;
  for (int i = threadIdx.x; i < total; i += blockDim.x) {
    const int x = x0 + i % nx, y = y0 + (i / nx) % ny, z = z0 + i / (nx * ny);
    const float v = tex3D<float>(pointTex, x + 0.5f, y + 0.5f, z + 0.5f);
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  __shared__ float slo[8], shi[8];
  if ((threadIdx.x & 31) == 0) {
    slo[threadIdx.x >> 5] = lo;
    shi[threadIdx.x >> 5] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
      lo = fminf(lo, slo[w]);
      hi = fmaxf(hi, shi[w]);
    }
    ranges[2 * cell] = lo;
    ranges[2 * cell + 1] = hi;
  }
}

__device__ __forceinline__ float tfCoord(float s, float lo, float hi)
{
  const float cs = fmaxf(lo, fminf(s, hi));
  return (cs - lo) * (1.f / (hi - lo));
}

__global__ void k_mcMajorants(const float *ranges,
    int numCells,
    const float4 *tf,
    int tfSize,
    float vlo,
    float vhi,
    float uniformOpacity,
    float *majorants,
    unsigned *emptyCells)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= numCells)
    return;
  const float lo = ranges[2 * c], hi = ranges[2 * c + 1];
  if (!(lo <= hi)) { // empty or all-NaN cell
    majorants[c] = 0.f;
    atomicAdd(emptyCells, 1u);
    return;
  }
  if (!tf) {
    majorants[c] = uniformOpacity;
    return;
  }
  int e0 = 0, e1 = tfSize - 1;
  if (vhi != vlo) {
    const float c0 = tfCoord(lo, vlo, vhi), c1 = tfCoord(hi, vlo, vhi);
    const float a = fminf(c0, c1), b = fmaxf(c0, c1);
    e0 = (int)floorf(a * tfSize - 0.5f) - 1;
    e1 = (int)floorf(b * tfSize - 0.5f) + 2;
    e0 = max(e0, 0);
    e1 = min(e1, tfSize - 1);
  }
  float m = 0.f;
  for (int e = e0; e <= e1; e++)
    m = fmaxf(m, tf[e].w);
  majorants[c] = m;
  if (m == 0.f)
    atomicAdd(emptyCells, 1u);
}

// --- delta-tracking grid (the reference's UniformGrid) -------------------
//
// UniformGrid::init/buildGrid/computeMaxOpacities
// (scene/volume/space_skipping/UniformGrid.cu:44-258): ceil(dims/16) cells
// spanning the field bounds [origin, origin + (dims - 1) spacing]. One
// thread per cell takes the max of 8 field taps at the object-space points
// (cell id +- 0.5) / cellDims (the reference passes these through the field
// sampler as positions, so they land near the field's first voxels), and
// splats it with float atomic min/max into every cell its bounds project
// onto. The dpt distance sampler reads these majorants, so they follow the
// reference's arithmetic, not the conservative skipping grid above.

__device__ __forceinline__ void atomicMinFloat(float *a, float v)
{
  if (!(v == v))
    return;
  if (v >= 0.f)
    atomicMin(reinterpret_cast<int *>(a), __float_as_int(v));
  else
    atomicMax(reinterpret_cast<unsigned *>(a), __float_as_uint(v));
}

__device__ __forceinline__ void atomicMaxFloat(float *a, float v)
{
  if (!(v == v))
    return;
  if (v >= 0.f)
    atomicMax(reinterpret_cast<int *>(a), __float_as_int(v));
  else
    atomicMin(reinterpret_cast<unsigned *>(a), __float_as_uint(v));
}

__device__ __forceinline__ int projectAxis(float v, float lo, float hi, int n)
{
  // projectOnGrid (gpu/uniformGrid.h:43-50): float -> int truncates
  const float v01 = __fdiv_rn(__fsub_rn(v, lo), __fsub_rn(hi, lo));
  return min(max(__float2int_rz(__fmul_rn(v01, float(n))), 0), n - 1);
}

__global__ void k_refGridInit(float *ranges, int cells)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cells)
    return;
  ranges[2 * c] = 1e30f;
  ranges[2 * c + 1] = -1e30f;
}

// The field sampler the reference grid build goes through: the structured
// field's texture at ((p - origin) + 0.5 spacing) * invSpacing
// (sampleSpatialField.h:54-78), or a NanoVDB grid (sampleSpatialField.h:
// 80-109).
struct RefTextureTap
{
  cudaTextureObject_t field;
  f3 origin, spacing, invSpacing;
  __device__ __forceinline__ float operator()(f3 p) const
  {
    const float cx = __fmul_rn(
        __fadd_rn(__fsub_rn(p.x, origin.x), __fmul_rn(0.5f, spacing.x)), invSpacing.x);
    const float cy = __fmul_rn(
        __fadd_rn(__fsub_rn(p.y, origin.y), __fmul_rn(0.5f, spacing.y)), invSpacing.y);
    const float cz = __fmul_rn(
        __fadd_rn(__fsub_rn(p.z, origin.z), __fmul_rn(0.5f, spacing.z)), invSpacing.z);
    return tex3D<float>(field, cx, cy, cz);
  }
};

struct RefNanovdbTap
{
  NvdbGPU grid;
  __device__ __forceinline__ float operator()(f3 p) const
  {
    return nvdb::sample(grid, p);
  }
};

template <typename Tap>
__global__ void k_refGridRanges(Tap tap, box3 bounds, int mx, int my, int mz, float *ranges)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= mx * my * mz)
    return;
  const int ix = c % mx, iy = (c / mx) % my, iz = c / (mx * my);
  const float ex = __fdiv_rn(__fsub_rn(bounds.hi.x, bounds.lo.x), float(mx));
  const float ey = __fdiv_rn(__fsub_rn(bounds.hi.y, bounds.lo.y), float(my));
  const float ez = __fdiv_rn(__fsub_rn(bounds.hi.z, bounds.lo.z), float(mz));
  const float lx = __fadd_rn(bounds.lo.x, __fmul_rn(float(ix), ex));
  const float ly = __fadd_rn(bounds.lo.y, __fmul_rn(float(iy), ey));
  const float lz = __fadd_rn(bounds.lo.z, __fmul_rn(float(iz), ez));
  const float ux = __fadd_rn(lx, ex), uy = __fadd_rn(ly, ey), uz = __fadd_rn(lz, ez);
  float value = -1e30f;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    // tap order of the reference: (-,-,-) (+,-,-) (+,+,-) (-,+,-), then z+
    const float ox = (k == 1 || k == 2 || k == 5 || k == 6) ? 0.5f : -0.5f;
    const float oy = (k == 2 || k == 3 || k == 6 || k == 7) ? 0.5f : -0.5f;
    const float oz = k >= 4 ? 0.5f : -0.5f;
    const f3 p = mk3(__fdiv_rn(__fadd_rn(float(ix), ox), float(mx)),
        __fdiv_rn(__fadd_rn(float(iy), oy), float(my)),
        __fdiv_rn(__fadd_rn(float(iz), oz), float(mz)));
    value = fmaxf(value, tap(p));
  }
  const int x0 = projectAxis(lx, bounds.lo.x, bounds.hi.x, mx);
  const int x1 = projectAxis(ux, bounds.lo.x, bounds.hi.x, mx);
  const int y0 = projectAxis(ly, bounds.lo.y, bounds.hi.y, my);
  const int y1 = projectAxis(uy, bounds.lo.y, bounds.hi.y, my);
  const int z0 = projectAxis(lz, bounds.lo.z, bounds.hi.z, mz);
  const int z1 = projectAxis(uz, bounds.lo.z, bounds.hi.z, mz);
  for (int z = z0; z <= z1; z++)
    for (int y = y0; y <= y1; y++)
      for (int x = x0; x <= x1; x++) {
        float *r = ranges + 2 * (((size_t)z * my + y) * mx + x);
        atomicMinFloat(r, value);
        atomicMaxFloat(r + 1, value);
      }
}

// computeMaxOpacitiesGPU (UniformGrid.cu:55-90) with the default TF range
// [0, 1]: max TF alpha over entries [int(lo (N-1)), int(hi (N-1)) + 1],
// read through the TF texture at entry centres.
__global__ void k_refMajorants(const float *ranges,
    int cells,
    cudaTextureObject_t tf,
    int tfSize,
    float uniformOpacity,
    float *majorants)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cells)
    return;
  const float lo = ranges[2 * c], hi = ranges[2 * c + 1];
  if (hi < lo) {
    majorants[c] = 0.f;
    return;
  }
  if (!tf) {
    majorants[c] = uniformOpacity;
    return;
  }
  const int n1 = tfSize - 1;
  const int e0 = min(max(__float2int_rz(__fmul_rn(lo, float(n1))), 0), n1);
  const int e1 = min(max(__float2int_rz(__fmul_rn(hi, float(n1))) + 1, 0), n1);
  float m = 0.f;
  for (int i = e0; i <= e1; i++)
    m = fmaxf(m, tex1D<float4>(tf, __fdiv_rn(float(i) + 0.5f, float(tfSize))).w);
  majorants[c] = m;
}

} // namespace

cudaError_t launchReferenceGridRanges(cudaTextureObject_t field,
    f3 origin,
    f3 spacing,
    f3 invSpacing,
    box3 bounds,
    const int mcDims[3],
    float *ranges,
    cudaStream_t s)
{
  const int cells = mcDims[0] * mcDims[1] * mcDims[2];
  if (!cells)
    return cudaSuccess;
  k_refGridInit<<<(cells + 255) / 256, 256, 0, s>>>(ranges, cells);
  k_refGridRanges<<<(cells + 127) / 128, 128, 0, s>>>(
      RefTextureTap{field, origin, spacing, invSpacing},
      bounds,
      mcDims[0],
      mcDims[1],
      mcDims[2],
      ranges);
  return cudaGetLastError();
}

namespace {

// one block per leaf, 729 threads: the 9^3 padded brick through the tree
// walk (the brick cache reads are then the walk's values)
__global__ void __launch_bounds__(729) k_nanovdbBricks(
    NvdbGPU grid, const int32_t *origins, uint32_t leaves, float *bricks)
{
  const uint32_t leaf = blockIdx.x;
  if (leaf >= leaves)
    return;
  const int t = threadIdx.x; // dx * 81 + dy * 9 + dz
  const int dx = t / 81, dy = (t / 9) % 9, dz = t % 9;
  grid.bricks = nullptr; // evaluate through the tree
  nvdb::Accessor a;
  bricks[size_t(leaf) * 729 + t] = nvdb::value(grid,
      a,
      origins[3 * leaf] + dx,
      origins[3 * leaf + 1] + dy,
      origins[3 * leaf + 2] + dz);
}

// one 256-thread block per table entry still unclassified: is the block's
// 9^3 region one value (compared bitwise)?
__global__ void __launch_bounds__(256) k_nanovdbClassifyBlocks(
    NvdbGPU grid, uint32_t entries, int32_t *table, float *fill)
{
  const uint32_t e = blockIdx.x;
  if (e >= entries || table[e] != kBlockUnclassified)
    return;
  const int bx = int(e % uint32_t(grid.blockDims[0]));
  const int by = int((e / uint32_t(grid.blockDims[0])) % uint32_t(grid.blockDims[1]));
  const int bz = int(e / (uint32_t(grid.blockDims[0]) * uint32_t(grid.blockDims[1])));
  const int ox = (grid.blockLo[0] + bx) * 8, oy = (grid.blockLo[1] + by) * 8,
            oz = (grid.blockLo[2] + bz) * 8;
  grid.bricks = nullptr; // evaluate through the tree
  __shared__ int varies;
  __shared__ float first;
  nvdb::Accessor a;
  if (threadIdx.x == 0) {
    first = nvdb::value(grid, a, ox, oy, oz);
    // a lerp of equal values returns the value itself only when it is
    // finite and not -0 (fmaf(w, 0, -0) is +0): other regions keep a brick
    varies = (!isfinite(first) || __float_as_uint(first) == 0x80000000u) ? 1 : 0;
  }
  __syncthreads();
  const uint32_t ref = __float_as_uint(first);
  for (int t = threadIdx.x; t < 729; t += blockDim.x) {
    const float v = nvdb::value(grid, a, ox + t / 81, oy + (t / 9) % 9, oz + t % 9);
    if (__float_as_uint(v) != ref)
      varies = 1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    table[e] = varies ? kBlockNeedsBrick : kBlockConstant;
    fill[e] = first;
  }
}

} // namespace

cudaError_t launchNanovdbClassifyBlocks(
    const NvdbGPU &grid, uint32_t entries, int32_t *table, float *fill, cudaStream_t s)
{
  if (!entries)
    return cudaSuccess;
  k_nanovdbClassifyBlocks<<<entries, 256, 0, s>>>(grid, entries, table, fill);
  return cudaGetLastError();
}

cudaError_t launchNanovdbBricks(
    const NvdbGPU &grid, const int32_t *origins, uint32_t leaves, float *bricks, cudaStream_t s)
{
  if (!leaves)
    return cudaSuccess;
  k_nanovdbBricks<<<leaves, 729, 0, s>>>(grid, origins, leaves, bricks);
  return cudaGetLastError();
}

cudaError_t launchReferenceGridRangesNanovdb(
    const NvdbGPU &grid, box3 bounds, const int mcDims[3], float *ranges, cudaStream_t s)
{
  const int cells = mcDims[0] * mcDims[1] * mcDims[2];
  if (!cells)
    return cudaSuccess;
  k_refGridInit<<<(cells + 255) / 256, 256, 0, s>>>(ranges, cells);
  k_refGridRanges<<<(cells + 127) / 128, 128, 0, s>>>(
      RefNanovdbTap{grid}, bounds, mcDims[0], mcDims[1], mcDims[2], ranges);
  return cudaGetLastError();
}

cudaError_t launchReferenceMajorants(const float *ranges,
    const int mcDims[3],
    cudaTextureObject_t tf,
    int tfSize,
    float uniformOpacity,
    float *majorants,
    cudaStream_t s)
{
  const int cells = mcDims[0] * mcDims[1] * mcDims[2];
  if (cells)
    k_refMajorants<<<(cells + 255) / 256, 256, 0, s>>>(
        ranges, cells, tf, tfSize, uniformOpacity, majorants);
  return cudaGetLastError();
}

cudaError_t launchTriangleBoxes(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    uint32_t n,
    box3 *boxes,
    cudaStream_t s)
{
  if (n)
    k_triBoxes<<<(n + 255) / 256, 256, 0, s>>>(geoms, refs, surfaces, n, boxes);
  return cudaGetLastError();
}

cudaError_t launchSphereBoxes(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    uint32_t n,
    box3 *boxes,
    cudaStream_t s)
{
  if (n)
    k_sphereBoxes<<<(n + 255) / 256, 256, 0, s>>>(geoms, refs, surfaces, n, boxes);
  return cudaGetLastError();
}

cudaError_t launchSegmentBoxes(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    uint32_t n,
    box3 *boxes,
    cudaStream_t s)
{
  if (n)
    k_segBoxes<<<(n + 255) / 256, 256, 0, s>>>(geoms, refs, surfaces, n, boxes);
  return cudaGetLastError();
}

cudaError_t launchGatherSegments(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    const uint32_t *order,
    uint32_t n,
    SegRecord *out,
    cudaStream_t s)
{
  if (n)
    k_gatherSegs<<<(n + 255) / 256, 256, 0, s>>>(geoms, refs, surfaces, order, n, out);
  return cudaGetLastError();
}

cudaError_t launchQuadIndices(
    const uint32_t *idx4, uint32_t numQuads, uint32_t *out, cudaStream_t s)
{
  if (numQuads)
    k_quadIndices<<<(numQuads + 255) / 256, 256, 0, s>>>(idx4, numQuads, out);
  return cudaGetLastError();
}

cudaError_t launchGatherTriangles(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    const uint32_t *order,
    uint32_t n,
    TriRecord *out,
    cudaStream_t s)
{
  if (n)
    k_gatherTris<<<(n + 255) / 256, 256, 0, s>>>(
        geoms, refs, surfaces, order, n, out);
  return cudaGetLastError();
}

cudaError_t launchGatherSpheres(const GeometryGPU *geoms,
    const uint2 *refs,
    const SurfaceGPU *surfaces,
    const uint32_t *order,
    uint32_t n,
    SphereRecord *out,
    cudaStream_t s)
{
  if (n)
    k_gatherSpheres<<<(n + 255) / 256, 256, 0, s>>>(
        geoms, refs, surfaces, order, n, out);
  return cudaGetLastError();
}

cudaError_t launchFillRefs(
    uint32_t surface, uint32_t count, uint2 *out, cudaStream_t s)
{
  if (count)
    k_fillRefs<<<(count + 255) / 256, 256, 0, s>>>(surface, count, out);
  return cudaGetLastError();
}

cudaError_t launchMacrocellRanges(cudaTextureObject_t field,
    const int dims[3],
    const int mcDims[3],
    float *ranges,
    cudaStream_t s)
{
  const int cells = mcDims[0] * mcDims[1] * mcDims[2];
  if (cells)
    k_mcRanges<<<cells, 256, 0, s>>>(field,
        dims[0],
        dims[1],
        dims[2],
        mcDims[0],
        mcDims[1],
        mcDims[2],
        ranges);
  return cudaGetLastError();
}

cudaError_t launchMacrocellMajorants(const float *ranges,
    const int mcDims[3],
    const float4 *tf,
    int tfSize,
    float valueLo,
    float valueHi,
    float uniformOpacity,
    float *majorants,
    unsigned *emptyCells,
    cudaStream_t s)
{
  const int cells = mcDims[0] * mcDims[1] * mcDims[2];
  if (cells)
    k_mcMajorants<<<(cells + 255) / 256, 256, 0, s>>>(ranges,
        cells,
        tf,
        tfSize,
        valueLo,
        valueHi,
        uniformOpacity,
        majorants,
        emptyCells);
  return cudaGetLastError();
}

} // namespace vrtx
