// Scivis volume integration (device code): the fixed-step emission-absorption
// marcher of the reference (devices/rtx/gpu/volumeIntegration.h:64-165,
// 318-350) with two additions that leave its results unchanged:
//  * in a volume with empty macrocells the march is driven by a 3D DDA over
//    the conservative macrocell grid, and samples in a cell whose majorant
//    is 0 (no voxel the trilinear filter can reach there maps to a non-zero
//    TF alpha) are not fetched: their contribution is exactly zero
//    (1 - pow(1 - 0, x) == 0), and the march position still advances by the
//    same repeated float additions, so every later sample sits where the
//    reference puts it;
//  * the volume "TLAS" is a flat list scanned for the nearest entry, in
//    place of the OptiX volume BVH (the lists here are short).
#pragma once

#include <curand_kernel.h>

#include "gpu_types.h"
#include "nvdb.cuh"

namespace vrtx {

typedef curandStatePhilox4_32_10_t RandState;

struct VolumeHitG
{
  int entry; // index into WorldGPU::volumes
  f3 localOrg, localDir;
  float tlo, thi;
};

// glm::min / glm::max on floats: the first operand where either is NaN
// (where fminf / fmaxf would return the other)
__device__ __forceinline__ float glmMin(float a, float b)
{
  return (b < a) ? b : a;
}
__device__ __forceinline__ float glmMax(float a, float b)
{
  return (a < b) ? b : a;
}

// Slab test in the volume's object space (Intersectors_ptx.cu:248-274):
// glm::min / glm::max per axis and glm::compMax / glm::compMin as left
// folds, so that a ray parallel to a bounding plane with its origin on it
// (a NaN slab) enters or misses as the reference's does; clamped to the ray
// interval [tmin, tmax] (gpu_math.h clamp).
__device__ __forceinline__ bool volumeSlab(const VolumeGPU &v,
    f3 worldOrg,
    f3 worldDir,
    float tmin,
    float tmax,
    VolumeHitG &h)
{
  const f3 lo = xfmPoint(v.worldToObject, worldOrg);
  const f3 ld = xfmVector(v.worldToObject, worldDir);
  const f3 inv = mk3(1.f / ld.x, 1.f / ld.y, 1.f / ld.z);
  const f3 mins = (v.bounds.lo - lo) * inv;
  const f3 maxs = (v.bounds.hi - lo) * inv;
  const f3 nears = mk3(glmMin(mins.x, maxs.x), glmMin(mins.y, maxs.y), glmMin(mins.z, maxs.z));
  const f3 fars = mk3(glmMax(mins.x, maxs.x), glmMax(mins.y, maxs.y), glmMax(mins.z, maxs.z));
  float t0 = glmMax(glmMax(nears.x, nears.y), nears.z);
  float t1 = glmMin(glmMin(fars.x, fars.y), fars.z);
  if (!(t0 < t1))
    return false;
  t0 = glmMax(tmin, glmMin(t0, tmax));
  t1 = glmMax(tmin, glmMin(t1, tmax));
  h.localOrg = lo;
  h.localDir = ld;
  h.tlo = t0;
  h.thi = t1;
  return true;
}

// Closest volume entry in [tmin, tmax], skipping `skip` (the reference's
// lastVolID/lastInstID test).
__device__ __forceinline__ bool intersectVolumes(const WorldGPU &w,
    f3 org,
    f3 dir,
    float tmin,
    float tmax,
    int skip,
    VolumeHitG &best)
{
  bool found = false;
  for (uint32_t i = 0; i < w.numVolumes; i++) {
    if ((int)i == skip)
      continue;
    VolumeHitG h;
    if (volumeSlab(w.volumes[i], org, dir, tmin, tmax, h)) {
      if (!found || h.tlo < best.tlo) {
        best = h;
        best.entry = (int)i;
        found = true;
      }
    }
  }
  return found;
}

__device__ __forceinline__ float sampleField(const VolumeGPU &v, f3 p)
{
  const f3 c = ((p - v.origin) + 0.5f * v.spacing) * v.invSpacing;
  return tex3D<float>(v.field, c.x, c.y, c.z);
}

// Field samplers the marchers are instantiated on (the reference's
// SpatialFieldSampler specialisations, gpu/sampleSpatialField.h:48-109).
struct TextureField
{
  __device__ __forceinline__ float operator()(const VolumeGPU &v, f3 p)
  {
    return sampleField(v, p);
  }
};

struct NanovdbField
{
  __device__ __forceinline__ float operator()(const VolumeGPU &v, f3 p)
  {
    return nvdb::sample(v.nvdb, p);
  }
};

__device__ __forceinline__ float4 classifySample(const VolumeGPU &v, float s)
{
  if (v.hasTF) {
    // position(s, valueRange) (gpu_math.h): clamp, then scale
    const float cs = fmaxf(v.valueLo, fminf(s, v.valueHi));
    const float coord = (cs - v.valueLo) * (1.f / (v.valueHi - v.valueLo));
    return tex1D<float4>(v.tf, coord);
  }
  return make_float4(
      v.uniformColor.x, v.uniformColor.y, v.uniformColor.z, v.uniformOpacity);
}

__device__ __forceinline__ float cellMajorant(const VolumeGPU &v, f3 p)
{
  if (!v.majorants)
    return 1.f;
  // voxel-space position -> macrocell (16 voxels per cell edge)
  const f3 q = (p - v.origin) * mk3(1.f / v.spacing.x, 1.f / v.spacing.y,
                                    1.f / v.spacing.z);
  const int cx = min(max((int)floorf(q.x * (1.f / 16.f)), 0), v.mcDims[0] - 1);
  const int cy = min(max((int)floorf(q.y * (1.f / 16.f)), 0), v.mcDims[1] - 1);
  const int cz = min(max((int)floorf(q.z * (1.f / 16.f)), 0), v.mcDims[2] - 1);
  return __ldg(v.majorants
      + ((size_t)cz * v.mcDims[1] + cy) * v.mcDims[0] + cx);
}

// One sample of the march: classify, composite front to back
// (volumeIntegration.h:46-103).
__device__ __forceinline__ void compositeSample(const VolumeGPU &v,
    float s,
    float exponent,
    f3 *color,
    float &opacity,
    float &transmittance)
{
  if (isnan(s))
    return;
  const float4 co = classifySample(v, s);
  const float stepT = powf(1.f - co.w, exponent);
  const float a = transmittance * (1.f - stepT);
  if (color)
    *color += a * mk3(co.x, co.y, co.z);
  opacity += a;
  transmittance *= stepT;
}

// The fixed-step march of a volume with empty macrocells, driven by a 3D
// DDA over the conservative skipping grid (16^3-voxel cells from the field
// origin): each cell gives the ray distance at which the ray leaves it; in
// a cell whose majorant is 0 the samples are only counted and the position
// advances by the same float additions, in a non-empty cell every sample is
// fetched and composited. The samples, their positions and the
// accumulation order are the plain march's, so the result is the same bit
// for bit. A sample within rounding of a cell face can be taken for either
// cell; the majorants cover one voxel of apron around each cell, so either
// cell's majorant bounds it.
template <typename Field>
__device__ __forceinline__ void marchCellsDDA(const VolumeGPU &v,
    Field &field,
    const VolumeHitG &h,
    float lower,
    float upper,
    float stepSize,
    float exponent,
    f3 *color,
    float &opacity,
    TravStats &st)
{
  float transmittance = 1.f;
  // voxel coordinates along the ray: q(t) = qo + qd * t
  const f3 inv = mk3(1.f / v.spacing.x, 1.f / v.spacing.y, 1.f / v.spacing.z);
  const f3 qo = (h.localOrg - v.origin) * inv;
  const f3 qd = h.localDir * inv;
  const f3 q0 = qo + qd * lower;
  int cell[3], stepDir[3];
  float tNext[3], tDelta[3];
  const float o[3] = {qo.x, qo.y, qo.z}, d[3] = {qd.x, qd.y, qd.z}, q[3] = {q0.x, q0.y, q0.z};
#pragma unroll
  for (int a = 0; a < 3; a++) {
    cell[a] = min(max((int)floorf(q[a] * (1.f / 16.f)), 0), v.mcDims[a] - 1);
    if (d[a] > 0.f) {
      stepDir[a] = 1;
      tNext[a] = (16.f * float(cell[a] + 1) - o[a]) / d[a];
      tDelta[a] = 16.f / d[a];
    } else if (d[a] < 0.f) {
      stepDir[a] = -1;
      tNext[a] = (16.f * float(cell[a]) - o[a]) / d[a];
      tDelta[a] = -16.f / d[a];
    } else {
      stepDir[a] = 0;
      tNext[a] = __int_as_float(0x7f800000);
      tDelta[a] = 0.f;
    }
  }
  bool inGrid = true;
  int guard = 0;
  while (guard < (1 << 24) && opacity < 0.99f && upper - lower >= 0.f) {
    const int a = tNext[0] <= tNext[1] ? (tNext[0] <= tNext[2] ? 0 : 2)
                                       : (tNext[1] <= tNext[2] ? 1 : 2);
    // past the grid (rounding at its far face): march the rest as non-empty
    const float tExit = inGrid ? tNext[a] : __int_as_float(0x7f800000);
    const float maj = inGrid
        ? __ldg(v.majorants + ((size_t)cell[2] * v.mcDims[1] + cell[1]) * v.mcDims[0] + cell[0])
        : 1.f;
    if (maj == 0.f) {
      for (; guard < (1 << 24) && lower <= tExit && upper - lower >= 0.f; guard++) {
        st.samples++;
        lower += stepSize;
      }
    } else {
      for (; guard < (1 << 24) && lower <= tExit && opacity < 0.99f && upper - lower >= 0.f;
           guard++) {
        st.samples++;
        st.fetches++;
        const float s = field(v, h.localOrg + h.localDir * lower);
        compositeSample(v, s, exponent, color, opacity, transmittance);
        lower += stepSize;
      }
    }
    if (!inGrid)
      break;
    cell[a] += stepDir[a];
    tNext[a] += tDelta[a];
    inGrid = cell[a] >= 0 && cell[a] < v.mcDims[a];
    guard++;
  }
}

// rayMarchVolume + _rayMarchVolume (volumeIntegration.h:64-126): returns the
// entry depth; accumulates into color (when non-null) and opacity.
template <typename Field>
__device__ __forceinline__ float rayMarchVolumeF(const VolumeGPU &v,
    Field &field,
    const VolumeHitG &h,
    RandState &rs,
    f3 *color,
    float &opacity,
    float invSamplingRate,
    TravStats &st)
{
  float lower = h.tlo;
  const float upper = h.thi;
  const float depth = lower;
  lower += v.stepSize * curand_uniform(&rs); // first jitter (unscaled step)
  const float stepSize = v.stepSize * invSamplingRate;
  const float exponent = stepSize * v.oneOverUnitDistance;
  lower += stepSize * curand_uniform(&rs); // second jitter
  float transmittance = 1.f;
  if (!(stepSize > 0.f))
    return depth;
  if (v.majorants) {
    marchCellsDDA(v, field, h, lower, upper, stepSize, exponent, color, opacity, st);
    return depth;
  }
  // Software-pipelined: the field fetch for the next position is issued
  // before the current sample is classified, so the two dependent texture
  // reads of consecutive samples overlap. Positions, the order of the
  // accumulation and the stopping rule are those of the plain loop.
  f3 p = h.localOrg + h.localDir * lower;
  bool want = cellMajorant(v, p) > 0.f;
  float s = want ? field(v, p) : 0.f;
  // bound the march (a ray through a 2^24-step box is not a real scene)
  for (int guard = 0; guard < (1 << 24) && opacity < 0.99f && upper - lower >= 0.f;
       guard++) {
    st.samples++;
    const float next = lower + stepSize;
    bool wantNext = false;
    float sNext = 0.f;
    if (upper - next >= 0.f) {
      const f3 pn = h.localOrg + h.localDir * next;
      wantNext = cellMajorant(v, pn) > 0.f;
      if (wantNext)
        sNext = field(v, pn);
    }
    if (want) {
      st.fetches++;
      if (!isnan(s)) {
        const float4 co = classifySample(v, s);
        const float stepT = powf(1.f - co.w, exponent);
        const float a = transmittance * (1.f - stepT);
        if (color)
          *color += a * mk3(co.x, co.y, co.z);
        opacity += a;
        transmittance *= stepT;
      }
    }
    lower = next;
    want = wantNext;
    s = sNext;
  }
  return depth;
}

// the field-type dispatch of rayMarchVolume (volumeIntegration.h:104-165);
// NV = false compiles the texture field only (worlds without NanoVDB fields)
template <bool NV = true>
__device__ __forceinline__ float rayMarchVolume(const VolumeGPU &v,
    const VolumeHitG &h,
    RandState &rs,
    f3 *color,
    float &opacity,
    float invSamplingRate,
    TravStats &st)
{
  if (NV && v.fieldKind == FIELD_NANOVDB) {
    NanovdbField f;
    return rayMarchVolumeF(v, f, h, rs, color, opacity, invSamplingRate, st);
  }
  TextureField f;
  return rayMarchVolumeF(v, f, h, rs, color, opacity, invSamplingRate, st);
}

// rayMarchAllVolumes (volumeIntegration.h:318-350).
template <bool NV = true>
__device__ __forceinline__ float rayMarchAllVolumes(const WorldGPU &w,
    RandState &rs,
    f3 org,
    f3 dir,
    float tmin,
    float tfar,
    float invSamplingRate,
    f3 &color,
    float &opacity,
    uint32_t &objID,
    uint32_t &instID,
    TravStats &st)
{
  float depth = tfar;
  if (w.numVolumes == 0)
    return depth;
  bool firstHit = true;
  int last = -1;
  do {
    VolumeHitG h;
    if (!intersectVolumes(w, org, dir, tmin, tfar, last, h))
      break;
    const VolumeGPU &v = w.volumes[h.entry];
    if (firstHit) {
      objID = v.id;
      instID = v.instId;
      firstHit = false;
    }
    depth = fminf(depth, h.tlo);
    h.thi = fminf(tfar, h.thi);
    rayMarchVolume<NV>(v, h, rs, &color, opacity, invSamplingRate, st);
    tmin = h.thi + 1e-3f;
    last = h.entry;
  } while (opacity < 0.99f);
  return depth;
}

// volumeAttenuation for shadow rays (DirectLight_ptx.cu:45-52,245-255): the
// any-hit march over every volume the shadow ray crosses, until >= 0.99.
__device__ __forceinline__ float volumeAttenuation(const WorldGPU &w,
    RandState &rs,
    f3 org,
    f3 dir,
    float tmin,
    float tmax,
    float invSamplingRate,
    TravStats &st)
{
  float a = 0.f;
  for (uint32_t i = 0; i < w.numVolumes; i++) {
    VolumeHitG h;
    if (!volumeSlab(w.volumes[i], org, dir, tmin, tmax, h))
      continue;
    h.entry = (int)i;
    rayMarchVolume(w.volumes[i], h, rs, nullptr, a, invSamplingRate, st);
    if (a >= 0.99f)
      break;
  }
  return a;
}

// dda3 (gpu/dda.h:44-122) over the delta-tracking grid (dims cells across
// `bounds`). Multiply-adds are written as fma so that the cell boundaries
// do not depend on the compiler's contraction choices.
template <typename F>
__device__ __forceinline__ void dda3(
    f3 org, f3 dir, float tlo, float thi, const int dims[3], box3 bounds, F func)
{
  const f3 rcp = mk3(dir.x != 0.f ? 1.f / dir.x : 0.f,
      dir.y != 0.f ? 1.f / dir.y : 0.f,
      dir.z != 0.f ? 1.f / dir.z : 0.f);
  const f3 lo = (bounds.lo - org) * rcp;
  const f3 hi = (bounds.hi - org) * rcp;
  const f3 tnear = fmin3(lo, hi);
  const f3 tfar = fmax3(lo, hi);
  // projectOnGrid (gpu/uniformGrid.h:43-50)
  int cx = min(max(__float2int_rz(__fmul_rn(__fdiv_rn(org.x - bounds.lo.x,
                                                bounds.hi.x - bounds.lo.x),
                                       float(dims[0]))),
                   0),
      dims[0] - 1);
  int cy = min(max(__float2int_rz(__fmul_rn(__fdiv_rn(org.y - bounds.lo.y,
                                                bounds.hi.y - bounds.lo.y),
                                       float(dims[1]))),
                   0),
      dims[1] - 1);
  int cz = min(max(__float2int_rz(__fmul_rn(__fdiv_rn(org.z - bounds.lo.z,
                                                bounds.hi.z - bounds.lo.z),
                                       float(dims[2]))),
                   0),
      dims[2] - 1);
  const f3 dist = mk3(__fdiv_rn(tfar.x - tnear.x, float(dims[0])),
      __fdiv_rn(tfar.y - tnear.y, float(dims[1])),
      __fdiv_rn(tfar.z - tnear.z, float(dims[2])));
  const int sx = dir.x > 0.f ? 1 : -1, sy = dir.y > 0.f ? 1 : -1,
            sz = dir.z > 0.f ? 1 : -1;
  const int stx = dir.x > 0.f ? dims[0] : -1, sty = dir.y > 0.f ? dims[1] : -1,
            stz = dir.z > 0.f ? dims[2] : -1;
  f3 tnext = mk3(
      __fmaf_rn(float(dir.x > 0.f ? cx + 1 : dims[0] - cx), dist.x, tnear.x),
      __fmaf_rn(float(dir.y > 0.f ? cy + 1 : dims[1] - cy), dist.y, tnear.y),
      __fmaf_rn(float(dir.z > 0.f ? cz + 1 : dims[2] - cz), dist.z, tnear.z));
  float t0 = fmaxf(tlo, 0.f);
  // every pass steps at least one axis; a cell walk ends within the sum of
  // the dims (the bound only guards against NaN coordinates)
  for (int guard = 0; guard < 4 * (dims[0] + dims[1] + dims[2]) + 8; guard++) {
    const float t1 = fminf(compMin(tnext), thi);
    const size_t cell = ((size_t)cz * dims[1] + cy) * dims[0] + cx;
    if (!func(cell, t0, t1))
      return;
    const float tc = compMin(tnext);
    if (tnext.x == tc) {
      tnext.x += dist.x;
      cx += sx;
      if (cx == stx)
        break;
    }
    if (tnext.y == tc) {
      tnext.y += dist.y;
      cy += sy;
      if (cy == sty)
        break;
    }
    if (tnext.z == tc) {
      tnext.z += dist.z;
      cz += sz;
      if (cz == stz)
        break;
    }
    t0 = t1;
  }
}

// _sampleDistance (volumeIntegration.h:167-238): Woodcock tracking inside
// each DDA cell against the cell majorant, t -= log(1-u)/majorant*stepSize.
template <typename Field>
__device__ __forceinline__ float sampleDistanceF(const VolumeGPU &v,
    Field &field,
    const VolumeHitG &h,
    RandState &rs,
    f3 &albedo,
    float &extinction,
    float &tr)
{
  const float stepSize = v.stepSize;
  float t_out = h.thi;
  tr = 1.f;
  const f3 org = mk3(__fmaf_rn(h.localDir.x, h.tlo, h.localOrg.x),
      __fmaf_rn(h.localDir.y, h.tlo, h.localOrg.y),
      __fmaf_rn(h.localDir.z, h.tlo, h.localOrg.z));
  const float tlo = 0.f, thi = h.thi - h.tlo;
  dda3(org, h.localDir, tlo, thi, v.mcDims, v.bounds, [&](size_t cell, float t0, float t1) {
    const float majorant = v.dptMajorants ? __ldg(v.dptMajorants + cell) : 1.f;
    float t = t0;
    // a cell ends after finitely many draws (t grows by a positive amount
    // each time unless a draw is exactly 0); the bound only guards that
    for (int guard = 0; guard < (1 << 20); guard++) {
      if (majorant <= 0.f)
        break;
      const float lg = logf(1.f - curand_uniform(&rs));
      t = __fmaf_rn(-__fdiv_rn(lg, majorant), stepSize, t);
      if (t >= t1)
        break;
      const float tt = t + h.tlo;
      const f3 p = mk3(__fmaf_rn(h.localDir.x, tt, h.localOrg.x),
          __fmaf_rn(h.localDir.y, tt, h.localOrg.y),
          __fmaf_rn(h.localDir.z, tt, h.localOrg.z));
      const float s = field(v, p);
      if (!isnan(s)) {
        const float4 co = classifySample(v, s);
        albedo = mk3(co.x, co.y, co.z);
        extinction = co.w;
        const float u = curand_uniform(&rs);
        if (extinction >= u * majorant) {
          tr = 0.f;
          t_out = t;
          return false;
        }
      }
    }
    return true;
  });
  return t_out + h.tlo;
}

// the field-type dispatch of sampleDistance (volumeIntegration.h:240-300)
template <bool NV = true>
__device__ __forceinline__ float sampleDistance(const VolumeGPU &v,
    const VolumeHitG &h,
    RandState &rs,
    f3 &albedo,
    float &extinction,
    float &tr)
{
  if (NV && v.fieldKind == FIELD_NANOVDB) {
    NanovdbField f;
    return sampleDistanceF(v, f, h, rs, albedo, extinction, tr);
  }
  TextureField f;
  return sampleDistanceF(v, f, h, rs, albedo, extinction, tr);
}

// sampleDistanceAllVolumes (volumeIntegration.h:352-389)
template <bool NV = true>
__device__ __forceinline__ float sampleDistanceAllVolumes(const WorldGPU &w,
    RandState &rs,
    f3 org,
    f3 dir,
    float tmin,
    float tfar,
    f3 &albedo,
    float &extinction,
    float &transmittance,
    uint32_t &objID,
    uint32_t &instID)
{
  float depth = tfar;
  transmittance = 1.f;
  int last = -1;
  for (uint32_t guard = 0; guard <= w.numVolumes; guard++) {
    VolumeHitG h;
    if (!intersectVolumes(w, org, dir, tmin, tfar, last, h))
      break;
    const VolumeGPU &v = w.volumes[h.entry];
    h.thi = fminf(tfar, h.thi);
    f3 alb = mk3(0.f, 0.f, 0.f);
    float ext = 0.f, tr = 0.f;
    const float d = sampleDistance<NV>(v, h, rs, alb, ext, tr);
    if (d < depth) {
      depth = d;
      albedo = alb;
      extinction = ext;
      transmittance = tr;
      objID = v.id;
      instID = v.instId;
    }
    tmin = h.thi + 1e-3f;
    last = h.entry;
  }
  return depth;
}

} // namespace vrtx
