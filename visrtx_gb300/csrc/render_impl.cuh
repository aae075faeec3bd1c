// Integrator device code and the per-pixel kernel template, shared by the
// translation units that instantiate it (render.cu: worlds with surfaces;
// render_volume.cu: volume-only worlds; render_ao.cu: the wavefront AO
// kernels). Every definition sits in an anonymous namespace, so each unit
// compiles its own copy of what it launches.
//
// Integrator kernels: one persistent kernel per renderer subtype.
//
// Each thread renders one pixel for all pixelSamples iterations, exactly as
// the reference's raygen programs do (one launch index per pixel, RNG state
// curand_init(y*w + x, 0, frameID*512) carried across the sample loop,
// createScreenSample.h:48-65), so the Philox stream each pixel consumes is
// the reference's. Warps pull 8x4 pixel tiles from a global counter (a
// per-warp work queue), which balances cheap background tiles against
// expensive ones without a second launch.
//
// Renderers follow:
//   directLight/default  renderer/DirectLight_ptx.cu:73-224, 294-418
//   raycast              renderer/Raycast_ptx.cu:60-179
//   ao                   renderer/AmbientOcclusion_ptx.cu:86-220
//   dpt                  renderer/DiffusePathTracer_ptx.cu:82-215
// with the output path of gpu/gpu_util.h:321-443.
#pragma once

#include "render.h"
#include "traverse.cuh"
#include "volume.cuh"

// Minimum resident 128-thread blocks per SM requested from ptxas for the
// integrator kernels (caps registers per thread at 65536 / (128 * value)).
#ifndef VRTX_RENDER_MIN_BLOCKS
#define VRTX_RENDER_MIN_BLOCKS 1
#endif
// The same for the any-hit queue kernel (8: <= 64 registers per thread).
#ifndef VRTX_AO_REFILL
#define VRTX_AO_REFILL 4
#endif

// leaf postponement in the AO any-hit kernel: a warp tests leaf groups once
// this percentage of its live lanes hold one (0: every step, no postponing);
// on the instanced AO bench 30 measured 681.6 Mrays/s against 667.4 at 50,
// 615.8 at 65 and 671.8 at 15
#ifndef VRTX_AO_LEAF_TURN
#define VRTX_AO_LEAF_TURN 30
#endif

// traversal steps per lane between the AO any-hit kernel's queue refills
// (3: fewer refill votes per node test; more leave lanes idle at a ray's end)
#ifndef VRTX_AO_STEPS
#define VRTX_AO_STEPS 3
#endif

// traversal stack entries of the AO any-hit kernel kept in shared memory
#ifndef VRTX_AO_SHARED_STACK
#define VRTX_AO_SHARED_STACK 16
#endif

// blocks per SM the per-pixel kernel is compiled for on worlds without
// surfaces (volume-only frames)
#ifndef VRTX_VOLUME_MIN_BLOCKS
#define VRTX_VOLUME_MIN_BLOCKS 8
#endif

// the same for volume-only worlds holding a NanoVDB field (the tree walk
// and its per-thread accessor need more registers than the texture fetch)
#ifndef VRTX_NANOVDB_MIN_BLOCKS
#define VRTX_NANOVDB_MIN_BLOCKS 4
#endif

// the same for the wavefront primary (closest-hit) kernels of "ao",
// "default" and "raycast" (5: <= 102 registers; a few spills, more warps)
#ifndef VRTX_PRIMARY_MIN_BLOCKS
#define VRTX_PRIMARY_MIN_BLOCKS 5
#endif

#ifndef VRTX_TRACE_MIN_BLOCKS
#define VRTX_TRACE_MIN_BLOCKS 8
#endif

namespace vrtx {

namespace {

constexpr float kFltMax = 3.402823466e+38f;

// --- ray generation ----------------------------------------------------------

__device__ __forceinline__ int computePixelX(int idx, int cb)
{
  return cb < 0 ? idx : idx * 2 + (cb & 0x1);
}
__device__ __forceinline__ int computePixelY(int idy, int cb)
{
  return cb < 0 ? idy : idy * 2 + ((cb >> 1) & 0x1);
}

__device__ __forceinline__ float mixf(float a, float b, float t)
{
  return a * (1.f - t) + b * t;
}

struct Ray
{
  f3 org, dir;
  float tmin, tmax;
};

// makePrimaryRay + cameraCreateRay (gpu/cameraCreateRay.h:38-81)
__device__ __forceinline__ Ray makePrimaryRay(const FrameParams &P,
    RandState &rs,
    int px,
    int py,
    bool centerPixel,
    float &screenX,
    float &screenY)
{
  const float4 r = curand_uniform4(&rs);
  const float sx0 = centerPixel ? (float)px : (float)px + r.x;
  const float sy0 = centerPixel ? (float)py : (float)py + r.y;
  screenX = sx0 * P.fb.invW;
  screenY = sy0 * P.fb.invH;
  const CameraGPU &c = P.camera;
  const float sx = mixf(c.region[0], c.region[2], screenX);
  const float sy = mixf(c.region[1], c.region[3], screenY);
  Ray ray;
  ray.tmin = 0.f;
  ray.tmax = kFltMax;
  if (c.type == CAMERA_PERSPECTIVE) {
    ray.org = c.pos;
    ray.dir = c.dir00 + sx * c.dirDu + sy * c.dirDv;
    if (c.scaledAperture > 0.f) {
      // uniformSampleDisk (gpu_math.h)
      const float rr = sqrtf(r.z) * c.scaledAperture;
      const float phi = 2.f * float(M_PI) * r.w;
      const float lx = rr * cosf(phi), ly = rr * sinf(phi);
      const f3 lp = (lx * c.dirDu) + ((ly * c.aspect) * c.dirDv);
      ray.org += lp;
      ray.dir = ray.dir - lp;
    }
    ray.dir = normalize(ray.dir);
  } else {
    ray.dir = c.dir;
    ray.org = c.pos00 + sx * c.posDu + sy * c.posDv;
  }
  return ray;
}

// --- hit population ----------------------------------------------------------

struct SurfaceHit
{
  float t;
  f3 hitpoint;
  f3 Ng, Ns;
  float epsilon;
  uint32_t primID; // geometry-local primitive index (OptiX primID)
  uint32_t surface;
  uint32_t instUserId;
  float u, v; // triangle barycentrics (v1, v2 weights); segments: u
};

// epsilonFrom (gpu_util.h:245-250)
__device__ __forceinline__ float epsilonFrom(f3 P, f3 dir, float t)
{
  const f3 aP = fabs3(P);
  const float m = fmaxf(fmaxf(fmaxf(aP.x, aP.y), aP.z), compMax(fabs3(dir)) * t);
  return m * 0x1.fp-21f;
}

// populateSurfaceHit + computeTangentSpace (gpu/populateHit.h:200-368)
__device__ __forceinline__ void populateSurfaceHit(
    const WorldGPU &w, const Ray &ray, const Hit &h, SurfaceHit &sh)
{
  const InstanceRecord &inst = w.instances[h.inst];
  const BLASDesc &blas = w.blas[inst.blas];
  sh.t = h.t;
  sh.u = h.u;
  sh.v = h.v;
  sh.hitpoint = ray.org + h.t * ray.dir;
  sh.epsilon = epsilonFrom(sh.hitpoint, ray.dir, h.t);
  sh.instUserId = inst.userId;
  f3 Ng, Ns;
  if (blas.type == GEOM_TRIANGLE) {
    const TriRecord tr = reinterpret_cast<const TriRecord *>(blas.prims)[h.rec];
    sh.primID = __float_as_uint(tr.v0.w);
    sh.surface = __float_as_uint(tr.v1.w);
    const f3 v0 = mk3(tr.v0.x, tr.v0.y, tr.v0.z);
    const f3 v1 = mk3(tr.v1.x, tr.v1.y, tr.v1.z);
    const f3 v2 = mk3(tr.v2.x, tr.v2.y, tr.v2.z);
    const GeometryGPU &g = w.geometries[w.surfaces[sh.surface].geometry];
    if (g.kind == KIND_QUAD) {
      // QUAD case (populateHit.h:267-279): unnormalised face normal, no
      // vertex normals
      Ng = cross(v1 - v0, v2 - v0);
      if (!h.front)
        Ng = -Ng;
      Ns = Ng;
    } else {
      Ng = normalize(cross(v1 - v0, v2 - v0));
      if (!h.front)
        Ng = -Ng;
      const float b0 = 1.f - h.u - h.v, b1 = h.u, b2 = h.v;
      if (g.normalsFV) {
        const uint32_t i0 = sh.primID * 3;
        Ns = b0 * g.normalsFV[i0] + b1 * g.normalsFV[i0 + 1]
            + b2 * g.normalsFV[i0 + 2];
      } else if (g.normals) {
        uint32_t i0, i1, i2;
        if (g.indices) {
          i0 = g.indices[3 * sh.primID];
          i1 = g.indices[3 * sh.primID + 1];
          i2 = g.indices[3 * sh.primID + 2];
        } else {
          i0 = 3 * sh.primID;
          i1 = i0 + 1;
          i2 = i0 + 2;
        }
        Ns = b0 * g.normals[i0] + b1 * g.normals[i1] + b2 * g.normals[i2];
      } else
        Ns = Ng;
      Ns = normalize(Ns);
      if (dot(Ng, Ns) < 0.f)
        Ns = -Ns;
    }
  } else if (blas.type == GEOM_SPHERE) {
    const SphereRecord sr =
        reinterpret_cast<const SphereRecord *>(blas.prims)[h.rec];
    sh.primID = sr.primID;
    sh.surface = sr.surface;
    const f3 lo = xfmPoint(inst.worldToObject, ray.org);
    const f3 ld = xfmVector(inst.worldToObject, ray.dir);
    const f3 hp = lo + h.t * ld;
    Ng = Ns = hp - mk3(sr.cr.x, sr.cr.y, sr.cr.z);
  } else {
    const SegRecord sr = reinterpret_cast<const SegRecord *>(blas.prims)[h.rec];
    sh.primID = sr.primID;
    sh.surface = sr.surface;
    if (blas.type == GEOM_CURVE) {
      // CURVE case (populateHit.h:292-303) with curveSurfaceNormal
      // (gpu/curveHelpers.h:91-107) at the object-space hit point
      const f3 p0 = mk3(sr.a.x, sr.a.y, sr.a.z);
      const f3 d = mk3(sr.b.x, sr.b.y, sr.b.z) - p0;
      const float rad = sr.a.w + (sr.b.w - sr.a.w) * h.u;
      const f3 ps = xfmPoint(inst.worldToObject, sh.hitpoint);
      f3 o1 = ps - (p0 + h.u * d);
      o1 = o1 - (dot(o1, d) / dot(d, d)) * d;
      o1 = o1 * (rad / sqrtf(dot(o1, o1)));
      Ng = Ns = normalize(o1);
    } else {
      // SPHERE / CONE / CYLINDER case: the intersector's normal attribute
      Ng = Ns = h.n;
    }
  }
  sh.Ng = normalize(xfmNormalTransposed(inst.worldToObject, Ng));
  sh.Ns = normalize(xfmNormalTransposed(inst.worldToObject, Ns));
}

// computeGeometryPrimId (gpu_util.h:309-315)
__device__ __forceinline__ uint32_t geometryPrimId(
    const WorldGPU &w, const SurfaceHit &sh)
{
  const GeometryGPU &g = w.geometries[w.surfaces[sh.surface].geometry];
  return g.primIds ? g.primIds[sh.primID] : sh.primID;
}

// The shading state of a hit (MatteShadingState / PhysicallyBasedShadingState)
struct MatteState
{
  f3 baseColor;
  float opacity;
  uint32_t type; // MaterialType
  float metallic, roughness, ior; // physicallyBased
};

// --- geometry attributes and material parameters ---------------------------

// attribute arithmetic, rounded per operation (no contraction) so that
// interpolated values feeding sampler coordinates are build-independent
__device__ __forceinline__ float4 f4add(float4 a, float4 b)
{
  return make_float4(
      __fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w));
}
__device__ __forceinline__ float4 f4sub(float4 a, float4 b)
{
  return make_float4(
      __fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z), __fsub_rn(a.w, b.w));
}
__device__ __forceinline__ float4 f4mul(float4 a, float s)
{
  return make_float4(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s), __fmul_rn(a.w, s));
}

// glm::convertLinearToSRGB (gamma 0.41666) on one channel
__device__ __forceinline__ float srgbEncode(float c)
{
  const float x = fminf(fmaxf(c, 0.f), 1.f);
  return x < 0.0031308f ? x * 12.92f : powf(x, 0.41666f) * 1.055f - 0.055f;
}

// getAttributeValue (gpu/evalMaterialParameters.h:60-99): element `offset`
// of an attribute array as a vec4 (missing channels 0, alpha 1; fixed-point
// normalised; sRGB8 values passed through the linear-to-sRGB conversion as
// the reference does)
__device__ __forceinline__ float4 attrValue(const AttrGPU &a, uint32_t offset, float4 uf)
{
  if (!a.data || offset == 0xFFFFFFFFu)
    return uf;
  switch (a.type) {
  case 240: { // FLOAT32
    const float *p = (const float *)a.data;
    return make_float4(p[offset], 0.f, 0.f, 1.f);
  }
  case 241: { // FLOAT32_VEC2
    const float *p = (const float *)a.data + 2 * (size_t)offset;
    return make_float4(p[0], p[1], 0.f, 1.f);
  }
  case 242: { // FLOAT32_VEC3
    const float *p = (const float *)a.data + 3 * (size_t)offset;
    return make_float4(p[0], p[1], p[2], 1.f);
  }
  case 243: // FLOAT32_VEC4
    return ((const float4 *)a.data)[offset];
  case 221: { // UFIXED8
    const uint8_t *p = (const uint8_t *)a.data;
    return make_float4(p[offset] / 255.f, 0.f, 0.f, 1.f);
  }
  case 223: { // UFIXED16
    const uint16_t *p = (const uint16_t *)a.data;
    return make_float4(p[offset] / 65535.f, 0.f, 0.f, 1.f);
  }
  case 260: // UFIXED8_VEC4
  case 261: { // UFIXED8_RGBA_SRGB
    const uint8_t *p = (const uint8_t *)a.data + 4 * (size_t)offset;
    float4 r = make_float4(p[0] / 255.f, p[1] / 255.f, p[2] / 255.f, p[3] / 255.f);
    if (a.type == 261)
      r = make_float4(srgbEncode(r.x), srgbEncode(r.y), srgbEncode(r.z), r.w);
    return r;
  }
  default:
    return uf;
  }
}

// readAttributeValue (gpu/evalMaterialParameters.h:131-263) for attribute
// slot `id` (0..3 attribute0..3, 4 color): per-vertex values interpolated
// per subtype, then per-primitive values, then the geometry's uniform value.
// (Instance attributes and face-varying attributes are not read.)
__device__ __forceinline__ float4 readAttribute(
    const WorldGPU &w, const SurfaceHit &sh, int id)
{
  const GeometryGPU &g = w.geometries[w.surfaces[sh.surface].geometry];
  const float4 uf = g.uattr[id];
  const AttrGPU &ap = g.vattr[id];
  const uint32_t prim = sh.primID;
  if (ap.data) {
    const float b0 = 1.f - sh.u - sh.v, b1 = sh.u, b2 = sh.v;
    switch (g.kind) {
    case KIND_TRIANGLE: {
      uint32_t i0, i1, i2;
      if (g.indices) {
        i0 = g.indices[3 * prim];
        i1 = g.indices[3 * prim + 1];
        i2 = g.indices[3 * prim + 2];
      } else {
        i0 = 3 * prim;
        i1 = i0 + 1;
        i2 = i0 + 2;
      }
      return f4add(f4add(f4mul(attrValue(ap, i0, uf), b0), f4mul(attrValue(ap, i1, uf), b1)),
          f4mul(attrValue(ap, i2, uf), b2));
    }
    case KIND_QUAD: {
      // corners (x, y, w, z) of the quad from its two triangles
      const uint32_t pair = prim & ~1u;
      const uint32_t x = g.indices[3 * pair], y = g.indices[3 * pair + 1],
                     wI = g.indices[3 * pair + 2], z = g.indices[3 * (pair + 1)];
      const float4 v0 = attrValue(ap, x, uf), v1 = attrValue(ap, y, uf);
      const float4 v2 = attrValue(ap, z, uf), v3 = attrValue(ap, wI, uf);
      const float qu = (prim & 1u) ? b1 : 1.f - b1;
      const float qv = (prim & 1u) ? b2 : 1.f - b2;
      const float4 l0 = f4add(v1, f4mul(f4sub(v0, v1), qu));
      const float4 l1 = f4add(v2, f4mul(f4sub(v3, v2), qu));
      return f4add(l1, f4mul(f4sub(l0, l1), qv));
    }
    case KIND_CYLINDER:
    case KIND_CONE: {
      const uint32_t i0 = g.indices ? g.indices[2 * prim] : 2 * prim;
      const uint32_t i1 = g.indices ? g.indices[2 * prim + 1] : 2 * prim + 1;
      // uvw = (0, u, 1 - u)
      return f4add(f4mul(attrValue(ap, i0, uf), 1.f - sh.u), f4mul(attrValue(ap, i1, uf), sh.u));
    }
    case KIND_CURVE: {
      const uint32_t i0 = g.indices ? g.indices[prim] : prim;
      return f4add(f4mul(attrValue(ap, i0, uf), 1.f - sh.u), f4mul(attrValue(ap, i0 + 1, uf), sh.u));
    }
    default: { // sphere
      const uint32_t i = g.indices ? g.indices[prim] : prim;
      return attrValue(ap, i, uf);
    }
    }
  }
  const AttrGPU &pp = g.pattr[id];
  if (pp.data)
    return attrValue(pp, g.kind == KIND_QUAD ? prim / 2 : prim, uf);
  return uf;
}

// column-major 4x4 times a vec4, plus an offset (glm's mat4 * vec4 sums
// the column products pairwise: (c0 + c1) + (c2 + c3)); rounded per
// operation, without contraction, so image lookups see the same coordinates
// on every build
__device__ __forceinline__ float4 affine4(const float *m, float4 v, float4 o)
{
  float r[4];
#pragma unroll
  for (int i = 0; i < 4; i++)
    r[i] = __fadd_rn(__fadd_rn(__fmul_rn(m[i], v.x), __fmul_rn(m[4 + i], v.y)),
        __fadd_rn(__fmul_rn(m[8 + i], v.z), __fmul_rn(m[12 + i], v.w)));
  return make_float4(
      __fadd_rn(r[0], o.x), __fadd_rn(r[1], o.y), __fadd_rn(r[2], o.z), __fadd_rn(r[3], o.w));
}

// evaluateSampler (gpu/evalMaterialParameters.h:291-334): the input
// attribute through the input map, an image lookup / the primitive array /
// the mapped value itself, then the output map
__device__ __forceinline__ float4 evaluateSampler(
    const WorldGPU &w, const SurfaceHit &sh, const SamplerGPU &sm)
{
  float4 r = make_float4(0.f, 0.f, 0.f, 1.f);
  const float4 tc = affine4(sm.inT, readAttribute(w, sh, (int)sm.attribute), sm.inO);
  switch (sm.type) {
  case SAMPLER_IMAGE1D:
    r = tex1D<float4>(sm.tex, tc.x);
    break;
  case SAMPLER_IMAGE2D:
    r = tex2D<float4>(sm.tex, tc.x, tc.y);
    break;
  case SAMPLER_IMAGE3D:
    r = tex3D<float4>(sm.tex, tc.x, tc.y, tc.z);
    break;
  case SAMPLER_PRIMITIVE:
    r = attrValue(sm.prim, sh.primID + sm.primOffset, r);
    break;
  case SAMPLER_TRANSFORM:
    r = tc;
    break;
  default:
    break;
  }
  return affine4(sm.outT, r, sm.outO);
}

// getMaterialParameter (gpu/evalMaterialParameters.h:336-374)
__device__ __forceinline__ float4 materialParam(const WorldGPU &w,
    const SurfaceHit &sh,
    uint32_t src,
    float4 value,
    uint32_t sampler)
{
  switch (src) {
  case PARAM_VALUE:
    return value;
  case PARAM_SAMPLER:
    return evaluateSampler(w, sh, w.samplers[sampler]);
  case PARAM_ATTRIB_0:
  case PARAM_ATTRIB_0 + 1:
  case PARAM_ATTRIB_0 + 2:
  case PARAM_ATTRIB_0 + 3:
    return readAttribute(w, sh, (int)(src - PARAM_ATTRIB_0));
  case PARAM_ATTRIB_COLOR:
    return readAttribute(w, sh, 4);
  case PARAM_WORLD_POSITION:
  case PARAM_OBJECT_POSITION: // world space, as the reference
    return make_float4(sh.hitpoint.x, sh.hitpoint.y, sh.hitpoint.z, 1.f);
  case PARAM_WORLD_NORMAL:
  case PARAM_OBJECT_NORMAL:
    return make_float4(sh.Ns.x, sh.Ns.y, sh.Ns.z, 1.f);
  default:
    return make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

__device__ __forceinline__ float4 materialParamSlot(
    const WorldGPU &w, const SurfaceHit &sh, const MaterialGPU &m, int slot)
{
  const MaterialParamGPU &p = m.params[slot];
  return materialParam(w, sh, p.src, p.value, p.sampler);
}

// The material's init callable (MatteShader_ptx.cu:38-49,
// PhysicallyBasedShader_ptx.cu:41-58): colour and opacity parameters,
// opacity = adjustedMaterialOpacity(color.w * opacity.x); physicallyBased
// also reads metallic, roughness and ior.
__device__ __forceinline__ MatteState matteInit(const WorldGPU &w, const SurfaceHit &sh)
{
  const MaterialGPU &m = w.materials[w.surfaces[sh.surface].material];
  MatteState s;
  float op;
  if (m.params[MP_COLOR].src == PARAM_VALUE && m.params[MP_OPACITY].src == PARAM_VALUE) {
    s.baseColor = m.color;
    op = m.opacity;
  } else {
    const float4 c = materialParamSlot(w, sh, m, MP_COLOR);
    const float o = materialParamSlot(w, sh, m, MP_OPACITY).x;
    s.baseColor = mk3(c.x, c.y, c.z);
    op = c.w * o;
  }
  s.opacity = m.alphaMode == ALPHA_OPAQUE
      ? 1.f
      : (m.alphaMode == ALPHA_BLEND ? op : (op < m.cutoff ? 0.f : 1.f));
  s.type = m.type;
  s.metallic = s.roughness = 0.f;
  s.ior = m.ior;
  if (m.type == MATERIAL_PBR) {
    s.metallic = materialParamSlot(w, sh, m, MP_METALLIC).x;
    s.roughness = materialParamSlot(w, sh, m, MP_ROUGHNESS).x;
  }
  return s;
}

// --- lights (gpu/sampleLight.h) ---------------------------------------------

struct LightSample
{
  f3 radiance;
  f3 dir;
  float dist;
  float pdf;
};

// glm::normalize: v * (1 / sqrt(dot(v, v)))
__device__ __forceinline__ f3 glmNormalize(f3 v)
{
  return v * (1.f / sqrtf(dot(v, v)));
}

// the HDRI radiance texture at uv (sampleHDRI, gpu_util.h:270-273)
__device__ __forceinline__ f3 hdriAt(const LightGPU &L, float u, float v)
{
  const float4 t = tex2D<float4>(L.hdriTex, u, v);
  return mk3(t.x, t.y, t.z);
}

// sampleHDRI(ld, rayDir) (gpu_util.h:275-288): the direction through the
// light's rotation, then spherical coordinates as texture coordinates
__device__ __forceinline__ f3 hdriRadiance(const LightGPU &L, f3 dir)
{
  const float *R = L.hdriRot;
  const f3 d = mk3(fmaf(R[2], dir.z, fmaf(R[1], dir.y, R[0] * dir.x)),
      fmaf(R[5], dir.z, fmaf(R[4], dir.y, R[3] * dir.x)),
      fmaf(R[8], dir.z, fmaf(R[7], dir.y, R[6] * dir.x)));
  // sphericalCoordsFromDirection (gpu_math.h:254-261)
  const float theta = acosf(fminf(fmaxf(d.z, -1.f), 1.f));
  const float p = atan2f(d.y, d.x);
  const float phi = p < 0.f ? p + 2.f * float(M_PI) : p;
  const float u = phi * (1.f / (2.f * float(M_PI)));
  const float v = theta * (1.f / float(M_PI));
  return hdriAt(L, u, v);
}

// getBackground (gpu_util.h:290-307): a visible HDRI, else the background
// image at loc (normalised coordinates), else the colour
__device__ __forceinline__ float4 backgroundOf(const FrameParams &P, f3 dir, float lx, float ly)
{
  const WorldGPU &w = P.world;
  if (w.hdri >= 0 && w.lights[w.hdri].visible) {
    const f3 r = hdriRadiance(w.lights[w.hdri], dir);
    return make_float4(r.x, r.y, r.z, 1.f);
  }
  if (P.renderer.backgroundTex)
    return tex2D<float4>(P.renderer.backgroundTex, lx, ly);
  return P.renderer.background;
}

// inverseSampleCDF (sampleLight.h:105-108): the first entry not below u
// (cub::LowerBound)
__device__ __forceinline__ int lowerBound(const float *cdf, int n, float u)
{
  int lo = 0, count = n;
  while (count > 0) {
    const int half = count >> 1;
    if (__ldg(cdf + lo + half) < u) {
      lo += half + 1;
      count -= half + 1;
    } else {
      count = half;
    }
  }
  return lo;
}

// sampleHDRILight (sampleLight.h:110-149)
__device__ __forceinline__ LightSample sampleHDRILight(const LightGPU &L, RandState &rs)
{
  const int W = (int)L.hdriW, H = (int)L.hdriH;
  const int y = lowerBound(L.marginalCDF, H, curand_uniform(&rs));
  // (a row index past the table only follows from a NaN CDF; clamped so
  // nothing reads outside it)
  const int x = lowerBound(L.conditionalCDF + (size_t)min(y, H - 1) * W, W, curand_uniform(&rs));
  const float u = fminf(fmaxf((float(x) + 0.5f) / float(W), 0.f), 1.f);
  const float v = fminf(fmaxf((float(y) + 0.5f) / float(H), 0.f), 1.f);
  const float theta = float(M_PI) * v, phi = float(M_PI) * (2.f * u);
  const f3 radiance = hdriAt(L, u, v);
  LightSample ls;
  ls.pdf = (radiance.x * 0.2126f + radiance.y * 0.7152f + radiance.z * 0.0722f) * L.pdfWeight;
  // sphericalCoordsToDirection, then row vector times the rotation
  const float sinTheta = sinf(theta);
  const f3 sd = mk3(sinTheta * cosf(phi), sinTheta * sinf(phi), cosf(theta));
  const float *R = L.hdriRot;
  ls.dir = mk3(fmaf(sd.z, R[6], fmaf(sd.y, R[3], sd.x * R[0])),
      fmaf(sd.z, R[7], fmaf(sd.y, R[4], sd.x * R[1])),
      fmaf(sd.z, R[8], fmaf(sd.y, R[5], sd.x * R[2])));
  ls.dist = 1e20f;
  ls.radiance = radiance * L.hdriScale;
  return ls;
}

// sampleLight (sampleLight.h:60-173) for a world-space hit point
__device__ __forceinline__ LightSample sampleLight(const LightGPU &L, f3 hitpoint, RandState &rs)
{
  LightSample ls;
  ls.pdf = 1.f;
  if (L.type == LIGHT_DIRECTIONAL) {
    ls.dir = L.dirToLight;
    ls.dist = __int_as_float(0x7f800000); // +inf
    ls.radiance = L.radiance;
  } else if (L.type == LIGHT_POINT) {
    const f3 d = L.position - hitpoint;
    ls.dist = sqrtf(dot(d, d));
    ls.dir = glmNormalize(d);
    ls.radiance = L.radiance;
  } else if (L.type == LIGHT_SPOT) {
    // the distance is taken of the normalised direction (sampleLight.h:87-88)
    ls.dir = glmNormalize(L.position - hitpoint);
    ls.dist = sqrtf(dot(ls.dir, ls.dir));
    float spot = dot(L.spotDir, -ls.dir);
    if (spot < L.cosOuter)
      spot = 0.f;
    else if (spot > L.cosInner)
      spot = 1.f;
    else {
      spot = (spot - L.cosOuter) / (L.cosInner - L.cosOuter);
      spot = spot * spot * (3.f - 2.f * spot);
    }
    ls.radiance = L.radiance * spot;
  } else {
    ls = sampleHDRILight(L, rs);
  }
  return ls;
}

// --- material evaluation (MatteShader_ptx.cu, PhysicallyBasedShader_ptx.cu)

__device__ __forceinline__ float pow2f(float f)
{
  return f * f;
}

__device__ __forceinline__ float pow5f(float f)
{
  return f * f * f * f * f;
}

__device__ __forceinline__ float heavisidef(float x)
{
  return x < 0.f ? 0.f : 1.f;
}

// shadeSurface: matte Lambert, or the physicallyBased Fresnel-Schlick +
// GGX + Smith model (PhysicallyBasedShader_ptx.cu:98-149)
__device__ __forceinline__ f3 shadeMaterial(
    const MatteState &s, f3 Ns, const LightSample &ls, f3 outgoing)
{
  if (s.type != MATERIAL_PBR) {
    const float NdotL = fmaxf(0.f, dot(Ns, ls.dir));
    return s.baseColor * float(M_1_PI) * NdotL * ls.radiance / ls.pdf;
  }
  const f3 H = glmNormalize(ls.dir + outgoing);
  const float NdotH = dot(Ns, H);
  const float NdotL = dot(Ns, ls.dir);
  const float NdotV = dot(Ns, outgoing);
  const float VdotH = dot(outgoing, H);
  const float LdotH = dot(ls.dir, H);
  const float f0s = pow2f((1.f - s.ior) / (1.f + s.ior));
  // glm::mix(a, b, t) = a * (1 - t) + b * t
  const f3 f0 = mk3(f0s, f0s, f0s) * (1.f - s.metallic) + s.baseColor * s.metallic;
  const float fw = pow5f(1.f - fabsf(VdotH));
  const f3 F = f0 + (mk3(1.f, 1.f, 1.f) - f0) * fw;
  const f3 diffuseColor = s.baseColor * (1.f - s.metallic) + mk3(0.f, 0.f, 0.f) * s.metallic;
  const f3 diffuseBRDF =
      (mk3(1.f, 1.f, 1.f) - F) * float(M_1_PI) * diffuseColor * fmaxf(0.f, NdotL);
  const float alpha = pow2f(s.roughness) * s.opacity;
  const float a2 = alpha * alpha;
  const float D = (a2 * heavisidef(NdotH))
      / (float(M_PI) * pow2f(NdotH * NdotH * (a2 - 1.f) + 1.f));
  const float G = ((2.f * fabsf(NdotL) * heavisidef(LdotH))
                      / (fabsf(NdotL) + sqrtf(a2 + (1.f - a2) * NdotL * NdotL)))
      * ((2.f * fabsf(NdotV) * heavisidef(VdotH))
          / (fabsf(NdotV) + sqrtf(a2 + (1.f - a2) * NdotV * NdotV)));
  const float denom = 4.f * fabsf(NdotV) * fabsf(NdotL);
  const f3 specularBRDF = denom != 0.f ? (F * D * G) / denom : mk3(0.f, 0.f, 0.f);
  return (diffuseBRDF + specularBRDF) * ls.radiance / ls.pdf;
}

struct NextRay
{
  f3 dir;
  f3 weight;
};

// nextRay: none for matte; for physicallyBased a direction in the cone of
// cos = 1 - roughness^2 around the mirror direction, weighted by
// baseColor * metallic (PhysicallyBasedShader_ptx.cu:60-84,
// uniformSampleCone gpu_math.h:299-312, computeOrthonormalBasis)
__device__ __forceinline__ NextRay materialNextRay(
    const MatteState &s, f3 Ns, f3 rayDir, RandState &rs)
{
  NextRay r;
  if (s.type != MATERIAL_PBR) {
    r.dir = mk3(0.f, 0.f, 0.f);
    r.weight = mk3(0.f, 0.f, 0.f);
    return r;
  }
  const f3 refl = rayDir - 2.f * dot(rayDir, Ns) * Ns;
  const float cosThetaMax = 1.f - s.roughness * s.roughness;
  const float s0 = curand_uniform(&rs), s1 = curand_uniform(&rs), s2 = curand_uniform(&rs);
  // phi in double (2.0f * M_PI promotes), then its float sine and cosine
  const float phi = float(2.0 * M_PI * double(s0));
  const float cosTheta = (1.f - s1) + s1 * cosThetaMax;
  const float sinTheta = sqrtf(1.f - cosTheta * cosTheta);
  const float d = powf(s2, 1.f / 3.f);
  const f3 cone = mk3(d * sinTheta * cosf(phi), d * sinTheta * sinf(phi), d * cosTheta);
  const f3 n = glmNormalize(refl);
  const float sign = n.z >= 0.f ? 1.f : -1.f;
  const float a = -1.f / (sign + n.z);
  const float b = n.x * n.y * a;
  const f3 u = mk3(1.f + sign * n.x * n.x * a, sign * b, -sign * n.x);
  const f3 v = mk3(b, sign + n.y * n.y * a, -n.y);
  r.dir = u * cone.x + v * cone.y + n * cone.z;
  r.weight = s.baseColor * s.metallic;
  return r;
}

__device__ __forceinline__ bool anyNan(f3 v)
{
  return isnan(v.x) || isnan(v.y) || isnan(v.z);
}

template <bool STATS>
__device__ __forceinline__ float surfaceAttenuation(const FrameParams &P,
    TravStats &st,
    f3 org,
    f3 dir,
    float tmin,
    float tmax)
{
  Hit h;
  float o;
  traverse<1, STATS>(
      P.world, org, dir, tmin, tmax, false, false, h, o, P.errorFlag, st);
  return o;
}

// randomDir(rs, normal) (gpu_util.h:190-208)
__device__ __forceinline__ f3 randomDir(RandState &rs, f3 n)
{
  const float4 r = curand_uniform4(&rs);
  const f3 d = normalize(mk3(2.f * r.x - 1.f, 2.f * r.y - 1.f, 2.f * r.z - 1.f));
  return dot(d, n) > 0.f ? d : -d;
}

// computeAO (gpu/computeAO.h:38-60)
template <bool STATS>
__device__ __forceinline__ float computeAO(const FrameParams &P,
    TravStats &st,
    RandState &rs,
    const SurfaceHit &hit,
    float dist,
    int numSamples)
{
  float weights = 0.f;
  float hits = 0.f;
  const f3 org = hit.hitpoint + (hit.epsilon * hit.Ng);
  for (int i = 0; i < numSamples; i++) {
    const f3 dir = randomDir(rs, hit.Ns);
    const float weight = fmaxf(0.f, dot(dir, hit.Ns));
    weights += weight;
    if (weight != 0.f)
      hits += weight * surfaceAttenuation<STATS>(P, st, org, dir, 0.f, dist);
  }
  return weights > 0.f ? 1.f - hits / weights : 0.f;
}

// shadeSurface (DirectLight_ptx.cu:73-224) for matte + directional/point
template <bool STATS>
__device__ __forceinline__ float4 shadeSurfaceDL(const FrameParams &P,
    TravStats &st,
    RandState &rs,
    const Ray &ray,
    const SurfaceHit &hit,
    int px,
    int py)
{
  const RendererGPU &rp = P.renderer;
  const WorldGPU &w = P.world;
  f3 shadePoint = hit.hitpoint + (hit.epsilon * hit.Ns);
  const float aoFactor = rp.aoSamples > 0
      ? computeAO<STATS>(P, st, rs, hit, rp.occlusionDistance, rp.aoSamples)
      : 1.f;
  f3 contrib = mk3(0.f, 0.f, 0.f);
  MatteState ms = matteInit(w, hit);
  const float opacity = ms.opacity;
  if (rp.ambientIntensity > 0.f)
    contrib = rp.ambientColor * rp.ambientIntensity * ms.baseColor;
  for (uint32_t l = 0; l < w.numLights; l++) {
    const LightSample ls = sampleLight(w.lights[l], hit.hitpoint, rs);
    if (ls.pdf == 0.f)
      continue;
    const float surface_o =
        1.f - surfaceAttenuation<STATS>(P, st, shadePoint, ls.dir, 0.f, ls.dist);
    const float volume_o = 1.f
        - volumeAttenuation(
            w, rs, shadePoint, ls.dir, 0.f, ls.dist, rp.invVolumeSamplingRate, st);
    const float attenuation = surface_o * volume_o;
    const f3 thisLight = shadeMaterial(ms, hit.Ns, ls, -ray.dir);
    if (anyNan(thisLight))
      continue;
    contrib += thisLight * attenuation;
  }
  contrib *= aoFactor;
  // bounce rays (DirectLight_ptx.cu:154-222): the material's next ray, up to
  // maxRayDepth closest hits, each shaded by the HDRI light or by the
  // background seen along the bounce; matte materials give no next ray
  f3 weight = mk3(1.f, 1.f, 1.f);
  f3 bounceDir = ray.dir;
  f3 Ns = hit.Ns;
  for (int depth = 0; depth < rp.maxRayDepth; depth++) {
    const NextRay nr = materialNextRay(ms, Ns, bounceDir, rs);
    if (!(fabsf(nr.dir.x) > 1.0e-8f && fabsf(nr.dir.y) > 1.0e-8f && fabsf(nr.dir.z) > 1.0e-8f))
      break;
    weight = weight * nr.weight;
    if (weight.x < 1.0e-12f && weight.y < 1.0e-12f && weight.z < 1.0e-12f)
      break;
    Ray br;
    br.org = shadePoint;
    br.dir = glmNormalize(nr.dir);
    br.tmin = 0.f;
    br.tmax = 3.402823466e+38f;
    Hit h;
    float unused;
    const bool found = traverse<0, STATS>(w,
        br.org,
        br.dir,
        br.tmin,
        br.tmax,
        rp.cullTriangleBF != 0,
        true,
        h,
        unused,
        P.errorFlag,
        st);
    bounceDir = br.dir;
    if (found) {
      SurfaceHit bh;
      populateSurfaceHit(w, br, h, bh);
      shadePoint = bh.hitpoint + (bh.epsilon * bh.Ns);
      LightSample ls;
      if (w.hdri >= 0 && w.lights[w.hdri].visible) {
        ls = sampleHDRILight(w.lights[w.hdri], rs);
      } else {
        // the bounce reads the background at the pixel position
        // (DirectLight_ptx.cu:196-200, ss.pixel)
        const float4 bg = backgroundOf(P, br.dir, float(px), float(py));
        ls.radiance = mk3(bg.x, bg.y, bg.z);
        ls.dir = br.dir;
        ls.dist = 1.f;
        ls.pdf = 1.f;
      }
      ms = matteInit(w, bh);
      Ns = bh.Ns;
      const f3 c = shadeMaterial(ms, bh.Ns, ls, -br.dir);
      if (anyNan(c))
        break;
      contrib += c * weight;
    } else {
      const float4 bg = backgroundOf(P, br.dir, float(px), float(py));
      contrib += mk3(bg.x, bg.y, bg.z) * weight;
      break;
    }
  }
  return make_float4(contrib.x, contrib.y, contrib.z, opacity);
}

struct SampleOut
{
  f3 color;
  float opacity;
  f3 albedo; // value accumulated into the albedo channel
  f3 normal;
  float depth;
  uint32_t primID, objID, instID;
};

// SURF = false: the world has no surface instances, so the surface
// traversal (and every shading branch behind a surface hit) compiles away;
// volume-only frames then run with far fewer registers per thread.
template <int RT, bool STATS, bool SURF, bool NV>
__device__ __forceinline__ void integrateSample(const FrameParams &P,
    TravStats &st,
    RandState &rs,
    int px,
    int py,
    SampleOut &o)
{
  const RendererGPU &rp = P.renderer;
  const WorldGPU &w = P.world;
  float scrX, scrY;
  Ray ray =
      makePrimaryRay(P, rs, px, py, RT == RENDERER_RAYCAST, scrX, scrY);
  const float tmax = ray.tmax;
  f3 outputColor = mk3(0.f, 0.f, 0.f);
  f3 outputNormal = ray.dir;
  float outputOpacity = 0.f;
  float depth = 1e30f;
  uint32_t primID = ~0u, objID = ~0u, instID = ~0u;
  bool firstHit = true;
  const bool cull = rp.cullTriangleBF != 0;

  while (outputOpacity < 0.99f) {
    ray.tmax = tmax;
    Hit h;
    float unused;
    // a primary / path ray against an empty surface set still counts
    if (!SURF)
      st.rays++;
    const bool found = SURF && traverse<0, STATS>(w,
        ray.org,
        ray.dir,
        ray.tmin,
        ray.tmax,
        cull,
        true,
        h,
        unused,
        P.errorFlag,
        st);
    f3 color = mk3(0.f, 0.f, 0.f);
    float opacity = 0.f;
    if (found) {
      SurfaceHit sh;
      populateSurfaceHit(w, ray, h, sh);
      uint32_t vObjID = ~0u, vInstID = ~0u;
      const float vDepth = rayMarchAllVolumes<NV>(w,
          rs,
          ray.org,
          ray.dir,
          ray.tmin,
          sh.t,
          rp.invVolumeSamplingRate,
          color,
          opacity,
          vObjID,
          vInstID,
          st);
      if (firstHit) {
        const bool volumeFirst = vDepth < sh.t;
        if (volumeFirst) {
          outputNormal = -ray.dir;
          depth = vDepth;
          primID = 0;
          objID = vObjID;
          instID = vInstID;
        } else {
          outputNormal = RT == RENDERER_DIRECT_LIGHT ? sh.Ns : sh.Ng;
          depth = sh.t;
          primID = geometryPrimId(w, sh);
          objID = w.surfaces[sh.surface].id;
          instID = sh.instUserId;
        }
        firstHit = false;
      }
      if (RT == RENDERER_DIRECT_LIGHT) {
        const float4 sr = shadeSurfaceDL<STATS>(P, st, rs, ray, sh, px, py);
        const f3 srgb = mk3(sr.x, sr.y, sr.z);
        if (anyNan(srgb)) {
          color = mk3(0.f, 0.f, 0.f);
          opacity = 0.f;
        } else {
          color = srgb;
          opacity = sr.w;
        }
        color += srgb * (1.f - opacity);
        opacity += sr.w * (1.f - opacity);
      } else if (RT == RENDERER_RAYCAST) {
        const MatteState ms = matteInit(w, sh);
        const f3 lighting = fabsf(dot(ray.dir, sh.Ns)) * rp.ambientColor;
        color += (ms.baseColor * lighting) * (1.f - opacity);
        opacity += ms.opacity * (1.f - opacity);
      } else { // AO
        const float aoFactor = rp.aoSamples > 0
            ? computeAO<STATS>(P, st, rs, sh, rp.occlusionDistance, rp.aoSamples)
            : 1.f;
        const MatteState ms = matteInit(w, sh);
        const f3 lighting = aoFactor * rp.ambientIntensity * rp.ambientColor;
        color += (ms.baseColor * lighting) * (1.f - opacity);
        opacity += ms.opacity * (1.f - opacity);
      }
      color *= opacity;
      outputColor += color * (1.f - outputOpacity);
      outputOpacity += opacity * (1.f - outputOpacity);
      ray.tmin = sh.t + sh.epsilon;
    } else {
      uint32_t vObjID = ~0u, vInstID = ~0u;
      const float volumeDepth = rayMarchAllVolumes<NV>(w,
          rs,
          ray.org,
          ray.dir,
          ray.tmin,
          ray.tmax,
          rp.invVolumeSamplingRate,
          color,
          opacity,
          vObjID,
          vInstID,
          st);
      if (firstHit) {
        depth = fminf(depth, volumeDepth);
        primID = 0;
        objID = vObjID;
        instID = vInstID;
      }
      color *= opacity;
      const float4 bg = backgroundOf(P, ray.dir, scrX, scrY);
      color += mk3(bg.x, bg.y, bg.z) * (1.f - opacity);
      opacity += bg.w * (1.f - opacity);
      outputColor += color * (1.f - outputOpacity);
      outputOpacity += opacity * (1.f - outputOpacity);
      break;
    }
  }
  o.color = outputColor;
  o.albedo = outputColor;
  o.opacity = outputOpacity;
  o.normal = outputNormal;
  o.depth = depth;
  o.primID = primID;
  o.objID = objID;
  o.instID = instID;
}

// computeOrthonormalBasis (gpu_util.h:210-222), Pixar ONB
__device__ __forceinline__ f3 onbMul(f3 n, f3 s)
{
  const float sign = n.z >= 0.f ? 1.f : -1.f;
  const float a = -1.f / (sign + n.z);
  const float b = n.x * n.y * a;
  const f3 u = mk3(1.f + sign * n.x * n.x * a, sign * b, -sign * n.x);
  const f3 v = mk3(b, sign + n.y * n.y * a, -n.y);
  return u * s.x + v * s.y + n * s.z;
}

// sampleUnitSphere (gpu_util.h:236-243)
__device__ __forceinline__ f3 sampleUnitSphere(RandState &rs, f3 n)
{
  const float cost = 1.f - 2.f * curand_uniform(&rs);
  const float sint = sqrtf(fmaxf(0.f, 1.f - cost * cost));
  const float phi = 2.f * float(M_PI) * curand_uniform(&rs);
  return onbMul(n, mk3(sint * cosf(phi), sint * sinf(phi), -cost));
}

// Diffuse path tracer raygen body (DiffusePathTracer_ptx.cu:82-215). The
// path state (depth, Lw) lives across the pixel's sample loop, as in the
// reference, where PathData is declared outside it.
struct PathData
{
  int depth;
  f3 Lw;
};

template <bool STATS, bool SURF, bool NV>
__device__ __forceinline__ void integrateDPT(const FrameParams &P,
    TravStats &st,
    RandState &rs,
    int px,
    int py,
    PathData &pd,
    SampleOut &o)
{
  const RendererGPU &rp = P.renderer;
  const WorldGPU &w = P.world;
  float scrX, scrY;
  Ray ray = makePrimaryRay(P, rs, px, py, false, scrX, scrY);
  const float tmax = ray.tmax;
  const float4 bg = backgroundOf(P, ray.dir, scrX, scrY);
  o.color = mk3(bg.x, bg.y, bg.z); // albedo channel value (outColor)
  o.normal = ray.dir;
  o.depth = tmax;
  o.primID = o.objID = o.instID = ~0u;
  const bool cull = rp.cullTriangleBF != 0;
  while (true) {
    Hit h;
    float unused;
    // a primary / path ray against an empty surface set still counts
    if (!SURF)
      st.rays++;
    const bool found = SURF && traverse<0, STATS>(w,
        ray.org,
        ray.dir,
        ray.tmin,
        ray.tmax,
        cull,
        false,
        h,
        unused,
        P.errorFlag,
        st);
    SurfaceHit sh;
    if (found)
      populateSurfaceHit(w, ray, h, sh);
    f3 volumeColor = mk3(0.f, 0.f, 0.f);
    float volumeOpacity = 0.f, Tr = 0.f;
    uint32_t vObjID = ~0u, vInstID = ~0u;
    const float volumeDepth = w.numVolumes
        ? sampleDistanceAllVolumes<NV>(w,
              rs,
              ray.org,
              ray.dir,
              ray.tmin,
              found ? sh.t : ray.tmax,
              volumeColor,
              volumeOpacity,
              Tr,
              vObjID,
              vInstID)
        : (found ? sh.t : ray.tmax);
    if (!w.numVolumes)
      Tr = 1.f;
    const bool volumeHit = Tr < 1.f && (!found || volumeDepth < sh.t);
    if (!found && !volumeHit)
      break;
    if (pd.depth++ >= rp.maxDepth) {
      pd.Lw = mk3(0.f, 0.f, 0.f);
      break;
    }
    f3 albedo;
    f3 pos;
    if (!volumeHit) {
      pos = sh.hitpoint + (sh.epsilon * sh.Ng);
      albedo = matteInit(w, sh).baseColor;
    } else {
      pos = ray.org + volumeDepth * ray.dir;
      albedo = volumeColor;
    }
    pd.Lw *= albedo;
    const float Pr = compMax(pd.Lw);
    if (Pr < .2f) {
      if (curand_uniform(&rs) > Pr) {
        pd.Lw = mk3(0.f, 0.f, 0.f);
        break;
      }
      pd.Lw = pd.Lw / Pr;
    }
    f3 scatterDir;
    if (!volumeHit) {
      scatterDir = randomDir(rs, sh.Ns);
      pd.Lw *= fmaxf(0.f, dot(scatterDir, sh.Ng));
    } else
      scatterDir = sampleUnitSphere(rs, -ray.dir);
    ray.org = pos;
    ray.dir = scatterDir;
    ray.tmin = 0.f;
    ray.tmax = rp.occlusionDistance;
  }
  const f3 Ld = mk3(rp.ambientIntensity, rp.ambientIntensity, rp.ambientIntensity);
  const f3 color = pd.depth ? pd.Lw * Ld : mk3(bg.x, bg.y, bg.z);
  // accumResults gets (color, 1) and outColor (the background) as albedo
  const f3 albedoOut = o.color;
  o.color = color;
  o.opacity = 1.f;
  o.albedo = albedoOut;
}

// --- output ------------------------------------------------------------------

__device__ __forceinline__ float4 tonemap(float4 v)
{
  const float m = fmaxf(0.f, fmaxf(v.x, fmaxf(v.y, v.z)));
  const float d = 1.f + m;
  return make_float4(v.x / d, v.y / d, v.z / d, v.w);
}

__device__ __forceinline__ float4 inverseTonemap(float4 v)
{
  const float d = fmaxf(1e-12f, 1.f - fmaxf(v.x, fmaxf(v.y, v.z)));
  return make_float4(v.x / d, v.y / d, v.z / d, v.w);
}

__device__ __forceinline__ float linearToSrgb(float c)
{
  return srgbEncode(c);
}

__device__ __forceinline__ uint32_t packUnorm4x8(float4 v)
{
  const uint32_t r = (uint32_t)roundf(fminf(fmaxf(v.x, 0.f), 1.f) * 255.f);
  const uint32_t g = (uint32_t)roundf(fminf(fmaxf(v.y, 0.f), 1.f) * 255.f);
  const uint32_t b = (uint32_t)roundf(fminf(fmaxf(v.z, 0.f), 1.f) * 255.f);
  const uint32_t a = (uint32_t)roundf(fminf(fmaxf(v.w, 0.f), 1.f) * 255.f);
  return r | (g << 8) | (b << 16) | (a << 24);
}

__device__ __forceinline__ void writeOutputColor(
    const FramebufferGPU &fb, float4 accum, uint32_t idx, int frameIDOffset)
{
  const float n = float(fb.frameID + frameIDOffset + 1);
  const float4 c =
      inverseTonemap(make_float4(accum.x / n, accum.y / n, accum.z / n, accum.w / n));
  if (fb.format == FORMAT_SRGB)
    fb.outColorU[idx] = packUnorm4x8(make_float4(
        linearToSrgb(c.x), linearToSrgb(c.y), linearToSrgb(c.z), c.w));
  else if (fb.format == FORMAT_UINT)
    fb.outColorU[idx] = packUnorm4x8(c);
  else
    fb.outColorF[idx] = c;
}

template <int RT, bool STATS, bool SURF, bool NV>
__device__ __forceinline__ void renderPixel(
    const FrameParams &P, TravStats &st, int lx, int ly)
{
  const FramebufferGPU &fb = P.fb;
  const int x = computePixelX(lx, fb.checkerboardID);
  const int y = computePixelY(ly, fb.checkerboardID);
  if (x >= (int)fb.w || y >= (int)fb.h)
    return;
  RandState rs;
  curand_init((unsigned long long)(y * (int)fb.w + x),
      0ull,
      (unsigned long long)fb.frameID * 512ull,
      &rs);
  const uint32_t idx = (uint32_t)x + (uint32_t)y * fb.w;
  float4 acc = fb.accum[idx];
  float curDepth = fb.depth ? fb.depth[idx] : 0.f;
  bool idsDirty = false;
  uint32_t oPrim = 0, oObj = 0, oInst = 0;
  f3 albedoAcc = mk3(0.f, 0.f, 0.f), normalAcc = mk3(0.f, 0.f, 0.f);
  const int iters = RT == RENDERER_RAYCAST ? 1 : P.renderer.numIterations;
  PathData pd;
  pd.depth = 0;
  pd.Lw = mk3(1.f, 1.f, 1.f);
  for (int i = 0; i < iters; i++) {
    SampleOut s;
    if (RT == RENDERER_DPT)
      integrateDPT<STATS, SURF, NV>(P, st, rs, x, y, pd, s);
    else
      integrateSample<RT, STATS, SURF, NV>(P, st, rs, x, y, s);
    const float4 tm = tonemap(make_float4(s.color.x, s.color.y, s.color.z, s.opacity));
    acc.x += tm.x;
    acc.y += tm.y;
    acc.z += tm.z;
    acc.w += tm.w;
    albedoAcc += s.albedo;
    normalAcc += s.normal;
    if (!fb.depth || s.depth < curDepth) {
      curDepth = s.depth;
      oPrim = s.primID;
      oObj = s.objID;
      oInst = s.instID;
      idsDirty = true;
    }
  }
  fb.accum[idx] = acc;
  if (fb.albedo)
    fb.albedo[idx] += albedoAcc;
  if (fb.normal)
    fb.normal[idx] += normalAcc;
  if (idsDirty) {
    if (fb.depth)
      fb.depth[idx] = curDepth;
    if (fb.primID)
      fb.primID[idx] = oPrim;
    if (fb.objID)
      fb.objID[idx] = oObj;
    if (fb.instID)
      fb.instID[idx] = oInst;
  }
  writeOutputColor(fb, acc, idx, iters - 1);
  if (fb.checkerboardID == 0 && fb.frameID + iters - 1 == 0) {
    // first-frame 2x2 splat (gpu_util.h:424-442)
    if (x + 1 < (int)fb.w)
      writeOutputColor(fb, acc, idx + 1, iters - 1);
    if (y + 1 < (int)fb.h)
      writeOutputColor(fb, acc, idx + fb.w, iters - 1);
    if (x + 1 < (int)fb.w && y + 1 < (int)fb.h)
      writeOutputColor(fb, acc, idx + fb.w + 1, iters - 1);
  }
}

__device__ __forceinline__ unsigned long long warpSum(unsigned long long v)
{
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int RT, bool STATS, bool SURF, bool NV>
__global__ void __launch_bounds__(128,
    SURF ? VRTX_RENDER_MIN_BLOCKS : (NV ? VRTX_NANOVDB_MIN_BLOCKS : VRTX_VOLUME_MIN_BLOCKS))
    k_render(const FrameParams P)
{
  const int lane = threadIdx.x & 31;
  const uint32_t numTiles = P.numTilesX * P.numTilesY;
  TravStats st{0u, 0u, 0u, 0u, 0u, 0u, 0u};
  while (true) {
    uint32_t t = 0;
    if (lane == 0)
      t = atomicAdd(P.workCounter, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= numTiles)
      break;
    const uint32_t tx = t % P.numTilesX, ty = t / P.numTilesX;
    const int lx = (int)(tx * 8 + (lane & 7));
    const int ly = (int)(ty * 4 + (lane >> 3));
    if (lx < (int)P.launchW && ly < (int)P.launchH)
      renderPixel<RT, STATS, SURF, NV>(P, st, lx, ly);
  }
  // per-warp totals: rays and volume samples always, traversal counters in
  // the counting build
  const unsigned long long rays = warpSum(st.rays);
  const unsigned long long smp = warpSum(st.samples), fet = warpSum(st.fetches);
  if (lane == 0) {
    atomicAdd(P.stats + 0, rays);
    if (smp)
      atomicAdd(P.stats + 5, smp);
    if (fet)
      atomicAdd(P.stats + 6, fet);
  }
  if (STATS) {
    const unsigned long long n = warpSum(st.nodes), t = warpSum(st.tris),
                             sp = warpSum(st.spheres), in = warpSum(st.instances);
    if (lane == 0) {
      atomicAdd(P.stats + 1, n);
      atomicAdd(P.stats + 2, t);
      atomicAdd(P.stats + 3, sp);
      atomicAdd(P.stats + 4, in);
    }
  }
}

template <int RT, bool STATS>
void launchSurface(const FrameParams &P, int *occ, int grid, cudaStream_t s)
{
  if (occ)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, k_render<RT, STATS, true, true>, 128, 0);
  else
    k_render<RT, STATS, true, true><<<grid, 128, 0, s>>>(P);
}

// worlds with surfaces: one kernel per renderer, volumes of either field kind
template <bool STATS>
void dispatchSurface(const FrameParams &P, int type, int *occ, int grid, cudaStream_t s)
{
  switch (type) {
  case RENDERER_RAYCAST:
    launchSurface<RENDERER_RAYCAST, STATS>(P, occ, grid, s);
    break;
  case RENDERER_AO:
    launchSurface<RENDERER_AO, STATS>(P, occ, grid, s);
    break;
  case RENDERER_DPT:
    launchSurface<RENDERER_DPT, STATS>(P, occ, grid, s);
    break;
  default:
    launchSurface<RENDERER_DIRECT_LIGHT, STATS>(P, occ, grid, s);
    break;
  }
}

} // namespace
} // namespace vrtx
