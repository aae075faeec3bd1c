// Device-side data layout of libvrtx: scene registries, acceleration
// structures, camera, renderer and framebuffer parameters.
//
// The fields follow the reference's GPU structs where they carry the same
// meaning (devices/rtx/gpu/gpu_objects.h: GeometryGPUData, SurfaceGPUData,
// CameraGPUData, RendererGPUData, FramebufferGPUData), re-laid out for this
// kernel design: no OptiX handles, explicit BVH8 nodes and primitive records.
#pragma once

#include "vmath.h"

namespace vrtx {

// ---------------------------------------------------------------------------
// Scene registries
// ---------------------------------------------------------------------------

// Primitive classes, one bottom-level structure each per group (the
// reference builds one GAS per class: triangles, curves, user primitives).
// Cylinders and cones are user primitives there; here each has its own
// structure because its leaf records and test differ.
enum GeomType : uint32_t
{
  GEOM_TRIANGLE = 0, // triangles and quads
  GEOM_SPHERE = 1,
  GEOM_CYLINDER = 2,
  GEOM_CONE = 3,
  GEOM_CURVE = 4, // round linear curve segments
  GEOM_NUM_TYPES = 5
};

// Geometry subtype, where it changes the hit population
enum GeomKind : uint32_t
{
  KIND_TRIANGLE = 0,
  KIND_QUAD = 1,
  KIND_SPHERE = 2,
  KIND_CYLINDER = 3,
  KIND_CONE = 4,
  KIND_CURVE = 5
};

// One geometry attribute array (Geometry.cpp:152-171): element type code
// (VRTX_FLOAT32.._VEC4, VRTX_UFIXED8 / _VEC4 / _RGBA_SRGB, VRTX_UFIXED16)
// and its channel count; data == NULL: not given.
struct AttrGPU
{
  const void *data;
  uint32_t type;
  uint32_t channels;
};

// Attribute slots in the reference's order: attribute0..3, color
constexpr int NUM_ATTRS = 5;

struct GeometryGPU
{
  uint32_t type; // GeomType (the class)
  uint32_t numPrims;
  const f3 *vertices; // vertex.position
  const uint32_t *indices; // triangle: uvec3 per prim or NULL (soup);
                           // quad: the generated uvec3 pairs (Quad.cpp:
                           // 115-141); sphere / curve: primitive.index or
                           // NULL; cylinder / cone: uvec2 per prim or NULL
  const f3 *normals; // triangle vertex.normal or NULL
  const f3 *normalsFV; // triangle faceVarying.normal or NULL
  const uint32_t *primIds; // primitive.id or NULL
  const float *radii; // sphere / cone / curve vertex.radius, cylinder
                      // primitive.radius, or NULL
  float radius; // uniform radius (sphere 0.01, cylinder / curve 1)
  uint32_t cullBackfaces; // VISRTX_TRIANGLE_BACK_FACE_CULLING extension
  uint32_t kind; // GeomKind
  uint32_t caps; // cylinder "caps" != "none"
  AttrGPU vattr[NUM_ATTRS]; // vertex.attribute0..3, vertex.color
  AttrGPU pattr[NUM_ATTRS]; // primitive.attribute0..3, primitive.color
  float4 uattr[NUM_ATTRS]; // uniform attribute0..3, color (default 0,0,0,1)
};

enum AlphaMode : int
{
  ALPHA_OPAQUE = 0,
  ALPHA_BLEND = 1,
  ALPHA_MASK = 2
};

// Where a material parameter comes from (MaterialParameterType of the
// reference): its value, a geometry attribute, or a hit quantity.
enum ParamSource : uint32_t
{
  PARAM_VALUE = 0,
  PARAM_ATTRIB_0 = 1, // .. PARAM_ATTRIB_3 = 4
  PARAM_ATTRIB_COLOR = 5,
  PARAM_WORLD_POSITION = 6,
  PARAM_WORLD_NORMAL = 7,
  PARAM_OBJECT_POSITION = 8,
  PARAM_OBJECT_NORMAL = 9,
  PARAM_SAMPLER = 10
};

enum SamplerType : uint32_t
{
  SAMPLER_NONE = 0,
  SAMPLER_IMAGE1D = 1,
  SAMPLER_IMAGE2D = 2,
  SAMPLER_IMAGE3D = 3,
  SAMPLER_TRANSFORM = 4,
  SAMPLER_PRIMITIVE = 5
};

// A material sampler (SamplerGPUData of the reference): its input attribute
// slot, input / output affine maps (column-major 4x4 + offset), and an image
// texture (float4, normalised coordinates) or a primitive array.
struct SamplerGPU
{
  uint32_t type; // SamplerType
  uint32_t attribute; // 0..3 attribute0..3, 4 color
  cudaTextureObject_t tex;
  float inT[16];
  float4 inO;
  float outT[16];
  float4 outO;
  AttrGPU prim; // primitive sampler: the array
  uint32_t primOffset;
  uint32_t pad;
};

enum MaterialType : uint32_t
{
  MATERIAL_MATTE = 0, // "matte" (Matte.cpp, shaders/MatteShader_ptx.cu)
  MATERIAL_PBR = 1 // "physicallyBased" (PBR.cpp, PhysicallyBasedShader_ptx.cu)
};

// material parameter slots: matte reads color and opacity, physicallyBased
// all four ("baseColor" in the color slot)
enum MaterialParamSlot : int
{
  MP_COLOR = 0,
  MP_OPACITY = 1,
  MP_METALLIC = 2,
  MP_ROUGHNESS = 3,
  MP_COUNT = 4
};

// one material parameter (MaterialParameter, gpu_objects.h): its value, the
// ParamSource that supplies it and, for PARAM_SAMPLER, the index into
// WorldGPU::samplers
struct MaterialParamGPU
{
  float4 value;
  uint32_t src;
  uint32_t sampler;
  uint32_t pad[2];
};

struct MaterialGPU
{
  uint32_t type; // MaterialType
  int alphaMode;
  float cutoff;
  float ior; // physicallyBased "ior" (1.5)
  f3 color; // the color value's rgb (default 0.8 grey, Matte.cpp:44)
  float opacity; // color.w * opacity of the values, before the alpha mode
  MaterialParamGPU params[MP_COUNT];
};

struct SurfaceGPU
{
  uint32_t geometry;
  uint32_t material;
  uint32_t id; // Surface "id" (default ~0u, Surface.cpp:44)
  uint32_t pad;
};

enum LightType : int
{
  LIGHT_DIRECTIONAL = 0,
  LIGHT_POINT = 1,
  LIGHT_SPOT = 2,
  LIGHT_HDRI = 3
};

struct LightGPU
{
  int type;
  f3 dirToLight; // directional: xfmVec(xfm, -direction) (sampleLight.h:60-70)
  f3 radiance; // color * irradiance (directional) or * intensity (point, spot)
  f3 position; // point, spot (instance-transformed)
  f3 spotDir; // spot: normalize(direction), not instance-transformed
  float cosOuter, cosInner; // spot: cos(openingAngle), cos(opening - 2 falloff)
  // hdri (HDRI.cu): radiance texture (linear, x repeat, y clamp), the
  // normalised marginal (H) and conditional (H x W) CDFs, the rotation whose
  // rows are (right, forward, up), scale, pdf weight, visibility
  cudaTextureObject_t hdriTex;
  const float *marginalCDF;
  const float *conditionalCDF;
  uint32_t hdriW, hdriH;
  float hdriRot[9];
  float hdriScale;
  float pdfWeight;
  uint32_t visible;
};

// ---------------------------------------------------------------------------
// Compressed 8-wide BVH (one 80-byte node = five 16-byte loads)
// ---------------------------------------------------------------------------
//
// Child boxes are quantised to 8 bits per plane relative to the node origin p
// with a per-axis power-of-two scale 2^e (e stored as a biased float
// exponent). Quantisation rounds outward, so every decoded child box
// contains the exact one. meta[i] == 0 marks an empty slot; an internal
// child has meta = 0b001'xxxxx with xxxxx = 24 + slot; a leaf child has meta
// = (unary prim count) << 5 | (offset of its first prim from primBase).
// Internal children are stored contiguously from childBase in slot order
// (imask bit i set <=> slot i is internal).
struct alignas(16) BVH8Node
{
  float px, py, pz;
  uint8_t ex, ey, ez, imask;
  uint32_t childBase;
  uint32_t primBase;
  uint8_t meta[8];
  uint8_t qlox[8], qloy[8], qloz[8];
  uint8_t qhix[8], qhiy[8], qhiz[8];
};
static_assert(sizeof(BVH8Node) == 80, "BVH8Node must be 80 bytes");

// Triangle leaf record: the three vertices, gathered in leaf order.
struct alignas(16) TriRecord
{
  float4 v0; // .w = primID (bit pattern) within its geometry
  float4 v1; // .w = global surface index (bit pattern)
  float4 v2; // .w unused
};

struct alignas(16) SphereRecord
{
  float4 cr; // center, radius
  uint32_t primID; // OptiX-style primitive index within the geometry
  uint32_t surface; // global surface index
  uint32_t pad[2];
};

// Cylinder / cone / curve leaf record: a segment with its end radii.
struct alignas(16) SegRecord
{
  float4 a; // p0, radius at p0 (cylinder: its one radius)
  float4 b; // p1, radius at p1
  uint32_t primID; // primitive index within the geometry
  uint32_t surface; // global surface index
  uint32_t caps; // cylinder end caps
  uint32_t pad;
};

// One bottom-level structure: one primitive class of a group.
struct BLASDesc
{
  const BVH8Node *nodes;
  const void *prims; // TriRecord*, SphereRecord* or SegRecord*
  uint32_t type; // GeomType
  uint32_t numPrims;
  box3 bounds;
};

// One top-level leaf: (instance, transform index, primitive class).
struct alignas(16) InstanceRecord
{
  xfm34 worldToObject;
  xfm34 objectToWorld;
  uint32_t blas; // index into the BLAS table
  uint32_t userId; // Instance "id" / id array entry (Instance.cpp:115-118)
  uint32_t pad[2];
};

// ---------------------------------------------------------------------------
// Volumes
// ---------------------------------------------------------------------------

enum FieldKind : uint32_t
{
  FIELD_STRUCTURED_REGULAR = 0,
  FIELD_NANOVDB = 1
};

// A NanoVDB grid in device memory (spatial_field/NvdbRegularField.cpp): the
// RootData of the grid buffer, its leaf codec (NanoVDB GridType: 1 float,
// 13 Fp4, 14 Fp8, 15 Fp16, 16 FpN), root tile count, background value and
// the float world -> index map (3x3 inverse matrix, row-major as stored,
// and translation).
struct NvdbGPU
{
  const uint8_t *root;
  uint32_t type;
  uint32_t tiles;
  float background;
  float inv[9];
  float vec[3];
  // brick cache (null: walk the tree): a dense table over leaf-block
  // coordinates [blockLo, blockLo + blockDims) (x fastest) giving each
  // block's brick slot (its 8^3 values and the one-voxel apron on the +
  // sides, 9^3 floats with x slowest) or kBlockConstant (the whole 9^3
  // region holds blockFill[block])
  const float *bricks;
  const int32_t *brickTable;
  const float *blockFill;
  int blockLo[3];
  int blockDims[3];
};

constexpr int32_t kBlockConstant = -2;
constexpr int32_t kBlockUnclassified = -3; // while the cache is built
constexpr int32_t kBlockNeedsBrick = -4; // while the cache is built

struct VolumeGPU
{
  cudaTextureObject_t field; // 3D texture, normalised coords, clamp
  cudaTextureObject_t tf; // 1D float4 texture, linear, clamp (0 = uniform)
  f3 origin;
  f3 spacing;
  f3 invSpacing; // 1 / (spacing * dims) (StructuredRegularField.cpp:188-189)
  box3 bounds; // [origin, origin + (dims - 1) * spacing]
  float stepSize; // min(spacing) / 2
  float oneOverUnitDistance;
  float valueLo, valueHi; // TF valueRange
  f3 uniformColor;
  float uniformOpacity;
  uint32_t id; // Volume "id"
  uint32_t instId; // instance user id
  uint32_t hasTF;
  uint32_t fieldKind; // FieldKind
  xfm34 worldToObject;
  // conservative macrocell majorants (max TF opacity reachable in a cell),
  // 16-voxel cells from the origin: empty-space skipping of the marcher
  const float *majorants;
  // the reference's delta-tracking majorants: mcDims cells spanning
  // `bounds` (UniformGrid.cu), read by the dpt distance sampler
  const float *dptMajorants;
  int mcDims[3];
  int dims[3]; // voxel dims
  NvdbGPU nvdb; // FIELD_NANOVDB
};

// ---------------------------------------------------------------------------
// Camera / renderer / framebuffer
// ---------------------------------------------------------------------------

enum CameraType : int
{
  CAMERA_PERSPECTIVE = 0,
  CAMERA_ORTHOGRAPHIC = 1
};

struct CameraGPU
{
  int type;
  float region[4]; // imageRegion (lo.x, lo.y, hi.x, hi.y)
  f3 pos;
  f3 dir;
  f3 dir00, dirDu, dirDv; // perspective (Perspective.cpp:51-58)
  float scaledAperture, aspect;
  f3 pos00, posDu, posDv; // orthographic (Orthographic.cpp:47-50)
};

enum RendererType : int
{
  RENDERER_DIRECT_LIGHT = 0, // "default", "directLight"
  RENDERER_RAYCAST = 1,
  RENDERER_AO = 2,
  RENDERER_DPT = 3 // "dpt", "diffuse_pathtracer"
};

struct RendererGPU
{
  int type;
  float4 background;
  f3 ambientColor;
  float ambientIntensity;
  float occlusionDistance;
  int cullTriangleBF;
  float invVolumeSamplingRate;
  int numIterations; // pixelSamples
  int maxRayDepth;
  int aoSamples;
  int maxDepth; // dpt
  float lightFalloff;
  // background image (RGBA8, normalised float reads, linear, clamp), 0:
  // the background colour
  cudaTextureObject_t backgroundTex;
};

enum FrameFormat : int
{
  FORMAT_SRGB = 0,
  FORMAT_UINT = 1,
  FORMAT_FLOAT = 2
};

struct FramebufferGPU
{
  uint32_t w, h;
  float invW, invH;
  int frameID;
  int checkerboardID;
  int format;
  float4 *accum;
  uint32_t *outColorU;
  float4 *outColorF;
  float *depth;
  uint32_t *primID;
  uint32_t *objID;
  uint32_t *instID;
  f3 *albedo;
  f3 *normal;
};

struct WorldGPU
{
  const BVH8Node *tlasNodes;
  const InstanceRecord *instances;
  uint32_t numInstances;
  uint32_t numLights;
  const BLASDesc *blas;
  const SurfaceGPU *surfaces;
  const GeometryGPU *geometries;
  const MaterialGPU *materials;
  const LightGPU *lights;
  const VolumeGPU *volumes;
  uint32_t numVolumes;
  uint32_t allOpaque; // every material is opaque: any-hit = first hit
  uint32_t allMatte; // no physicallyBased material: no bounce rays
  uint32_t hasSegments; // some BLAS holds cylinders, cones or curves
  const SamplerGPU *samplers; // the materials' samplers
  uint32_t hasNanovdb; // some volume samples a NanoVDB field
  int hdri; // index into lights of the world's HDRI light, -1: none
  // Traversal loop bound per ray (node steps). A well-formed BVH ends far
  // below it; a ray that reaches it stops, counts as a miss and sets bit 1
  // of the frame's error flag. Frames set it from "vrtx.maxTraversalSteps".
  uint32_t maxTraversalSteps = 1u << 22;
};

// Per-thread work counters. Rays and volume samples are counted by every
// kernel; node visits and primitive tests only by the counting builds.
struct TravStats
{
  uint32_t nodes; // BVH8 nodes visited (TLAS + BLAS)
  uint32_t tris; // triangle tests
  uint32_t spheres; // sphere tests
  uint32_t instances; // BLAS entries
  uint32_t rays; // traversals
  uint32_t samples; // volume march positions (the reference's samples)
  uint32_t fetches; // of which fetched and classified (not skipped)
};

struct FrameParams
{
  WorldGPU world;
  CameraGPU camera;
  RendererGPU renderer;
  FramebufferGPU fb;
  uint32_t *workCounter; // persistent scheduling counter (zeroed per launch)
  uint32_t *errorFlag; // bit 0: traversal stack overflow, bit 1: a ray
                       // reached world.maxTraversalSteps
  unsigned long long *stats; // [0] rays, [1] nodes, [2] tri tests,
                             // [3] sphere tests, [4] BLAS entries,
                             // [5] volume samples, [6] volume fetches;
                             // [8..12] = [0..4] of the AO any-hit kernel
  uint32_t numTilesX, numTilesY;
  uint32_t launchW, launchH; // checkerboarding halves these
};

} // namespace vrtx
