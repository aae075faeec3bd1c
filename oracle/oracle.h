/*
 * oracle.h -- CPU oracle for the VisRTX hot path. TEST INFRASTRUCTURE ONLY:
 * tests, the smoke check and bench.py's CPU-baseline/reference legs call it
 * as the checker; libvrtx never links or calls it.
 *
 * It restates, on the CPU, the reference's algorithms for ray generation,
 * ray/primitive intersection, the default/raycast/ao/dpt integrators, the
 * scivis volume marcher and the frame output path (citations per function
 * in oracle.cpp), plus an FP64 marcher and FP64 adjoint for the
 * differentiable marcher of this library.
 *
 * Parity status: the reference cannot be built here (OptiX and the
 * ANARI-SDK are absent) and ships no golden images or known-answer tests,
 * so the end-to-end algorithm is "parity unpinned". The third-party
 * arithmetic at its boundary is pinned separately: Philox4x32-10 against the
 * SC'11 paper's algorithm and against curand outputs captured on the GPU,
 * and the texture-filter emulation against tex1D/tex3D outputs captured on
 * the GPU (tests/golden/). NanoVDB field sampling is pinned to the NanoVDB
 * library the reference vendors (external/nanovdb): its builder made the
 * golden grids and its sampler the golden values, which the reader here
 * reproduces bit for bit (oracle/ref_nvdb.cpp, tests/golden/nvdb_golden.npz).
 * The reference's own host-compilable code on the path pins more of it:
 * its TF discretisation helpers (utility/colorMapHelpers.h), its
 * gpu/gpu_math.h helpers for the thin-lens aperture, the HDRI direction map
 * and the physically based cone sample, its macrocell projection
 * (gpu/uniformGrid.h), its macrocell walk (gpu/dda.h, compiled with
 * contraction on, as nvcc builds it), its primary-ray generation
 * (gpu/cameraCreateRay.h, compiled without contraction, as the oracle and
 * the library's kernels round it), its structured-field sampler
 * (gpu/sampleSpatialField.h), its image staging
 * (utility/CudaImageTexture.cpp), and the glm calls of its frame colour
 * write and volume entry, compiled in place (oracle/ref_*.cpp), made the
 * fixtures tests/golden/*_golden.npz, which the functions here reproduce
 * bit for bit.
 */
#ifndef VRTX_ORACLE_H
#define VRTX_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* --- RNG ----------------------------------------------------------------- */

/* Philox4x32-10 block function (Salmon et al., SC'11). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* curand-style Philox stream: init(seed, subsequence, offset), then n
 * draws. kind 0: curand() raw u32; 1: curand_uniform; 2: curand_uniform4
 * (n must be a multiple of 4). out is uint32 or float accordingly. */
void orc_philox_stream(uint64_t seed,
    uint64_t subsequence,
    uint64_t offset,
    int kind,
    int n,
    void *out);

/* --- texture filter emulation (parity mode) ------------------------------ */

/* Linear-filtered, clamped, normalised-coordinate fetches from a 1D table
 * of `comps`-component floats and from a 3D float field. mode 1: the
 * texture unit's arithmetic (coordinates truncated to 21 fractional bits,
 * 8-bit weights split into integer corner weights, one rounding of the
 * exact sum; bit-exact against GPU captures); mode 0: FP32 lerps with
 * weights rounded to 8 bits (the textbook form). */
void orc_tex1d(const float *table, int n, int comps, float coord, int mode,
    float *out);
float orc_tex3d(const float *vox, const int dims[3], const float coord[3], int mode);
/* Float4 texture fetch of `ndim` dimensions (dims[ndim]), filter 0 point /
 * 1 linear, wrap[k] 0 clamp / 1 repeat / 2 mirror, as the image samplers
 * and the HDRI map are read; and the RGBA8 normalised-float linear clamped
 * fetch of the background image. */
void orc_tex_float4(const float *texels, int ndim, const int dims[3], int filter,
    const int wrap[3], const float coord[3], float out[4]);
void orc_tex_rgba8(const uint8_t *texels, int w, int h, const float coord[2], float out[4]);
/* The same fetch as orc_tex_float4 from RGBA8 texels read as normalised
 * float (8-bit image samplers): point b / 255, linear the texture unit's
 * integer filter scaled to 16 bits. */
void orc_tex_unorm8(const uint8_t *texels, int ndim, const int dims[3], int filter,
    const int wrap[3], const float coord[3], float out[4]);
/* The read of a single-channel 16-bit normalised texture (texels as
 * integers; scale 65535 for UFIXED16, 32767 for FIXED16): linear filtering
 * rounds the integer weighted sum once, F / 256 half up. */
float orc_tex_norm16(const int32_t *texels, int ndim, const int dims[3], int filter,
    const int wrap[3], const float coord[3], int scale);

/* --- NanoVDB fields ------------------------------------------------------ */

/* Samples a NanoVDB grid buffer (NanoVDB 32.7 layout; leaf codecs float,
 * Fp4, Fp8, Fp16, FpN) at n world-space points the way the reference's
 * field sampler does (gpu/sampleSpatialField.h:80-109: the grid's float
 * inverse map, then first-order interpolation of the 2x2x2 voxel stencil).
 * fused = 0 rounds the leaf decode and the interpolation separately, as the
 * NanoVDB library compiled for the host does; fused = 1 evaluates them as
 * fused multiply-adds, as the reference's device build (and libvrtx) does.
 * Returns 0, or -1 for a buffer this reader does not accept. */
int orc_nvdb_sample(const uint8_t *grid, const float *xyz, int n, int fused, float *out);

/* --- scene ---------------------------------------------------------------- */

/* A geometry attribute array: element type code (this library's VRTX_*
 * values: 240..243 float32 x1..x4, 221 ufixed8, 223 ufixed16, 260 ufixed8
 * x4, 261 sRGB ufixed8 x4) and channel count; data NULL: absent. */
typedef struct OrcAttr {
  const void *data;
  int type;
  int channels;
} OrcAttr;

/* A material sampler: type 1 image1D, 2 image2D, 3 image3D, 4 transform,
 * 5 primitive; input attribute slot; column-major in / out maps; the image
 * as staged (orc_stage_image): float4 texels (image) or RGBA8 texels read
 * as normalised float (image8), x fastest, with its dims, filter
 * (0 nearest, 1 linear) and wrap modes (0 clampToEdge, 1 repeat,
 * 2 mirrorRepeat); or the primitive array and offset. */
typedef struct OrcSampler {
  int type;
  int attribute;
  float inT[16], inO[4], outT[16], outO[4];
  const float *image;
  const uint8_t *image8;
  int dims[3];
  int filter;
  int wrap[3];
  OrcAttr prim;
  uint32_t primOffset;
} OrcSampler;

typedef struct OrcSurface {
  int type; /* 0 triangle, 1 sphere, 2 quad, 3 cylinder, 4 cone, 5 curve */
  const float *vertices; /* vec3 */
  /* uvec3 per triangle, uvec4 per quad, uvec2 per cylinder / cone, u32 per
   * sphere / curve; NULL: implicit */
  const uint32_t *indices;
  uint32_t numPrims; /* quads count two triangles each */
  const float *normals; /* vertex.normal (vec3) or NULL */
  const uint32_t *primIds; /* primitive.id or NULL */
  /* per-vertex radius (sphere, cone, curve) or per-primitive radius
   * (cylinder), or NULL */
  const float *radii;
  float radius;
  int cullBackfaces;
  uint32_t id; /* Surface id */
  float color[3];
  float opacity;
  int alphaMode; /* 0 opaque, 1 blend, 2 mask */
  float cutoff;
  int caps; /* cylinder end caps */
  /* attributes: slots attribute0..3, color */
  OrcAttr vattr[5]; /* vertex.* */
  OrcAttr pattr[5]; /* primitive.* */
  float uattr[5][4]; /* uniform (default 0, 0, 0, 1) */
  /* matte parameter sources: 0 value, 1..4 attribute0..3, 5 color,
   * 6 worldPosition, 7 worldNormal, 8 objectPosition, 9 objectNormal */
  int colorSrc, opacitySrc; /* 10: the sampler below */
  float colorW; /* w of the colour value */
  OrcSampler colorSampler, opacitySampler;
  /* 0 matte, 1 physicallyBased (color = baseColor) */
  int materialType;
  float metallic, roughness, ior;
  int metallicSrc, roughnessSrc;
  OrcSampler metallicSampler, roughnessSampler;
} OrcSurface;

typedef struct OrcInstance {
  float xfm[12]; /* 3 rows x 4 */
  uint32_t userId;
  int firstSurface;
  int numSurfaces;
} OrcInstance;

typedef struct OrcLight {
  int type; /* 0 directional, 1 point, 2 spot, 3 hdri */
  float direction[3]; /* directional: direction of travel; spot: its axis */
  float position[3];
  float radiance[3]; /* color * irradiance / intensity */
  float cosOuter, cosInner; /* spot */
  /* hdri: W x H float RGB radiance (x fastest), direction, up, scale,
   * visibility */
  const float *hdri;
  int hdriW, hdriH;
  float hdriDirection[3], hdriUp[3];
  float hdriScale;
  int hdriVisible;
} OrcLight;

typedef struct OrcVolume {
  const float *field; /* dims[0] fastest */
  int dims[3];
  float origin[3], spacing[3];
  int filterLinear;
  const float *tf; /* 256 x RGBA, NULL = uniform */
  float valueRange[2];
  float unitDistance;
  float uniformColor[3];
  float uniformOpacity;
  uint32_t id;
  uint32_t instId;
  float xfm[12];
  /* non-NULL: a NanoVDB field (the grid buffer); field, dims, origin,
   * spacing and filterLinear are then unused */
  const uint8_t *nvdb;
} OrcVolume;

/* The reference's delta-tracking majorants of one volume (dpt renderer):
 * ceil(dims/16) cells, x fastest (UniformGrid.cu). */
void orc_dpt_majorants(const OrcVolume *volume, int round, float *out);

typedef struct OrcScene {
  const OrcSurface *surfaces;
  int numSurfaces;
  const OrcInstance *instances;
  int numInstances;
  const OrcLight *lights;
  int numLights;
  const OrcVolume *volumes;
  int numVolumes;
} OrcScene;

typedef struct OrcCamera {
  int type; /* 0 perspective, 1 orthographic */
  float position[3], direction[3], up[3];
  float fovy, aspect, height;
  float imageRegion[4];
  float apertureRadius, focusDistance;
} OrcCamera;

typedef struct OrcRenderer {
  int type; /* 0 default/directLight, 1 raycast, 2 ao, 3 dpt */
  float background[4];
  float ambientColor[3];
  float ambientRadiance;
  float occlusionDistance;
  int cullTriangleBackfaces;
  float volumeSamplingRate;
  int pixelSamples;
  int ambientSamples;
  int maxDepth;
  int maxRayDepth; /* bounce rays of the default renderer */
  /* background image (W x H, x fastest) of element type bgType (this
   * library's codes: 242/243 float32 x3/x4, 260 ufixed8 x4, 261 sRGB8 x4),
   * NULL: the background colour */
  const void *bgImage;
  int bgType, bgW, bgH;
} OrcRenderer;

typedef struct OrcFrame {
  int width, height;
  int frameID; /* sample index base (RNG offset = frameID * 512) */
  int colorFormat; /* 0 sRGB rgba8, 1 linear rgba8, 2 float4 */
  int rowBegin, rowEnd; /* launch rows to render */
  /* outputs (full-frame buffers; only rows in range are written) */
  float *accum; /* float4, in/out */
  void *color; /* u32 or float4 */
  float *depth; /* in/out (cleared to FLT_MAX by the caller) */
  uint32_t *primId, *objId, *instId;
  /* statistics: rays traced (primary + secondary) */
  uint64_t raysTraced;
  int checkerboardID; /* -1: off; 0..3: which pixel of each 2x2 block */
  float *albedo, *normal; /* vec3 accumulations (in/out) or NULL */
  /* statistics: volume march positions (the reference's samples) */
  uint64_t volumeSamples;
} OrcFrame;

/* Renders rows [rowBegin, rowEnd). volumeMode 0: parity (texture
 * emulation, float32 like the reference), 1: clean FP64 volumes.
 * threads <= 0 uses all hardware threads. Returns 0 on success. */
/* Builds the oracle's acceleration structures for `scene` once (the scene
 * arrays must stay alive); render with orc_render_prepared, free with
 * orc_release. */
void *orc_prepare(const OrcScene *scene);
void orc_release(void *prepared);
int orc_render_prepared(void *prepared,
    const OrcCamera *camera,
    const OrcRenderer *renderer,
    OrcFrame *frame,
    int volumeMode,
    int texRound,
    int threads);

int orc_render(const OrcScene *scene,
    const OrcCamera *camera,
    const OrcRenderer *renderer,
    OrcFrame *frame,
    int volumeMode,
    int texRound,
    int threads);

/* uniformSampleDisk (gpu_math.h:292-297) on n (radius, s0, s1) triples
 * -> n (x, y); sphericalCoordsFromDirection (gpu_math.h:254-261) on n
 * directions -> n (theta, phi): the oracle's own thin-lens and HDRI
 * helpers. */
void orc_uniform_sample_disk(const float *in3, int n, float *out2);
void orc_spherical_from_dir(const float *dir3, int n, float *out2);
/* uniformSampleCone (gpu_math.h:299-312) on n (cosThetaMax, s0, s1, s2)
 * -> n directions: the physically based material's next-ray sample. */
void orc_uniform_sample_cone(const float *in4, int n, float *out3);
/* projectOnGrid (uniformGrid.h:43-50) of n points onto a dims3 grid over
 * box6 (lo xyz, hi xyz) -> n integer cells. */
void orc_project_on_grid(const float *p3, int n, const int *dims3, const float *box6, int *out3);
/* An image sampler's staging (Image2D.cpp:70-78, CudaImageTexture.cpp:43-111)
 * of n texels of element type et (this library's codes: 240..243 float32
 * x1..x4, 221 ufixed8, 223 ufixed16, 260 ufixed8 x4, 261 sRGB ufixed8 x4):
 * float types to outFloat (n x 4, missing channels 0, alpha 1), returning
 * 1; the others to outBytes (n x 4 RGBA8, missing channels 0, alpha 255),
 * returning 0; -1 for another type. */
int orc_stage_image(int et, const void *texels, uint64_t n, float *outFloat, uint8_t *outBytes);
/* The renderer's background image staging (Renderer.cpp:173-179,
 * CudaImageTexture.cpp:43-93) of n texels of et (242 / 243 float32 x3 / x4,
 * 260 ufixed8 x4, 261 sRGB ufixed8 x4) to out (n x 4 RGBA8); -1 for another
 * type. */
int orc_stage_background(int et, const void *texels, uint64_t n, uint8_t *out);
/* The structured-regular field's texture coordinates
 * (sampleSpatialField.h:54-78, invSpacing as StructuredRegularField.cpp:
 * 188-189) of n world points p3 for a field of origin3, spacing3 over dims3
 * voxels -> out3 (n x 3). */
void orc_field_coords(const float *origin3, const float *spacing3, const int *dims3,
    const float *p3, int n, float *out3);
/* intersectVolume's slab interval (Intersectors_ptx.cu:248-274), the
 * volume's entry, for n local rays (org xyz, dir xyz, tmin, tmax) against
 * box6 (lo xyz, hi xyz): hit[i] 1 or 0, t01[2i..2i+1] the clamped interval
 * on a hit (0, 0 otherwise). */
void orc_volume_interval(const float *rays8, int n, const float *box6, int *hit, float *t01);
/* makePrimaryRay + cameraCreateRay (cameraCreateRay.h:38-81) for n
 * samples (pixel x, pixel y, r0..r3: the uniform4 draw) of a camera record
 * (30 floats: region 4, pos 3, dir 3, dir_00 3, dir_du 3, dir_dv 3,
 * scaledAperture, aspect, pos_00 3, pos_du 3, pos_dv 3; type 0
 * perspective, 1 orthographic) over a frame of 1 / invW x 1 / invH pixels
 * -> out n x (org xyz, dir xyz, screen xy). */
void orc_primary_rays(const float *cam,
    int type,
    const float *samples,
    int n,
    float invW,
    float invH,
    int centerPixel,
    float *out);
/* dda3 (dda.h:43-122) for n rays (org xyz, dir xyz, tlo, thi) over a dims3
 * grid spanning box6: counts[i] cells per ray (at most maxCells), their
 * linear indices in cells[i * maxCells ...] and intervals in
 * t01[2 * (i * maxCells + k) ...]; returns the total. */
int orc_dda_walk(const float *rays8,
    int n,
    const int *dims3,
    const float *box6,
    int maxCells,
    int *counts,
    long long *cells,
    float *t01);

/* The frame's colour write (gpu_util.h:370-389) of n accumulated RGBA
 * colours after frameID + 1 samples: format 0 sRGB rgba8, 1 linear
 * rgba8, packed into out (n uint32). */
void orc_write_colors(const float *accum, int n, int frameID, int format, uint32_t *out);

/* TF discretisation of the reference (TransferFunction1D.cpp:101-150):
 * color (nc x 3 or 4 floats), opacity (no floats) -> 256 x RGBA; where an
 * array is absent the uniform colour (4 floats, NULL: white) / opacity
 * stand in. */
void orc_discretize_tf(const float *color,
    int nc,
    int colorComps,
    const float *opacity,
    int no,
    float valueLo,
    float valueHi,
    const float *uniformColor4,
    float uniformOpacity,
    float *out256x4);

/* Counts node visits and primitive tests of a closest-hit traversal over a
 * libvrtx BVH8 (one BLAS: nodes + triangle records, as copied by
 * vrtxDebugCopyAccel) for the given rays (org/dir/tmax, 7 floats each). */
void orc_bvh8_count(const void *nodes,
    const void *triRecords,
    const float *rays,
    int numRays,
    uint64_t *nodeVisits,
    uint64_t *primTests,
    float *tHit);

/* --- differentiable marcher, FP64 ----------------------------------------- */

typedef struct OrcDMVolume {
  const double *density;
  int dims[3];
  const double *tf; /* tfSize x 4 */
  int tfSize;
  double opacityScale, step, unitDistance, valueLo, valueHi;
} OrcDMVolume;

typedef struct OrcDMView {
  int width, height;
  double eye[3], d00[3], du[3], dv[3], background[3];
} OrcDMView;

/* Forward image (3 doubles per pixel); when gradImage != NULL, also the
 * adjoint: gradDensity (dims), gradTf (tfSize x 4), gradScale (1),
 * accumulated. */
void orc_dm(const OrcDMVolume *vol,
    const OrcDMView *view,
    double *image,
    const double *gradImage,
    double *gradDensity,
    double *gradTf,
    double *gradScale,
    int threads);

#ifdef __cplusplus
}
#endif

#endif
