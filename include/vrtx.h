/*
 * vrtx.h -- C ABI of libvrtx, a GB300-native (sm_103a) implementation of the
 * VisRTX ANARI device's hot path: BVH traversal over triangles, spheres and
 * instances, and emission-absorption ray marching through structured-regular
 * volumes with a 1D transfer function.
 *
 * Every entry point is plain C: opaque handles, plain pointers and sizes. No
 * C++ or torch type crosses this boundary and no exception escapes it; errors
 * are reported through the status callback given to vrtxNewDevice (the ANARI
 * convention) and, where a call returns a value, through that value.
 *
 * Each declaration names the reference interface it replaces as
 * file:line within the VisRTX project (devices/rtx/...). Object subtypes,
 * parameter names, frame channel names and their defaults are the
 * reference's; data type codes are this library's own (VRTX_*), named after
 * the ANARI data types they stand for.
 */
#ifndef VRTX_H
#define VRTX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define VRTX_API __declspec(dllexport)
#else
#define VRTX_API __attribute__((visibility("default")))
#endif

/* ------------------------------------------------------------------------ */
/* Handles                                                                  */
/* ------------------------------------------------------------------------ */

typedef struct VRTXDevice_st *VRTXDevice;
typedef struct VRTXObject_st *VRTXObject;
typedef VRTXObject VRTXArray;
typedef VRTXObject VRTXFrame;

/* ------------------------------------------------------------------------ */
/* Data types (ANARIDataType stand-ins)                                     */
/* ------------------------------------------------------------------------ */

typedef enum VRTXDataType {
  VRTX_UNKNOWN = 0,
  VRTX_STRING = 1,
  VRTX_VOID_POINTER = 2,
  VRTX_BOOL = 3,
  VRTX_FUNCTION_POINTER = 4, /* frameCompletionCallback */
  VRTX_MEMORY_DELETER = 5,
  VRTX_STRING_LIST = 6, /* const char *const *, NULL-terminated */

  VRTX_OBJECT = 100,
  VRTX_ARRAY1D = 101,
  VRTX_ARRAY2D = 102,
  VRTX_ARRAY3D = 103,
  VRTX_CAMERA = 104,
  VRTX_FRAME = 105,
  VRTX_GEOMETRY = 106,
  VRTX_GROUP = 107,
  VRTX_INSTANCE = 108,
  VRTX_LIGHT = 109,
  VRTX_MATERIAL = 110,
  VRTX_RENDERER = 111,
  VRTX_SURFACE = 112,
  VRTX_SAMPLER = 113,
  VRTX_SPATIAL_FIELD = 114,
  VRTX_VOLUME = 115,
  VRTX_WORLD = 116,
  VRTX_DEVICE = 117, /* object type of the device itself (feature queries) */

  VRTX_INT32 = 200,
  VRTX_INT32_VEC2 = 201,
  VRTX_INT8 = 202,
  VRTX_UINT8 = 203, /* raw bytes, e.g. a NanoVDB grid buffer */
  VRTX_UINT32 = 210,
  VRTX_UINT32_VEC2 = 211,
  VRTX_UINT32_VEC3 = 212,
  VRTX_UINT32_VEC4 = 213,
  VRTX_UINT64 = 214,
  VRTX_FIXED8 = 220,
  VRTX_UFIXED8 = 221,
  VRTX_FIXED16 = 222,
  VRTX_UFIXED16 = 223,
  VRTX_FLOAT16 = 230,
  VRTX_BFLOAT16 = 231,
  VRTX_FLOAT32 = 240,
  VRTX_FLOAT32_VEC2 = 241,
  VRTX_FLOAT32_VEC3 = 242,
  VRTX_FLOAT32_VEC4 = 243,
  VRTX_FLOAT32_BOX1 = 244,
  VRTX_FLOAT32_BOX2 = 245,
  VRTX_FLOAT32_BOX3 = 246,
  VRTX_FLOAT32_MAT3x4 = 247, /* ANARI_FLOAT32_MAT4x3: 4 columns of vec3 */
  VRTX_FLOAT32_MAT4 = 248,
  VRTX_FLOAT64 = 250,
  VRTX_FLOAT64_BOX1 = 251,
  VRTX_UFIXED8_VEC4 = 260,
  VRTX_UFIXED8_RGBA_SRGB = 261,
  VRTX_DATA_TYPE = 270 /* a parameter whose value is a VRTXDataType */
} VRTXDataType;

typedef enum VRTXStatusSeverity {
  VRTX_SEVERITY_FATAL_ERROR = 0,
  VRTX_SEVERITY_ERROR = 1,
  VRTX_SEVERITY_WARNING = 2,
  VRTX_SEVERITY_PERFORMANCE_WARNING = 3,
  VRTX_SEVERITY_INFO = 4,
  VRTX_SEVERITY_DEBUG = 5
} VRTXStatusSeverity;

typedef enum VRTXWaitMask {
  VRTX_NO_WAIT = 0,
  VRTX_WAIT = 1
} VRTXWaitMask;

/* ANARIStatusCallback: same argument order as the ANARI status callback. */
typedef void (*VRTXStatusCallback)(const void *userPtr,
    VRTXDevice device,
    VRTXObject source,
    int sourceType,
    int severity,
    int code,
    const char *message);

/* ANARIMemoryDeleter */
typedef void (*VRTXMemoryDeleter)(const void *userPtr, const void *appMemory);

/* ANARIFrameCompletionCallback */
typedef void (*VRTXFrameCompletionCallback)(
    const void *userPtr, VRTXDevice device, VRTXFrame frame);

/* ------------------------------------------------------------------------ */
/* Library / device                                                         */
/* ------------------------------------------------------------------------ */

/* Replaces makeVisRTXDevice (VisRTXLibrary.cpp:76-80,
 * include/anari/ext/visrtx/visrtx.h:49-51). CUDA is initialised lazily on
 * the first object creation, as VisRTXDevice::initDevice does
 * (VisRTXDevice.cpp:435-458). Returns NULL only when out of host memory.
 * Every ANARI object call (arrays, objects, parameters, frames) runs on
 * the device's GPU ("cudaDevice", fixed when the device initialises) and
 * leaves the calling thread's current CUDA device as it was
 * (CUDADeviceScope, VisRTXDevice.cpp:790-814); objects may be created and
 * used from any thread. The vrtxDM* calls are the exception: they run on
 * the calling thread's current device, the one that owns their pointers. */
VRTX_API VRTXDevice vrtxNewDevice(
    VRTXStatusCallback statusCallback, const void *statusCallbackUserData);

/* Device parameters ("cudaDevice", "forceInit", "statusCallback"); replaces
 * VisRTXDevice::deviceSetParameter / deviceCommitParameters
 * (VisRTXDevice.cpp:460-478). "cudaDevice" set after the device has
 * initialised is reported as a warning and ignored; with "forceInit" the
 * commit initialises CUDA instead of the first object creation. This
 * library also takes "vrtx.failFrameAllocations" (INT32 N, no reference
 * counterpart): the next N frame allocations fail on the host, without a
 * CUDA call, to test error handling; such a frame reports the failure, is
 * skipped by render, and allocates again at its next commit. */
VRTX_API void vrtxDeviceSetParameter(
    VRTXDevice d, const char *name, int type, const void *mem);
VRTX_API void vrtxDeviceCommitParameters(VRTXDevice d);

/* Releases the device and every object it still owns. */
VRTX_API void vrtxDeviceRelease(VRTXDevice d);

/* Device properties ("version": INT32, "visrtx": BOOL, "extension":
 * STRING_LIST, written as one const char *const * pointer); replaces
 * VisRTXDevice::deviceGetProperty (VisRTXDevice.cpp:520-552). Returns 1 when
 * the property was written. */
VRTX_API int vrtxDeviceGetProperty(VRTXDevice d,
    const char *name,
    int type,
    void *mem,
    uint64_t size,
    uint32_t waitMask);

/* 1 when the build has a usable CUDA device, 0 otherwise (after init). */
VRTX_API int vrtxDeviceIsValid(VRTXDevice d);

/* ------------------------------------------------------------------------ */
/* Feature queries                                                          */
/* ------------------------------------------------------------------------ */

/* The subtypes this library creates for an object type (VRTX_CAMERA ...
 * VRTX_VOLUME), as a static NULL-terminated list; NULL for types without
 * subtypes. Replaces VisRTXDevice::getObjectSubtypes
 * (VisRTXDevice.cpp:296-299). */
VRTX_API const char *const *vrtxGetObjectSubtypes(VRTXDevice d, int objectType);

/* The reference's extension flags (visrtx.h:55-64), one int per feature. */
typedef struct VRTXExtensions {
  int VISRTX_ARRAY_CUDA;
  int VISRTX_CUDA_OUTPUT_BUFFERS;
  int VISRTX_INSTANCE_ATTRIBUTES;
  int VISRTX_MATERIAL_MDL;
  int VISRTX_SPATIAL_FIELD_NANOVDB;
  int VISRTX_TRIANGLE_BACK_FACE_CULLING;
  int VISRTX_TRIANGLE_FACE_VARYING_ATTRIBUTES;
} VRTXExtensions;

/* Fill *ext from the features of one object subtype; returns 1 when the
 * subtype is known, else 0 (ext untouched). Replaces
 * visrtxGetObjectExtensions (VisRTXFeatureUtility.cpp:66-80). */
VRTX_API int vrtxGetObjectExtensions(
    VRTXExtensions *ext, VRTXDevice d, int objectType, const char *subtype);

/* Fill *ext from the device's "extension" list; returns 1 on success.
 * object: the device itself (NULL) -- the reference reads the property of
 * the object it is given, and only the device has one. Replaces
 * visrtxGetInstanceExtensions (VisRTXFeatureUtility.cpp:82-99). */
VRTX_API int vrtxGetInstanceExtensions(
    VRTXExtensions *ext, VRTXDevice d, VRTXObject object);

/* ------------------------------------------------------------------------ */
/* Arrays                                                                   */
/* ------------------------------------------------------------------------ */

/* Replace VisRTXDevice::newArray1D/2D/3D (VisRTXDevice.cpp:131-188) with the
 * ownership rules of Array.cpp:69-119: appMemory != NULL and deleter == NULL
 * -> shared; appMemory != NULL and deleter != NULL -> captured;
 * appMemory == NULL -> managed (fill through vrtxMapArray). appMemory may be
 * CUDA device memory (NV_ARRAY_CUDA, detected as Array.cpp:38-65 does). */
VRTX_API VRTXArray vrtxNewArray1D(VRTXDevice d,
    const void *appMemory,
    VRTXMemoryDeleter deleter,
    const void *userData,
    int elementType,
    uint64_t numItems1);
VRTX_API VRTXArray vrtxNewArray2D(VRTXDevice d,
    const void *appMemory,
    VRTXMemoryDeleter deleter,
    const void *userData,
    int elementType,
    uint64_t numItems1,
    uint64_t numItems2);
VRTX_API VRTXArray vrtxNewArray3D(VRTXDevice d,
    const void *appMemory,
    VRTXMemoryDeleter deleter,
    const void *userData,
    int elementType,
    uint64_t numItems1,
    uint64_t numItems2,
    uint64_t numItems3);

/* Replace VisRTXDevice::mapArray / unmapArray (VisRTXDevice.cpp:190-200). */
VRTX_API void *vrtxMapArray(VRTXDevice d, VRTXArray a);
VRTX_API void vrtxUnmapArray(VRTXDevice d, VRTXArray a);

/* ------------------------------------------------------------------------ */
/* Object creation (VisRTXDevice.cpp:202-292)                               */
/* ------------------------------------------------------------------------ */

VRTX_API VRTXObject vrtxNewCamera(VRTXDevice d, const char *subtype);
VRTX_API VRTXObject vrtxNewGeometry(VRTXDevice d, const char *subtype);
VRTX_API VRTXObject vrtxNewLight(VRTXDevice d, const char *subtype);
VRTX_API VRTXObject vrtxNewMaterial(VRTXDevice d, const char *subtype);
VRTX_API VRTXObject vrtxNewRenderer(VRTXDevice d, const char *subtype);
VRTX_API VRTXObject vrtxNewSampler(VRTXDevice d, const char *subtype);
VRTX_API VRTXObject vrtxNewSpatialField(VRTXDevice d, const char *subtype);
VRTX_API VRTXObject vrtxNewVolume(VRTXDevice d, const char *subtype);
VRTX_API VRTXObject vrtxNewSurface(VRTXDevice d);
VRTX_API VRTXObject vrtxNewGroup(VRTXDevice d);
VRTX_API VRTXObject vrtxNewInstance(VRTXDevice d, const char *subtype);
VRTX_API VRTXObject vrtxNewWorld(VRTXDevice d);
VRTX_API VRTXFrame vrtxNewFrame(VRTXDevice d);

/* ------------------------------------------------------------------------ */
/* Parameters, commit, reference counting (helium::BaseDevice semantics)     */
/* ------------------------------------------------------------------------ */

/* mem points at the value; for object-typed parameters it points at the
 * VRTXObject handle, for VRTX_STRING it is the C string itself. */
VRTX_API void vrtxSetParameter(VRTXDevice d,
    VRTXObject o,
    const char *name,
    int type,
    const void *mem);
VRTX_API void vrtxUnsetParameter(VRTXDevice d, VRTXObject o, const char *name);
VRTX_API void vrtxUnsetAllParameters(VRTXDevice d, VRTXObject o);
VRTX_API void vrtxCommitParameters(VRTXDevice d, VRTXObject o);
VRTX_API void vrtxRelease(VRTXDevice d, VRTXObject o);
VRTX_API void vrtxRetain(VRTXDevice d, VRTXObject o);

/* Object properties: World/Group "bounds" (World.cpp:100-118,
 * Group.cpp:65-86), Frame "duration"/"numSamples"/"nextFrameReset"
 * (Frame.cu:163-193), "valid" on any object. Returns 1 when written. */
VRTX_API int vrtxGetProperty(VRTXDevice d,
    VRTXObject o,
    const char *name,
    int type,
    void *mem,
    uint64_t size,
    uint32_t waitMask);

/* ------------------------------------------------------------------------ */
/* Frame operations                                                         */
/* ------------------------------------------------------------------------ */

/* Replaces VisRTXDevice::renderFrame -> Frame::renderFrame
 * (VisRTXDevice.cpp:360-366, frame/Frame.cu:195-310). Asynchronous on the
 * device's CUDA stream. */
VRTX_API void vrtxRenderFrame(VRTXDevice d, VRTXFrame f);

/* Replaces Frame::frameReady (Frame.cu:425-432): 1 when the last render has
 * finished; with VRTX_WAIT it blocks until then. */
VRTX_API int vrtxFrameReady(VRTXDevice d, VRTXFrame f, uint32_t waitMask);

/* Replaces Frame::discardFrame (no-op in the reference). */
VRTX_API void vrtxDiscardFrame(VRTXDevice d, VRTXFrame f);

/* Replaces Frame::map (Frame.cu:312-423). Channels: "channel.color",
 * "channel.depth", "channel.primitiveId", "channel.objectId",
 * "channel.instanceId", "channel.albedo", "channel.normal" (host copies) and
 * the same names with a "CUDA" suffix (device pointers owned by the frame,
 * valid until the next render or frame change). Unknown or disabled channels
 * return NULL with width = height = 0 and pixelType = VRTX_UNKNOWN. */
VRTX_API const void *vrtxMapFrame(VRTXDevice d,
    VRTXFrame f,
    const char *channel,
    uint32_t *width,
    uint32_t *height,
    int *pixelType);
VRTX_API void vrtxUnmapFrame(VRTXDevice d, VRTXFrame f, const char *channel);

/* ------------------------------------------------------------------------ */
/* Introspection used by tests, the benchmark and the roofline accounting.   */
/* These have no ANARI counterpart; they expose what the reference keeps     */
/* inside OptiX (BVH layout, traversal statistics).                          */
/* ------------------------------------------------------------------------ */

/* Copies the world's acceleration structures for the last render to host
 * memory so a CPU traversal can count node visits on the same BVH. kind: 0 =
 * TLAS nodes, 1 = BLAS nodes (all BLASes, concatenated), 2 = BLAS triangle
 * records, 3 = instance records, 4 = sphere records, 5 = BLAS table. Returns
 * the number of bytes (call with dst = NULL to query). */
VRTX_API uint64_t vrtxDebugCopyAccel(
    VRTXDevice d, VRTXObject world, int kind, void *dst, uint64_t capacity);

/* Image texels as the device stages them at commit, computed on the host
 * (no device, no GPU), for checking. background = 0: an image sampler's
 * image, n texels of elementType (FLOAT32..FLOAT32_VEC4, UFIXED8,
 * UFIXED16, UFIXED8_VEC4, UFIXED8_RGBA_SRGB); float types go to outFloat
 * as n x 4 floats (missing channels 0, alpha 1) and return 1; every other
 * type goes to outBytes as n x 4 bytes that the texture reads as
 * normalised float (8-bit values as they are, sRGB bytes -- alpha too --
 * linearised and truncated to 8 bits, 16-bit values truncated from
 * (c / 65535) * 255; missing channels 0, alpha 255) and returns 0.
 * background = 1: the renderer's background image (FLOAT32_VEC3/4,
 * UFIXED8_VEC4, UFIXED8_RGBA_SRGB) to outBytes as n x 4 bytes (floats
 * truncated from c * 255, clamped to [0, 255]), returning 0. Replaces
 * Image1D/2D/3D::finalize's and Renderer::finalize's staging
 * (scene/surface/material/sampler/Image2D.cpp:70-78, Renderer.cpp:173-179,
 * utility/CudaImageTexture.cpp:43-111) as a separate entry for checking.
 * Returns -1 for an unsupported type or a missing buffer. */
VRTX_API int vrtxDebugStageImage(int elementType,
    int background,
    const void *texels,
    uint64_t n,
    float *outFloat,
    uint8_t *outBytes);

/* The 256-entry RGBA table a transferFunction1D volume's colour / opacity
 * arrays discretise to at commit, computed on the host (no device, no GPU):
 * the colour array (numColor >= 2 entries of colorComponents = 3 or 4
 * floats) and the opacity array (numOpacity >= 2 floats) spread uniformly
 * over [valueLo, valueHi]; either may be NULL, the uniform colour (4 floats)
 * / opacity then stand in, as the volume's "color" / "opacity" values do.
 * Writes 256 x 4 floats to out. Replaces
 * TransferFunction1D::discritizeTFData (TransferFunction1D.cpp:101-150) as a
 * separate entry for checking. Returns 0, or -1 for invalid arguments. */
VRTX_API int vrtxDebugDiscretizeTF(const float *color,
    int numColor,
    int colorComponents,
    const float *opacity,
    int numOpacity,
    float valueLo,
    float valueHi,
    const float *uniformColor,
    float uniformOpacity,
    float *out);

/* The frame's colour write (the end of every render kernel: the
 * accumulation divided by frameID + 1 samples, inverse-tonemapped and
 * packed as sRGB rgba8 for format 0 or linear rgba8 for format 1) applied
 * on the device's GPU to n accumulated RGBA colours (4 floats each, host
 * memory), packed into out (n uint32, host memory). Replaces
 * writeOutputColor (gpu/gpu_util.h:370-389) as a separate entry for
 * checking. Returns 0, or a negative code after reporting the error. */
VRTX_API int vrtxDebugWriteColors(VRTXDevice d,
    const float *accum,
    uint32_t n,
    int frameID,
    int format,
    uint32_t *out);

/* Sorts n (key, value) pairs held in host memory with the BVH builder's
 * Morton sort (a stable LSD radix sort by the low `bits` bits of the keys,
 * bits in 1..64), through device copies on the device's stream. Replaces
 * nothing in the reference: its sort is inside optixAccelBuild
 * (optix_visrtx.cpp:288-372). Returns 0, or a negative code after
 * reporting the error. */
VRTX_API int vrtxDebugRadixSort(
    VRTXDevice d, uint64_t *keys, uint32_t *vals, uint32_t n, int bits);

/* Milliseconds spent in the last BVH / macrocell-grid build of a world
 * (host wall clock around the device build, synchronised). */
VRTX_API float vrtxWorldBuildMilliseconds(VRTXDevice d, VRTXObject world);

/* Device milliseconds of the last frame's integrator kernel alone (CUDA
 * events on the device stream), and the number of kernels the last
 * renderFrame launched. */
VRTX_API float vrtxFrameKernelMilliseconds(VRTXDevice d, VRTXFrame f);
VRTX_API int vrtxFrameKernelLaunches(VRTXDevice d, VRTXFrame f);

/* The CUDA stream (cudaStream_t) the device renders on. */
VRTX_API void *vrtxDeviceStream(VRTXDevice d);

/* ------------------------------------------------------------------------ */
/* Differentiable volume marcher. No reference counterpart: VisRTX has no    */
/* gradient path; this is the emission-absorption model of its scivis        */
/* marcher (devices/rtx/gpu/volumeIntegration.h:64-103) made differentiable. */
/*                                                                          */
/* Model, per pixel ray in voxel space (voxel i's centre at coordinate i,   */
/* box [0, dims-1]): samples at t_k = t_in + (k + 0.5) * step inside the box; */
/* s_k = trilinear(density, p_k); x = clamp((s-lo)/(hi-lo), 0, 1)*(N-1);     */
/* (rgb, A) = lerp(tf[floor x], tf[floor x + 1]); alpha = min(A * scale,    */
/* 0.999); sigma_k = (step/unit) * log(1 - alpha) (<= 0); log T_{k+1} =      */
/* log T_k + sigma_k (Kahan-compensated); pixel = sum T_k (1 - e^sigma_k)   */
/* rgb_k + T_end * background. Marching stops once T < 1e-3.                */
/*                                                                          */
/* All pointers are CUDA device pointers; work is queued on `stream` (a     */
/* cudaStream_t, NULL = legacy default stream) on the calling thread's     */
/* current device, the one that owns the pointers. One launch covers every */
/* view: views are cut into tiles that persistent blocks pull from a queue. */
/* ------------------------------------------------------------------------ */

typedef struct VRTXDMVolume {
  const void *density;   /* dims[0] fastest; fp32, fp16 or bf16 */
  int densityType;       /* VRTX_FLOAT32, VRTX_FLOAT16 or VRTX_BFLOAT16 */
  int dims[3];
  const void *tf;        /* tfSize x RGBA, of type tfType */
  int tfSize;            /* 2..256 */
  float opacityScale;    /* multiplies TF alpha */
  float step;            /* sample spacing, voxels */
  float unitDistance;    /* voxels */
  float valueLo, valueHi;/* density range mapped onto the TF */
  float *gradDensity;    /* fp32, same dims; backward only, may be NULL */
  float *gradTf;         /* fp32, tfSize x 4; backward only, may be NULL */
  float *gradOpacityScale; /* one fp32; backward only, may be NULL */
  const float *opacityScaleDevice; /* when not NULL, read instead of
                                      opacityScale (device scalar) */
  int flags;             /* VRTX_DM_* bits, 0 by default */
  int tfType;            /* VRTX_FLOAT32 (or 0), VRTX_FLOAT16 or VRTX_BFLOAT16;
                            entries are read in fp32, gradTf stays fp32 */
} VRTXDMVolume;

/* Backward pass: one atomic add per gradient term per sample instead of
 * per-thread run-length accumulation (consecutive samples of a ray that
 * stay in one trilinear cell / one TF segment summed in registers first).
 * Both give the same gradients up to float summation order. */
#define VRTX_DM_PLAIN 1

typedef struct VRTXDMView {
  int volume;            /* index into the volume array */
  int width, height;
  float eye[3];          /* camera position, voxel space */
  float d00[3], du[3], dv[3]; /* ray dir = normalize(d00 + (x+.5) du + (y+.5) dv) */
  float background[3];
  int64_t pixelOffset;   /* first pixel of this view in image/state */
} VRTXDMView;

/* Forward. image: 3 floats per pixel. state: 2 floats per pixel (final
 * log-transmittance, and the sample count stored as an int32 bit pattern);
 * the backward pass reads it. tileW x tileH pixels per work item
 * (tileW * tileH a multiple of 32, at most 256). Returns 0, or a negative
 * code after reporting the error through the device's status callback. */
VRTX_API int vrtxDMForward(VRTXDevice d,
    const VRTXDMVolume *volumes,
    int numVolumes,
    const VRTXDMView *views,
    int numViews,
    float *image,
    float *state,
    int tileW,
    int tileH,
    void *stream);

/* Backward: reverse-order march from each pixel's stored end state;
 * accumulates (adds) into the gradient buffers named in volumes[]. */
VRTX_API int vrtxDMBackward(VRTXDevice d,
    const VRTXDMVolume *volumes,
    int numVolumes,
    const VRTXDMView *views,
    int numViews,
    const float *image,
    const float *state,
    const float *gradImage,
    int tileW,
    int tileH,
    void *stream);

/* Plans: the volume/view descriptors uploaded once (stream-ordered on
 * `stream`) so that vrtxDMPlanForward / vrtxDMPlanBackward issue only a
 * counter reset and one kernel each, and can be captured into a CUDA graph.
 * Buffers named in the descriptors must outlive the plan. Returns NULL
 * after reporting invalid arguments. */
typedef struct VRTXDMPlan_st *VRTXDMPlan;
VRTX_API VRTXDMPlan vrtxDMPlanCreate(VRTXDevice d,
    const VRTXDMVolume *volumes,
    int numVolumes,
    const VRTXDMView *views,
    int numViews,
    int tileW,
    int tileH,
    void *stream);
VRTX_API int vrtxDMPlanForward(
    VRTXDMPlan plan, float *image, float *state, void *stream);
VRTX_API int vrtxDMPlanBackward(VRTXDMPlan plan,
    const float *state,
    const float *gradImage,
    void *stream);
/* One training step of an L2 image loss in a single persistent launch:
 * every pixel of every view is marched forward, its loss gradient
 * 2 * lossScale * (pixel - target) is formed in registers, and the same
 * thread runs the adjoint at once, adding into the plan's gradient buffers
 * (as vrtxDMPlanBackward would with that gradImage). target: 3 floats per
 * pixel, the plan's image layout. image (may be NULL) receives the pixels;
 * loss (a device float, may be NULL) has lossScale * sum((pixel -
 * target)^2) added to it. No per-pixel state is written and no loss kernel
 * runs between the passes. No reference counterpart (VisRTX has no
 * gradient path). Returns 0, or a negative code after reporting the
 * error. */
VRTX_API int vrtxDMPlanStepL2(VRTXDMPlan plan,
    const float *target,
    float lossScale,
    float *image,
    float *loss,
    void *stream);
/* The plan's launch shape: resident blocks per SM of both kernels (0: as
 * many as fit, the default) and work items each block takes from the queue
 * per atomic fetch (1..64 consecutive tiles, default 1). Results do not
 * depend on it beyond float summation order of the gradient reductions.
 * No reference counterpart (the differentiable marcher is this library's
 * own). Returns 0, or a negative code after reporting the error. */
VRTX_API int vrtxDMPlanSetLaunch(VRTXDMPlan plan, int blocksPerSM, int tilesPerFetch);
VRTX_API void vrtxDMPlanRelease(VRTXDMPlan plan);

/* The forward pass of vrtxDMForward for callers that cannot allocate
 * device memory: code whose memory comes from an allocator that is not
 * CUDA's (a host application's pool, a plugin sandbox), or code running
 * where cudaMalloc must not be called. No counterpart in the reference
 * (VisRTX has no gradient path).
 *
 * Same arguments and results as vrtxDMForward. It allocates nothing: its
 * scratch (the launch counter and the volume/view descriptors) is one
 * fixed-size device array inside the library, at most 64 volumes and 4096
 * views per call (about 400 KB, held on every GPU that loads the library
 * until the process exits); larger requests are rejected with an error.
 * The first call on a device looks up that array's device address; make
 * that first call before any stream capture. The address is kept for the
 * life of the process and does not survive a cudaDeviceReset. Every call
 * copies its descriptors from host memory it frees on return, so a call
 * on a stream that is capturing is rejected with an error. All calls share
 * the array: calls that overlap on the GPU (unordered streams) race on
 * it. */
VRTX_API int vrtxDMForwardNoAlloc(VRTXDevice d,
    const VRTXDMVolume *volumes,
    int numVolumes,
    const VRTXDMView *views,
    int numViews,
    float *image,
    float *state,
    int tileW,
    int tileH,
    void *stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* VRTX_H */
