/*
 * anari_visrtx.h -- the ANARI-facing face of libvrtx: the ANARI 1.0 C API
 * calls a VisRTX application makes, and VisRTX's own exported functions
 * (include/anari/ext/visrtx/visrtx.h:49-73 in the VisRTX project), each
 * forwarding to the vrtx* C ABI of include/vrtx.h.
 *
 * The ANARI-SDK is not part of this build, so the names, handle types,
 * signatures and enum values below are written from the public ANARI 1.0
 * specification (its C API chapter and its type table). An application
 * written against the ANARI C API compiles against this header and links
 * against libvrtx.so instead of libanari + libanari_library_visrtx.so; a
 * prebuilt one links unchanged where its anari_enums.h carries these
 * values.
 *
 * What is left out: the SDK's C++ library entry point
 * (ANARI_DEFINE_LIBRARY_ENTRYPOINT, VisRTXLibrary.cpp:70-74), whose ABI is
 * the SDK's C++ classes; anariGetObjectInfo / anariGetParameterInfo return
 * NULL (no introspection tables).
 */
#ifndef ANARI_VISRTX_H
#define ANARI_VISRTX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define ANARI_SHIM_API __declspec(dllexport)
#else
#define ANARI_SHIM_API __attribute__((visibility("default")))
#endif

/* --- handles ------------------------------------------------------------- */

typedef struct _ANARILibrary *ANARILibrary;
typedef struct _ANARIDevice *ANARIDevice;
typedef struct _ANARIObject *ANARIObject;
typedef ANARIObject ANARIArray;
typedef ANARIObject ANARIArray1D;
typedef ANARIObject ANARIArray2D;
typedef ANARIObject ANARIArray3D;
typedef ANARIObject ANARICamera;
typedef ANARIObject ANARIFrame;
typedef ANARIObject ANARIGeometry;
typedef ANARIObject ANARIGroup;
typedef ANARIObject ANARIInstance;
typedef ANARIObject ANARILight;
typedef ANARIObject ANARIMaterial;
typedef ANARIObject ANARIRenderer;
typedef ANARIObject ANARISampler;
typedef ANARIObject ANARISpatialField;
typedef ANARIObject ANARISurface;
typedef ANARIObject ANARIVolume;
typedef ANARIObject ANARIWorld;

typedef int ANARIDataType;
typedef int ANARIStatusSeverity;
typedef int ANARIStatusCode;
typedef uint32_t ANARIWaitMask;

/* --- data types (the ANARI 1.0 type table) --------------------------------- */

#define ANARI_UNKNOWN 0
#define ANARI_DATA_TYPE 100
#define ANARI_STRING 101
#define ANARI_VOID_POINTER 102
#define ANARI_BOOL 103
#define ANARI_STRING_LIST 150
#define ANARI_DATA_TYPE_LIST 151
#define ANARI_PARAMETER_LIST 152
#define ANARI_FUNCTION_POINTER 200
#define ANARI_MEMORY_DELETER 201
#define ANARI_STATUS_CALLBACK 202
#define ANARI_LIBRARY 500
#define ANARI_DEVICE 501
#define ANARI_OBJECT 502
#define ANARI_ARRAY 503
#define ANARI_ARRAY1D 504
#define ANARI_ARRAY2D 505
#define ANARI_ARRAY3D 506
#define ANARI_CAMERA 507
#define ANARI_FRAME 508
#define ANARI_GEOMETRY 509
#define ANARI_GROUP 510
#define ANARI_INSTANCE 511
#define ANARI_LIGHT 512
#define ANARI_MATERIAL 513
#define ANARI_RENDERER 514
#define ANARI_SURFACE 515
#define ANARI_SAMPLER 516
#define ANARI_SPATIAL_FIELD 517
#define ANARI_VOLUME 518
#define ANARI_WORLD 519
#define ANARI_INT8 1000
#define ANARI_UINT8 1004
#define ANARI_INT16 1008
#define ANARI_UINT16 1012
#define ANARI_INT32 1016
#define ANARI_INT32_VEC2 1017
#define ANARI_UINT32 1020
#define ANARI_UINT32_VEC2 1021
#define ANARI_UINT32_VEC3 1022
#define ANARI_UINT32_VEC4 1023
#define ANARI_INT64 1024
#define ANARI_UINT64 1028
#define ANARI_FIXED8 1032
#define ANARI_UFIXED8 1036
#define ANARI_UFIXED8_VEC4 1039
#define ANARI_FIXED16 1040
#define ANARI_UFIXED16 1044
#define ANARI_FLOAT16 1064
#define ANARI_FLOAT32 1068
#define ANARI_FLOAT32_VEC2 1069
#define ANARI_FLOAT32_VEC3 1070
#define ANARI_FLOAT32_VEC4 1071
#define ANARI_FLOAT64 1072
#define ANARI_UFIXED8_RGBA_SRGB 2003
#define ANARI_FLOAT32_BOX1 2008
#define ANARI_FLOAT32_BOX2 2009
#define ANARI_FLOAT32_BOX3 2010
#define ANARI_FLOAT64_BOX1 2012
#define ANARI_FLOAT32_MAT4 2022
#define ANARI_FLOAT32_MAT3x4 2024

#define ANARI_SEVERITY_FATAL_ERROR 1
#define ANARI_SEVERITY_ERROR 2
#define ANARI_SEVERITY_WARNING 3
#define ANARI_SEVERITY_PERFORMANCE_WARNING 4
#define ANARI_SEVERITY_INFO 5
#define ANARI_SEVERITY_DEBUG 6

#define ANARI_STATUS_NO_ERROR 0
#define ANARI_STATUS_UNKNOWN_ERROR 1

#define ANARI_NO_WAIT 0
#define ANARI_WAIT 1

/* --- callbacks ----------------------------------------------------------- */

typedef void (*ANARIStatusCallback)(const void *userData,
    ANARIDevice device,
    ANARIObject source,
    ANARIDataType sourceType,
    ANARIStatusSeverity severity,
    ANARIStatusCode code,
    const char *message);
typedef void (*ANARIMemoryDeleter)(const void *userData, const void *appMemory);
typedef void (*ANARIFrameCompletionCallback)(
    const void *userData, ANARIDevice device, ANARIFrame frame);

/* --- VisRTX's exported functions (visrtx.h:49-73, VisRTXLibrary.cpp:76-80) */

/* A device on CUDA device 0 (or "cudaDevice" set before the first object);
 * forwards to vrtxNewDevice. */
ANARI_SHIM_API ANARIDevice makeVisRTXDevice(
    ANARIStatusCallback defaultCallback, const void *userPtr);

typedef struct
{
  int VISRTX_ARRAY_CUDA;
  int VISRTX_CUDA_OUTPUT_BUFFERS;
  int VISRTX_INSTANCE_ATTRIBUTES;
  int VISRTX_MATERIAL_MDL;
  int VISRTX_SPATIAL_FIELD_NANOVDB;
  int VISRTX_TRIANGLE_BACK_FACE_CULLING;
  int VISRTX_TRIANGLE_FACE_VARYING_ATTRIBUTES;
} VisRTXExtensions;

/* visrtxGetObjectExtensions / visrtxGetInstanceExtensions
 * (VisRTXFeatureUtility.cpp:66-99); forward to vrtxGetObjectExtensions /
 * vrtxGetInstanceExtensions. */
ANARI_SHIM_API int visrtxGetObjectExtensions(VisRTXExtensions *extensions,
    ANARIDevice device,
    ANARIDataType objectType,
    const char *objectSubtype);
ANARI_SHIM_API int visrtxGetInstanceExtensions(
    VisRTXExtensions *extensions, ANARIDevice device, ANARIObject object);

/* --- the ANARI C API (the calls of a VisRTX application) ------------------ */

/* "visrtx" (or "default", "environment"): a library whose only device type
 * is "visrtx" (also answered to "default"). */
ANARI_SHIM_API ANARILibrary anariLoadLibrary(const char *name,
    ANARIStatusCallback statusCallback,
    const void *statusCallbackUserData);
ANARI_SHIM_API void anariUnloadLibrary(ANARILibrary library);
ANARI_SHIM_API const char **anariGetDeviceSubtypes(ANARILibrary library);
ANARI_SHIM_API ANARIDevice anariNewDevice(ANARILibrary library, const char *type);

ANARI_SHIM_API ANARIArray1D anariNewArray1D(ANARIDevice device,
    const void *appMemory,
    ANARIMemoryDeleter deleter,
    const void *userData,
    ANARIDataType dataType,
    uint64_t numItems1);
ANARI_SHIM_API ANARIArray2D anariNewArray2D(ANARIDevice device,
    const void *appMemory,
    ANARIMemoryDeleter deleter,
    const void *userData,
    ANARIDataType dataType,
    uint64_t numItems1,
    uint64_t numItems2);
ANARI_SHIM_API ANARIArray3D anariNewArray3D(ANARIDevice device,
    const void *appMemory,
    ANARIMemoryDeleter deleter,
    const void *userData,
    ANARIDataType dataType,
    uint64_t numItems1,
    uint64_t numItems2,
    uint64_t numItems3);
ANARI_SHIM_API void *anariMapArray(ANARIDevice device, ANARIArray array);
ANARI_SHIM_API void anariUnmapArray(ANARIDevice device, ANARIArray array);

ANARI_SHIM_API ANARILight anariNewLight(ANARIDevice device, const char *type);
ANARI_SHIM_API ANARICamera anariNewCamera(ANARIDevice device, const char *type);
ANARI_SHIM_API ANARIGeometry anariNewGeometry(ANARIDevice device, const char *type);
ANARI_SHIM_API ANARISpatialField anariNewSpatialField(ANARIDevice device, const char *type);
ANARI_SHIM_API ANARIVolume anariNewVolume(ANARIDevice device, const char *type);
ANARI_SHIM_API ANARISurface anariNewSurface(ANARIDevice device);
ANARI_SHIM_API ANARIMaterial anariNewMaterial(ANARIDevice device, const char *type);
ANARI_SHIM_API ANARISampler anariNewSampler(ANARIDevice device, const char *type);
ANARI_SHIM_API ANARIGroup anariNewGroup(ANARIDevice device);
ANARI_SHIM_API ANARIInstance anariNewInstance(ANARIDevice device, const char *type);
ANARI_SHIM_API ANARIWorld anariNewWorld(ANARIDevice device);
ANARI_SHIM_API ANARIRenderer anariNewRenderer(ANARIDevice device, const char *type);
ANARI_SHIM_API ANARIFrame anariNewFrame(ANARIDevice device);
/* objectType: "camera", "geometry", "light", "material", "renderer",
 * "sampler", "spatialField", "volume", "instance", "surface", "group",
 * "world" or "frame". */
ANARI_SHIM_API ANARIObject anariNewObject(
    ANARIDevice device, const char *objectType, const char *type);

/* object == (ANARIObject)device sets a device parameter ("cudaDevice",
 * "forceInit", "statusCallback", "statusCallbackUserData"). */
ANARI_SHIM_API void anariSetParameter(ANARIDevice device,
    ANARIObject object,
    const char *name,
    ANARIDataType dataType,
    const void *mem);
ANARI_SHIM_API void anariUnsetParameter(
    ANARIDevice device, ANARIObject object, const char *name);
ANARI_SHIM_API void anariUnsetAllParameters(ANARIDevice device, ANARIObject object);
/* A managed array set as the parameter and mapped; its memory is written by
 * the application until anariUnmapParameterArray. elementStride receives
 * the element size in bytes. */
ANARI_SHIM_API void *anariMapParameterArray1D(ANARIDevice device,
    ANARIObject object,
    const char *name,
    ANARIDataType dataType,
    uint64_t numElements1,
    uint64_t *elementStride);
ANARI_SHIM_API void *anariMapParameterArray2D(ANARIDevice device,
    ANARIObject object,
    const char *name,
    ANARIDataType dataType,
    uint64_t numElements1,
    uint64_t numElements2,
    uint64_t *elementStride);
ANARI_SHIM_API void *anariMapParameterArray3D(ANARIDevice device,
    ANARIObject object,
    const char *name,
    ANARIDataType dataType,
    uint64_t numElements1,
    uint64_t numElements2,
    uint64_t numElements3,
    uint64_t *elementStride);
ANARI_SHIM_API void anariUnmapParameterArray(
    ANARIDevice device, ANARIObject object, const char *name);
ANARI_SHIM_API void anariCommitParameters(ANARIDevice device, ANARIObject object);
/* anariRelease(device, (ANARIObject)device) releases the device. */
ANARI_SHIM_API void anariRelease(ANARIDevice device, ANARIObject object);
ANARI_SHIM_API void anariRetain(ANARIDevice device, ANARIObject object);

ANARI_SHIM_API const char **anariGetObjectSubtypes(
    ANARIDevice device, ANARIDataType objectType);
ANARI_SHIM_API const void *anariGetObjectInfo(ANARIDevice device,
    ANARIDataType objectType,
    const char *objectSubtype,
    const char *infoName,
    ANARIDataType infoType);
ANARI_SHIM_API const void *anariGetParameterInfo(ANARIDevice device,
    ANARIDataType objectType,
    const char *objectSubtype,
    const char *parameterName,
    ANARIDataType parameterType,
    const char *infoName,
    ANARIDataType infoType);
/* object == (ANARIObject)device reads a device property. */
ANARI_SHIM_API int anariGetProperty(ANARIDevice device,
    ANARIObject object,
    const char *name,
    ANARIDataType type,
    void *mem,
    uint64_t size,
    ANARIWaitMask mask);

ANARI_SHIM_API const void *anariMapFrame(ANARIDevice device,
    ANARIFrame frame,
    const char *channel,
    uint32_t *width,
    uint32_t *height,
    ANARIDataType *pixelType);
ANARI_SHIM_API void anariUnmapFrame(ANARIDevice device, ANARIFrame frame, const char *channel);
ANARI_SHIM_API void anariRenderFrame(ANARIDevice device, ANARIFrame frame);
ANARI_SHIM_API int anariFrameReady(ANARIDevice device, ANARIFrame frame, ANARIWaitMask mask);
ANARI_SHIM_API void anariDiscardFrame(ANARIDevice device, ANARIFrame frame);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* ANARI_VISRTX_H */
