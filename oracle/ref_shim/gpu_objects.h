// Test infrastructure: a host stand-in for the reference's
// devices/rtx/gpu/gpu_objects.h, which needs OptiX, curand and the ANARI-SDK
// (none present here). oracle/build.py puts it ahead of the reference's own
// header only when it compiles the harnesses oracle/ref_dda.cpp,
// oracle/ref_camera.cpp and oracle/ref_field.cpp. It declares what those
// reference headers use from gpu_objects.h and nothing else:
//  * the launch-index queries of gpu_debug.h's debug() / crosshair(), here a
//    launch of one pixel;
//  * the camera record cameraCreateRay reads (the same member names; the
//    perspective and orthographic parts side by side rather than in a
//    union, since the harness fills them by name);
//  * the frame record and screen sample makePrimaryRay reads, with
//    curand_uniform4 returning the four numbers the harness put in the
//    sample's generator state, so that a harness call chooses the
//    sub-pixel offset and aperture sample;
//  * the spatial-field record the field sampler of gpu/sampleSpatialField.h
//    reads (structured-regular and NanoVDB parts side by side), and the
//    frame's field registry it indexes.
// The vector, box and ray types come from the reference's own
// gpu/gpu_math.h.
#pragma once

#include "gpu/gpu_math.h"

#include <glm/ext/vector_uint2.hpp>

#if __has_include(<texture_types.h>)
#include <texture_types.h>
#else
typedef unsigned long long cudaTextureObject_t; // CUDA's texture handle type
#endif

namespace visrtx_host_shim {
struct LaunchIndex
{
  unsigned x, y, z;
};
} // namespace visrtx_host_shim

inline visrtx_host_shim::LaunchIndex optixGetLaunchIndex()
{
  return {0u, 0u, 0u};
}

inline visrtx_host_shim::LaunchIndex optixGetLaunchDimensions()
{
  return {1u, 1u, 1u};
}

// CUDA's float4 (its own where CUDA's headers are on the include path) and a
// generator whose next uniform4 draw is preset
#if __has_include(<vector_types.h>)
#include <vector_types.h>
#else
struct float4
{
  float x, y, z, w;
};
#endif

namespace visrtx_host_shim {
struct PresetUniform4
{
  ::float4 next;
};
} // namespace visrtx_host_shim

inline ::float4 curand_uniform4(visrtx_host_shim::PresetUniform4 *s)
{
  return s->next;
}

namespace visrtx {

using RandState = visrtx_host_shim::PresetUniform4;

enum class CameraType
{
  PERSPECTIVE,
  ORTHOGRAPHIC,
  UNKNOWN
};

struct PerspectiveCameraGPUData
{
  vec3 dir_du;
  vec3 dir_dv;
  vec3 dir_00;
  float scaledAperture;
  float aspect;
};

struct OrthographicCameraGPUData
{
  vec3 pos_du;
  vec3 pos_dv;
  vec3 pos_00;
};

struct CameraGPUData
{
  CameraType type{CameraType::UNKNOWN};
  vec4 region;
  vec3 pos;
  vec3 dir;
  vec3 up;
  PerspectiveCameraGPUData perspective;
  OrthographicCameraGPUData orthographic;
};

using DeviceObjectIndex = int32_t;

enum class SpatialFieldType
{
  STRUCTURED_REGULAR,
  NANOVDB_REGULAR,
  UNKNOWN
};

struct StructuredRegularData
{
  cudaTextureObject_t texObj;
  vec3 origin;
  vec3 spacing;
  vec3 invSpacing;
};

struct NVdbRegularData
{
  vec3 origin;
  vec3 voxelSize;
  int gridType;
  const void *gridData;
};

struct SpatialFieldGPUData
{
  SpatialFieldType type{SpatialFieldType::UNKNOWN};
  struct
  {
    StructuredRegularData structuredRegular;
    NVdbRegularData nvdbRegular;
  } data;
};

struct FramebufferGPUData
{
  glm::vec2 invSize;
};

struct FrameGPUData
{
  FramebufferGPUData fb;
  CameraGPUData *camera;
  struct
  {
    const SpatialFieldGPUData *fields;
  } registry;
};

struct ScreenSample
{
  glm::uvec2 pixel;
  glm::vec2 screen;
  mutable RandState rs;
  const FrameGPUData *frameData;
};

} // namespace visrtx
