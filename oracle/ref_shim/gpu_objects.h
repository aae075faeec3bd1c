// Test infrastructure: a host stand-in for the reference's
// devices/rtx/gpu/gpu_objects.h, which needs OptiX, curand and the ANARI-SDK
// (none present here). It is put ahead of the reference's own header only
// when oracle/build.py compiles oracle/ref_dda.cpp, which needs from it no
// more than gpu_debug.h does: the launch-index queries of debug() /
// crosshair(), here a launch of one pixel. The vector, box and ray types
// come from the reference's own gpu/gpu_math.h.
#pragma once

#include "gpu/gpu_math.h"

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
