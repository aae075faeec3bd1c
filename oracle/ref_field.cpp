// Test infrastructure: a harness around the reference's own structured-field
// sampler (devices/rtx/gpu/sampleSpatialField.h:54-78,
// SpatialFieldSampler<cudaTextureObject_t>: the world location to the 3D
// texture coordinate the field's texture is read at), compiled unchanged
// into oracle/_ref/libfieldref.so by oracle/build.py, only where the
// reference tree is present, and used only by
// tests/golden/make_field_golden.py.
//
// The header includes gpu_objects.h, which needs OptiX; oracle/build.py
// compiles this file through oracle/_ref/gpu_inc/gpu/, where
// oracle/ref_shim/gpu_objects.h stands in for it (the field record by the
// reference's member names). The texture fetch itself is the texture unit's
// (pinned separately by GPU captures), so the tex3D below only records the
// coordinate the sampler hands it.
#include <texture_types.h>

namespace {
struct TexCoord
{
  float x, y, z;
};
TexCoord g_lastFetch;
} // namespace

template <typename T>
T tex3D(cudaTextureObject_t, float x, float y, float z)
{
  g_lastFetch = {x, y, z};
  return T(0);
}

#include "gpu/sampleSpatialField.h"

// The texture coordinates the sampler computes for n world points p3 of a
// field with the given origin and spacing over dims3 voxels. invSpacing is
// set as StructuredRegularField::gpuData computes it
// (StructuredRegularField.cpp:188-189: vec3(1) / (spacing * vec3(dims)));
// that file needs the ANARI-SDK and is not compiled here.
extern "C" void fieldref_coords(const float *origin3,
    const float *spacing3,
    const int *dims3,
    const float *p3,
    int n,
    float *out3)
{
  using namespace visrtx;
  SpatialFieldGPUData sf;
  sf.type = SpatialFieldType::STRUCTURED_REGULAR;
  auto &s = sf.data.structuredRegular;
  s.texObj = 0;
  s.origin = vec3(origin3[0], origin3[1], origin3[2]);
  s.spacing = vec3(spacing3[0], spacing3[1], spacing3[2]);
  s.invSpacing = vec3(1.f) / (s.spacing * vec3(dims3[0], dims3[1], dims3[2]));
  SpatialFieldSampler<cudaTextureObject_t> sampler(sf);
  for (int i = 0; i < n; i++) {
    sampler(vec3(p3[3 * i], p3[3 * i + 1], p3[3 * i + 2]));
    out3[3 * i] = g_lastFetch.x;
    out3[3 * i + 1] = g_lastFetch.y;
    out3[3 * i + 2] = g_lastFetch.z;
  }
}
