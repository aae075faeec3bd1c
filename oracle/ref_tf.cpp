// Test infrastructure: a harness around the reference's own transfer-function
// helpers (devices/rtx/utility/colorMapHelpers.h: generateLinearPositions,
// getInterpolatedValue, with gpu/gpu_math.h's box1 / position / contains and
// the vendored glm), compiled from those headers where they lie into
// oracle/_ref/libtfref.so by oracle/build.py, only where the reference tree
// is present, and used only by tests/golden/make_tf_golden.py,
// tests/golden/make_math_golden.py (the gpu_math.h and uniformGrid.h
// helpers after it) and tests/golden/make_volume_interval_golden.py
// (intersectVolume's glm calls, at the end).
//
// tfref_discretize repeats the call sequence of
// TransferFunction1D::discritizeTFData (TransferFunction1D.cpp:101-150): the
// colour and opacity knots placed uniformly over the value range, each of
// the tfDim entries sampled at p = i / (tfDim - 1), the entry (rgb, a * o)
// with a = 1 for vec3 colours, and the uniform colour / opacity where an
// array is absent. That file itself needs the ANARI-SDK and cannot be built
// here; the arithmetic it calls is the helpers', compiled unchanged.
#define GLM_ENABLE_EXPERIMENTAL
#include "gpu/uniformGrid.h"
#include "utility/colorMapHelpers.h"

#include <glm/gtx/component_wise.hpp>

#include <vector>

extern "C" void tfref_discretize(const float *color,
    int numColor,
    int colorComps,
    const float *opacity,
    int numOpacity,
    float lo,
    float hi,
    const float *uniformColor,
    float uniformOpacity,
    int tfDim,
    float *out)
{
  using namespace visrtx;
  const box1 range(lo, hi);
  std::vector<float> cPos, oPos;
  Span<float> cPositions, oPositions;
  if (color) {
    cPos = generateLinearPositions((size_t)numColor, range);
    cPositions = make_Span(cPos.data(), cPos.size());
  }
  if (opacity) {
    oPos = generateLinearPositions((size_t)numOpacity, range);
    oPositions = make_Span(oPos.data(), oPos.size());
  }
  for (int i = 0; i < tfDim; i++) {
    const float p = float(i) / (tfDim - 1);
    vec4 c(uniformColor[0], uniformColor[1], uniformColor[2], uniformColor[3]);
    if (color) {
      if (colorComps == 3)
        c = vec4(getInterpolatedValue(
                     reinterpret_cast<const vec3 *>(color), cPositions, range, p),
            1.f);
      else
        c = getInterpolatedValue(
            reinterpret_cast<const vec4 *>(color), cPositions, range, p);
    }
    const float o = opacity
        ? getInterpolatedValue(opacity, oPositions, range, p)
        : uniformOpacity;
    out[4 * i + 0] = c.x;
    out[4 * i + 1] = c.y;
    out[4 * i + 2] = c.z;
    out[4 * i + 3] = c.w * o;
  }
}

// The reference's own gpu/gpu_math.h helpers on the thin-lens, HDRI and
// physically based next-ray paths (uniformSampleDisk :292-297,
// sphericalCoordsFromDirection :254-261, uniformSampleCone below),
// compiled unchanged, on n inputs.
extern "C" void mathref_uniform_sample_disk(const float *in3, int n, float *out2)
{
  for (int i = 0; i < n; i++) {
    const visrtx::vec2 r = visrtx::uniformSampleDisk(
        in3[3 * i], visrtx::vec2(in3[3 * i + 1], in3[3 * i + 2]));
    out2[2 * i] = r.x;
    out2[2 * i + 1] = r.y;
  }
}

extern "C" void mathref_spherical_from_dir(const float *dir3, int n, float *out2)
{
  for (int i = 0; i < n; i++) {
    const visrtx::vec2 r = visrtx::sphericalCoordsFromDirection(
        visrtx::vec3(dir3[3 * i], dir3[3 * i + 1], dir3[3 * i + 2]));
    out2[2 * i] = r.x;
    out2[2 * i + 1] = r.y;
  }
}

// uniformSampleCone (gpu/gpu_math.h:299-312), compiled unchanged
extern "C" void mathref_uniform_sample_cone(const float *in4, int n, float *out3)
{
  for (int i = 0; i < n; i++) {
    const visrtx::vec3 r = visrtx::uniformSampleCone(
        in4[4 * i], visrtx::vec3(in4[4 * i + 1], in4[4 * i + 2], in4[4 * i + 3]));
    out3[3 * i] = r.x;
    out3[3 * i + 1] = r.y;
    out3[3 * i + 2] = r.z;
  }
}

// projectOnGrid (gpu/uniformGrid.h:43-50), compiled unchanged, for points
// inside the box (outside it the host's float-to-int conversion is not
// defined)
extern "C" void mathref_project_on_grid(
    const float *p3, int n, const int *dims3, const float *box6, int *out3)
{
  const visrtx::ivec3 dims(dims3[0], dims3[1], dims3[2]);
  const visrtx::box3 b(visrtx::vec3(box6[0], box6[1], box6[2]),
      visrtx::vec3(box6[3], box6[4], box6[5]));
  for (int i = 0; i < n; i++) {
    const visrtx::ivec3 c = visrtx::projectOnGrid(
        visrtx::vec3(p3[3 * i], p3[3 * i + 1], p3[3 * i + 2]), dims, b);
    out3[3 * i] = c.x;
    out3[3 * i + 1] = c.y;
    out3[3 * i + 2] = c.z;
  }
}

// intersectVolume's slab interval (scene/Intersectors_ptx.cu:248-274): its
// calls repeated over the vendored glm (glm::min / glm::max of the slab
// vectors, glm::compMax / glm::compMin) and gpu_math.h's range clamp, for n
// local rays (org xyz, dir xyz, tmin, tmax) against box6. That file is an
// OptiX program and cannot be built here; the arithmetic it calls is glm's
// and gpu_math.h's, compiled unchanged.
extern "C" void mathref_volume_interval(
    const float *rays8, int n, const float *box6, int *hit, float *t01)
{
  using namespace visrtx;
  const box3 bounds(vec3(box6[0], box6[1], box6[2]), vec3(box6[3], box6[4], box6[5]));
  for (int i = 0; i < n; i++) {
    const float *r = rays8 + 8 * i;
    const vec3 org(r[0], r[1], r[2]), dir(r[3], r[4], r[5]);
    const vec3 mins = (bounds.lower - org) * (1.f / dir);
    const vec3 maxs = (bounds.upper - org) * (1.f / dir);
    const vec3 nears = glm::min(mins, maxs);
    const vec3 fars = glm::max(mins, maxs);
    box1 t(glm::compMax(nears), glm::compMin(fars));
    hit[i] = t.lower < t.upper ? 1 : 0;
    if (hit[i]) {
      const box1 rayt{r[6], r[7]};
      t.lower = visrtx::clamp(t.lower, rayt);
      t.upper = visrtx::clamp(t.upper, rayt);
    }
    t01[2 * i] = hit[i] ? t.lower : 0.f;
    t01[2 * i + 1] = hit[i] ? t.upper : 0.f;
  }
}
