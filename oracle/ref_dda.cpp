// Test infrastructure: a harness around the reference's own macrocell walk
// (devices/rtx/gpu/dda.h:43-122, dda3), compiled unchanged from the header
// where it lies into oracle/_ref/libddaref.so by oracle/build.py, only where
// the reference tree is present, and used only by
// tests/golden/make_dda_golden.py.
//
// dda.h includes gpu_objects.h, which needs OptiX. oracle/build.py therefore
// compiles this file through oracle/_ref/gpu_inc/gpu/, a directory of links
// to the reference's dda.h, gpu_debug.h, gpu_math.h, gpu_decl.h and
// uniformGrid.h beside a link to oracle/ref_shim/gpu_objects.h (the launch
// queries gpu_debug.h calls); every other line is the reference's.
//
// The names below are the ones dda.h takes from its CUDA translation unit:
// the scalar min / max that CUDA declares globally, and glm's component-wise
// compMin, which the reference's volume integration brings in before dda.h
// (through gpu/gpu_util.h). The reference's GPU build contracts
// tnear + float(c) * dist into a fused multiply-add (nvcc's default
// -fmad=true); oracle/build.py compiles this file with contraction on, so
// that the host walk rounds as that build does.
#define GLM_ENABLE_EXPERIMENTAL
#include <glm/common.hpp>
#include <glm/gtx/component_wise.hpp>

#include <algorithm>
using std::max;
using std::min;

#include "gpu/dda.h"

// ddaref_walk runs dda3 for n rays over one grid and records, per visited
// cell, the linear cell index and the interval [t0, t1] the walk hands its
// callback. A ray's walk stops after maxCells cells (the callback returns
// false), as the delta-tracking loop stops once it has found a collision.
extern "C" int ddaref_walk(const float *rays8, // org xyz, dir xyz, tlo, thi
    int n,
    const int *dims3,
    const float *box6,
    int maxCells,
    int *counts, // n: cells visited per ray
    long long *cells, // n * maxCells
    float *t01) // n * maxCells * 2
{
  using namespace visrtx;
  const ivec3 dims(dims3[0], dims3[1], dims3[2]);
  const box3 bounds(
      vec3(box6[0], box6[1], box6[2]), vec3(box6[3], box6[4], box6[5]));
  int total = 0;
  for (int i = 0; i < n; i++) {
    const float *r = rays8 + 8 * i;
    Ray ray;
    ray.org = vec3(r[0], r[1], r[2]);
    ray.dir = vec3(r[3], r[4], r[5]);
    ray.t = box1(r[6], r[7]);
    int k = 0;
    dda3(ray, dims, bounds, [&](size_t cell, float t0, float t1) {
      const size_t j = (size_t)i * maxCells + k;
      cells[j] = (long long)cell;
      t01[2 * j] = t0;
      t01[2 * j + 1] = t1;
      return ++k < maxCells;
    });
    counts[i] = k;
    total += k;
  }
  return total;
}
