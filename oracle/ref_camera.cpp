// Test infrastructure: a harness around the reference's own primary-ray
// generation (devices/rtx/gpu/cameraCreateRay.h:38-81, makePrimaryRay and
// cameraCreateRay, with gpu_math.h's uniformSampleDisk for the thin lens),
// compiled unchanged from the header where it lies into
// oracle/_ref/libcamref.so by oracle/build.py, only where the reference tree
// is present, and used only by tests/golden/make_camera_golden.py.
//
// cameraCreateRay.h includes gpu_objects.h, which needs OptiX and curand;
// oracle/build.py compiles this file through the same directory of links as
// oracle/ref_dda.cpp, where oracle/ref_shim/gpu_objects.h stands in for it
// (the camera, frame and screen-sample records by member name, and a
// curand_uniform4 that returns the numbers this harness presets). It is
// compiled without floating-point contraction: each operation rounds once,
// as in the oracle and in the library's kernels (built with -fmad=false).
#include "gpu/cameraCreateRay.h"

// Camera record, 30 floats: region (4), pos (3), dir (3), dir_00 (3),
// dir_du (3), dir_dv (3), scaledAperture, aspect, pos_00 (3), pos_du (3),
// pos_dv (3). type 0 perspective, 1 orthographic. samples: n x (pixel x,
// pixel y, r0, r1, r2, r3). out: n x (org xyz, dir xyz, screen xy).
extern "C" void camref_primary_rays(const float *cam,
    int type,
    const float *samples,
    int n,
    float invW,
    float invH,
    int centerPixel,
    float *out)
{
  using namespace visrtx;
  CameraGPUData c;
  c.type = type == 0 ? CameraType::PERSPECTIVE : CameraType::ORTHOGRAPHIC;
  c.region = vec4(cam[0], cam[1], cam[2], cam[3]);
  c.pos = vec3(cam[4], cam[5], cam[6]);
  c.dir = vec3(cam[7], cam[8], cam[9]);
  c.up = vec3(0.f);
  c.perspective.dir_00 = vec3(cam[10], cam[11], cam[12]);
  c.perspective.dir_du = vec3(cam[13], cam[14], cam[15]);
  c.perspective.dir_dv = vec3(cam[16], cam[17], cam[18]);
  c.perspective.scaledAperture = cam[19];
  c.perspective.aspect = cam[20];
  c.orthographic.pos_00 = vec3(cam[21], cam[22], cam[23]);
  c.orthographic.pos_du = vec3(cam[24], cam[25], cam[26]);
  c.orthographic.pos_dv = vec3(cam[27], cam[28], cam[29]);
  FrameGPUData frame;
  frame.fb.invSize = vec2(invW, invH);
  frame.camera = &c;
  for (int i = 0; i < n; i++) {
    const float *s = samples + 6 * i;
    ScreenSample ss;
    ss.pixel = glm::uvec2((unsigned)s[0], (unsigned)s[1]);
    ss.screen = vec2(0.f);
    ss.rs.next = {s[2], s[3], s[4], s[5]};
    ss.frameData = &frame;
    const Ray r = makePrimaryRay(ss, centerPixel != 0);
    float *o = out + 8 * i;
    o[0] = r.org.x;
    o[1] = r.org.y;
    o[2] = r.org.z;
    o[3] = r.dir.x;
    o[4] = r.dir.y;
    o[5] = r.dir.z;
    o[6] = ss.screen.x;
    o[7] = ss.screen.y;
  }
}
