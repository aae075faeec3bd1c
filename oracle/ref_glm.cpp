// Test infrastructure: the reference's output colour encoding
// (gpu/gpu_util.h:370-389, writeOutputColor: the accumulation divided by the
// sample count, inverse-tonemapped, then glm::packUnorm4x8 of
// glm::convertLinearToSRGB for sRGB frames, of the colour itself for UINT
// frames), with the two glm calls taken from the glm the reference vendors
// (external/glm, header-only), compiled where it lies into
// oracle/_ref/libglmref.so by oracle/build.py, only where the reference tree
// is present, and used only by tests/golden/make_color_golden.py. The
// tonemap arithmetic of gpu_util.h:324-334 is restated (that header needs
// OptiX); the conversions are glm's own code.
#include <glm/gtc/color_space.hpp>
#include <glm/packing.hpp>
#include <glm/vec4.hpp>

#include <algorithm>
#include <cstdint>

extern "C" void glmref_write_color(
    const float *accum, int n, int frameID, int format, uint32_t *out)
{
  for (int i = 0; i < n; i++) {
    glm::vec4 v(accum[4 * i], accum[4 * i + 1], accum[4 * i + 2], accum[4 * i + 3]);
    v = v / float(frameID + 1);
    const float m = std::max(v.x, std::max(v.y, v.z));
    const glm::vec3 rgb = glm::vec3(v) / std::max(1e-12f, 1.f - m);
    const glm::vec4 c(rgb, v.w);
    out[i] = format == 0 ? glm::packUnorm4x8(glm::convertLinearToSRGB(c))
                         : glm::packUnorm4x8(c);
  }
}
