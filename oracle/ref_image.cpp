// Test infrastructure: a harness around the reference's own image staging
// (devices/rtx/utility/CudaImageTexture.cpp:43-111, convertComponentUint8 /
// convertComponentFloat and transformToStagingBufferUint8 / Float: how an
// image sampler's image, and the renderer's background image, become the
// texels of a CUDA array), compiled unchanged into oracle/_ref/libimgref.so
// by oracle/build.py, only where the reference tree is present, and used
// only by tests/golden/make_image_golden.py.
//
// The .cpp includes its header CudaImageTexture.h, which needs the
// ANARI-SDK's helium; oracle/build.py compiles this file through
// oracle/_ref/gpu_inc/, where utility/ holds links to the reference's
// CudaImageTexture.cpp and AnariTypeHelpers.h beside a link to
// oracle/ref_shim/CudaImageTexture.h (an array of host bytes), and
// oracle/ref_shim/anari/anari.h names the data types. The staging
// functions are file-local (static) in the .cpp, so this file includes it.
// Its other functions (CUDA array and texture creation) compile but are
// never called: there is no GPU here.
#include "utility/CudaImageTexture.cpp"

namespace {

using namespace visrtx;

// kind: 0 float32, 1 ufixed8, 2 ufixed16, 3 ufixed32, 4 ufixed8 sRGB
template <int NC>
int stageUint8(int kind, const void *data, size_t count, uint8_t *out)
{
  const ANARIDataType t = ANARI_UINT8; // element type: unused by the staging
  const Array a(t, data, count);
  switch (kind) {
  case 0:
    transformToStagingBufferUint8<NC, float>(a, out);
    return 0;
  case 1:
    transformToStagingBufferUint8<NC, uint8_t>(a, out);
    return 0;
  case 2:
    transformToStagingBufferUint8<NC, uint16_t>(a, out);
    return 0;
  case 3:
    transformToStagingBufferUint8<NC, uint32_t>(a, out);
    return 0;
  case 4:
    transformToStagingBufferUint8<NC, uint8_t, true>(a, out);
    return 0;
  default:
    return -1;
  }
}

template <int NC>
int stageFloat(int kind, const void *data, size_t count, float *out)
{
  const Array a(ANARI_FLOAT32, data, count);
  switch (kind) {
  case 0:
    transformToStagingBufferFloat<NC, float>(a, out);
    return 0;
  case 1:
    transformToStagingBufferFloat<NC, uint8_t>(a, out);
    return 0;
  case 2:
    transformToStagingBufferFloat<NC, uint16_t>(a, out);
    return 0;
  case 3:
    transformToStagingBufferFloat<NC, uint32_t>(a, out);
    return 0;
  case 4:
    transformToStagingBufferFloat<NC, uint8_t, true>(a, out);
    return 0;
  default:
    return -1;
  }
}

} // namespace

// The 8-bit staging of `count` texels of nc components of the given kind
// into out (count * nc bytes; count * 4 for nc = 3, alpha 255 added).
extern "C" int imgref_stage_uint8(
    int kind, int nc, const void *data, size_t count, uint8_t *out)
{
  switch (nc) {
  case 1:
    return stageUint8<1>(kind, data, count, out);
  case 2:
    return stageUint8<2>(kind, data, count, out);
  case 3:
    return stageUint8<3>(kind, data, count, out);
  case 4:
    return stageUint8<4>(kind, data, count, out);
  default:
    return -1;
  }
}

// The float staging, laid out as the 8-bit one (alpha 1 added for nc = 3).
extern "C" int imgref_stage_float(
    int kind, int nc, const void *data, size_t count, float *out)
{
  switch (nc) {
  case 1:
    return stageFloat<1>(kind, data, count, out);
  case 2:
    return stageFloat<2>(kind, data, count, out);
  case 3:
    return stageFloat<3>(kind, data, count, out);
  case 4:
    return stageFloat<4>(kind, data, count, out);
  default:
    return -1;
  }
}

// The reference's choice of staging for an image sampler's image
// (scene/surface/material/sampler/Image2D.cpp:70-78 and its 1D / 3D
// siblings: float element types as float, every other as 8-bit read as
// normalised float), by its own isFloat test: 1 for float staging.
extern "C" int imgref_sampler_uses_float(int kind)
{
  static const ANARIDataType types[5] = {ANARI_FLOAT32_VEC4,
      ANARI_UFIXED8_VEC4,
      ANARI_UFIXED16,
      ANARI_UFIXED32,
      ANARI_UFIXED8_RGBA_SRGB};
  return kind >= 0 && kind < 5 && isFloat(types[kind]) ? 1 : 0;
}
