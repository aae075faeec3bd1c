// Test infrastructure: a host stand-in for the reference's
// devices/rtx/utility/CudaImageTexture.h, whose array/Array.h needs the
// ANARI-SDK's helium library (not present here). oracle/build.py links it
// beside the reference's own CudaImageTexture.cpp only when it compiles
// oracle/ref_image.cpp. It declares what that .cpp uses: CUDA's runtime
// types, glm's sRGB conversion, the vector names of gpu/gpu_math.h, an
// image array that hands out its element type, element count and host
// bytes, the standard headers the real header brings in through helium
// (<algorithm>, <vector>), and the prototypes of the .cpp's staging
// functions, which it calls before it defines them.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cassert>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include <glm/gtc/color_space.hpp>

#include "gpu/gpu_math.h"
#include "utility/AnariTypeHelpers.h"

namespace visrtx {

class Array
{
 public:
  Array(ANARIDataType type, const void *data, size_t count)
      : m_type(type), m_data(data), m_count(count)
  {}
  ANARIDataType elementType() const
  {
    return m_type;
  }
  size_t totalSize() const
  {
    return m_count;
  }
  const void *data() const
  {
    return m_data;
  }

 private:
  ANARIDataType m_type;
  const void *m_data;
  size_t m_count;
};

int countCudaChannels(const cudaChannelFormatDesc &desc);
cudaTextureAddressMode stringToAddressMode(const std::string &str);
void makeCudaArrayUint8(cudaArray_t &cuArray, const Array &array, uvec2 size);
void makeCudaArrayFloat(cudaArray_t &cuArray, const Array &array, uvec2 size);
void makeCudaArrayUint8(cudaArray_t &cuArray, const Array &array, uvec3 size);
void makeCudaArrayFloat(cudaArray_t &cuArray, const Array &array, uvec3 size);
void makeCudaCompressedTextureArray(cudaArray_t &cuArray,
    const uvec2 &size,
    const Array &array,
    const cudaChannelFormatKind channelFormatKind);

} // namespace visrtx
