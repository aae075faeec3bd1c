// Test infrastructure: a host stand-in for the ANARI-SDK's <anari/anari.h>
// (not present here), put on the include path only when oracle/build.py
// compiles oracle/ref_image.cpp. It declares the data-type names that the
// reference's utility/AnariTypeHelpers.h and utility/CudaImageTexture.cpp
// switch on, with distinct values local to that harness (the harness picks
// its staging by these names, never by a number from outside it).
#pragma once

typedef int ANARIDataType;

enum : int
{
  ANARI_INT8 = 1,
  ANARI_UINT8,
  ANARI_UFIXED8,
  ANARI_UFIXED8_VEC2,
  ANARI_UFIXED8_VEC3,
  ANARI_UFIXED8_VEC4,
  ANARI_UFIXED8_R_SRGB,
  ANARI_UFIXED8_RA_SRGB,
  ANARI_UFIXED8_RGB_SRGB,
  ANARI_UFIXED8_RGBA_SRGB,
  ANARI_UFIXED16,
  ANARI_UFIXED16_VEC2,
  ANARI_UFIXED16_VEC3,
  ANARI_UFIXED16_VEC4,
  ANARI_UFIXED32,
  ANARI_UFIXED32_VEC2,
  ANARI_UFIXED32_VEC3,
  ANARI_UFIXED32_VEC4,
  ANARI_FLOAT16,
  ANARI_FLOAT16_VEC2,
  ANARI_FLOAT16_VEC3,
  ANARI_FLOAT16_VEC4,
  ANARI_FLOAT32,
  ANARI_FLOAT32_VEC2,
  ANARI_FLOAT32_VEC3,
  ANARI_FLOAT32_VEC4,
  ANARI_FLOAT64,
  ANARI_FLOAT64_VEC2,
  ANARI_FLOAT64_VEC3,
  ANARI_FLOAT64_VEC4
};
