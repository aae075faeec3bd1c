// Captures, on a GPU, the texture unit's filtering for every texture
// configuration the reference's hot path samples and libvrtx creates, as
// binary records on the file named by argv[1] (read by gen_tex_sweep.py):
//  * 3D single-channel fields, linear and nearest, clamped, normalised
//    coordinates, from float32 and from normalised 8/16-bit integers
//    (sampleSpatialField.h:66-71, StructuredRegularField.cpp:98-159);
//  * the 1D float4 TF table (volumeIntegration.h:53);
//  * float4 image samplers in 1D/2D/3D with clamp, repeat and mirror
//    addressing (sampler/Image*.cpp, utility/CudaImageTexture.cpp);
//  * the HDRI light's float4 map (repeat in x, clamp in y) and the RGBA8
//    background image read as normalised float (HDRI.cu, Renderer.cpp).
// Inputs: axis ramps (texel value = its index on one axis), one-hot
// corners and seeded random texels, sampled at seeded random coordinates
// and at fine sweeps across one texel.
//
// Record: int32 header[16] = {dim, nx, ny, nz, channels, format, filter,
// addr0, addr1, addr2, K, tag, 0, 0, 0, 0}, then the texels as stored
// (nx*ny*nz*channels elements of the format's size), then K*dim float
// coordinates, then K*(channels == 1 ? 1 : 4) float results.
// format: 0 float32, 1 uint8 normalised, 2 uint16 normalised, 3 int8
// normalised, 4 int16 normalised. filter: 0 point, 1 linear. addr:
// cudaTextureAddressMode values.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#define CK(x)                                                                  \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess) {                                                   \
      std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));            \
      std::exit(1);                                                            \
    }                                                                          \
  } while (0)

template <int DIM, typename T>
__global__ void k_fetch(cudaTextureObject_t t, const float *c, int n, float *out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  T v;
  if (DIM == 1)
    v = tex1D<T>(t, c[i]);
  else if (DIM == 2)
    v = tex2D<T>(t, c[2 * i], c[2 * i + 1]);
  else
    v = tex3D<T>(t, c[3 * i], c[3 * i + 1], c[3 * i + 2]);
  if constexpr (sizeof(T) == sizeof(float)) {
    out[i] = *(const float *)&v;
  } else {
    const float4 f = *(const float4 *)&v;
    out[4 * i] = f.x;
    out[4 * i + 1] = f.y;
    out[4 * i + 2] = f.z;
    out[4 * i + 3] = f.w;
  }
}

static unsigned g_seed = 20240611u;
static unsigned lcg()
{
  g_seed = g_seed * 1664525u + 1013904223u;
  return g_seed;
}
static float u01()
{
  return (lcg() >> 8) * (1.0f / 16777216.0f);
}

struct Spec
{
  int dim, n[3], ch, format, filter, addr[3], tag;
};

static size_t elemSize(int format)
{
  return format == 0 ? 4 : (format == 1 || format == 3 ? 1 : 2);
}

static FILE *g_out;

// texels: n0*n1*n2*ch elements of the format (raw bytes); coords: K*dim
static void record(const Spec &s, const std::vector<uint8_t> &texels,
    const std::vector<float> &coords)
{
  const int K = (int)coords.size() / s.dim;
  cudaChannelFormatKind kind = s.format == 0 ? cudaChannelFormatKindFloat
      : (s.format == 1 || s.format == 2)      ? cudaChannelFormatKindUnsigned
                                              : cudaChannelFormatKindSigned;
  const int bits = (int)elemSize(s.format) * 8;
  cudaChannelFormatDesc desc = cudaCreateChannelDesc(bits,
      s.ch > 1 ? bits : 0,
      s.ch > 2 ? bits : 0,
      s.ch > 3 ? bits : 0,
      kind);
  cudaArray_t arr;
  const size_t rowBytes = (size_t)s.n[0] * s.ch * elemSize(s.format);
  if (s.dim == 3) {
    CK(cudaMalloc3DArray(&arr, &desc, make_cudaExtent(s.n[0], s.n[1], s.n[2])));
    cudaMemcpy3DParms cp{};
    cp.srcPtr = make_cudaPitchedPtr((void *)texels.data(), rowBytes, s.n[0], s.n[1]);
    cp.dstArray = arr;
    cp.extent = make_cudaExtent(s.n[0], s.n[1], s.n[2]);
    cp.kind = cudaMemcpyHostToDevice;
    CK(cudaMemcpy3D(&cp));
  } else {
    CK(cudaMallocArray(&arr, &desc, s.n[0], s.dim == 2 ? s.n[1] : 0));
    CK(cudaMemcpy2DToArray(arr, 0, 0, texels.data(), rowBytes, rowBytes,
        s.dim == 2 ? s.n[1] : 1, cudaMemcpyHostToDevice));
  }
  cudaResourceDesc rd{};
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = arr;
  cudaTextureDesc td{};
  for (int k = 0; k < 3; k++)
    td.addressMode[k] = (cudaTextureAddressMode)s.addr[k];
  td.filterMode = s.filter ? cudaFilterModeLinear : cudaFilterModePoint;
  td.readMode = s.format == 0 ? cudaReadModeElementType : cudaReadModeNormalizedFloat;
  td.normalizedCoords = 1;
  cudaTextureObject_t tex;
  CK(cudaCreateTextureObject(&tex, &rd, &td, nullptr));
  const int outC = s.ch == 1 ? 1 : 4;
  float *dC, *dV;
  CK(cudaMalloc(&dC, sizeof(float) * coords.size()));
  CK(cudaMalloc(&dV, sizeof(float) * (size_t)K * outC));
  CK(cudaMemcpy(dC, coords.data(), sizeof(float) * coords.size(), cudaMemcpyHostToDevice));
  const int blocks = (K + 127) / 128;
  if (s.ch == 1) {
    if (s.dim == 1)
      k_fetch<1, float><<<blocks, 128>>>(tex, dC, K, dV);
    else if (s.dim == 2)
      k_fetch<2, float><<<blocks, 128>>>(tex, dC, K, dV);
    else
      k_fetch<3, float><<<blocks, 128>>>(tex, dC, K, dV);
  } else {
    if (s.dim == 1)
      k_fetch<1, float4><<<blocks, 128>>>(tex, dC, K, dV);
    else if (s.dim == 2)
      k_fetch<2, float4><<<blocks, 128>>>(tex, dC, K, dV);
    else
      k_fetch<3, float4><<<blocks, 128>>>(tex, dC, K, dV);
  }
  CK(cudaGetLastError());
  std::vector<float> vals((size_t)K * outC);
  CK(cudaMemcpy(vals.data(), dV, sizeof(float) * vals.size(), cudaMemcpyDeviceToHost));
  CK(cudaDestroyTextureObject(tex));
  CK(cudaFreeArray(arr));
  CK(cudaFree(dC));
  CK(cudaFree(dV));
  int32_t hdr[16] = {s.dim, s.n[0], s.n[1], s.n[2], s.ch, s.format, s.filter,
      s.addr[0], s.addr[1], s.addr[2], K, s.tag, 0, 0, 0, 0};
  std::fwrite(hdr, 4, 16, g_out);
  std::fwrite(texels.data(), 1, texels.size(), g_out);
  std::fwrite(coords.data(), 4, coords.size(), g_out);
  std::fwrite(vals.data(), 4, vals.size(), g_out);
}

static std::vector<uint8_t> floats(const std::vector<float> &v)
{
  std::vector<uint8_t> b(v.size() * 4);
  std::memcpy(b.data(), v.data(), b.size());
  return b;
}

static std::vector<float> randomCoords(int K, int dim, float lo, float hi)
{
  std::vector<float> c((size_t)K * dim);
  for (auto &x : c)
    x = lo + (hi - lo) * u01();
  return c;
}

enum Tag
{
  RAMP = 1,
  ONEHOT = 2,
  RANDOM = 3,
  BOUNDARY = 4
};

int main(int argc, char **argv)
{
  g_out = std::fopen(argc > 1 ? argv[1] : "tex_sweep.bin", "wb");
  if (!g_out)
    return 1;
  const int CL = cudaAddressModeClamp, WR = cudaAddressModeWrap, MI = cudaAddressModeMirror;
  const int K = 1024;

  // 3D float fields: axis ramps (sizes with and without a power of two)
  for (int N : {3, 100, 512})
    for (int axis = 0; axis < 3; axis++) {
      Spec s{3, {2, 2, 2}, 1, 0, 1, {CL, CL, CL}, RAMP};
      s.n[axis] = N;
      std::vector<float> vol((size_t)s.n[0] * s.n[1] * s.n[2]);
      for (int z = 0; z < s.n[2]; z++)
        for (int y = 0; y < s.n[1]; y++)
          for (int x = 0; x < s.n[0]; x++) {
            const int idx[3] = {x, y, z};
            vol[((size_t)z * s.n[1] + y) * s.n[0] + x] = (float)idx[axis];
          }
      std::vector<float> c(3 * K, 0.5f);
      const int cell = N / 2 - 1;
      for (int k = 0; k < K; k++)
        c[3 * k + axis] = k < K / 2
            ? u01()
            : ((float)cell + 0.5f + (float)(k - K / 2) / (float)(K / 2)) / (float)N;
      record(s, floats(vol), c);
    }
  // 3D one-hot corners of a 2x2x2 texture
  {
    const std::vector<float> c = randomCoords(K, 3, -0.1f, 1.1f);
    for (int q = 0; q < 8; q++) {
      std::vector<float> vol(8, 0.f);
      vol[q] = 1.f;
      record(Spec{3, {2, 2, 2}, 1, 0, 1, {CL, CL, CL}, ONEHOT}, floats(vol), c);
    }
  }
  // 3D random float fields, linear and nearest
  for (int filter : {1, 0}) {
    std::vector<float> vol(8 * 7 * 6);
    for (auto &v : vol)
      v = u01() * 2.f - 0.5f;
    record(Spec{3, {8, 7, 6}, 1, 0, filter, {CL, CL, CL}, RANDOM}, floats(vol),
        randomCoords(4 * K, 3, -0.1f, 1.1f));
  }
  // nearest: coordinates within a few ulps of texel boundaries
  {
    std::vector<float> vol(8 * 7 * 6);
    for (auto &v : vol)
      v = u01();
    const int n[3] = {8, 7, 6};
    std::vector<float> c(3 * K);
    for (int k = 0; k < K; k++)
      for (int a = 0; a < 3; a++) {
        const int edge = (int)(lcg() % (unsigned)(n[a] + 1));
        const float e = ((float)(int)(lcg() % 65u) - 32.f) * 1.2e-7f;
        c[3 * k + a] = (float)edge / (float)n[a] + e;
      }
    record(Spec{3, {8, 7, 6}, 1, 0, 0, {CL, CL, CL}, BOUNDARY}, floats(vol), c);
  }
  // 3D normalised-integer fields (UFIXED8/16, FIXED8/16), linear and nearest
  for (int format : {1, 2, 3, 4})
    for (int filter : {1, 0}) {
      const int n = 6 * 5 * 4;
      std::vector<uint8_t> raw(n * elemSize(format));
      for (auto &b : raw)
        b = (uint8_t)(lcg() >> 24);
      record(Spec{3, {6, 5, 4}, 1, format, filter, {CL, CL, CL}, RANDOM}, raw,
          randomCoords(K, 3, -0.1f, 1.1f));
    }
  // 1D float4 tables: clamp (the TF), repeat, mirror; linear and nearest
  for (int addr : {CL, WR, MI})
    for (int filter : {1, 0}) {
      std::vector<float> t(4 * 13);
      for (auto &v : t)
        v = u01();
      record(Spec{1, {13, 1, 1}, 4, 0, filter, {addr, addr, addr}, RANDOM}, floats(t),
          randomCoords(K, 1, addr == CL ? -0.1f : -2.f, addr == CL ? 1.1f : 2.f));
    }
  {
    std::vector<float> t(4 * 256);
    for (auto &v : t)
      v = u01();
    record(Spec{1, {256, 1, 1}, 4, 0, 1, {CL, CL, CL}, RANDOM}, floats(t),
        randomCoords(K, 1, -0.05f, 1.05f));
  }
  // 2D float4: ramps, one-hot corners, random tables per address mode
  for (int N : {3, 100})
    for (int axis = 0; axis < 2; axis++) {
      Spec s{2, {2, 2, 1}, 4, 0, 1, {CL, CL, CL}, RAMP};
      s.n[axis] = N;
      std::vector<float> t((size_t)4 * s.n[0] * s.n[1]);
      for (int y = 0; y < s.n[1]; y++)
        for (int x = 0; x < s.n[0]; x++)
          for (int c = 0; c < 4; c++)
            t[4 * (y * s.n[0] + x) + c] = (float)(axis ? y : x);
      std::vector<float> c(2 * K, 0.5f);
      const int cell = N / 2 - 1;
      for (int k = 0; k < K; k++)
        c[2 * k + axis] = k < K / 2
            ? u01()
            : ((float)cell + 0.5f + (float)(k - K / 2) / (float)(K / 2)) / (float)N;
      record(s, floats(t), c);
    }
  {
    const std::vector<float> c = randomCoords(K, 2, -0.1f, 1.1f);
    for (int q = 0; q < 4; q++) {
      std::vector<float> t(16, 0.f);
      for (int c4 = 0; c4 < 4; c4++)
        t[4 * q + c4] = 1.f;
      record(Spec{2, {2, 2, 1}, 4, 0, 1, {CL, CL, CL}, ONEHOT}, floats(t), c);
    }
  }
  for (int addr : {CL, WR, MI})
    for (int filter : {1, 0}) {
      std::vector<float> t(4 * 7 * 5);
      for (auto &v : t)
        v = u01() * 2.f - 0.5f;
      record(Spec{2, {7, 5, 1}, 4, 0, filter, {addr, addr, addr}, RANDOM}, floats(t),
          randomCoords(K, 2, addr == CL ? -0.1f : -2.f, addr == CL ? 1.1f : 2.f));
    }
  // HDRI map: repeat in x, clamp in y
  {
    std::vector<float> t(4 * 16 * 8);
    for (auto &v : t)
      v = u01() * 4.f;
    record(Spec{2, {16, 8, 1}, 4, 0, 1, {WR, CL, CL}, RANDOM}, floats(t),
        randomCoords(K, 2, -0.5f, 1.5f));
  }
  // RGBA8 background image, normalised float read
  {
    std::vector<uint8_t> t(4 * 9 * 7);
    for (auto &b : t)
      b = (uint8_t)(lcg() >> 24);
    record(Spec{2, {9, 7, 1}, 4, 1, 1, {CL, CL, CL}, RANDOM}, t,
        randomCoords(K, 2, -0.1f, 1.1f));
  }
  // 3D float4 image samplers per address mode
  for (int addr : {CL, WR, MI})
    for (int filter : {1, 0}) {
      std::vector<float> t(4 * 5 * 4 * 3);
      for (auto &v : t)
        v = u01();
      record(Spec{3, {5, 4, 3}, 4, 0, filter, {addr, addr, addr}, RANDOM}, floats(t),
          randomCoords(K, 3, addr == CL ? -0.1f : -2.f, addr == CL ? 1.1f : 2.f));
    }
  std::fclose(g_out);
  CK(cudaDeviceSynchronize());
  std::printf("ok\n");
  return 0;
}
