// Captures, on a GPU, the third-party arithmetic the reference's hot path
// stands on, as JSON on stdout (read by gen_cuda_fixtures.py):
//  * curand Philox4_32_10 streams: curand_init(seed, subsequence, offset)
//    followed by curand(), curand_uniform() or curand_uniform4() draws
//    (gpu/createScreenSample.h:58, cameraCreateRay.h:76, gpu_util.h:199);
//  * hardware linear filtering of a clamped, normalised-coordinate 3D float
//    texture and a 1D float4 texture (sampleSpatialField.h:70,
//    volumeIntegration.h:53).
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include <cstdio>
#include <vector>

struct Case
{
  unsigned long long seed, subsequence, offset;
  int kind;
};

__global__ void k_draws(const Case *cases, int n, int per, unsigned *out)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n)
    return;
  curandStatePhilox4_32_10_t s;
  curand_init(cases[c].seed, cases[c].subsequence, cases[c].offset, &s);
  unsigned *o = out + (size_t)c * per;
  if (cases[c].kind == 0) {
    for (int i = 0; i < per; i++)
      o[i] = curand(&s);
  } else if (cases[c].kind == 1) {
    for (int i = 0; i < per; i++)
      o[i] = __float_as_uint(curand_uniform(&s));
  } else {
    for (int i = 0; i + 3 < per; i += 4) {
      const float4 r = curand_uniform4(&s);
      o[i] = __float_as_uint(r.x);
      o[i + 1] = __float_as_uint(r.y);
      o[i + 2] = __float_as_uint(r.z);
      o[i + 3] = __float_as_uint(r.w);
    }
  }
}

__global__ void k_tex3(cudaTextureObject_t t, const float *coords, int n, float *out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    out[i] = tex3D<float>(t, coords[3 * i], coords[3 * i + 1], coords[3 * i + 2]);
}

__global__ void k_tex1(cudaTextureObject_t t, const float *coords, int n, float4 *out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    out[i] = tex1D<float4>(t, coords[i]);
}

static unsigned lcg(unsigned &s)
{
  s = s * 1664525u + 1013904223u;
  return s;
}

static float u01(unsigned &s)
{
  return (lcg(s) >> 8) * (1.0f / 16777216.0f);
}

int main()
{
  // --- curand --------------------------------------------------------------
  std::vector<Case> cases;
  const unsigned long long seeds[] = {0ull, 1ull, 12345ull, 196607ull, 0x123456789abcull};
  const unsigned long long offsets[] = {0ull, 1ull, 3ull, 512ull, 4096ull * 512ull + 68ull};
  for (unsigned long long sd : seeds)
    for (unsigned long long off : offsets)
      for (int kind = 0; kind < 3; kind++)
        cases.push_back(Case{sd, sd == 1ull ? 7ull : 0ull, off, kind});
  const int per = 16;
  Case *dCases;
  unsigned *dOut;
  cudaMalloc(&dCases, sizeof(Case) * cases.size());
  cudaMalloc(&dOut, sizeof(unsigned) * per * cases.size());
  cudaMemcpy(dCases, cases.data(), sizeof(Case) * cases.size(), cudaMemcpyHostToDevice);
  k_draws<<<(int)(cases.size() + 63) / 64, 64>>>(dCases, (int)cases.size(), per, dOut);
  std::vector<unsigned> draws(per * cases.size());
  cudaMemcpy(draws.data(), dOut, sizeof(unsigned) * draws.size(), cudaMemcpyDeviceToHost);

  // --- 3D texture --------------------------------------------------------------
  const int nx = 8, ny = 7, nz = 6;
  unsigned s = 2024u;
  std::vector<float> vol(nx * ny * nz);
  for (auto &v : vol)
    v = u01(s) * 2.f - 0.5f;
  cudaArray_t arr;
  cudaChannelFormatDesc desc = cudaCreateChannelDesc<float>();
  cudaMalloc3DArray(&arr, &desc, make_cudaExtent(nx, ny, nz));
  cudaMemcpy3DParms cp{};
  cp.srcPtr = make_cudaPitchedPtr(vol.data(), nx * sizeof(float), nx, ny);
  cp.dstArray = arr;
  cp.extent = make_cudaExtent(nx, ny, nz);
  cp.kind = cudaMemcpyHostToDevice;
  cudaMemcpy3D(&cp);
  cudaResourceDesc rd{};
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = arr;
  cudaTextureDesc td{};
  td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
  td.filterMode = cudaFilterModeLinear;
  td.readMode = cudaReadModeElementType;
  td.normalizedCoords = 1;
  cudaTextureObject_t tex3;
  cudaCreateTextureObject(&tex3, &rd, &td, nullptr);
  const int nc = 400;
  std::vector<float> coords(3 * nc);
  for (auto &c : coords)
    c = u01(s) * 1.2f - 0.1f;
  float *dC, *dV;
  cudaMalloc(&dC, sizeof(float) * coords.size());
  cudaMalloc(&dV, sizeof(float) * nc);
  cudaMemcpy(dC, coords.data(), sizeof(float) * coords.size(), cudaMemcpyHostToDevice);
  k_tex3<<<(nc + 127) / 128, 128>>>(tex3, dC, nc, dV);
  std::vector<float> vals(nc);
  cudaMemcpy(vals.data(), dV, sizeof(float) * nc, cudaMemcpyDeviceToHost);

  // --- 1D float4 texture (a 256-entry TF) -------------------------------------
  const int nt = 256;
  std::vector<float> table(4 * nt);
  for (auto &v : table)
    v = u01(s);
  cudaArray_t arr1;
  cudaChannelFormatDesc d4 = cudaCreateChannelDesc<float4>();
  cudaMallocArray(&arr1, &d4, nt);
  cudaMemcpy2DToArray(arr1, 0, 0, table.data(), nt * 16, nt * 16, 1, cudaMemcpyHostToDevice);
  cudaResourceDesc rd1{};
  rd1.resType = cudaResourceTypeArray;
  rd1.res.array.array = arr1;
  cudaTextureDesc td1{};
  td1.addressMode[0] = cudaAddressModeClamp;
  td1.filterMode = cudaFilterModeLinear;
  td1.readMode = cudaReadModeElementType;
  td1.normalizedCoords = 1;
  cudaTextureObject_t tex1;
  cudaCreateTextureObject(&tex1, &rd1, &td1, nullptr);
  const int n1 = 300;
  std::vector<float> c1(n1);
  for (auto &c : c1)
    c = u01(s) * 1.1f - 0.05f;
  float *dC1;
  float4 *dV1;
  cudaMalloc(&dC1, sizeof(float) * n1);
  cudaMalloc(&dV1, sizeof(float4) * n1);
  cudaMemcpy(dC1, c1.data(), sizeof(float) * n1, cudaMemcpyHostToDevice);
  k_tex1<<<(n1 + 127) / 128, 128>>>(tex1, dC1, n1, dV1);
  std::vector<float> v1(4 * n1);
  cudaMemcpy(v1.data(), dV1, sizeof(float4) * n1, cudaMemcpyDeviceToHost);
  if (cudaDeviceSynchronize() != cudaSuccess) {
    std::fprintf(stderr, "CUDA error: %s\n", cudaGetErrorString(cudaGetLastError()));
    return 1;
  }

  // --- JSON ---------------------------------------------------------------------
  std::printf("{\"curand\": [");
  for (size_t c = 0; c < cases.size(); c++) {
    std::printf("%s{\"seed\": %llu, \"subsequence\": %llu, \"offset\": %llu, \"kind\": %d, "
                "\"bits\": [",
        c ? ", " : "",
        cases[c].seed,
        cases[c].subsequence,
        cases[c].offset,
        cases[c].kind);
    for (int i = 0; i < per; i++)
      std::printf("%s%u", i ? ", " : "", draws[c * per + i]);
    std::printf("]}");
  }
  std::printf("], \"tex3\": {\"dims\": [%d, %d, %d], \"volume\": [", nx, ny, nz);
  for (size_t i = 0; i < vol.size(); i++)
    std::printf("%s%.9g", i ? ", " : "", vol[i]);
  std::printf("], \"coords\": [");
  for (int i = 0; i < nc; i++)
    std::printf("%s[%.9g, %.9g, %.9g]", i ? ", " : "", coords[3 * i], coords[3 * i + 1],
        coords[3 * i + 2]);
  std::printf("], \"values\": [");
  for (int i = 0; i < nc; i++)
    std::printf("%s%.9g", i ? ", " : "", vals[i]);
  std::printf("]}, \"tex1\": {\"table\": [");
  for (size_t i = 0; i < table.size(); i++)
    std::printf("%s%.9g", i ? ", " : "", table[i]);
  std::printf("], \"coords\": [");
  for (int i = 0; i < n1; i++)
    std::printf("%s%.9g", i ? ", " : "", c1[i]);
  std::printf("], \"values\": [");
  for (int i = 0; i < 4 * n1; i++)
    std::printf("%s%.9g", i ? ", " : "", v1[i]);
  std::printf("]}}\n");
  return 0;
}
