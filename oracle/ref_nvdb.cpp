// Test infrastructure: a harness around the NanoVDB library that the
// reference vendors (external/nanovdb, NanoVDB 32.7.0, header-only). It is
// compiled from those headers where they lie into oracle/_ref/libnvdbref.so
// by oracle/build.py, only where the reference tree is present, and is used
// only by the tests and by tests/golden/make_nvdb_golden.py:
//  * nvdbref_build: NanoVDB's own builder (tools::build::Grid +
//    tools::createNanoGrid) turns a dense block into a grid buffer of type
//    Float / Fp4 / Fp8 / Fp16 / FpN, giving golden grid buffers;
//  * nvdbref_sample: samples a buffer exactly as the reference's field
//    sampler does (gpu/sampleSpatialField.h:80-109: worldToIndexF of the
//    location, then a first-order SampleFromVoxels over the grid accessor);
//  * nvdbref_validate: NanoVDB's GridValidator (CheckMode::Full) on a
//    buffer, which pins this library's own grid writer to the format.
#include <nanovdb/GridHandle.h>
#include <nanovdb/HostBuffer.h>
#include <nanovdb/NanoVDB.h>
#include <nanovdb/math/SampleFromVoxels.h>
#include <nanovdb/tools/CreateNanoGrid.h>
#include <nanovdb/tools/GridBuilder.h>
#include <nanovdb/tools/GridValidator.h>

#include <cstdint>
#include <cstring>

namespace {

using SrcGrid = nanovdb::tools::build::Grid<float>;

template <typename BuildT>
nanovdb::GridHandle<> convert(const SrcGrid &g);

template <>
nanovdb::GridHandle<> convert<float>(const SrcGrid &g)
{
  return nanovdb::tools::createNanoGrid<SrcGrid, float>(g);
}

template <typename BuildT>
nanovdb::GridHandle<> convert(const SrcGrid &g)
{
  return nanovdb::tools::createNanoGrid<SrcGrid, BuildT>(g);
}

nanovdb::GridHandle<> hostHandle(const uint8_t *buf, size_t size)
{
  auto hb = nanovdb::HostBuffer::create(size);
  std::memcpy(hb.data(), buf, size);
  return nanovdb::GridHandle<>(std::move(hb));
}

template <typename BuildT>
int sampleAll(const nanovdb::GridHandle<> &h, const float *xyz, int n, float *out)
{
  const auto *grid = h.grid<BuildT>();
  if (!grid)
    return -1;
  const auto acc = grid->getAccessor();
  for (int i = 0; i < n; i++) {
    auto smp = nanovdb::math::createSampler<1>(acc);
    const nanovdb::Vec3d loc(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    out[i] = smp(nanovdb::math::Vec3d(grid->worldToIndexF(loc)));
  }
  return 0;
}

template <typename BuildT>
int validate(const nanovdb::GridHandle<> &h)
{
  const auto *grid = h.grid<BuildT>();
  if (!grid)
    return 0;
  return nanovdb::tools::isValid(grid, nanovdb::CheckMode::Full, false) ? 1 : 0;
}

} // namespace

extern "C" {

// Builds a grid from a dense (nz, ny, nx) block whose voxel (0, 0, 0) sits at
// index (ox, oy, oz): voxels with active[i] != 0 are set (active) to
// dense[i]; the map is a uniform scale plus a translation. Returns the
// buffer size, copying the buffer into `out` when `cap` suffices; 0 on an
// unsupported type.
size_t nvdbref_build(int type,
    const float *dense,
    const uint8_t *active,
    int nx,
    int ny,
    int nz,
    int ox,
    int oy,
    int oz,
    float background,
    double voxelSize,
    const double *translation,
    uint8_t *out,
    size_t cap)
{
  SrcGrid g(background, "density", nanovdb::GridClass::FogVolume);
  g.setTransform(voxelSize, nanovdb::Vec3d(translation[0], translation[1], translation[2]));
  auto acc = g.getAccessor();
  for (int z = 0; z < nz; z++)
    for (int y = 0; y < ny; y++)
      for (int x = 0; x < nx; x++) {
        const size_t i = ((size_t)z * ny + y) * nx + x;
        if (active[i])
          acc.setValue(nanovdb::Coord(ox + x, oy + y, oz + z), dense[i]);
      }
  nanovdb::GridHandle<> h;
  switch (type) {
  case 1:
    h = convert<float>(g);
    break;
  case 13:
    h = convert<nanovdb::Fp4>(g);
    break;
  case 14:
    h = convert<nanovdb::Fp8>(g);
    break;
  case 15:
    h = convert<nanovdb::Fp16>(g);
    break;
  case 16:
    h = convert<nanovdb::FpN>(g);
    break;
  default:
    return 0;
  }
  if (out && cap >= h.size())
    std::memcpy(out, h.data(), h.size());
  return h.size();
}

// Samples n world-space points; returns 0, or -1 for a grid type the
// reference's marcher does not dispatch.
int nvdbref_sample(const uint8_t *buf, size_t size, const float *xyz, int n, float *out)
{
  const auto h = hostHandle(buf, size);
  const auto *md = h.gridMetaData();
  if (!md)
    return -1;
  switch (md->gridType()) {
  case nanovdb::GridType::Float:
    return sampleAll<float>(h, xyz, n, out);
  case nanovdb::GridType::Fp4:
    return sampleAll<nanovdb::Fp4>(h, xyz, n, out);
  case nanovdb::GridType::Fp8:
    return sampleAll<nanovdb::Fp8>(h, xyz, n, out);
  case nanovdb::GridType::Fp16:
    return sampleAll<nanovdb::Fp16>(h, xyz, n, out);
  case nanovdb::GridType::FpN:
    return sampleAll<nanovdb::FpN>(h, xyz, n, out);
  default:
    return -1;
  }
}

// 1 when NanoVDB's full validation accepts the buffer.
int nvdbref_validate(const uint8_t *buf, size_t size)
{
  const auto h = hostHandle(buf, size);
  const auto *md = h.gridMetaData();
  if (!md)
    return 0;
  switch (md->gridType()) {
  case nanovdb::GridType::Float:
    return validate<float>(h);
  case nanovdb::GridType::Fp4:
    return validate<nanovdb::Fp4>(h);
  case nanovdb::GridType::Fp8:
    return validate<nanovdb::Fp8>(h);
  case nanovdb::GridType::Fp16:
    return validate<nanovdb::Fp16>(h);
  case nanovdb::GridType::FpN:
    return validate<nanovdb::FpN>(h);
  default:
    return 0;
  }
}

} // extern "C"
