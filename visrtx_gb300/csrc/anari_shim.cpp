// The ANARI C API and VisRTX's exported functions (include/anari_visrtx.h)
// over the vrtx* C ABI (include/vrtx.h). An ANARIDevice is the library's
// device handle and every other ANARI handle is its object handle; what is
// here is translation: ANARI type codes to and from the library's own, the
// status reports of devices made here (ANARI source types and severities),
// the device taking parameters and properties as an object, and parameter
// arrays mapped in place. No rendering state lives here.
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <utility>

#include "../../include/anari_visrtx.h"
#include "../../include/vrtx.h"

namespace vrtx {
// device.cpp: makes a device report status with translated codes (kind 0:
// the source's object type, kind 1: the severity)
void setReportCodes(VRTXDevice d, int (*map)(int kind, int value));
} // namespace vrtx

namespace {

// parameter arrays handed out by anariMapParameterArray*, per (device,
// object, parameter name)
std::mutex g_mapMutex;
std::map<std::tuple<ANARIDevice, ANARIObject, std::string>, VRTXArray> g_mapped;

struct ShimLibrary
{
  ANARIStatusCallback cb = nullptr;
  const void *cbUser = nullptr;
};

VRTXDevice VD(ANARIDevice d)
{
  return reinterpret_cast<VRTXDevice>(d);
}

VRTXObject VO(ANARIObject o)
{
  return reinterpret_cast<VRTXObject>(o);
}

ANARIObject AO(VRTXObject o)
{
  return reinterpret_cast<ANARIObject>(o);
}

// ANARI type code <-> the library's (pairs of the two type tables)
const int kTypes[][2] = {
    {ANARI_UNKNOWN, VRTX_UNKNOWN},
    {ANARI_DATA_TYPE, VRTX_DATA_TYPE},
    {ANARI_STRING, VRTX_STRING},
    {ANARI_VOID_POINTER, VRTX_VOID_POINTER},
    {ANARI_BOOL, VRTX_BOOL},
    {ANARI_STRING_LIST, VRTX_STRING_LIST},
    {ANARI_FUNCTION_POINTER, VRTX_FUNCTION_POINTER},
    {ANARI_MEMORY_DELETER, VRTX_MEMORY_DELETER},
    {ANARI_DEVICE, VRTX_DEVICE},
    {ANARI_OBJECT, VRTX_OBJECT},
    {ANARI_ARRAY, VRTX_OBJECT},
    {ANARI_ARRAY1D, VRTX_ARRAY1D},
    {ANARI_ARRAY2D, VRTX_ARRAY2D},
    {ANARI_ARRAY3D, VRTX_ARRAY3D},
    {ANARI_CAMERA, VRTX_CAMERA},
    {ANARI_FRAME, VRTX_FRAME},
    {ANARI_GEOMETRY, VRTX_GEOMETRY},
    {ANARI_GROUP, VRTX_GROUP},
    {ANARI_INSTANCE, VRTX_INSTANCE},
    {ANARI_LIGHT, VRTX_LIGHT},
    {ANARI_MATERIAL, VRTX_MATERIAL},
    {ANARI_RENDERER, VRTX_RENDERER},
    {ANARI_SURFACE, VRTX_SURFACE},
    {ANARI_SAMPLER, VRTX_SAMPLER},
    {ANARI_SPATIAL_FIELD, VRTX_SPATIAL_FIELD},
    {ANARI_VOLUME, VRTX_VOLUME},
    {ANARI_WORLD, VRTX_WORLD},
    {ANARI_INT8, VRTX_INT8},
    {ANARI_UINT8, VRTX_UINT8},
    {ANARI_INT32, VRTX_INT32},
    {ANARI_INT32_VEC2, VRTX_INT32_VEC2},
    {ANARI_UINT32, VRTX_UINT32},
    {ANARI_UINT32_VEC2, VRTX_UINT32_VEC2},
    {ANARI_UINT32_VEC3, VRTX_UINT32_VEC3},
    {ANARI_UINT32_VEC4, VRTX_UINT32_VEC4},
    {ANARI_UINT64, VRTX_UINT64},
    {ANARI_FIXED8, VRTX_FIXED8},
    {ANARI_UFIXED8, VRTX_UFIXED8},
    {ANARI_UFIXED8_VEC4, VRTX_UFIXED8_VEC4},
    {ANARI_FIXED16, VRTX_FIXED16},
    {ANARI_UFIXED16, VRTX_UFIXED16},
    {ANARI_FLOAT16, VRTX_FLOAT16},
    {ANARI_FLOAT32, VRTX_FLOAT32},
    {ANARI_FLOAT32_VEC2, VRTX_FLOAT32_VEC2},
    {ANARI_FLOAT32_VEC3, VRTX_FLOAT32_VEC3},
    {ANARI_FLOAT32_VEC4, VRTX_FLOAT32_VEC4},
    {ANARI_FLOAT64, VRTX_FLOAT64},
    {ANARI_UFIXED8_RGBA_SRGB, VRTX_UFIXED8_RGBA_SRGB},
    {ANARI_FLOAT32_BOX1, VRTX_FLOAT32_BOX1},
    {ANARI_FLOAT32_BOX2, VRTX_FLOAT32_BOX2},
    {ANARI_FLOAT32_BOX3, VRTX_FLOAT32_BOX3},
    {ANARI_FLOAT64_BOX1, VRTX_FLOAT64_BOX1},
    {ANARI_FLOAT32_MAT4, VRTX_FLOAT32_MAT4},
    {ANARI_FLOAT32_MAT3x4, VRTX_FLOAT32_MAT3x4},
};

int toVrtx(int a)
{
  for (const auto &p : kTypes)
    if (p[0] == a)
      return p[1];
  return -1;
}

int toAnari(int v)
{
  for (const auto &p : kTypes)
    if (p[1] == v && p[0] != ANARI_ARRAY)
      return p[0];
  return ANARI_UNKNOWN;
}

// the device's status reports in ANARI codes: source type and severity
int reportCode(int kind, int v)
{
  return kind == 0 ? toAnari(v) : v + 1;
}

ANARIDevice newDevice(ANARIStatusCallback cb, const void *user)
{
  VRTXDevice d = vrtxNewDevice(reinterpret_cast<VRTXStatusCallback>(cb), user);
  if (d)
    vrtx::setReportCodes(d, reportCode);
  return reinterpret_cast<ANARIDevice>(d);
}

bool isDevice(ANARIDevice d, ANARIObject o)
{
  return reinterpret_cast<void *>(d) == reinterpret_cast<void *>(o);
}

const char *const kDeviceSubtypes[] = {"visrtx", "default", nullptr};

VRTXArray newArray(ANARIDevice device,
    int dims,
    const void *mem,
    ANARIMemoryDeleter deleter,
    const void *user,
    ANARIDataType type,
    uint64_t n1,
    uint64_t n2,
    uint64_t n3)
{
  if (!device)
    return nullptr;
  const int t = toVrtx(type);
  VRTXDevice d = VD(device);
  auto del = reinterpret_cast<VRTXMemoryDeleter>(deleter);
  if (dims == 1)
    return vrtxNewArray1D(d, mem, del, user, t, n1);
  if (dims == 2)
    return vrtxNewArray2D(d, mem, del, user, t, n1, n2);
  return vrtxNewArray3D(d, mem, del, user, t, n1, n2, n3);
}

void *mapParameterArray(ANARIDevice device,
    ANARIObject object,
    const char *name,
    ANARIDataType type,
    int dims,
    uint64_t n1,
    uint64_t n2,
    uint64_t n3,
    uint64_t *stride)
{
  if (!device || !object || !name)
    return nullptr;
  VRTXDevice d = VD(device);
  VRTXArray a = newArray(device, dims, nullptr, nullptr, nullptr, type, n1, n2, n3);
  if (!a)
    return nullptr;
  vrtxSetParameter(d, VO(object), name, dims == 1 ? VRTX_ARRAY1D
          : dims == 2                                  ? VRTX_ARRAY2D
                                                       : VRTX_ARRAY3D,
      &a);
  void *p = vrtxMapArray(d, a);
  if (stride) {
    uint64_t bytes = 0;
    switch (toVrtx(type)) {
    case VRTX_UINT8:
    case VRTX_INT8:
    case VRTX_UFIXED8:
    case VRTX_FIXED8:
      bytes = 1;
      break;
    case VRTX_FLOAT16:
    case VRTX_UFIXED16:
    case VRTX_FIXED16:
      bytes = 2;
      break;
    case VRTX_FLOAT32:
    case VRTX_UINT32:
    case VRTX_INT32:
    case VRTX_UFIXED8_VEC4:
    case VRTX_UFIXED8_RGBA_SRGB:
      bytes = 4;
      break;
    case VRTX_FLOAT32_VEC2:
    case VRTX_UINT32_VEC2:
    case VRTX_INT32_VEC2:
    case VRTX_FLOAT64:
    case VRTX_UINT64:
      bytes = 8;
      break;
    case VRTX_FLOAT32_VEC3:
    case VRTX_UINT32_VEC3:
      bytes = 12;
      break;
    case VRTX_FLOAT32_VEC4:
    case VRTX_UINT32_VEC4:
      bytes = 16;
      break;
    case VRTX_FLOAT32_MAT4:
      bytes = 64;
      break;
    default:
      bytes = sizeof(void *);
      break;
    }
    *stride = bytes;
  }
  std::lock_guard<std::mutex> lock(g_mapMutex);
  const auto key = std::make_tuple(device, object, std::string(name));
  auto it = g_mapped.find(key);
  if (it != g_mapped.end()) {
    vrtxUnmapArray(d, it->second);
    vrtxRelease(d, it->second);
  }
  g_mapped[key] = a;
  return p;
}

template <typename F>
VRTXObject byType(ANARIDevice device, F f)
{
  return device ? f(VD(device)) : nullptr;
}

} // namespace

extern "C" {

// --- VisRTX's exported functions ---------------------------------------------

ANARI_SHIM_API ANARIDevice makeVisRTXDevice(ANARIStatusCallback cb, const void *user)
{
  return newDevice(cb, user);
}

ANARI_SHIM_API int visrtxGetObjectExtensions(
    VisRTXExtensions *ext, ANARIDevice device, ANARIDataType objectType, const char *subtype)
{
  if (!device)
    return 0;
  return vrtxGetObjectExtensions(reinterpret_cast<VRTXExtensions *>(ext),
      VD(device),
      toVrtx(objectType),
      subtype);
}

ANARI_SHIM_API int visrtxGetInstanceExtensions(
    VisRTXExtensions *ext, ANARIDevice device, ANARIObject object)
{
  if (!device)
    return 0;
  return vrtxGetInstanceExtensions(reinterpret_cast<VRTXExtensions *>(ext),
      VD(device),
      isDevice(device, object) ? nullptr : VO(object));
}

// --- library and device --------------------------------------------------------

ANARI_SHIM_API ANARILibrary anariLoadLibrary(
    const char *name, ANARIStatusCallback cb, const void *user)
{
  if (name && std::strcmp(name, "visrtx") != 0 && std::strcmp(name, "default") != 0
      && std::strcmp(name, "environment") != 0)
    return nullptr;
  auto *lib = new (std::nothrow) ShimLibrary();
  if (!lib)
    return nullptr;
  lib->cb = cb;
  lib->cbUser = user;
  return reinterpret_cast<ANARILibrary>(lib);
}

ANARI_SHIM_API void anariUnloadLibrary(ANARILibrary library)
{
  delete reinterpret_cast<ShimLibrary *>(library);
}

ANARI_SHIM_API const char **anariGetDeviceSubtypes(ANARILibrary)
{
  return const_cast<const char **>(kDeviceSubtypes);
}

ANARI_SHIM_API ANARIDevice anariNewDevice(ANARILibrary library, const char *type)
{
  if (!library)
    return nullptr;
  if (type && std::strcmp(type, "visrtx") != 0 && std::strcmp(type, "default") != 0)
    return nullptr;
  const auto *lib = reinterpret_cast<ShimLibrary *>(library);
  return newDevice(lib->cb, lib->cbUser);
}

// --- arrays -------------------------------------------------------------------

ANARI_SHIM_API ANARIArray1D anariNewArray1D(ANARIDevice device,
    const void *mem,
    ANARIMemoryDeleter deleter,
    const void *user,
    ANARIDataType type,
    uint64_t n1)
{
  return AO(newArray(device, 1, mem, deleter, user, type, n1, 1, 1));
}

ANARI_SHIM_API ANARIArray2D anariNewArray2D(ANARIDevice device,
    const void *mem,
    ANARIMemoryDeleter deleter,
    const void *user,
    ANARIDataType type,
    uint64_t n1,
    uint64_t n2)
{
  return AO(newArray(device, 2, mem, deleter, user, type, n1, n2, 1));
}

ANARI_SHIM_API ANARIArray3D anariNewArray3D(ANARIDevice device,
    const void *mem,
    ANARIMemoryDeleter deleter,
    const void *user,
    ANARIDataType type,
    uint64_t n1,
    uint64_t n2,
    uint64_t n3)
{
  return AO(newArray(device, 3, mem, deleter, user, type, n1, n2, n3));
}

ANARI_SHIM_API void *anariMapArray(ANARIDevice device, ANARIArray array)
{
  return device ? vrtxMapArray(VD(device), VO(array)) : nullptr;
}

ANARI_SHIM_API void anariUnmapArray(ANARIDevice device, ANARIArray array)
{
  if (device)
    vrtxUnmapArray(VD(device), VO(array));
}

// --- objects --------------------------------------------------------------------

ANARI_SHIM_API ANARILight anariNewLight(ANARIDevice device, const char *type)
{
  return AO(byType(device, [&](VRTXDevice d) { return vrtxNewLight(d, type); }));
}

ANARI_SHIM_API ANARICamera anariNewCamera(ANARIDevice device, const char *type)
{
  return AO(byType(device, [&](VRTXDevice d) { return vrtxNewCamera(d, type); }));
}

ANARI_SHIM_API ANARIGeometry anariNewGeometry(ANARIDevice device, const char *type)
{
  return AO(byType(device, [&](VRTXDevice d) { return vrtxNewGeometry(d, type); }));
}

ANARI_SHIM_API ANARISpatialField anariNewSpatialField(ANARIDevice device, const char *type)
{
  return AO(byType(device, [&](VRTXDevice d) { return vrtxNewSpatialField(d, type); }));
}

ANARI_SHIM_API ANARIVolume anariNewVolume(ANARIDevice device, const char *type)
{
  return AO(byType(device, [&](VRTXDevice d) { return vrtxNewVolume(d, type); }));
}

ANARI_SHIM_API ANARISurface anariNewSurface(ANARIDevice device)
{
  return AO(byType(device, [&](VRTXDevice d) { return vrtxNewSurface(d); }));
}

ANARI_SHIM_API ANARIMaterial anariNewMaterial(ANARIDevice device, const char *type)
{
  return AO(byType(device, [&](VRTXDevice d) { return vrtxNewMaterial(d, type); }));
}

ANARI_SHIM_API ANARISampler anariNewSampler(ANARIDevice device, const char *type)
{
  return AO(byType(device, [&](VRTXDevice d) { return vrtxNewSampler(d, type); }));
}

ANARI_SHIM_API ANARIGroup anariNewGroup(ANARIDevice device)
{
  return AO(byType(device, [&](VRTXDevice d) { return vrtxNewGroup(d); }));
}

ANARI_SHIM_API ANARIInstance anariNewInstance(ANARIDevice device, const char *type)
{
  return AO(byType(device, [&](VRTXDevice d) { return vrtxNewInstance(d, type); }));
}

ANARI_SHIM_API ANARIWorld anariNewWorld(ANARIDevice device)
{
  return AO(byType(device, [&](VRTXDevice d) { return vrtxNewWorld(d); }));
}

ANARI_SHIM_API ANARIRenderer anariNewRenderer(ANARIDevice device, const char *type)
{
  return AO(byType(device, [&](VRTXDevice d) { return vrtxNewRenderer(d, type); }));
}

ANARI_SHIM_API ANARIFrame anariNewFrame(ANARIDevice device)
{
  return AO(byType(device, [&](VRTXDevice d) { return vrtxNewFrame(d); }));
}

ANARI_SHIM_API ANARIObject anariNewObject(
    ANARIDevice device, const char *objectType, const char *type)
{
  if (!device || !objectType)
    return nullptr;
  const std::string t(objectType);
  if (t == "camera")
    return anariNewCamera(device, type);
  if (t == "geometry")
    return anariNewGeometry(device, type);
  if (t == "light")
    return anariNewLight(device, type);
  if (t == "material")
    return anariNewMaterial(device, type);
  if (t == "renderer")
    return anariNewRenderer(device, type);
  if (t == "sampler")
    return anariNewSampler(device, type);
  if (t == "spatialField")
    return anariNewSpatialField(device, type);
  if (t == "volume")
    return anariNewVolume(device, type);
  if (t == "instance")
    return anariNewInstance(device, type);
  if (t == "surface")
    return anariNewSurface(device);
  if (t == "group")
    return anariNewGroup(device);
  if (t == "world")
    return anariNewWorld(device);
  if (t == "frame")
    return anariNewFrame(device);
  return nullptr;
}

// --- parameters -------------------------------------------------------------------

ANARI_SHIM_API void anariSetParameter(ANARIDevice device,
    ANARIObject object,
    const char *name,
    ANARIDataType type,
    const void *mem)
{
  if (!device || !object || !name)
    return;
  VRTXDevice d = VD(device);
  if (isDevice(device, object)) {
    vrtxDeviceSetParameter(d, name, toVrtx(type), mem);
    return;
  }
  const int t = toVrtx(type);
  if (t == VRTX_DATA_TYPE && mem) {
    // a parameter whose value is a data type ("channel.color", ...)
    const int32_t v = toVrtx(*reinterpret_cast<const int32_t *>(mem));
    vrtxSetParameter(d, VO(object), name, t, &v);
    return;
  }
  vrtxSetParameter(d, VO(object), name, t, mem);
}

ANARI_SHIM_API void anariUnsetParameter(ANARIDevice device, ANARIObject object, const char *name)
{
  if (device && !isDevice(device, object))
    vrtxUnsetParameter(VD(device), VO(object), name);
}

ANARI_SHIM_API void anariUnsetAllParameters(ANARIDevice device, ANARIObject object)
{
  if (device && !isDevice(device, object))
    vrtxUnsetAllParameters(VD(device), VO(object));
}

ANARI_SHIM_API void *anariMapParameterArray1D(ANARIDevice device,
    ANARIObject object,
    const char *name,
    ANARIDataType type,
    uint64_t n1,
    uint64_t *stride)
{
  return mapParameterArray(device, object, name, type, 1, n1, 1, 1, stride);
}

ANARI_SHIM_API void *anariMapParameterArray2D(ANARIDevice device,
    ANARIObject object,
    const char *name,
    ANARIDataType type,
    uint64_t n1,
    uint64_t n2,
    uint64_t *stride)
{
  return mapParameterArray(device, object, name, type, 2, n1, n2, 1, stride);
}

ANARI_SHIM_API void *anariMapParameterArray3D(ANARIDevice device,
    ANARIObject object,
    const char *name,
    ANARIDataType type,
    uint64_t n1,
    uint64_t n2,
    uint64_t n3,
    uint64_t *stride)
{
  return mapParameterArray(device, object, name, type, 3, n1, n2, n3, stride);
}

ANARI_SHIM_API void anariUnmapParameterArray(
    ANARIDevice device, ANARIObject object, const char *name)
{
  if (!device || !name)
    return;
  std::lock_guard<std::mutex> lock(g_mapMutex);
  auto it = g_mapped.find(std::make_tuple(device, object, std::string(name)));
  if (it == g_mapped.end())
    return;
  vrtxUnmapArray(VD(device), it->second);
  vrtxRelease(VD(device), it->second); // the parameter keeps its reference
  g_mapped.erase(it);
}

ANARI_SHIM_API void anariCommitParameters(ANARIDevice device, ANARIObject object)
{
  if (!device)
    return;
  if (isDevice(device, object))
    vrtxDeviceCommitParameters(VD(device));
  else
    vrtxCommitParameters(VD(device), VO(object));
}

ANARI_SHIM_API void anariRelease(ANARIDevice device, ANARIObject object)
{
  if (!device)
    return;
  if (isDevice(device, object)) {
    {
      std::lock_guard<std::mutex> lock(g_mapMutex);
      for (auto it = g_mapped.begin(); it != g_mapped.end();) {
        if (std::get<0>(it->first) == device) {
          vrtxUnmapArray(VD(device), it->second);
          vrtxRelease(VD(device), it->second);
          it = g_mapped.erase(it);
        } else {
          ++it;
        }
      }
    }
    vrtxDeviceRelease(VD(device));
    return;
  }
  vrtxRelease(VD(device), VO(object));
}

ANARI_SHIM_API void anariRetain(ANARIDevice device, ANARIObject object)
{
  if (device && !isDevice(device, object))
    vrtxRetain(VD(device), VO(object));
}

// --- queries --------------------------------------------------------------------

ANARI_SHIM_API const char **anariGetObjectSubtypes(ANARIDevice device, ANARIDataType objectType)
{
  if (!device)
    return nullptr;
  return const_cast<const char **>(
      vrtxGetObjectSubtypes(VD(device), toVrtx(objectType)));
}

ANARI_SHIM_API const void *anariGetObjectInfo(
    ANARIDevice, ANARIDataType, const char *, const char *, ANARIDataType)
{
  return nullptr;
}

ANARI_SHIM_API const void *anariGetParameterInfo(ANARIDevice,
    ANARIDataType,
    const char *,
    const char *,
    ANARIDataType,
    const char *,
    ANARIDataType)
{
  return nullptr;
}

ANARI_SHIM_API int anariGetProperty(ANARIDevice device,
    ANARIObject object,
    const char *name,
    ANARIDataType type,
    void *mem,
    uint64_t size,
    ANARIWaitMask mask)
{
  if (!device || !name)
    return 0;
  if (isDevice(device, object))
    return vrtxDeviceGetProperty(VD(device), name, toVrtx(type), mem, size, mask);
  return vrtxGetProperty(VD(device), VO(object), name, toVrtx(type), mem, size, mask);
}

// --- frames -----------------------------------------------------------------------

ANARI_SHIM_API const void *anariMapFrame(ANARIDevice device,
    ANARIFrame frame,
    const char *channel,
    uint32_t *width,
    uint32_t *height,
    ANARIDataType *pixelType)
{
  if (!device) {
    if (width)
      *width = 0;
    if (height)
      *height = 0;
    if (pixelType)
      *pixelType = ANARI_UNKNOWN;
    return nullptr;
  }
  int t = VRTX_UNKNOWN;
  const void *p = vrtxMapFrame(VD(device), VO(frame), channel, width, height, &t);
  if (pixelType)
    *pixelType = toAnari(t);
  return p;
}

ANARI_SHIM_API void anariUnmapFrame(ANARIDevice device, ANARIFrame frame, const char *channel)
{
  if (device)
    vrtxUnmapFrame(VD(device), VO(frame), channel);
}

ANARI_SHIM_API void anariRenderFrame(ANARIDevice device, ANARIFrame frame)
{
  if (device)
    vrtxRenderFrame(VD(device), VO(frame));
}

ANARI_SHIM_API int anariFrameReady(ANARIDevice device, ANARIFrame frame, ANARIWaitMask mask)
{
  return device ? vrtxFrameReady(VD(device), VO(frame), mask) : 1;
}

ANARI_SHIM_API void anariDiscardFrame(ANARIDevice device, ANARIFrame frame)
{
  if (device)
    vrtxDiscardFrame(VD(device), VO(frame));
}

} // extern "C"
