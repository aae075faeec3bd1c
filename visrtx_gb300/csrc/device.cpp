// libvrtx host side: object model, world build and the C ABI (include/vrtx.h).
//
// Mirrors the VisRTX device's object layer (devices/rtx/VisRTXDevice.cpp,
// array/, camera/, frame/Frame.cu, renderer/Renderer.cpp, scene/) for the
// hot path: same subtypes, parameter names, defaults and error behaviour
// (status callback, null handles, skipped renders), with OptiX replaced by
// the kernels of bvh.cu, scene.cu and the render*.cu units.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <set>

#include <nvtx3/nvToolsExt.h>

#include "objects.h"
#include "radix_sort.h"

namespace vrtx {

static std::atomic<uint64_t> g_stamp{1};
uint64_t newStamp()
{
  return g_stamp.fetch_add(1) + 1;
}

size_t sizeOfType(int t)
{
  switch (t) {
  case VRTX_BOOL:
    return 4;
  case VRTX_INT32:
  case VRTX_UINT32:
  case VRTX_FLOAT32:
  case VRTX_DATA_TYPE:
    return 4;
  case VRTX_INT32_VEC2:
  case VRTX_UINT32_VEC2:
  case VRTX_FLOAT32_VEC2:
  case VRTX_FLOAT32_BOX1:
    return 8;
  case VRTX_UINT32_VEC3:
  case VRTX_FLOAT32_VEC3:
    return 12;
  case VRTX_UINT32_VEC4:
  case VRTX_FLOAT32_VEC4:
  case VRTX_FLOAT32_BOX2:
    return 16;
  case VRTX_FLOAT32_BOX3:
    return 24;
  case VRTX_FLOAT32_MAT3x4:
    return 48;
  case VRTX_FLOAT32_MAT4:
    return 64;
  case VRTX_FLOAT64:
    return 8;
  case VRTX_FLOAT64_BOX1:
    return 16;
  case VRTX_FIXED8:
  case VRTX_UFIXED8:
  case VRTX_INT8:
  case VRTX_UINT8:
    return 1;
  case VRTX_FIXED16:
  case VRTX_UFIXED16:
  case VRTX_FLOAT16:
  case VRTX_BFLOAT16:
    return 2;
  case VRTX_UFIXED8_VEC4:
  case VRTX_UFIXED8_RGBA_SRGB:
    return 4;
  case VRTX_VOID_POINTER:
  case VRTX_FUNCTION_POINTER:
  case VRTX_MEMORY_DELETER:
    return sizeof(void *);
  default:
    if (isObjectType(t))
      return sizeof(void *);
    return 0;
  }
}

bool isObjectType(int t)
{
  return t >= VRTX_OBJECT && t <= VRTX_WORLD;
}

const char *typeName(int t)
{
  switch (t) {
  case VRTX_CAMERA:
    return "ANARICamera";
  case VRTX_FRAME:
    return "ANARIFrame";
  case VRTX_GEOMETRY:
    return "ANARIGeometry";
  case VRTX_GROUP:
    return "ANARIGroup";
  case VRTX_INSTANCE:
    return "ANARIInstance";
  case VRTX_LIGHT:
    return "ANARILight";
  case VRTX_MATERIAL:
    return "ANARIMaterial";
  case VRTX_RENDERER:
    return "ANARIRenderer";
  case VRTX_SURFACE:
    return "ANARISurface";
  case VRTX_SPATIAL_FIELD:
    return "ANARISpatialField";
  case VRTX_VOLUME:
    return "ANARIVolume";
  case VRTX_WORLD:
    return "ANARIWorld";
  case VRTX_ARRAY1D:
  case VRTX_ARRAY2D:
  case VRTX_ARRAY3D:
    return "ANARIArray";
  default:
    return "ANARIObject";
  }
}

// ---------------------------------------------------------------------------
// NVTX ranges under the reference's names (utility/instrument.cpp:39-54,
// call sites Frame.cu:201-306), so a profile timeline reads the same.
// Without a profiler attached the calls do nothing measurable.
// ---------------------------------------------------------------------------

struct NvtxRange
{
  explicit NvtxRange(const char *name)
  {
    nvtxRangePushA(name);
  }
  ~NvtxRange()
  {
    nvtxRangePop();
  }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

// ---------------------------------------------------------------------------
// Device
// ---------------------------------------------------------------------------

void Device::report(const Object *src, int severity, const char *msg)
{
  if (!cb)
    return;
  int type = src ? src->type : 0;
  if (reportMap) {
    type = reportMap(0, type);
    severity = reportMap(1, severity);
  }
  cb(cbPtr,
      reinterpret_cast<VRTXDevice>(this),
      reinterpret_cast<VRTXObject>(const_cast<Object *>(src)),
      type,
      severity,
      0,
      msg);
}

// the ANARI entry points (anari_shim.cpp) make their devices report ANARI
// codes
void setReportCodes(VRTXDevice d, int (*map)(int kind, int value))
{
  if (d)
    reinterpret_cast<Device *>(d)->reportMap = map;
}

// Lazy CUDA init (VisRTXDevice::initDevice, VisRTXDevice.cpp:435-458).
bool Device::init()
{
  std::lock_guard<std::recursive_mutex> lock(mutex);
  if (initTried)
    return initOk;
  initTried = true;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    report(nullptr,
        VRTX_SEVERITY_FATAL_ERROR,
        "no CUDA device found: libvrtx has no CPU path");
    return false;
  }
  cudaDevice = desiredDevice;
  if (cudaDevice < 0 || cudaDevice >= n) {
    report(nullptr, VRTX_SEVERITY_FATAL_ERROR, "invalid 'cudaDevice'");
    return false;
  }
  if (cudaSetDevice(cudaDevice) != cudaSuccess
      || cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking)
          != cudaSuccess) {
    report(nullptr, VRTX_SEVERITY_FATAL_ERROR, "CUDA initialisation failed");
    return false;
  }
  cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, cudaDevice);
  // keep freed stream-ordered memory in the pool between frames
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, cudaDevice) == cudaSuccess) {
    uint64_t thresh = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thresh);
  }
  initOk = true;
  return true;
}

// ---------------------------------------------------------------------------
// Object
// ---------------------------------------------------------------------------

Object::Object(Device *d, int t, const std::string &st)
    : dev(d), type(t), subtype(st)
{}

Object::~Object()
{
  for (auto &p : pending)
    if (p.second.obj)
      releaseObj(p.second.obj);
  for (auto &p : params)
    if (p.second.obj)
      releaseObj(p.second.obj);
}

void retainObj(Object *o)
{
  if (o)
    o->refs++;
}

void releaseObj(Object *o)
{
  if (o && --o->refs == 0) {
    Device *d = o->dev;
    {
      std::lock_guard<std::recursive_mutex> lock(d->mutex);
      auto it = std::find(d->live.begin(), d->live.end(), o);
      if (it != d->live.end())
        d->live.erase(it);
    }
    delete o;
  }
}

void Object::report(int severity, const char *fmt, ...) const
{
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  dev->report(this, severity, buf);
}

void Object::setParam(const std::string &name, int t, const void *mem)
{
  Param p;
  p.type = t;
  if (isObjectType(t)) {
    Object *o = mem ? *reinterpret_cast<Object *const *>(mem) : nullptr;
    retainObj(o);
    p.obj = o;
  } else if (t == VRTX_STRING) {
    p.str = mem ? (const char *)mem : "";
  } else {
    const size_t sz = sizeOfType(t);
    if (sz == 0 || !mem) {
      report(VRTX_SEVERITY_WARNING,
          "ignoring parameter '%s' of unsupported type %d",
          name.c_str(),
          t);
      return;
    }
    p.bytes.resize(sz);
    std::memcpy(p.bytes.data(), mem, sz);
  }
  auto it = pending.find(name);
  if (it != pending.end() && it->second.obj)
    releaseObj(it->second.obj);
  pending[name] = std::move(p);
}

void Object::unsetParam(const std::string &name)
{
  auto it = pending.find(name);
  if (it == pending.end())
    return;
  if (it->second.obj)
    releaseObj(it->second.obj);
  pending.erase(it);
}

void Object::unsetAll()
{
  for (auto &p : pending)
    if (p.second.obj)
      releaseObj(p.second.obj);
  pending.clear();
}

void Object::commitParams()
{
  for (auto &p : params)
    if (p.second.obj)
      releaseObj(p.second.obj);
  params = pending;
  for (auto &p : params)
    if (p.second.obj)
      retainObj(p.second.obj);
  commitStamp = newStamp();
  commit();
  dev->markChanged();
}

bool Object::has(const std::string &name, int t) const
{
  auto it = params.find(name);
  return it != params.end() && it->second.type == t;
}

Object *Object::getObject(const std::string &name, int t) const
{
  auto it = params.find(name);
  if (it == params.end() || !it->second.obj)
    return nullptr;
  Object *o = it->second.obj;
  if (t == VRTX_OBJECT || o->type == t)
    return o;
  if ((t == VRTX_ARRAY1D || t == VRTX_ARRAY2D || t == VRTX_ARRAY3D)
      && o->type == t)
    return o;
  return nullptr;
}

std::string Object::getString(const std::string &name, const std::string &def) const
{
  auto it = params.find(name);
  if (it == params.end() || it->second.type != VRTX_STRING)
    return def;
  return it->second.str;
}

bool Object::getProperty(
    const std::string &name, int t, void *mem, uint64_t size, uint32_t)
{
  if (name == "valid" && t == VRTX_BOOL && size >= 4) {
    int32_t v = isValid() ? 1 : 0;
    std::memcpy(mem, &v, 4);
    return true;
  }
  return false;
}

// ---------------------------------------------------------------------------
// Array (array/Array.cpp:38-297)
// ---------------------------------------------------------------------------

Array::Array(Device *d,
    int dims,
    const void *mem,
    VRTXMemoryDeleter del,
    const void *delPtr,
    int et,
    uint64_t n1,
    uint64_t n2,
    uint64_t n3)
    : Object(d,
          dims == 1 ? VRTX_ARRAY1D : (dims == 2 ? VRTX_ARRAY2D : VRTX_ARRAY3D)),
      elemType(et),
      n{n1, n2, n3},
      appMem(mem),
      deleter(del),
      deleterPtr(delPtr)
{
  if (!appMem)
    owned.resize(bytes());
  else if (d->initOk) {
    // NV_ARRAY_CUDA: application device pointers are used in place
    // getPointerAddressSpace (Array.cpp:38-65): device memory of this GPU
    // and managed memory are used in place; another GPU's memory is foreign
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, appMem) == cudaSuccess) {
      if (attr.type == cudaMemoryTypeManaged
          || (attr.type == cudaMemoryTypeDevice && attr.device == d->cudaDevice))
        appIsDevice = true;
      else if (attr.type == cudaMemoryTypeDevice)
        appIsForeign = true;
    }
    cudaGetLastError();
  }
  dataStamp = newStamp();
  refreshHandles();
}

void Array::settleHostReads()
{
  if (hostReadQueued && Object::dev->initOk)
    cudaStreamSynchronize(Object::dev->stream);
  hostReadQueued = false;
}

Array::~Array()
{
  settleHostReads();
  for (auto *h : handles)
    releaseObj(h);
  if (dptr && devBytes)
    cudaFreeAsync(dptr, Object::dev->stream);
  if (deleter && appMem)
    deleter(deleterPtr, appMem);
}

const void *Array::hostData() const
{
  if (appIsDevice || appIsForeign)
    return nullptr;
  return appMem ? appMem : owned.data();
}

const void *Array::deviceData()
{
  if (appIsDevice)
    return appMem;
  if (!Object::dev->initOk)
    return nullptr;
  const size_t b = bytes();
  if (b == 0)
    return nullptr;
  if (devStamp >= dataStamp && dptr)
    return dptr;
  // stream-ordered from the device's pool (kept between frames): a scene
  // rebuilt every frame reuses its buffers without cudaMalloc / cudaFree
  // round trips, and a release does not synchronise the device
  if (devBytes < b) {
    if (dptr)
      cudaFreeAsync(dptr, Object::dev->stream);
    dptr = nullptr;
    devBytes = 0;
    if (cudaMallocAsync(&dptr, b, Object::dev->stream) != cudaSuccess) {
      report(VRTX_SEVERITY_ERROR, "device allocation of %zu bytes failed", b);
      cudaGetLastError();
      return nullptr;
    }
    devBytes = b;
  }
  // a foreign array comes from the other GPU through unified addressing
  cudaMemcpyAsync(dptr,
      appIsForeign ? appMem : hostData(),
      b,
      appIsForeign ? cudaMemcpyDefault : cudaMemcpyHostToDevice,
      Object::dev->stream);
  if (!appIsForeign && appMem)
    hostReadQueued = true;
  devStamp = dataStamp;
  return dptr;
}

void *Array::map()
{
  if (appIsDevice || appIsForeign)
    return const_cast<void *>(appMem);
  return const_cast<void *>(hostData());
}

void Array::unmap()
{
  dataStamp = newStamp();
  refreshHandles();
  Object::dev->markChanged();
}

void Array::privatize()
{
  if (!appMem || deleter || appIsDevice || appIsForeign)
    return;
  settleHostReads();
  owned.assign((const uint8_t *)appMem, (const uint8_t *)appMem + bytes());
  appMem = nullptr;
}

void Array::refreshHandles()
{
  for (auto *h : handles)
    releaseObj(h);
  handles.clear();
  if (!isObjectType(elemType) || appIsDevice || appIsForeign)
    return;
  const Object *const *p = reinterpret_cast<const Object *const *>(hostData());
  if (!p)
    return;
  for (uint64_t i = 0; i < count(); i++) {
    Object *o = const_cast<Object *>(p[i]);
    retainObj(o);
    handles.push_back(o);
  }
}

// ---------------------------------------------------------------------------
// Camera (camera/Camera.cpp:68-76, Perspective.cpp:40-72,
// Orthographic.cpp:38-52)
// ---------------------------------------------------------------------------

void Camera::commit()
{
  float region[4] = {0.f, 0.f, 1.f, 1.f};
  if (has("imageRegion", VRTX_FLOAT32_BOX2))
    std::memcpy(region, params["imageRegion"].bytes.data(), 16);
  for (int i = 0; i < 4; i++)
    gpu.region[i] = region[i];
  gpu.pos = get<f3>("position", VRTX_FLOAT32_VEC3, f3{0.f, 0.f, 0.f});
  gpu.dir = normalize(get<f3>("direction", VRTX_FLOAT32_VEC3, f3{0.f, 0.f, 1.f}));
  const f3 up = normalize(get<f3>("up", VRTX_FLOAT32_VEC3, f3{0.f, 1.f, 0.f}));
  const float aspect = get<float>("aspect", VRTX_FLOAT32, 1.f);
  if (subtype == "orthographic") {
    gpu.type = CAMERA_ORTHOGRAPHIC;
    const float height = get<float>("height", VRTX_FLOAT32, 1.f);
    const float sx = height * aspect, sy = height;
    gpu.posDu = normalize(cross(gpu.dir, up)) * sx;
    gpu.posDv = normalize(cross(gpu.posDu, gpu.dir)) * sy;
    gpu.pos00 = gpu.pos - 0.5f * gpu.posDu - 0.5f * gpu.posDv;
  } else {
    if (subtype != "perspective")
      report(VRTX_SEVERITY_WARNING,
          "unknown camera subtype '%s', using perspective",
          subtype.c_str());
    gpu.type = CAMERA_PERSPECTIVE;
    const float fovy =
        get<float>("fovy", VRTX_FLOAT32, 60.f * float(M_PI) / 180.f);
    const float ipy = 2.f * tanf(0.5f * fovy);
    const float ipx = ipy * aspect;
    f3 du = normalize(cross(gpu.dir, up)) * ipx;
    f3 dv = normalize(cross(du, gpu.dir)) * ipy;
    f3 d00 = gpu.dir - .5f * du - .5f * dv;
    const float focusDistance = get<float>("focusDistance", VRTX_FLOAT32, 1.f);
    const float apertureRadius =
        get<float>("apertureRadius", VRTX_FLOAT32, 0.f) / (ipx * focusDistance);
    if (apertureRadius > 0.f) {
      du *= focusDistance;
      dv *= focusDistance;
      d00 *= focusDistance;
    }
    gpu.dirDu = du;
    gpu.dirDv = dv;
    gpu.dir00 = d00;
    gpu.scaledAperture = apertureRadius;
    gpu.aspect = aspect;
  }
}

// ---------------------------------------------------------------------------
// Geometry (scene/surface/geometry/Triangle.cpp:42-175, Sphere.cu:40-115)
// ---------------------------------------------------------------------------

static Array *arrayParam(Object *o, const char *name, int elemType)
{
  auto *a = static_cast<Array *>(o->getObject(name, VRTX_ARRAY1D));
  if (!a)
    return nullptr;
  if (a->elemType != elemType) {
    o->report(VRTX_SEVERITY_WARNING,
        "'%s' array has element type %d, expected %d; ignored",
        name,
        a->elemType,
        elemType);
    return nullptr;
  }
  return a;
}

// Channels of an attribute element type this device reads (0: not one)
static uint32_t attrChannels(int t)
{
  switch (t) {
  case VRTX_FLOAT32:
  case VRTX_UFIXED8:
  case VRTX_UFIXED16:
    return 1;
  case VRTX_FLOAT32_VEC2:
    return 2;
  case VRTX_FLOAT32_VEC3:
    return 3;
  case VRTX_FLOAT32_VEC4:
  case VRTX_UFIXED8_VEC4:
  case VRTX_UFIXED8_RGBA_SRGB:
    return 4;
  default:
    return 0;
  }
}

static Array *attrArray(Object *o, const std::string &name)
{
  auto *a = static_cast<Array *>(o->getObject(name, VRTX_ARRAY1D));
  if (!a)
    return nullptr;
  if (!attrChannels(a->elemType)) {
    o->report(VRTX_SEVERITY_WARNING,
        "'%s' array has an element type this device does not read; ignored",
        name.c_str());
    return nullptr;
  }
  return a;
}

Geometry::~Geometry()
{
  if (quadIndices && Object::dev->initOk)
    cudaFree(quadIndices);
}

int Geometry::geomClass() const
{
  if (subtype == "sphere")
    return GEOM_SPHERE;
  if (subtype == "cylinder")
    return GEOM_CYLINDER;
  if (subtype == "cone")
    return GEOM_CONE;
  if (subtype == "curve")
    return GEOM_CURVE;
  return GEOM_TRIANGLE; // triangle, quad
}

uint32_t Geometry::kind() const
{
  if (subtype == "quad")
    return KIND_QUAD;
  if (subtype == "sphere")
    return KIND_SPHERE;
  if (subtype == "cylinder")
    return KIND_CYLINDER;
  if (subtype == "cone")
    return KIND_CONE;
  if (subtype == "curve")
    return KIND_CURVE;
  return KIND_TRIANGLE;
}

// Parameters per subtype: Triangle.cpp, Quad.cpp:40-47, Sphere.cu:45-55,
// Cylinder.cpp:42-51, Cone.cpp:40-48, Curve.cpp:45-53.
void Geometry::commit()
{
  vertex = arrayParam(this, "vertex.position", VRTX_FLOAT32_VEC3);
  normal = normalFV = radius = index = nullptr;
  cull = caps = false;
  const uint32_t nv = vertex ? (uint32_t)vertex->count() : 0;
  if (subtype == "sphere") {
    index = arrayParam(this, "primitive.index", VRTX_UINT32);
    radius = arrayParam(this, "vertex.radius", VRTX_FLOAT32);
    globalRadius = get<float>("radius", VRTX_FLOAT32, 0.01f);
    numPrims = index ? (uint32_t)index->count() : nv;
  } else if (subtype == "cylinder") {
    index = arrayParam(this, "primitive.index", VRTX_UINT32_VEC2);
    radius = arrayParam(this, "primitive.radius", VRTX_FLOAT32);
    globalRadius = get<float>("radius", VRTX_FLOAT32, 1.f);
    caps = getString("caps", "none") != "none";
    numPrims = index ? (uint32_t)index->count() : nv / 2;
  } else if (subtype == "cone") {
    index = arrayParam(this, "primitive.index", VRTX_UINT32_VEC2);
    radius = arrayParam(this, "vertex.radius", VRTX_FLOAT32);
    if (!radius)
      report(VRTX_SEVERITY_WARNING,
          "missing required parameter 'vertex.radius' on cone geometry");
    numPrims = index ? (uint32_t)index->count() : nv / 2;
  } else if (subtype == "curve") {
    index = arrayParam(this, "primitive.index", VRTX_UINT32);
    radius = arrayParam(this, "vertex.radius", VRTX_FLOAT32);
    globalRadius = get<float>("radius", VRTX_FLOAT32, 1.f);
    // without an index the reference numbers segments 0 .. n/2 - 1, each
    // from vertex i to i + 1 (Curve.cpp:88-99)
    numPrims = index ? (uint32_t)index->count() : nv / 2;
  } else if (subtype == "quad") {
    index = arrayParam(this, "primitive.index", VRTX_UINT32_VEC4);
    normal = arrayParam(this, "vertex.normal", VRTX_FLOAT32_VEC3);
    cull = get<int32_t>("cullBackfaces", VRTX_BOOL, 0) != 0;
    if (!index && nv % 4 != 0) {
      report(VRTX_SEVERITY_ERROR,
          "'vertex.position' on quad geometry is a non-multiple of 4 without "
          "'primitive.index' present");
      vertex = nullptr;
    }
    // two triangles per quad (Quad.cpp:115-141)
    numPrims = 2 * (index ? (uint32_t)index->count() : nv / 4);
  } else {
    if (subtype != "triangle")
      report(VRTX_SEVERITY_WARNING,
          "geometry subtype '%s' is not supported by this device",
          subtype.c_str());
    index = arrayParam(this, "primitive.index", VRTX_UINT32_VEC3);
    normal = arrayParam(this, "vertex.normal", VRTX_FLOAT32_VEC3);
    normalFV = arrayParam(this, "faceVarying.normal", VRTX_FLOAT32_VEC3);
    cull = get<int32_t>("cullBackfaces", VRTX_BOOL, 0) != 0;
    numPrims = index ? (uint32_t)index->count() : nv / 3;
  }
  primId = arrayParam(this, "primitive.id", VRTX_UINT32);
  // attributes (Geometry.cpp:108-126,152-171): vertex.* per subtype,
  // primitive.*, and uniform FLOAT32_VEC4 values
  static const char *names[NUM_ATTRS] = {
      "attribute0", "attribute1", "attribute2", "attribute3", "color"};
  for (int k = 0; k < NUM_ATTRS; k++) {
    vattr[k] = attrArray(this, std::string("vertex.") + names[k]);
    pattr[k] = attrArray(this, std::string("primitive.") + names[k]);
    float u[4] = {0.f, 0.f, 0.f, 1.f};
    if (has(names[k], VRTX_FLOAT32_VEC4))
      std::memcpy(u, params[names[k]].bytes.data(), 16);
    uattr[k] = make_float4(u[0], u[1], u[2], u[3]);
  }
  if (!vertex)
    report(VRTX_SEVERITY_WARNING,
        "missing required parameter 'vertex.position' on %s geometry",
        subtype.c_str());
}

bool Geometry::isValid() const
{
  if (!vertex)
    return false;
  if (subtype == "cone")
    return radius != nullptr;
  return subtype == "triangle" || subtype == "sphere" || subtype == "quad"
      || subtype == "cylinder" || subtype == "curve";
}

uint64_t Geometry::deepStamp() const
{
  uint64_t s = commitStamp;
  for (const Array *a : {vertex, index, normal, normalFV, primId, radius})
    if (a)
      s = std::max(s, a->deepStamp());
  for (int k = 0; k < NUM_ATTRS; k++)
    for (const Array *a : {vattr[k], pattr[k]})
      if (a)
        s = std::max(s, a->deepStamp());
  return s;
}

GeometryGPU Geometry::gpuData()
{
  GeometryGPU g{};
  g.type = (uint32_t)geomClass();
  g.kind = kind();
  g.numPrims = numPrims;
  g.vertices = vertex ? (const f3 *)vertex->deviceData() : nullptr;
  g.indices = index ? (const uint32_t *)index->deviceData() : nullptr;
  if (g.kind == KIND_QUAD) {
    const uint64_t want = deepStamp();
    if (!quadIndices || quadStamp < want) {
      if (quadIndices)
        cudaFree(quadIndices);
      quadIndices = nullptr;
      if (numPrims
          && cudaMalloc(&quadIndices, sizeof(uint32_t) * 3 * (size_t)numPrims)
              == cudaSuccess) {
        launchQuadIndices(g.indices, numPrims / 2, quadIndices, Object::dev->stream);
        quadStamp = want;
      } else {
        cudaGetLastError();
        quadIndices = nullptr;
      }
    }
    g.indices = quadIndices;
  }
  g.normals = normal ? (const f3 *)normal->deviceData() : nullptr;
  g.normalsFV = normalFV ? (const f3 *)normalFV->deviceData() : nullptr;
  g.primIds = primId ? (const uint32_t *)primId->deviceData() : nullptr;
  g.radii = radius ? (const float *)radius->deviceData() : nullptr;
  g.radius = globalRadius;
  g.cullBackfaces = cull ? 1u : 0u;
  g.caps = caps ? 1u : 0u;
  for (int k = 0; k < NUM_ATTRS; k++) {
    for (int which = 0; which < 2; which++) {
      Array *a = which ? pattr[k] : vattr[k];
      AttrGPU &o = which ? g.pattr[k] : g.vattr[k];
      o.data = a ? a->deviceData() : nullptr;
      o.type = a ? (uint32_t)a->elemType : 0u;
      o.channels = a ? attrChannels(a->elemType) : 0u;
    }
    g.uattr[k] = uattr[k];
  }
  return g;
}

// ---------------------------------------------------------------------------
// Material (Matte.cpp:39-53) and Light (Directional.cpp:38-55, Light.cpp)
// ---------------------------------------------------------------------------

// Matte::commitParameters (Matte.cpp:39-53) and PBR::commitParameters
// (PBR.cpp:39-62): each parameter a value, a sampler or a string naming an
// attribute / hit quantity (populateMaterialParameter, Material.cpp)
void Material::commit()
{
  const bool pbr = subtype == "physicallyBased";
  if (subtype != "matte" && !pbr)
    report(VRTX_SEVERITY_WARNING,
        "material subtype '%s' is evaluated as matte",
        subtype.c_str());
  gpu = MaterialGPU{};
  gpu.type = pbr ? MATERIAL_PBR : MATERIAL_MATTE;
  auto source = [&](const char *name) -> uint32_t {
    if (!has(name, VRTX_STRING))
      return PARAM_VALUE;
    const std::string a = getString(name, "");
    if (a == "attribute0")
      return PARAM_ATTRIB_0;
    if (a == "attribute1")
      return PARAM_ATTRIB_0 + 1;
    if (a == "attribute2")
      return PARAM_ATTRIB_0 + 2;
    if (a == "attribute3")
      return PARAM_ATTRIB_0 + 3;
    if (a == "color")
      return PARAM_ATTRIB_COLOR;
    if (a == "worldPosition")
      return PARAM_WORLD_POSITION;
    if (a == "worldNormal")
      return PARAM_WORLD_NORMAL;
    if (a == "objectPosition")
      return PARAM_OBJECT_POSITION;
    if (a == "objectNormal")
      return PARAM_OBJECT_NORMAL;
    report(VRTX_SEVERITY_WARNING,
        "unknown attribute '%s' for material parameter '%s'",
        a.c_str(),
        name);
    return PARAM_VALUE;
  };
  const char *colorName = pbr ? "baseColor" : "color";
  float c[4] = {0.8f, 0.8f, 0.8f, 1.f};
  if (has(colorName, VRTX_FLOAT32_VEC4))
    std::memcpy(c, params[colorName].bytes.data(), 16);
  else if (has(colorName, VRTX_FLOAT32_VEC3))
    std::memcpy(c, params[colorName].bytes.data(), 12);
  gpu.color = f3{c[0], c[1], c[2]};
  const float op = get<float>("opacity", VRTX_FLOAT32, 1.f);
  gpu.opacity = c[3] * op;
  const char *names[MP_COUNT] = {colorName, "opacity", "metallic", "roughness"};
  const float4 values[MP_COUNT] = {make_float4(c[0], c[1], c[2], c[3]),
      make_float4(op, 0.f, 0.f, 1.f),
      make_float4(get<float>("metallic", VRTX_FLOAT32, 1.f), 0.f, 0.f, 1.f),
      make_float4(get<float>("roughness", VRTX_FLOAT32, 1.f), 0.f, 0.f, 1.f)};
  const int slots = pbr ? MP_COUNT : 2;
  for (int k = 0; k < MP_COUNT; k++) {
    samplers[k] = nullptr;
    gpu.params[k].value = values[k];
    gpu.params[k].src = PARAM_VALUE;
    if (k >= slots)
      continue;
    gpu.params[k].src = source(names[k]);
    samplers[k] = static_cast<Sampler *>(getObject(names[k], VRTX_SAMPLER));
    if (samplers[k])
      gpu.params[k].src = PARAM_SAMPLER;
  }
  gpu.ior = get<float>("ior", VRTX_FLOAT32, 1.5f);
  gpu.cutoff = get<float>("alphaCutoff", VRTX_FLOAT32, 0.5f);
  const std::string mode = getString("alphaMode", "opaque");
  gpu.alphaMode = mode == "blend" ? ALPHA_BLEND
                                  : (mode == "mask" ? ALPHA_MASK : ALPHA_OPAQUE);
}

uint64_t Material::deepStamp() const
{
  uint64_t s = commitStamp;
  for (const Sampler *sm : samplers)
    if (sm)
      s = std::max(s, sm->deepStamp());
  return s;
}

// ---------------------------------------------------------------------------
// Sampler (Sampler.cpp:68-95, Image1D/2D/3D.cpp, TransformSampler.cpp,
// PrimitiveSampler.cpp)
// ---------------------------------------------------------------------------

Sampler::~Sampler()
{
  cleanup();
}

void Sampler::cleanup()
{
  if (Object::dev->initOk) {
    if (tex)
      cudaDestroyTextureObject(tex);
    if (cuArray)
      cudaFreeArray(cuArray);
  }
  tex = 0;
  cuArray = nullptr;
  builtStamp = 0;
}

uint32_t Sampler::type() const
{
  if (subtype == "image1D")
    return SAMPLER_IMAGE1D;
  if (subtype == "image2D")
    return SAMPLER_IMAGE2D;
  if (subtype == "image3D")
    return SAMPLER_IMAGE3D;
  if (subtype == "transform")
    return SAMPLER_TRANSFORM;
  if (subtype == "primitive")
    return SAMPLER_PRIMITIVE;
  return SAMPLER_NONE;
}

void Sampler::commit()
{
  const std::string a = getString("inAttribute", "attribute0");
  attribute = a == "attribute1" ? 1u
      : a == "attribute2"       ? 2u
      : a == "attribute3"       ? 3u
      : a == "color"            ? 4u
                                : 0u;
  const float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  std::memcpy(inT, ident, sizeof(ident));
  std::memcpy(outT, ident, sizeof(ident));
  if (has("inTransform", VRTX_FLOAT32_MAT4))
    std::memcpy(inT, params["inTransform"].bytes.data(), 64);
  if (has("outTransform", VRTX_FLOAT32_MAT4))
    std::memcpy(outT, params["outTransform"].bytes.data(), 64);
  float o[4] = {0, 0, 0, 0};
  if (has("inOffset", VRTX_FLOAT32_VEC4))
    std::memcpy(o, params["inOffset"].bytes.data(), 16);
  inO = make_float4(o[0], o[1], o[2], o[3]);
  float q[4] = {0, 0, 0, 0};
  if (has("outOffset", VRTX_FLOAT32_VEC4))
    std::memcpy(q, params["outOffset"].bytes.data(), 16);
  outO = make_float4(q[0], q[1], q[2], q[3]);
  filter = getString("filter", "linear");
  // image1D reads "wrapMode", image2D / image3D "wrapMode1/2/3"
  wrap[0] = getString(type() == SAMPLER_IMAGE1D ? "wrapMode" : "wrapMode1", "clampToEdge");
  wrap[1] = getString("wrapMode2", "clampToEdge");
  wrap[2] = getString("wrapMode3", "clampToEdge");
  image = nullptr;
  primArray = nullptr;
  const uint32_t t = type();
  if (t == SAMPLER_IMAGE1D)
    image = static_cast<Array *>(getObject("image", VRTX_ARRAY1D));
  else if (t == SAMPLER_IMAGE2D)
    image = static_cast<Array *>(getObject("image", VRTX_ARRAY2D));
  else if (t == SAMPLER_IMAGE3D)
    image = static_cast<Array *>(getObject("image", VRTX_ARRAY3D));
  else if (t == SAMPLER_PRIMITIVE) {
    primArray = static_cast<Array *>(getObject("array", VRTX_ARRAY1D));
    primOffset = (uint32_t)get<uint64_t>("offset", VRTX_UINT64, get<uint32_t>("offset", VRTX_UINT32, 0u));
  } else if (t == SAMPLER_NONE)
    report(VRTX_SEVERITY_WARNING, "sampler subtype '%s' is not supported", subtype.c_str());
  if ((t == SAMPLER_IMAGE1D || t == SAMPLER_IMAGE2D || t == SAMPLER_IMAGE3D) && !image)
    report(VRTX_SEVERITY_WARNING, "missing required parameter 'image' on %s sampler",
        subtype.c_str());
}

bool Sampler::isValid() const
{
  const uint32_t t = type();
  if (t == SAMPLER_TRANSFORM)
    return true;
  if (t == SAMPLER_PRIMITIVE)
    return primArray != nullptr;
  return t != SAMPLER_NONE && image != nullptr;
}

uint64_t Sampler::deepStamp() const
{
  uint64_t s = commitStamp;
  for (const Array *a : {image, primArray})
    if (a)
      s = std::max(s, a->deepStamp());
  return s;
}

static cudaTextureAddressMode addressMode(const std::string &w)
{
  // stringToAddressMode (utility/CudaImageTexture.cpp:129-137)
  if (w == "repeat")
    return cudaAddressModeWrap;
  if (w == "mirrorRepeat")
    return cudaAddressModeMirror;
  return cudaAddressModeClamp;
}

// glm::convertSRGBToLinear of one component, as the reference's image
// staging calls it (glm's sRGB curve with gamma 2.4)
static float srgbToLinear(float x)
{
  return x <= 0.04045f ? x * 0.07739938080495356f
                       : std::pow((x + 0.055f) * 0.94786729857819905f, 2.4f);
}

// One component of the reference's 8-bit staging (convertComponentUint8,
// utility/CudaImageTexture.cpp:43-57): 8-bit values as they are, sRGB-encoded
// bytes linearised and truncated back to 8 bits, 16-bit values truncated
// from (c / 65535) * 255.
static uint8_t stageComponentUint8(int et, const uint8_t *texel, uint32_t c)
{
  if (et == VRTX_UFIXED16) {
    uint16_t v;
    std::memcpy(&v, texel + 2 * c, 2);
    return (uint8_t)((v / 65535.f) * 255.f);
  }
  if (et == VRTX_UFIXED8_RGBA_SRGB)
    return (uint8_t)(srgbToLinear(texel[c] / 255.f) * 255.f);
  return texel[c];
}

// An image sampler's texels as the reference stages them
// (Image1D/2D/3D::finalize, scene/surface/material/sampler/Image2D.cpp:70-78,
// with transformToStagingBuffer{Float,Uint8},
// utility/CudaImageTexture.cpp:76-111): float element types as float texels,
// every other as 8-bit texels that the texture reads as normalised float,
// all four components of an sRGB texel (alpha too) linearised. The n texels
// of src (element type et, ch channels) go to f4 (n x 4 floats, missing
// channels 0, alpha 1) or to u8 (n x 4 bytes, missing channels 0, alpha 255),
// which is what a fetch of the reference's ch-channel array returns; true
// for float staging.
static bool stageSamplerImage(
    int et, uint32_t ch, const uint8_t *src, size_t n, std::vector<float> &f4, std::vector<uint8_t> &u8)
{
  if (et >= VRTX_FLOAT32 && et <= VRTX_FLOAT32_VEC4) {
    f4.assign(4 * n, 0.f);
    for (size_t i = 0; i < n; i++) {
      std::memcpy(&f4[4 * i], src + i * ch * 4, ch * 4);
      if (ch < 4)
        f4[4 * i + 3] = 1.f;
    }
    return true;
  }
  const size_t bytes = et == VRTX_UFIXED16 ? 2 : 1;
  u8.assign(4 * n, 0);
  for (size_t i = 0; i < n; i++) {
    const uint8_t *t = src + i * ch * bytes;
    for (uint32_t c = 0; c < ch; c++)
      u8[4 * i + c] = stageComponentUint8(et, t, c);
    if (ch < 4)
      u8[4 * i + 3] = 255;
  }
  return false;
}

// Image samplers: the image staged as the reference stages it
// (stageSamplerImage) into a float4 or an RGBA8 cudaArray, with a
// normalised-coordinate texture of the sampler's filter and wrap modes,
// RGBA8 read as normalised float.
bool Sampler::ensureBuilt()
{
  const uint32_t t = type();
  if (t != SAMPLER_IMAGE1D && t != SAMPLER_IMAGE2D && t != SAMPLER_IMAGE3D)
    return true;
  if (!image)
    return false;
  const uint64_t want = deepStamp();
  if (builtStamp >= want && tex)
    return true;
  cleanup();
  const uint32_t ch = attrChannels(image->elemType);
  if (!ch) {
    report(VRTX_SEVERITY_WARNING, "image sampler: unsupported image element type");
    return false;
  }
  const size_t n = (size_t)image->n[0] * image->n[1] * image->n[2];
  std::vector<uint8_t> host(image->bytes());
  if (const void *h = image->hostData())
    std::memcpy(host.data(), h, host.size());
  else {
    // device-resident or other-GPU images: the upload is stream-ordered on
    // the device stream, which the synchronous read-back must follow
    const void *d = image->deviceData();
    cudaStreamSynchronize(Object::dev->stream);
    cudaMemcpy(host.data(), d, host.size(), cudaMemcpyDefault);
  }
  std::vector<float> f4;
  std::vector<uint8_t> u8;
  const bool isFloat = stageSamplerImage(image->elemType, ch, host.data(), n, f4, u8);
  const int bits = isFloat ? 32 : 8;
  cudaChannelFormatDesc desc = cudaCreateChannelDesc(bits, bits, bits, bits,
      isFloat ? cudaChannelFormatKindFloat : cudaChannelFormatKindUnsigned);
  const cudaExtent ext = make_cudaExtent(image->n[0],
      t >= SAMPLER_IMAGE2D ? image->n[1] : 0,
      t == SAMPLER_IMAGE3D ? image->n[2] : 0);
  if (cudaMalloc3DArray(&cuArray, &desc, ext) != cudaSuccess) {
    cudaGetLastError();
    cuArray = nullptr;
    report(VRTX_SEVERITY_ERROR, "image sampler: cudaMalloc3DArray failed");
    return false;
  }
  cudaMemcpy3DParms cp{};
  cp.srcPtr = make_cudaPitchedPtr(isFloat ? (void *)f4.data() : (void *)u8.data(),
      image->n[0] * (isFloat ? 16 : 4),
      image->n[0],
      t >= SAMPLER_IMAGE2D ? image->n[1] : 1);
  cp.dstArray = cuArray;
  cp.extent = make_cudaExtent(image->n[0],
      t >= SAMPLER_IMAGE2D ? image->n[1] : 1,
      t == SAMPLER_IMAGE3D ? image->n[2] : 1);
  cp.kind = cudaMemcpyHostToDevice;
  cudaMemcpy3D(&cp);
  cudaResourceDesc rd{};
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = cuArray;
  cudaTextureDesc td{};
  for (int k = 0; k < 3; k++)
    td.addressMode[k] = addressMode(wrap[k]);
  td.filterMode = filter == "nearest" ? cudaFilterModePoint : cudaFilterModeLinear;
  td.readMode = isFloat ? cudaReadModeElementType : cudaReadModeNormalizedFloat;
  td.normalizedCoords = 1;
  cudaCreateTextureObject(&tex, &rd, &td, nullptr);
  builtStamp = want;
  return cudaGetLastError() == cudaSuccess;
}

SamplerGPU Sampler::gpuData() const
{
  SamplerGPU g{};
  g.type = type();
  g.attribute = attribute;
  g.tex = tex;
  std::memcpy(g.inT, inT, 64);
  std::memcpy(g.outT, outT, 64);
  g.inO = inO;
  g.outO = outO;
  if (primArray) {
    g.prim.data = const_cast<Array *>(primArray)->deviceData();
    g.prim.type = (uint32_t)primArray->elemType;
    g.prim.channels = attrChannels(primArray->elemType);
    if (!g.prim.channels)
      g.prim.data = nullptr;
  }
  g.primOffset = primOffset;
  return g;
}

Light::~Light()
{
  cleanup();
}

void Light::cleanup()
{
  if (gpu.hdriTex)
    cudaDestroyTextureObject(gpu.hdriTex);
  if (cuArray)
    cudaFreeArray(cuArray);
  if (cdfs)
    cudaFree(cdfs);
  gpu.hdriTex = 0;
  gpu.marginalCDF = gpu.conditionalCDF = nullptr;
  cuArray = nullptr;
  cdfs = nullptr;
  builtStamp = 0;
}

// Light::commitParameters and the subtypes (Directional.cpp:38-55,
// Point.cpp:38-55, Spot.cpp:38-70, HDRI.cu:92-131)
void Light::commit()
{
  const f3 color = get<f3>("color", VRTX_FLOAT32_VEC3, f3{1.f, 1.f, 1.f});
  auto intensity = [&]() {
    const float power = get<float>("power", VRTX_FLOAT32, 1.f);
    return std::min(std::max(get<float>("intensity", VRTX_FLOAT32, power), 0.f),
        3.402823466e+38f);
  };
  const LightGPU old = gpu;
  gpu = LightGPU{};
  gpu.hdriTex = old.hdriTex;
  gpu.marginalCDF = old.marginalCDF;
  gpu.conditionalCDF = old.conditionalCDF;
  radiance = nullptr;
  builtStamp = 0;
  if (subtype == "point") {
    gpu.type = LIGHT_POINT;
    gpu.position = get<f3>("position", VRTX_FLOAT32_VEC3, f3{0.f, 0.f, 0.f});
    gpu.radiance = color * intensity();
  } else if (subtype == "spot") {
    gpu.type = LIGHT_SPOT;
    gpu.position = get<f3>("position", VRTX_FLOAT32_VEC3, f3{0.f, 0.f, 0.f});
    gpu.spotDir = normalize(get<f3>("direction", VRTX_FLOAT32_VEC3, f3{0.f, 0.f, -1.f}));
    const float opening = get<float>("openingAngle", VRTX_FLOAT32, float(M_PI));
    const float falloff = get<float>("falloffAngle", VRTX_FLOAT32, 0.1f);
    const float inner = opening - 2.f * falloff;
    if (inner < 0.f)
      report(VRTX_SEVERITY_WARNING, "falloffAngle should be smaller than half of openingAngle");
    gpu.cosOuter = std::cos(opening);
    gpu.cosInner = std::cos(inner);
    gpu.radiance = color * intensity();
  } else if (subtype == "hdri") {
    gpu.type = LIGHT_HDRI;
    radiance = static_cast<Array *>(getObject("radiance", VRTX_ARRAY2D));
    if (!radiance)
      report(VRTX_SEVERITY_WARNING, "missing required parameter 'radiance' on HDRI light");
    hdriDirection = get<f3>("direction", VRTX_FLOAT32_VEC3, f3{1.f, 0.f, 0.f});
    hdriUp = get<f3>("up", VRTX_FLOAT32_VEC3, f3{0.f, 0.f, 1.f});
    gpu.hdriScale = get<float>("scale", VRTX_FLOAT32, 1.f);
    gpu.visible = get<int32_t>("visible", VRTX_BOOL, 1) != 0 ? 1u : 0u;
    gpu.radiance = color;
  } else {
    if (subtype != "directional")
      report(VRTX_SEVERITY_WARNING,
          "light subtype '%s' is not supported; using directional",
          subtype.c_str());
    gpu.type = LIGHT_DIRECTIONAL;
    const f3 d =
        normalize(get<f3>("direction", VRTX_FLOAT32_VEC3, f3{0.f, 0.f, -1.f}));
    const float irr = std::min(std::max(get<float>("irradiance", VRTX_FLOAT32, 1.f), 0.f),
        3.402823466e+38f);
    gpu.dirToLight = -d; // transformed per instance at world build
    gpu.radiance = color * irr;
  }
}

bool Light::isValid() const
{
  if (gpu.type != LIGHT_HDRI)
    return true;
  return radiance && radiance->elemType == VRTX_FLOAT32_VEC3;
}

uint64_t Light::deepStamp() const
{
  return std::max(commitStamp, radiance ? radiance->deepStamp() : 0);
}

// HDRI::finalize / gpuData / generateCDFTables (HDRI.cu:98-170, 218-319):
// the radiance as a float4 texture (linear, x repeat, y clamp); luminance
// weighted by sin(theta) of each row; row sums; marginal and per-row
// conditional inclusive scans, normalised by their last entries; the pdf
// weight total / (2 pi^2 W H); the rotation rows (right, forward, up). The
// scans run here in order (the reference's device scans associate
// differently; the tables differ only by rounding).
bool Light::ensureBuilt()
{
  if (gpu.type != LIGHT_HDRI)
    return true;
  if (!isValid()) {
    if (radiance)
      report(VRTX_SEVERITY_WARNING, "HDRI radiance must be a FLOAT32_VEC3 Array2D");
    return false;
  }
  const uint64_t want = deepStamp();
  if (builtStamp && builtStamp >= want)
    return true;
  cleanup();
  const int W = (int)radiance->n[0], H = (int)radiance->n[1];
  if (W < 1 || H < 1)
    return false;
  std::vector<float> rgb((size_t)W * H * 3);
  if (const void *h = radiance->hostData())
    std::memcpy(rgb.data(), h, rgb.size() * sizeof(float));
  else {
    const void *d = radiance->deviceData();
    cudaStreamSynchronize(Object::dev->stream);
    cudaMemcpy(rgb.data(), d, rgb.size() * sizeof(float), cudaMemcpyDeviceToHost);
  }
  std::vector<float> lum((size_t)W * H), rowSums(H), cdf((size_t)H + (size_t)W * H);
  for (int y = 0; y < H; y++) {
    const float sinTheta = std::sin(float(M_PI) * (float(y) + 0.5f) / float(H));
    for (int x = 0; x < W; x++) {
      const float *p = &rgb[3 * ((size_t)y * W + x)];
      lum[(size_t)y * W + x] = sinTheta * (p[0] * 0.2126f + p[1] * 0.7152f + p[2] * 0.0722f);
    }
    float sum = 0.f;
    for (int x = 0; x < W; x++)
      sum += lum[(size_t)y * W + x];
    rowSums[y] = sum;
  }
  float *marginal = cdf.data(), *conditional = cdf.data() + H;
  float acc = 0.f;
  for (int y = 0; y < H; y++)
    marginal[y] = acc += rowSums[y];
  for (int y = 0; y < H; y++) {
    float r = 0.f;
    for (int x = 0; x < W; x++)
      conditional[(size_t)y * W + x] = r += lum[(size_t)y * W + x];
  }
  const float total = marginal[H - 1];
  gpu.pdfWeight = total / (2.0f * float(M_PI) * float(M_PI) * float(W) * float(H));
  for (int y = 0; y < H; y++)
    marginal[y] = marginal[y] / total;
  for (int y = 0; y < H; y++) {
    const float rowTotal = conditional[(size_t)y * W + W - 1];
    for (int x = 0; x < W; x++)
      conditional[(size_t)y * W + x] = conditional[(size_t)y * W + x] / rowTotal;
  }
  if (cudaMalloc(&cdfs, cdf.size() * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    cdfs = nullptr;
    return false;
  }
  cudaMemcpy(cdfs, cdf.data(), cdf.size() * sizeof(float), cudaMemcpyHostToDevice);
  std::vector<float> rgba((size_t)W * H * 4);
  for (size_t i = 0; i < (size_t)W * H; i++) {
    rgba[4 * i] = rgb[3 * i];
    rgba[4 * i + 1] = rgb[3 * i + 1];
    rgba[4 * i + 2] = rgb[3 * i + 2];
    rgba[4 * i + 3] = 1.f;
  }
  cudaChannelFormatDesc desc = cudaCreateChannelDesc(32, 32, 32, 32, cudaChannelFormatKindFloat);
  if (cudaMallocArray(&cuArray, &desc, W, H) != cudaSuccess) {
    cudaGetLastError();
    cuArray = nullptr;
    return false;
  }
  cudaMemcpy2DToArray(cuArray, 0, 0, rgba.data(), W * 16, W * 16, H, cudaMemcpyHostToDevice);
  cudaResourceDesc rd{};
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = cuArray;
  cudaTextureDesc td{};
  td.addressMode[0] = cudaAddressModeWrap;
  td.addressMode[1] = cudaAddressModeClamp;
  td.filterMode = cudaFilterModeLinear;
  td.readMode = cudaReadModeElementType;
  td.normalizedCoords = 1;
  cudaCreateTextureObject(&gpu.hdriTex, &rd, &td, nullptr);
  gpu.marginalCDF = cdfs;
  gpu.conditionalCDF = cdfs + H;
  gpu.hdriW = (uint32_t)W;
  gpu.hdriH = (uint32_t)H;
  // up = -normalize(up); forward = -normalize(cross(up, direction));
  // right = normalize(cross(forward, up)); rows (right, forward, up)
  const f3 up = -normalize(hdriUp);
  const f3 forward = -normalize(cross(up, hdriDirection));
  const f3 right = normalize(cross(forward, up));
  const f3 rows[3] = {right, forward, up};
  for (int r = 0; r < 3; r++) {
    gpu.hdriRot[3 * r] = rows[r].x;
    gpu.hdriRot[3 * r + 1] = rows[r].y;
    gpu.hdriRot[3 * r + 2] = rows[r].z;
  }
  builtStamp = want;
  return cudaGetLastError() == cudaSuccess;
}

// ---------------------------------------------------------------------------
// Surface (Surface.cpp:41-118)
// ---------------------------------------------------------------------------

void Surface::commit()
{
  id = get<uint32_t>("id", VRTX_UINT32, ~0u);
  geometry = static_cast<Geometry *>(getObject("geometry", VRTX_GEOMETRY));
  material = static_cast<Material *>(getObject("material", VRTX_MATERIAL));
  if (!material)
    report(VRTX_SEVERITY_WARNING, "missing 'material' on ANARISurface");
  if (!geometry)
    report(VRTX_SEVERITY_WARNING, "missing 'geometry' on ANARISurface");
}

bool Surface::isValid() const
{
  return geometry && material && geometry->isValid();
}

uint64_t Surface::deepStamp() const
{
  uint64_t s = commitStamp;
  if (geometry)
    s = std::max(s, geometry->deepStamp());
  if (material)
    s = std::max(s, material->deepStamp());
  return s;
}

// ---------------------------------------------------------------------------
// Group / Instance
// ---------------------------------------------------------------------------

static Array *objectArrayParam(Object *o, const char *name)
{
  auto *a = static_cast<Array *>(o->getObject(name, VRTX_ARRAY1D));
  if (a && !isObjectType(a->elemType))
    return nullptr;
  return a;
}

void Group::commit()
{
  surfaces = objectArrayParam(this, "surface");
  volumes = objectArrayParam(this, "volume");
  lights = objectArrayParam(this, "light");
}

template <typename T>
static std::vector<T *> validOf(Array *a, int type)
{
  std::vector<T *> out;
  if (!a)
    return out;
  for (Object *o : a->handles)
    if (o && o->type == type && o->isValid())
      out.push_back(static_cast<T *>(o));
  return out;
}

std::vector<Surface *> Group::validSurfaces() const
{
  return validOf<Surface>(surfaces, VRTX_SURFACE);
}
std::vector<Volume *> Group::validVolumes() const
{
  return validOf<Volume>(volumes, VRTX_VOLUME);
}
std::vector<Light *> Group::validLights() const
{
  return validOf<Light>(lights, VRTX_LIGHT);
}

uint64_t Group::deepStamp() const
{
  uint64_t s = commitStamp;
  for (Array *a : {surfaces, volumes, lights}) {
    if (!a)
      continue;
    s = std::max(s, a->deepStamp());
    for (Object *o : a->handles)
      if (o)
        s = std::max(s, o->deepStamp());
  }
  return s;
}

bool Group::getProperty(
    const std::string &name, int t, void *mem, uint64_t size, uint32_t mask)
{
  return Object::getProperty(name, t, mem, size, mask);
}

void Instance::commit()
{
  group = static_cast<Group *>(getObject("group", VRTX_GROUP));
  xfmArray = static_cast<Array *>(getObject("transform", VRTX_ARRAY1D));
  if (xfmArray && xfmArray->elemType != VRTX_FLOAT32_MAT4) {
    report(VRTX_SEVERITY_WARNING,
        "'transform' array elements need to be FLOAT32_MAT4");
    xfmArray = nullptr;
  }
  idArray = static_cast<Array *>(getObject("id", VRTX_ARRAY1D));
  if (idArray && idArray->elemType != VRTX_UINT32) {
    report(VRTX_SEVERITY_WARNING, "'id' array elements need to be UINT32");
    idArray = nullptr;
  }
  id = get<uint32_t>("id", VRTX_UINT32, ~0u);
  const float identity[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  std::memcpy(xfm, identity, sizeof(xfm));
  if (has("transform", VRTX_FLOAT32_MAT4)) {
    const float *m = reinterpret_cast<const float *>(params["transform"].bytes.data());
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 4; c++)
        xfm[r * 4 + c] = m[c * 4 + r];
  } else if (has("transform", VRTX_FLOAT32_MAT3x4)) {
    const float *m = reinterpret_cast<const float *>(params["transform"].bytes.data());
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 4; c++)
        xfm[r * 4 + c] = m[c * 3 + r];
  }
  if (!group)
    report(VRTX_SEVERITY_WARNING, "missing 'group' on ANARIInstance");
}

uint64_t Instance::deepStamp() const
{
  uint64_t s = commitStamp;
  if (group)
    s = std::max(s, group->deepStamp());
  if (xfmArray)
    s = std::max(s, xfmArray->deepStamp());
  if (idArray)
    s = std::max(s, idArray->deepStamp());
  return s;
}

size_t Instance::numTransforms() const
{
  return xfmArray ? (size_t)xfmArray->count() : 1;
}

void Instance::transform(size_t i, float out[12]) const
{
  if (xfmArray) {
    const float *m =
        reinterpret_cast<const float *>(xfmArray->hostData()) + 16 * i;
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 4; c++)
        out[r * 4 + c] = m[c * 4 + r];
  } else
    std::memcpy(out, xfm, sizeof(xfm));
}

uint32_t Instance::userID(size_t i) const
{
  if (xfmArray && idArray && i < idArray->count())
    return reinterpret_cast<const uint32_t *>(idArray->hostData())[i];
  return id;
}

static void invertAffine(const float m[12], xfm34 &out)
{
  const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6],
               g = m[8], h = m[9], k = m[10];
  const double A = e * k - f * h, B = -(d * k - f * g), C = d * h - e * g;
  double det = a * A + b * B + c * C;
  if (det == 0.0)
    det = 1e-30;
  const double inv[3][3] = {{A / det, -(b * k - c * h) / det, (b * f - c * e) / det},
      {B / det, (a * k - c * g) / det, -(a * f - c * d) / det},
      {C / det, -(a * h - b * g) / det, (a * e - b * d) / det}};
  const double t[3] = {m[3], m[7], m[11]};
  for (int r = 0; r < 3; r++) {
    for (int cc = 0; cc < 3; cc++)
      out.r[r][cc] = (float)inv[r][cc];
    out.r[r][3] =
        (float)(-(inv[r][0] * t[0] + inv[r][1] * t[1] + inv[r][2] * t[2]));
  }
}

// ---------------------------------------------------------------------------
// Spatial field (StructuredRegularField.cpp:64-192)
// ---------------------------------------------------------------------------

SpatialField::~SpatialField()
{
  cleanup();
}

void SpatialField::cleanup()
{
  if (tex)
    cudaDestroyTextureObject(tex);
  if (pointTex)
    cudaDestroyTextureObject(pointTex);
  if (cuArray)
    cudaFreeArray(cuArray);
  if (ranges)
    cudaFree(ranges);
  if (refRanges)
    cudaFree(refRanges);
  if (gridDev)
    cudaFree(gridDev);
  if (bricks)
    cudaFree(bricks);
  if (brickTable)
    cudaFree(brickTable);
  if (blockFill)
    cudaFree(blockFill);
  bricks = nullptr;
  brickTable = nullptr;
  blockFill = nullptr;
  tex = pointTex = 0;
  cuArray = nullptr;
  ranges = nullptr;
  refRanges = nullptr;
  gridDev = nullptr;
  nvdbGPU = NvdbGPU{};
  builtStamp = 0;
}

void SpatialField::commit()
{
  nanovdb = subtype == "nanovdb";
  if (nanovdb) {
    // NvdbRegularField::commitParameters (NvdbRegularField.cpp:63-67)
    filter = getString("filter", "linear");
    data = static_cast<Array *>(getObject("data", VRTX_ARRAY1D));
    // libvrtx tuning parameter: the brick cache (on by default)
    useBricks = get<int32_t>("vrtx.brickCache", VRTX_BOOL, 1) != 0;
    if (!data)
      report(VRTX_SEVERITY_WARNING,
          "missing required parameter 'data' on NanoVDB regular spatial field");
    else if (data->elemType != VRTX_UINT8)
      report(VRTX_SEVERITY_WARNING,
          "invalid data array type encountered in NanoVDB spatial field (%d)",
          data->elemType);
    builtStamp = 0;
    return;
  }
  if (subtype != "structuredRegular")
    report(VRTX_SEVERITY_WARNING,
        "spatial field subtype '%s' is not supported",
        subtype.c_str());
  origin = get<f3>("origin", VRTX_FLOAT32_VEC3, f3{0.f, 0.f, 0.f});
  spacing = get<f3>("spacing", VRTX_FLOAT32_VEC3, f3{1.f, 1.f, 1.f});
  filter = getString("filter", "linear");
  data = static_cast<Array *>(getObject("data", VRTX_ARRAY3D));
  if (!data)
    report(VRTX_SEVERITY_WARNING,
        "missing required parameter 'data' on structuredRegular spatial field");
  builtStamp = 0;
}

static bool validFieldType(int t)
{
  return t == VRTX_FIXED8 || t == VRTX_UFIXED8 || t == VRTX_FIXED16
      || t == VRTX_UFIXED16 || t == VRTX_FLOAT32;
}

bool SpatialField::isValid() const
{
  if (nanovdb)
    return data && data->elemType == VRTX_UINT8;
  return data && validFieldType(data->elemType);
}

uint64_t SpatialField::deepStamp() const
{
  return std::max(commitStamp, data ? data->deepStamp() : 0);
}

box3 SpatialField::bounds() const
{
  if (nanovdb)
    return gridBounds; // the grid's world bbox (NvdbRegularField.cpp:105-108)
  if (!isValid())
    return box3{{0.f, 0.f, 0.f}, {1.f, 1.f, 1.f}};
  return box3{origin,
      origin
          + f3{(float(data->n[0]) - 1.f) * spacing.x,
              (float(data->n[1]) - 1.f) * spacing.y,
              (float(data->n[2]) - 1.f) * spacing.z}};
}

float SpatialField::stepSize() const
{
  if (nanovdb) // NvdbRegularField::stepSize: compMin(voxelSize) / 2
    return std::min(gridVoxel.x, std::min(gridVoxel.y, gridVoxel.z)) / 2.f;
  return std::min(spacing.x / 2.f, std::min(spacing.y / 2.f, spacing.z / 2.f));
}

// Host-side check of a NanoVDB grid buffer before any kernel reads it: the
// header (magic, major version 32, one grid, a leaf codec the marcher
// dispatches: float, Fp4, Fp8, Fp16, FpN), and every root tile, internal
// slot and leaf the tree links to lying inside the buffer on a 32-byte
// boundary (NanoVDB's alignment), so the device walk never leaves it.
static bool checkNanovdb(
    const uint8_t *b, size_t size, std::string &why, std::vector<int32_t> *leafOrigins)
{
  auto rd64 = [&](size_t o) {
    uint64_t v;
    std::memcpy(&v, b + o, 8);
    return v;
  };
  auto rd32 = [&](size_t o) {
    uint32_t v;
    std::memcpy(&v, b + o, 4);
    return v;
  };
  if (size < 672 + 64 + 64) {
    why = "buffer smaller than a grid header";
    return false;
  }
  const uint64_t magic = rd64(0);
  if (magic != 0x304244566F6E614EULL && magic != 0x314244566F6E614EULL) {
    why = "not a NanoVDB grid (magic number)";
    return false;
  }
  if ((rd32(16) >> 21) != 32u) {
    why = "unsupported NanoVDB major version";
    return false;
  }
  if (rd32(28) != 1u) {
    why = "VisRTX NanoVDB support's a single grid per file";
    return false;
  }
  const uint32_t type = rd32(636);
  if (type != 1u && (type < 13u || type > 16u)) {
    why = "unsupported NanoVDB grid type (float, Fp4, Fp8, Fp16 and FpN are)";
    return false;
  }
  const uint64_t gridSize = rd64(32);
  if (gridSize > size) {
    why = "grid size exceeds the buffer";
    return false;
  }
  const int64_t rootOff = (int64_t)rd64(672 + 24);
  auto inside = [&](int64_t off, size_t len) {
    return off >= 0 && (off & 31) == 0 && (uint64_t)off + len <= gridSize;
  };
  const int64_t root = 672 + rootOff;
  if (!inside(root, 64)) {
    why = "root node outside the buffer";
    return false;
  }
  const uint32_t tiles = rd32(root + 24);
  if (!inside(root, 64 + 32ull * tiles)) {
    why = "root tiles outside the buffer";
    return false;
  }
  const size_t fixedLeaf = type == 1u ? 96 + 2048
      : type == 13u                   ? 96 + 256
      : type == 14u                   ? 96 + 512
      : type == 15u                   ? 96 + 1024
                                      : 0;
  for (uint32_t t = 0; t < tiles; t++) {
    const uint64_t key = rd64(root + 64 + 32 * t);
    const int64_t child = (int64_t)rd64(root + 64 + 32 * t + 8);
    if (!child)
      continue;
    // RootData::KeyToCoord: 21 bits per axis, x highest
    const int32_t ux = int32_t(uint32_t((key >> 42) & 0x1FFFFF) << 12);
    const int32_t uy = int32_t(uint32_t((key >> 21) & 0x1FFFFF) << 12);
    const int32_t uz = int32_t(uint32_t(key & 0x1FFFFF) << 12);
    const int64_t up = root + child;
    if (!inside(up, 270400)) {
      why = "upper node outside the buffer";
      return false;
    }
    for (uint32_t nu = 0; nu < 32768; nu++) {
      if (!((rd64(up + 4128 + 8 * (nu >> 6)) >> (nu & 63)) & 1))
        continue;
      const int64_t lo = up + (int64_t)rd64(up + 8256 + 8 * nu);
      if (!inside(lo, 33856)) {
        why = "lower node outside the buffer";
        return false;
      }
      for (uint32_t nl = 0; nl < 4096; nl++) {
        if (!((rd64(lo + 544 + 8 * (nl >> 6)) >> (nl & 63)) & 1))
          continue;
        const int64_t leaf = lo + (int64_t)rd64(lo + 1088 + 8 * nl);
        if (!inside(leaf, 96)) {
          why = "leaf outside the buffer";
          return false;
        }
        const size_t len = fixedLeaf ? fixedLeaf : 96 + (64u << (b[leaf + 15] >> 5));
        if ((b[leaf + 15] >> 5) > 4 || !inside(leaf, len)) {
          why = "leaf outside the buffer";
          return false;
        }
        if (leafOrigins) {
          leafOrigins->push_back(ux + int32_t(((nu >> 10) & 31u) << 7) + int32_t(((nl >> 8) & 15u) << 3));
          leafOrigins->push_back(uy + int32_t(((nu >> 5) & 31u) << 7) + int32_t(((nl >> 4) & 15u) << 3));
          leafOrigins->push_back(uz + int32_t((nu & 31u) << 7) + int32_t((nl & 15u) << 3));
        }
      }
    }
  }
  return true;
}

// NvdbRegularField::finalize / buildGrid (NvdbRegularField.cpp:69-149): the
// grid copied to device memory, the bounds and voxel size from its header,
// and the delta-tracking grid over its index bbox.
bool SpatialField::buildNanovdb()
{
  cudaStream_t s = Object::dev->stream;
  const size_t size = data->bytes();
  std::vector<uint8_t> host(size);
  if (const void *h = data->hostData())
    std::memcpy(host.data(), h, size);
  else if (const void *d = data->deviceData()) {
    cudaStreamSynchronize(s);
    cudaMemcpy(host.data(), d, size, cudaMemcpyDeviceToHost);
  } else
    return false;
  std::string why;
  std::vector<int32_t> origins;
  if (!checkNanovdb(host.data(), size, why, &origins)) {
    report(VRTX_SEVERITY_WARNING, "NanoVDB spatial field: %s", why.c_str());
    return false;
  }
  if (cudaMalloc(&gridDev, size) != cudaSuccess) {
    cudaGetLastError();
    gridDev = nullptr;
    report(VRTX_SEVERITY_ERROR, "device allocation of %zu bytes failed", size);
    return false;
  }
  cudaMemcpyAsync(gridDev, host.data(), size, cudaMemcpyHostToDevice, s);
  auto rdf = [&](size_t o) {
    float v;
    std::memcpy(&v, host.data() + o, 4);
    return v;
  };
  auto rdd = [&](size_t o) {
    double v;
    std::memcpy(&v, host.data() + o, 8);
    return v;
  };
  auto rdi = [&](size_t o) {
    int32_t v;
    std::memcpy(&v, host.data() + o, 4);
    return v;
  };
  int64_t rootOff;
  std::memcpy(&rootOff, host.data() + 672 + 24, 8);
  const size_t root = 672 + (size_t)rootOff;
  nvdbGPU.root = gridDev + root;
  std::memcpy(&nvdbGPU.type, host.data() + 636, 4);
  std::memcpy(&nvdbGPU.tiles, host.data() + root + 24, 4);
  nvdbGPU.background = rdf(root + 28);
  for (int k = 0; k < 9; k++)
    nvdbGPU.inv[k] = rdf(296 + 36 + 4 * k);
  for (int k = 0; k < 3; k++)
    nvdbGPU.vec[k] = rdf(296 + 72 + 4 * k);
  gridBounds = box3{{float(rdd(560)), float(rdd(568)), float(rdd(576))},
      {float(rdd(584)), float(rdd(592)), float(rdd(600))}};
  gridVoxel = f3{float(rdd(608)), float(rdd(616)), float(rdd(624))};
  for (int k = 0; k < 3; k++)
    dims[k] = rdi(root + 12 + 4 * k) - rdi(root + 4 * k) + 1; // indexBBox().dim()
  mcDims[0] = (dims[0] + 15) / 16;
  mcDims[1] = (dims[1] + 15) / 16;
  mcDims[2] = (dims[2] + 15) / 16;
  const size_t cells = (size_t)mcDims[0] * mcDims[1] * mcDims[2];
  if (cudaMalloc(&refRanges, 2 * cells * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    refRanges = nullptr;
    return false;
  }
  if (useBricks)
    buildNanovdbBricks(origins);
  launchReferenceGridRangesNanovdb(nvdbGPU, gridBounds, mcDims, refRanges, s);
  return cudaGetLastError() == cudaSuccess;
}

// The brick cache of a NanoVDB field, a dense table over leaf-block
// coordinates (the blocks of every leaf plus one block below on each axis,
// x fastest) whose entries are
//   slot >= 0  a brick: the block's 8^3 values and the one-voxel apron on
//              the +x/+y/+z sides, 9^3 floats with x slowest;
//   -2         a block whose 9^3 region holds one value (in blockFill);
// every value produced by the device tree walk itself. A stencil then reads
// one brick (or one value) whatever leaves or tiles it straddles, with the
// walk's values bit for bit. Leaf blocks get bricks; other blocks are
// classified on the device and get a brick only where their region is not
// constant. Skipped (the sampler walks the tree) when the table would exceed
// 2^26 entries or the bricks do not fit.
void SpatialField::buildNanovdbBricks(const std::vector<int32_t> &origins)
{
  const size_t n = origins.size() / 3;
  if (!n)
    return;
  int32_t lo[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, hi[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
  for (size_t i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) {
      lo[k] = std::min(lo[k], (origins[3 * i + k] >> 3) - 1);
      hi[k] = std::max(hi[k], origins[3 * i + k] >> 3);
    }
  const size_t dims[3] = {size_t(hi[0] - lo[0] + 1), size_t(hi[1] - lo[1] + 1),
      size_t(hi[2] - lo[2] + 1)};
  const size_t entries = dims[0] * dims[1] * dims[2];
  if (entries > (size_t(1) << 26))
    return;
  std::vector<int32_t> table(entries, kBlockUnclassified);
  for (size_t i = 0; i < n; i++) {
    const size_t bx = size_t((origins[3 * i] >> 3) - lo[0]);
    const size_t by = size_t((origins[3 * i + 1] >> 3) - lo[1]);
    const size_t bz = size_t((origins[3 * i + 2] >> 3) - lo[2]);
    table[(bz * dims[1] + by) * dims[0] + bx] = int32_t(i);
  }
  cudaStream_t s = Object::dev->stream;
  auto fail = [&]() {
    cudaGetLastError();
    report(VRTX_SEVERITY_PERFORMANCE_WARNING,
        "NanoVDB brick cache not built; sampling walks the tree");
    for (void *p : {(void *)brickTable, (void *)bricks, (void *)blockFill})
      if (p)
        cudaFree(p);
    brickTable = nullptr;
    bricks = nullptr;
    blockFill = nullptr;
  };
  if (cudaMalloc(&brickTable, entries * sizeof(int32_t)) != cudaSuccess
      || cudaMalloc(&blockFill, entries * sizeof(float)) != cudaSuccess) {
    fail();
    return;
  }
  NvdbGPU g = nvdbGPU;
  for (int k = 0; k < 3; k++) {
    g.blockLo[k] = lo[k];
    g.blockDims[k] = (int)dims[k];
  }
  // classify the blocks without a leaf: constant region or brick
  cudaMemcpyAsync(brickTable, table.data(), entries * sizeof(int32_t), cudaMemcpyHostToDevice, s);
  launchNanovdbClassifyBlocks(g, (uint32_t)entries, brickTable, blockFill, s);
  cudaMemcpyAsync(table.data(), brickTable, entries * sizeof(int32_t), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  std::vector<int32_t> brickOrigins(origins);
  for (size_t e = 0; e < entries; e++) {
    if (table[e] != kBlockNeedsBrick)
      continue;
    table[e] = int32_t(brickOrigins.size() / 3);
    const size_t bx = e % dims[0], by = (e / dims[0]) % dims[1], bz = e / (dims[0] * dims[1]);
    brickOrigins.push_back((lo[0] + int32_t(bx)) * 8);
    brickOrigins.push_back((lo[1] + int32_t(by)) * 8);
    brickOrigins.push_back((lo[2] + int32_t(bz)) * 8);
  }
  const size_t slots = brickOrigins.size() / 3;
  int32_t *dOrigins = nullptr;
  if (cudaMalloc(&bricks, slots * 729 * sizeof(float)) != cudaSuccess
      || cudaMalloc(&dOrigins, brickOrigins.size() * sizeof(int32_t)) != cudaSuccess) {
    if (dOrigins)
      cudaFree(dOrigins);
    fail();
    return;
  }
  cudaMemcpyAsync(brickTable, table.data(), entries * sizeof(int32_t), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dOrigins,
      brickOrigins.data(),
      brickOrigins.size() * sizeof(int32_t),
      cudaMemcpyHostToDevice,
      s);
  launchNanovdbBricks(nvdbGPU, dOrigins, (uint32_t)slots, bricks, s);
  cudaStreamSynchronize(s);
  cudaFree(dOrigins);
  g.bricks = bricks;
  g.brickTable = brickTable;
  g.blockFill = blockFill;
  nvdbGPU = g;
}

bool SpatialField::ensureBuilt()
{
  if (!isValid())
    return false;
  const uint64_t want = deepStamp();
  if (builtStamp && builtStamp >= want)
    return true;
  cleanup();
  if (nanovdb) {
    if (!buildNanovdb())
      return false;
    builtStamp = want;
    return true;
  }
  cudaStream_t s = Object::dev->stream;
  const int et = data->elemType;
  dims[0] = (int)data->n[0];
  dims[1] = (int)data->n[1];
  dims[2] = (int)data->n[2];
  const int bits = (int)sizeOfType(et) * 8;
  const cudaChannelFormatKind kind = et == VRTX_FLOAT32
      ? cudaChannelFormatKindFloat
      : ((et == VRTX_UFIXED8 || et == VRTX_UFIXED16)
              ? cudaChannelFormatKindUnsigned
              : cudaChannelFormatKindSigned);
  cudaChannelFormatDesc desc = cudaCreateChannelDesc(bits, 0, 0, 0, kind);
  if (cudaMalloc3DArray(&cuArray, &desc, make_cudaExtent(dims[0], dims[1], dims[2]))
      != cudaSuccess) {
    cudaGetLastError();
    report(VRTX_SEVERITY_ERROR, "cudaMalloc3DArray failed for field data");
    cuArray = nullptr;
    return false;
  }
  // host-resident voxels go straight into the texture array (no linear
  // device copy); device and other-GPU arrays are copied from device memory
  cudaMemcpy3DParms cp{};
  const void *host = data->hostData();
  const void *src = host ? host : data->deviceData();
  if (!src) {
    report(VRTX_SEVERITY_ERROR, "field data is not readable");
    return false;
  }
  cp.srcPtr = make_cudaPitchedPtr(const_cast<void *>(src),
      dims[0] * sizeOfType(et),
      dims[0],
      dims[1]);
  cp.dstArray = cuArray;
  cp.extent = make_cudaExtent(dims[0], dims[1], dims[2]);
  cp.kind = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  cudaMemcpy3DAsync(&cp, s);
  if (host && data->appMem)
    data->hostReadQueued = true;
  cudaResourceDesc rd{};
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = cuArray;
  cudaTextureDesc td{};
  td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
  td.filterMode = filter == "nearest" ? cudaFilterModePoint : cudaFilterModeLinear;
  td.readMode = et == VRTX_FLOAT32 ? cudaReadModeElementType
                                   : cudaReadModeNormalizedFloat;
  td.normalizedCoords = 1;
  cudaCreateTextureObject(&tex, &rd, &td, nullptr);
  cudaTextureDesc tp = td;
  tp.filterMode = cudaFilterModePoint;
  tp.normalizedCoords = 0;
  cudaCreateTextureObject(&pointTex, &rd, &tp, nullptr);
  mcDims[0] = (dims[0] + 15) / 16;
  mcDims[1] = (dims[1] + 15) / 16;
  mcDims[2] = (dims[2] + 15) / 16;
  const size_t cells = (size_t)mcDims[0] * mcDims[1] * mcDims[2];
  if (cudaMalloc(&ranges, 2 * cells * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    ranges = nullptr;
    return false;
  }
  launchMacrocellRanges(pointTex, dims, mcDims, ranges, s);
  if (cudaMalloc(&refRanges, 2 * cells * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    refRanges = nullptr;
    return false;
  }
  const f3 invSpacing{1.f / (spacing.x * float(dims[0])),
      1.f / (spacing.y * float(dims[1])),
      1.f / (spacing.z * float(dims[2]))};
  launchReferenceGridRanges(
      tex, origin, spacing, invSpacing, bounds(), mcDims, refRanges, s);
  builtStamp = want;
  return cudaGetLastError() == cudaSuccess;
}

// ---------------------------------------------------------------------------
// Volume: transferFunction1D / scivis (scene/volume/TransferFunction1D.cpp,
// utility/colorMapHelpers.h)
// ---------------------------------------------------------------------------

Volume::~Volume()
{
  cleanup();
}

void Volume::cleanup()
{
  if (tfTex)
    cudaDestroyTextureObject(tfTex);
  if (tfArray)
    cudaFreeArray(tfArray);
  if (tfDev)
    cudaFree(tfDev);
  if (majorants)
    cudaFree(majorants);
  if (dptMajorants)
    cudaFree(dptMajorants);
  tfTex = 0;
  tfArray = nullptr;
  tfDev = nullptr;
  majorants = nullptr;
  dptMajorants = nullptr;
  builtStamp = 0;
}

void Volume::commit()
{
  if (subtype != "transferFunction1D" && subtype != "scivis")
    report(VRTX_SEVERITY_WARNING,
        "volume subtype '%s' is not supported",
        subtype.c_str());
  id = get<uint32_t>("id", VRTX_UINT32, ~0u);
  // "vrtx.emptySpaceSkipping" false: march every sample with a fetch (the
  // plain fixed-step loop); results are the same either way
  emptySpaceSkipping = get<int32_t>("vrtx.emptySpaceSkipping", VRTX_BOOL, 1) != 0;
  field = static_cast<SpatialField *>(getObject("value", VRTX_SPATIAL_FIELD));
  color = static_cast<Array *>(getObject("color", VRTX_ARRAY1D));
  opacity = static_cast<Array *>(getObject("opacity", VRTX_ARRAY1D));
  float uc[4] = {1.f, 1.f, 1.f, 1.f};
  if (has("color", VRTX_FLOAT32_VEC3))
    std::memcpy(uc, params["color"].bytes.data(), 12);
  if (has("color", VRTX_FLOAT32_VEC4))
    std::memcpy(uc, params["color"].bytes.data(), 16);
  uniformColor = f3{uc[0], uc[1], uc[2]};
  uniformColorW = uc[3];
  uniformOpacity = get<float>("opacity", VRTX_FLOAT32, 1.f) * uc[3];
  unitDistance = get<float>("unitDistance", VRTX_FLOAT32, 1.f);
  if (has("valueRange", VRTX_FLOAT32_VEC2) || has("valueRange", VRTX_FLOAT32_BOX1)) {
    const auto &b = params.count("valueRange") ? params["valueRange"].bytes
                                               : std::vector<uint8_t>();
    std::memcpy(valueRange, b.data(), 8);
  }
  if (has("valueRange", VRTX_FLOAT64_BOX1)) {
    double d[2];
    std::memcpy(d, params["valueRange"].bytes.data(), 16);
    valueRange[0] = float(d[0]);
    valueRange[1] = float(d[1]);
  }
  if (!field)
    report(VRTX_SEVERITY_WARNING,
        "missing parameter 'value' on transferFunction1D ANARIVolume");
  builtStamp = 0;
}

bool Volume::isValid() const
{
  return field && field->isValid();
}

uint64_t Volume::deepStamp() const
{
  uint64_t s = commitStamp;
  if (field)
    s = std::max(s, field->deepStamp());
  if (color)
    s = std::max(s, color->deepStamp());
  if (opacity)
    s = std::max(s, opacity->deepStamp());
  return s;
}

// position(v, r) (gpu_math.h): clamp, then (v - lo) * (1 / size)
static float positionIn(float v, float lo, float hi)
{
  v = std::max(lo, std::min(v, hi));
  return (v - lo) * (1.f / (hi - lo));
}

// generateLinearPositions (colorMapHelpers.h:43-61)
static std::vector<float> linearPositions(size_t n, float lo, float hi)
{
  std::vector<float> p(n);
  p.front() = 0.f;
  p.back() = 1.f;
  const float w = 1.f / float(n - 1);
  for (size_t i = 1; i + 1 < n; i++)
    p[i] = p[i - 1] + w;
  for (auto &v : p)
    v = v * (hi - lo) + lo;
  return p;
}

// getInterpolatedValue (colorMapHelpers.h:63-73) on nc-component values
static void interpolated(const float *values,
    int nc,
    const std::vector<float> &pos,
    float lo,
    float hi,
    float p,
    float *out)
{
  for (size_t i = 0; i + 1 < pos.size(); i++) {
    const float a = positionIn(pos[i], lo, hi);
    const float b = positionIn(pos[i + 1], lo, hi);
    if (p >= a && p <= b) {
      const float t = positionIn(p, a, b);
      for (int c = 0; c < nc; c++)
        out[c] = values[i * nc + c] * (1.f - t) + values[(i + 1) * nc + c] * t;
      return;
    }
  }
  const size_t k = p <= positionIn(pos[0], lo, hi) ? 0 : pos.size() - 1;
  for (int c = 0; c < nc; c++)
    out[c] = values[k * nc + c];
}

// discritizeTFData (TransferFunction1D.cpp:101-150): n entries sampled at
// i / (n - 1), entry = (rgb, c.w * o); the colour array (nc = 3 or 4
// components) or the opacity array may be absent (NULL), and the uniform
// colour / opacity stand in for it.
static void discretizeTF(const float *cvals,
    int numColor,
    int nc,
    const float *ovals,
    int numOpacity,
    float lo,
    float hi,
    const float uniformColor[4],
    float uniformOpacity,
    int n,
    float *out)
{
  std::vector<float> cpos, opos;
  if (cvals)
    cpos = linearPositions((size_t)numColor, lo, hi);
  if (ovals)
    opos = linearPositions((size_t)numOpacity, lo, hi);
  for (int i = 0; i < n; i++) {
    const float p = float(i) / float(n - 1);
    float c[4] = {uniformColor[0], uniformColor[1], uniformColor[2], uniformColor[3]};
    if (cvals) {
      float v[4] = {0.f, 0.f, 0.f, 1.f};
      interpolated(cvals, nc, cpos, lo, hi, p, v);
      c[0] = v[0];
      c[1] = v[1];
      c[2] = v[2];
      c[3] = nc == 4 ? v[3] : 1.f;
    }
    float o = uniformOpacity;
    if (ovals)
      interpolated(ovals, 1, opos, lo, hi, p, &o);
    out[4 * i + 0] = c[0];
    out[4 * i + 1] = c[1];
    out[4 * i + 2] = c[2];
    out[4 * i + 3] = c[3] * o;
  }
}

void Volume::discretize()
{
  const int N = 256;
  tf.assign(N * 4, 0.f);
  const float *cvals = nullptr;
  int cnc = 0;
  if (color && color->count() >= 2
      && (color->elemType == VRTX_FLOAT32_VEC3
          || color->elemType == VRTX_FLOAT32_VEC4)) {
    cvals = reinterpret_cast<const float *>(color->hostData());
    cnc = color->elemType == VRTX_FLOAT32_VEC3 ? 3 : 4;
  } else if (color)
    report(VRTX_SEVERITY_WARNING, "unusable tf1D color array type set");
  const float *ovals = nullptr;
  if (opacity && opacity->count() >= 2 && opacity->elemType == VRTX_FLOAT32)
    ovals = reinterpret_cast<const float *>(opacity->hostData());
  const float uc[4] = {uniformColor.x, uniformColor.y, uniformColor.z, uniformColorW};
  discretizeTF(cvals,
      cvals ? (int)color->count() : 0,
      cnc,
      ovals,
      ovals ? (int)opacity->count() : 0,
      valueRange[0],
      valueRange[1],
      uc,
      uniformOpacity,
      N,
      tf.data());
}

bool Volume::ensureBuilt()
{
  if (!isValid() || !field->ensureBuilt())
    return false;
  const uint64_t want = deepStamp();
  if (builtStamp && builtStamp >= want)
    return true;
  cleanup();
  cudaStream_t s = Object::dev->stream;
  const bool hasTF = color != nullptr || opacity != nullptr;
  if (hasTF) {
    discretize();
    cudaChannelFormatDesc desc =
        cudaCreateChannelDesc(32, 32, 32, 32, cudaChannelFormatKindFloat);
    if (cudaMallocArray(&tfArray, &desc, 256) != cudaSuccess) {
      cudaGetLastError();
      tfArray = nullptr;
      return false;
    }
    cudaMemcpy2DToArrayAsync(tfArray,
        0,
        0,
        tf.data(),
        256 * sizeof(float4),
        256 * sizeof(float4),
        1,
        cudaMemcpyHostToDevice,
        s);
    cudaResourceDesc rd{};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = tfArray;
    cudaTextureDesc td{};
    td.addressMode[0] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    cudaCreateTextureObject(&tfTex, &rd, &td, nullptr);
    cudaMalloc(&tfDev, 256 * sizeof(float4));
    cudaMemcpyAsync(
        tfDev, tf.data(), 256 * sizeof(float4), cudaMemcpyHostToDevice, s);
  }
  const size_t cells =
      (size_t)field->mcDims[0] * field->mcDims[1] * field->mcDims[2];
  hasEmptyCells = false;
  if (!field->ranges) {
    // no skipping grid (NanoVDB fields): only the delta-tracking majorants
    if (cudaMalloc(&dptMajorants, cells * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      dptMajorants = nullptr;
      return false;
    }
    launchReferenceMajorants(
        field->refRanges, field->mcDims, tfTex, 256, uniformOpacity, dptMajorants, s);
    builtStamp = want;
    return cudaGetLastError() == cudaSuccess;
  }
  if (cudaMalloc(&majorants, cells * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    majorants = nullptr;
    return false;
  }
  unsigned *dEmpty = nullptr;
  unsigned empty = 0;
  if (cudaMalloc(&dEmpty, sizeof(unsigned)) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cudaMemsetAsync(dEmpty, 0, sizeof(unsigned), s);
  launchMacrocellMajorants(field->ranges,
      field->mcDims,
      tfDev,
      256,
      valueRange[0],
      valueRange[1],
      uniformOpacity,
      majorants,
      dEmpty,
      s);
  cudaMemcpyAsync(&empty, dEmpty, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  cudaFree(dEmpty);
  // without empty cells the skipping grid never skips: the marcher then
  // does not consult it
  hasEmptyCells = empty > 0;
  if (cudaMalloc(&dptMajorants, cells * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    dptMajorants = nullptr;
    return false;
  }
  launchReferenceMajorants(
      field->refRanges, field->mcDims, tfTex, 256, uniformOpacity, dptMajorants, s);
  builtStamp = want;
  return cudaGetLastError() == cudaSuccess;
}

// ---------------------------------------------------------------------------
// World (scene/World.cpp:100-442, Group.cpp:189-266, optix_visrtx.cpp)
// ---------------------------------------------------------------------------

World::~World()
{
  freeBuilt();
  if (zeroInstance)
    releaseObj(zeroInstance);
  if (zeroGroup)
    releaseObj(zeroGroup);
}

void World::commit()
{
  instances = objectArrayParam(this, "instance");
  zeroSurfaces = objectArrayParam(this, "surface");
  zeroVolumes = objectArrayParam(this, "volume");
  zeroLights = objectArrayParam(this, "light");
  id = get<uint32_t>("id", VRTX_UINT32, ~0u);
  // libvrtx tuning parameters: primitives per BVH8 leaf slot (1..3)
  maxLeaf[GEOM_TRIANGLE] = get<int32_t>("vrtx.maxLeafTriangles", VRTX_INT32, 1);
  maxLeaf[GEOM_SPHERE] = get<int32_t>("vrtx.maxLeafSpheres", VRTX_INT32, 1);
  if (!zeroGroup) {
    zeroGroup = new Group(Object::dev, VRTX_GROUP);
    zeroInstance = new Instance(Object::dev, VRTX_INSTANCE, "transform");
  }
  zeroGroup->surfaces = zeroSurfaces;
  zeroGroup->volumes = zeroVolumes;
  zeroGroup->lights = zeroLights;
  zeroGroup->commitStamp = commitStamp;
  zeroInstance->group = zeroGroup;
  zeroInstance->id = id;
  const float identity[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  std::memcpy(zeroInstance->xfm, identity, sizeof(identity));
  zeroInstance->commitStamp = commitStamp;
  builtStamp = 0;
}

std::vector<Instance *> World::instanceList() const
{
  std::vector<Instance *> out;
  if (instances)
    for (Object *o : instances->handles)
      if (o && o->type == VRTX_INSTANCE && o->isValid())
        out.push_back(static_cast<Instance *>(o));
  if (zeroGroup && (zeroSurfaces || zeroVolumes || zeroLights))
    out.push_back(zeroInstance);
  return out;
}

uint64_t World::deepStamp() const
{
  uint64_t s = commitStamp;
  if (instances) {
    s = std::max(s, instances->deepStamp());
    for (Object *o : instances->handles)
      if (o)
        s = std::max(s, o->deepStamp());
  }
  if (zeroGroup)
    s = std::max(s, zeroGroup->deepStamp());
  return s;
}

void World::freeBuilt()
{
  cudaStream_t s = Object::dev->stream;
  for (auto &b : blases) {
    freeBVH8(b.bvh, s);
    if (b.records)
      cudaFreeAsync(b.records, s);
  }
  blases.clear();
  freeBVH8(tlas, s);
  for (void *p : allocations)
    cudaFreeAsync(p, s);
  allocations.clear();
  gpu = WorldGPU{};
  builtStamp = 0;
}

template <typename T>
static T *uploadVec(World *w, const std::vector<T> &v, cudaStream_t s)
{
  if (v.empty())
    return nullptr;
  T *p = nullptr;
  if (cudaMallocAsync((void **)&p, sizeof(T) * v.size(), s) != cudaSuccess)
    return nullptr;
  cudaMemcpyAsync(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s);
  w->allocations.push_back(p);
  return p;
}

static box3 xfmBox(const float m[12], const box3 &b)
{
  box3 o = emptyBox();
  for (int i = 0; i < 8; i++) {
    const f3 p{(i & 1) ? b.hi.x : b.lo.x,
        (i & 2) ? b.hi.y : b.lo.y,
        (i & 4) ? b.hi.z : b.lo.z};
    const f3 q{m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3],
        m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
        m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]};
    extend(o, q);
  }
  return o;
}

bool World::rebuild()
{
  const auto t0 = std::chrono::steady_clock::now();
  cudaStream_t s = Object::dev->stream;
  freeBuilt();
  const auto insts = instanceList();

  std::vector<Surface *> surfaces;
  std::map<Surface *, uint32_t> surfIdx;
  std::vector<Geometry *> geoms;
  std::map<Geometry *, uint32_t> geomIdx;
  std::vector<Material *> mats;
  std::map<Material *, uint32_t> matIdx;
  std::vector<Group *> groups;
  std::map<Group *, std::vector<Surface *>> groupSurfaces;
  for (Instance *inst : insts) {
    Group *g = inst->group;
    if (groupSurfaces.count(g))
      continue;
    groups.push_back(g);
    auto ss = g->validSurfaces();
    groupSurfaces[g] = ss;
    for (Surface *sf : ss) {
      if (surfIdx.count(sf))
        continue;
      surfIdx[sf] = (uint32_t)surfaces.size();
      surfaces.push_back(sf);
      if (!geomIdx.count(sf->geometry)) {
        geomIdx[sf->geometry] = (uint32_t)geoms.size();
        geoms.push_back(sf->geometry);
      }
      if (!matIdx.count(sf->material)) {
        matIdx[sf->material] = (uint32_t)mats.size();
        mats.push_back(sf->material);
      }
    }
  }

  std::vector<GeometryGPU> hGeoms;
  for (Geometry *g : geoms)
    hGeoms.push_back(g->gpuData());
  std::vector<MaterialGPU> hMats;
  std::vector<SamplerGPU> hSamplers;
  std::map<Sampler *, uint32_t> samplerIdx;
  auto samplerSlot = [&](Sampler *sm) -> uint32_t {
    if (!sm || !sm->isValid() || !sm->ensureBuilt())
      return ~0u;
    auto it = samplerIdx.find(sm);
    if (it != samplerIdx.end())
      return it->second;
    const uint32_t k = (uint32_t)hSamplers.size();
    samplerIdx[sm] = k;
    hSamplers.push_back(sm->gpuData());
    return k;
  };
  bool allOpaque = true, allMatte = true;
  for (Material *m : mats) {
    MaterialGPU mg = m->gpu;
    for (int k = 0; k < MP_COUNT; k++) {
      if (mg.params[k].src != PARAM_SAMPLER)
        continue;
      mg.params[k].sampler = samplerSlot(m->samplers[k]);
      if (mg.params[k].sampler == ~0u)
        mg.params[k].src = PARAM_VALUE;
    }
    hMats.push_back(mg);
    if (m->gpu.alphaMode != ALPHA_OPAQUE)
      allOpaque = false;
    if (m->gpu.type == MATERIAL_PBR)
      allMatte = false;
  }
  std::vector<SurfaceGPU> hSurfs;
  for (Surface *sf : surfaces)
    hSurfs.push_back(SurfaceGPU{
        geomIdx[sf->geometry], matIdx[sf->material], sf->id, 0u});
  GeometryGPU *dGeoms = uploadVec(this, hGeoms, s);
  MaterialGPU *dMats = uploadVec(this, hMats, s);
  SamplerGPU *dSamplers = hSamplers.empty() ? nullptr : uploadVec(this, hSamplers, s);
  SurfaceGPU *dSurfs = uploadVec(this, hSurfs, s);

  // BLAS per (group, primitive class)
  std::map<Group *, std::array<int, GEOM_NUM_TYPES>> groupBlas;
  std::vector<BLASDesc> hBlas;
  for (Group *g : groups) {
    std::array<int, GEOM_NUM_TYPES> ids;
    ids.fill(-1);
    for (int cls = 0; cls < GEOM_NUM_TYPES; cls++) {
      uint32_t n = 0;
      for (Surface *sf : groupSurfaces[g])
        if (sf->geometry->geomClass() == cls)
          n += sf->geometry->numPrims;
      if (n == 0)
        continue;
      uint2 *refs = nullptr;
      box3 *boxes = nullptr;
      cudaMallocAsync((void **)&refs, sizeof(uint2) * n, s);
      cudaMallocAsync((void **)&boxes, sizeof(box3) * n, s);
      uint32_t off = 0;
      for (Surface *sf : groupSurfaces[g]) {
        if (sf->geometry->geomClass() != cls)
          continue;
        launchFillRefs(surfIdx[sf], sf->geometry->numPrims, refs + off, s);
        off += sf->geometry->numPrims;
      }
      if (cls == GEOM_TRIANGLE)
        launchTriangleBoxes(dGeoms, refs, dSurfs, n, boxes, s);
      else if (cls == GEOM_SPHERE)
        launchSphereBoxes(dGeoms, refs, dSurfs, n, boxes, s);
      else
        launchSegmentBoxes(dGeoms, refs, dSurfs, n, boxes, s);
      BLASBuild b;
      b.type = (uint32_t)cls;
      b.numPrims = n;
      cudaError_t err = buildBVH8(boxes, n, s, b.bvh, maxLeaf[cls]);
      if (err == cudaSuccess) {
        const size_t recBytes = cls == GEOM_TRIANGLE
            ? sizeof(TriRecord)
            : (cls == GEOM_SPHERE ? sizeof(SphereRecord) : sizeof(SegRecord));
        cudaMallocAsync(&b.records, recBytes * b.bvh.numPrims, s);
        if (cls == GEOM_TRIANGLE)
          launchGatherTriangles(dGeoms,
              refs,
              dSurfs,
              b.bvh.primOrder,
              b.bvh.numPrims,
              (TriRecord *)b.records,
              s);
        else if (cls == GEOM_SPHERE)
          launchGatherSpheres(dGeoms,
              refs,
              dSurfs,
              b.bvh.primOrder,
              b.bvh.numPrims,
              (SphereRecord *)b.records,
              s);
        else
          launchGatherSegments(dGeoms,
              refs,
              dSurfs,
              b.bvh.primOrder,
              b.bvh.numPrims,
              (SegRecord *)b.records,
              s);
      }
      cudaFreeAsync(refs, s);
      cudaFreeAsync(boxes, s);
      if (err != cudaSuccess) {
        report(VRTX_SEVERITY_ERROR,
            "BVH build failed: %s",
            cudaGetErrorString(err));
        cudaGetLastError();
        continue;
      }
      ids[cls] = (int)hBlas.size();
      BLASDesc d{};
      d.nodes = b.bvh.nodes;
      d.prims = b.records;
      d.type = b.type;
      d.numPrims = b.bvh.numPrims;
      d.bounds = b.bvh.bounds;
      hBlas.push_back(d);
      blases.push_back(b);
    }
    groupBlas[g] = ids;
  }
  BLASDesc *dBlas = uploadVec(this, hBlas, s);

  // top level: one record per (instance, transform, class)
  std::vector<InstanceRecord> recs;
  std::vector<box3> recBoxes;
  std::vector<LightGPU> lights;
  int hdriIndex = -1;
  std::vector<VolumeGPU> vols;
  worldBounds = emptyBox();
  for (Instance *inst : insts) {
    Group *g = inst->group;
    const auto ids = groupBlas[g];
    const auto gl = g->validLights();
    const auto gv = g->validVolumes();
    for (size_t t = 0; t < inst->numTransforms(); t++) {
      float m[12];
      inst->transform(t, m);
      InstanceRecord r{};
      invertAffine(m, r.worldToObject);
      for (int i = 0; i < 12; i++)
        r.objectToWorld.r[i / 4][i % 4] = m[i];
      r.userId = inst->userID(t);
      for (int cls = 0; cls < GEOM_NUM_TYPES; cls++) {
        if (ids[cls] < 0)
          continue;
        r.blas = (uint32_t)ids[cls];
        recs.push_back(r);
        const box3 wb = xfmBox(m, hBlas[ids[cls]].bounds);
        recBoxes.push_back(wb);
        extend(worldBounds, wb);
      }
      for (Light *l : gl) {
        if (!l->ensureBuilt())
          continue;
        LightGPU lg = l->gpu;
        if (lg.type == LIGHT_HDRI) {
          // the first HDRI light is the world's (World.cpp:466-480); its
          // instance transform is not applied (sampleLight.h:110-149)
          if (hdriIndex < 0)
            hdriIndex = (int)lights.size();
        } else if (lg.type == LIGHT_DIRECTIONAL)
          lg.dirToLight = f3{m[0] * l->gpu.dirToLight.x + m[1] * l->gpu.dirToLight.y
                  + m[2] * l->gpu.dirToLight.z,
              m[4] * l->gpu.dirToLight.x + m[5] * l->gpu.dirToLight.y
                  + m[6] * l->gpu.dirToLight.z,
              m[8] * l->gpu.dirToLight.x + m[9] * l->gpu.dirToLight.y
                  + m[10] * l->gpu.dirToLight.z};
        else
          lg.position = f3{m[0] * lg.position.x + m[1] * lg.position.y
                  + m[2] * lg.position.z + m[3],
              m[4] * lg.position.x + m[5] * lg.position.y + m[6] * lg.position.z
                  + m[7],
              m[8] * lg.position.x + m[9] * lg.position.y + m[10] * lg.position.z
                  + m[11]};
        lights.push_back(lg);
      }
      for (Volume *v : gv) {
        if (!v->ensureBuilt())
          continue;
        SpatialField *f = v->field;
        VolumeGPU vg{};
        vg.field = f->tex;
        vg.fieldKind = f->nanovdb ? FIELD_NANOVDB : FIELD_STRUCTURED_REGULAR;
        vg.nvdb = f->nvdbGPU;
        vg.tf = v->tfTex;
        vg.hasTF = v->tfTex ? 1u : 0u;
        vg.origin = f->origin;
        vg.spacing = f->spacing;
        vg.invSpacing = f3{1.f / (f->spacing.x * float(f->dims[0])),
            1.f / (f->spacing.y * float(f->dims[1])),
            1.f / (f->spacing.z * float(f->dims[2]))};
        vg.bounds = f->bounds();
        vg.stepSize = f->stepSize();
        vg.oneOverUnitDistance = 1.f / v->unitDistance;
        vg.valueLo = v->valueRange[0];
        vg.valueHi = v->valueRange[1];
        vg.uniformColor = v->uniformColor;
        vg.uniformOpacity = v->uniformOpacity;
        vg.id = v->id;
        vg.instId = inst->userID(t);
        vg.worldToObject = r.worldToObject;
        vg.majorants =
            v->hasEmptyCells && v->emptySpaceSkipping ? v->majorants : nullptr;
        vg.dptMajorants = v->dptMajorants;
        for (int k = 0; k < 3; k++) {
          vg.mcDims[k] = f->mcDims[k];
          vg.dims[k] = f->dims[k];
        }
        vols.push_back(vg);
        extend(worldBounds, xfmBox(m, vg.bounds));
      }
    }
  }

  // TLAS over instance records
  InstanceRecord *dRecs = nullptr;
  if (!recs.empty()) {
    box3 *dBoxes = nullptr;
    cudaMallocAsync((void **)&dBoxes, sizeof(box3) * recBoxes.size(), s);
    cudaMemcpyAsync(dBoxes,
        recBoxes.data(),
        sizeof(box3) * recBoxes.size(),
        cudaMemcpyHostToDevice,
        s);
    cudaError_t err = buildBVH8(dBoxes, (uint32_t)recBoxes.size(), s, tlas, 1);
    cudaFreeAsync(dBoxes, s);
    if (err != cudaSuccess) {
      report(VRTX_SEVERITY_ERROR, "TLAS build failed: %s", cudaGetErrorString(err));
      return false;
    }
    std::vector<uint32_t> order(tlas.numPrims);
    cudaMemcpyAsync(order.data(),
        tlas.primOrder,
        sizeof(uint32_t) * order.size(),
        cudaMemcpyDeviceToHost,
        s);
    cudaStreamSynchronize(s);
    std::vector<InstanceRecord> sorted(order.size());
    for (size_t i = 0; i < order.size(); i++)
      sorted[i] = recs[order[i]];
    dRecs = uploadVec(this, sorted, s);
  }

  gpu.tlasNodes = tlas.nodes;
  gpu.instances = dRecs;
  gpu.numInstances = (uint32_t)recs.size();
  gpu.blas = dBlas;
  gpu.surfaces = dSurfs;
  gpu.geometries = dGeoms;
  gpu.materials = dMats;
  gpu.samplers = dSamplers;
  gpu.lights = uploadVec(this, lights, s);
  gpu.numLights = (uint32_t)lights.size();
  gpu.hdri = hdriIndex;
  gpu.volumes = uploadVec(this, vols, s);
  gpu.numVolumes = (uint32_t)vols.size();
  gpu.allOpaque = allOpaque ? 1u : 0u;
  gpu.allMatte = allMatte ? 1u : 0u;
  gpu.hasNanovdb = 0u;
  for (const VolumeGPU &v : vols)
    if (v.fieldKind == FIELD_NANOVDB)
      gpu.hasNanovdb = 1u;
  gpu.hasSegments = 0u;
  for (const BLASDesc &b : hBlas)
    if (b.type >= GEOM_CYLINDER)
      gpu.hasSegments = 1u;
  const cudaError_t err = cudaStreamSynchronize(s);
  builtStamp = deepStamp();
  buildMs = std::chrono::duration<float, std::milli>(
      std::chrono::steady_clock::now() - t0)
                .count();
  if (err != cudaSuccess) {
    report(VRTX_SEVERITY_ERROR, "world build failed: %s", cudaGetErrorString(err));
    return false;
  }
  return true;
}

bool World::getProperty(
    const std::string &name, int t, void *mem, uint64_t size, uint32_t mask)
{
  if (name == "bounds" && t == VRTX_FLOAT32_BOX3 && size >= 24) {
    if (Object::dev->initOk && (builtStamp == 0 || deepStamp() > builtStamp))
      rebuild();
    std::memcpy(mem, &worldBounds, 24);
    return true;
  }
  return Object::getProperty(name, t, mem, size, mask);
}

// ---------------------------------------------------------------------------
// Renderer (renderer/Renderer.cpp:152-207, DirectLight.cpp, AmbientOcclusion
// .cpp, Raycast.cpp, DiffusePathTracer.cpp)
// ---------------------------------------------------------------------------

Renderer::~Renderer()
{
  if (gpu.backgroundTex)
    cudaDestroyTextureObject(gpu.backgroundTex);
  if (bgArray)
    cudaFreeArray(bgArray);
}

uint64_t Renderer::deepStamp() const
{
  return std::max(commitStamp, bgImage ? bgImage->deepStamp() : 0);
}

// The background image's n texels (element type et, nc = 3 or 4 channels)
// staged as RGBA8 (Array2D::acquireCUDAArrayUint8 with
// transformToStagingBufferUint8, utility/CudaImageTexture.cpp:43-93): float
// components truncated from c * 255 (clamped to [0, 255] here, where the
// reference's conversion is undefined), sRGB-encoded bytes (alpha too)
// linearised, other bytes as they are; alpha 255 for three channels.
static void stageBackgroundImage(int et, int nc, const uint8_t *raw, size_t n, uint8_t *rgba)
{
  for (size_t i = 0; i < n; i++) {
    for (int c = 0; c < 4; c++) {
      uint8_t v = 255;
      if (c < nc) {
        if (et == VRTX_FLOAT32_VEC3 || et == VRTX_FLOAT32_VEC4) {
          float f;
          std::memcpy(&f, raw + 4 * (i * nc + c), 4);
          const float s = f * 255.f;
          v = (uint8_t)(s >= 255.f ? 255.f : (s > 0.f ? s : 0.f));
        } else {
          v = stageComponentUint8(et, raw + i * 4, c);
        }
      }
      rgba[i * 4 + c] = v;
    }
  }
}

static int backgroundChannels(int et)
{
  return et == VRTX_FLOAT32_VEC3 ? 3
      : (et == VRTX_FLOAT32_VEC4 || et == VRTX_UFIXED8_VEC4 || et == VRTX_UFIXED8_RGBA_SRGB) ? 4
                                                                                            : 0;
}

// Renderer::finalize with Array2D::acquireCUDAArrayUint8
// (utility/CudaImageTexture.cpp:43-93,139-190): the image staged as RGBA8
// (float components truncated from c * 255, clamped to [0, 255] here;
// sRGB-encoded bytes, alpha too, linearised first; three channels get alpha
// 255), a normalised-float, linear, clamped texture read at the sample's
// screen position
bool Renderer::ensureBackground()
{
  if (!bgImage) {
    if (gpu.backgroundTex)
      cudaDestroyTextureObject(gpu.backgroundTex);
    if (bgArray)
      cudaFreeArray(bgArray);
    gpu.backgroundTex = 0;
    bgArray = nullptr;
    return true;
  }
  const uint64_t want = deepStamp();
  if (bgStamp && bgStamp >= want && gpu.backgroundTex)
    return true;
  if (gpu.backgroundTex)
    cudaDestroyTextureObject(gpu.backgroundTex);
  if (bgArray)
    cudaFreeArray(bgArray);
  gpu.backgroundTex = 0;
  bgArray = nullptr;
  const int et = bgImage->elemType;
  const int nc = backgroundChannels(et);
  if (!nc) {
    report(VRTX_SEVERITY_WARNING,
        "background image: element type %d is not supported (FLOAT32_VEC3/4, "
        "UFIXED8_VEC4, UFIXED8_RGBA_SRGB are)",
        et);
    return false;
  }
  const size_t W = bgImage->n[0], H = bgImage->n[1];
  std::vector<uint8_t> raw(bgImage->bytes());
  if (const void *h = bgImage->hostData())
    std::memcpy(raw.data(), h, raw.size());
  else {
    const void *d = bgImage->deviceData();
    cudaStreamSynchronize(Object::dev->stream);
    cudaMemcpy(raw.data(), d, raw.size(), cudaMemcpyDeviceToHost);
  }
  std::vector<uint8_t> rgba(W * H * 4);
  stageBackgroundImage(et, nc, raw.data(), W * H, rgba.data());
  cudaChannelFormatDesc desc = cudaCreateChannelDesc<uchar4>();
  if (cudaMallocArray(&bgArray, &desc, W, H) != cudaSuccess) {
    cudaGetLastError();
    bgArray = nullptr;
    return false;
  }
  cudaMemcpy2DToArray(bgArray, 0, 0, rgba.data(), W * 4, W * 4, H, cudaMemcpyHostToDevice);
  cudaResourceDesc rd{};
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = bgArray;
  cudaTextureDesc td{};
  td.addressMode[0] = td.addressMode[1] = cudaAddressModeClamp;
  td.filterMode = cudaFilterModeLinear;
  td.readMode = cudaReadModeNormalizedFloat;
  td.normalizedCoords = 1;
  cudaCreateTextureObject(&gpu.backgroundTex, &rd, &td, nullptr);
  bgStamp = want;
  return cudaGetLastError() == cudaSuccess;
}

void Renderer::commit()
{
  RendererGPU &r = gpu;
  float defaultAmbient = 0.f;
  if (subtype == "raycast")
    r.type = RENDERER_RAYCAST;
  else if (subtype == "ao") {
    r.type = RENDERER_AO;
    defaultAmbient = 1.f;
  } else if (subtype == "dpt" || subtype == "diffuse_pathtracer") {
    r.type = RENDERER_DPT;
    defaultAmbient = 1.f;
  } else {
    if (subtype != "default" && subtype != "directLight")
      report(VRTX_SEVERITY_WARNING,
          "unknown renderer subtype '%s', using 'default'",
          subtype.c_str());
    r.type = RENDERER_DIRECT_LIGHT;
  }
  float bg[4] = {0.f, 0.f, 0.f, 1.f};
  if (has("background", VRTX_FLOAT32_VEC4))
    std::memcpy(bg, params["background"].bytes.data(), 16);
  r.background = make_float4(bg[0], bg[1], bg[2], bg[3]);
  bgImage = static_cast<Array *>(getObject("background", VRTX_ARRAY2D));
  bgStamp = 0;
  spp = get<int32_t>("pixelSamples", VRTX_INT32, 1);
  r.maxRayDepth = get<int32_t>("maxRayDepth", VRTX_INT32, 5);
  r.ambientColor = get<f3>("ambientColor", VRTX_FLOAT32_VEC3, f3{1.f, 1.f, 1.f});
  r.ambientIntensity = get<float>("ambientRadiance", VRTX_FLOAT32, defaultAmbient);
  r.occlusionDistance = get<float>("ambientOcclusionDistance", VRTX_FLOAT32, 1e20f);
  checkerboard = get<int32_t>("checkerboarding", VRTX_BOOL, 0) != 0;
  sampleLimit = get<int32_t>("sampleLimit", VRTX_INT32, 128);
  r.cullTriangleBF = get<int32_t>("cullTriangleBackfaces", VRTX_BOOL, 0) != 0;
  const float vsr = std::min(
      std::max(get<float>("volumeSamplingRate", VRTX_FLOAT32, 0.125f), 1e-3f),
      10.f);
  r.invVolumeSamplingRate = 1.f / vsr;
  if (checkerboard)
    spp = 1;
  r.aoSamples = 0;
  if (r.type == RENDERER_DIRECT_LIGHT || r.type == RENDERER_AO)
    r.aoSamples = std::min(std::max(get<int32_t>("ambientSamples", VRTX_INT32, 1), 0), 256);
  r.lightFalloff =
      std::min(std::max(get<float>("lightFalloff", VRTX_FLOAT32, 1.f), 0.f), 1.f);
  r.maxDepth = std::min(std::max(get<int32_t>("maxDepth", VRTX_INT32, 5), 1), 256);
  if (r.type == RENDERER_RAYCAST)
    sampleLimit = 1; // single-shot renderer (Raycast.cpp:46-51)
  r.numIterations = std::max(spp, 1);
}

bool Renderer::isValid() const
{
  return true;
}

// ---------------------------------------------------------------------------
// Frame (frame/Frame.cu)
// ---------------------------------------------------------------------------

Frame::~Frame()
{
  if (Object::dev->initOk) {
    wait();
    freeBuffers();
    for (cudaEvent_t e : {evStart, evEnd, evKStart, evKEnd})
      if (e)
        cudaEventDestroy(e);
    for (cudaEvent_t e : traceEvents)
      cudaEventDestroy(e);
    cudaStream_t s = Object::dev->stream;
    if (workCounter)
      cudaFreeAsync(workCounter, s);
    if (errorFlag)
      cudaFreeAsync(errorFlag, s);
    if (stats)
      cudaFreeAsync(stats, s);
    if (scratch)
      cudaFreeAsync(scratch, s);
  }
}

// A frame allocation from the device's pool, or a failure the device was
// told to inject ("vrtx.failFrameAllocations": host-side fault injection for
// tests of the error path; no CUDA call is made for an injected failure).
cudaError_t Frame::frameAlloc(void **p, size_t bytes, cudaStream_t s)
{
  std::atomic<int> &inject = Object::dev->failFrameAllocs;
  for (int k = inject.load(); k > 0;)
    if (inject.compare_exchange_weak(k, k - 1)) {
      *p = nullptr;
      return cudaErrorMemoryAllocation;
    }
  const cudaError_t e = cudaMallocAsync(p, bytes, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
  }
  return e;
}

// Frame buffers and counters come from the device's stream-ordered pool:
// a frame created, resized or released every step reuses pool memory
// instead of cudaMalloc / cudaFree round trips that synchronise the device.
void Frame::freeBuffers()
{
  for (void *&b : buffers) {
    if (b)
      cudaFreeAsync(b, Object::dev->stream);
    b = nullptr;
  }
  fb = FramebufferGPU{};
}

void Frame::commit()
{
  renderer = static_cast<Renderer *>(getObject("renderer", VRTX_RENDERER));
  camera = static_cast<Camera *>(getObject("camera", VRTX_CAMERA));
  world = static_cast<World *>(getObject("world", VRTX_WORLD));
  callback = get<VRTXFrameCompletionCallback>(
      "frameCompletionCallback", VRTX_FUNCTION_POINTER, nullptr);
  callbackPtr =
      get<const void *>("frameCompletionCallbackUserData", VRTX_VOID_POINTER, nullptr);
  colorType =
      get<int32_t>("channel.color", VRTX_DATA_TYPE, VRTX_UFIXED8_RGBA_SRGB);
  uint32_t sz[2] = {10, 10};
  if (has("size", VRTX_UINT32_VEC2))
    std::memcpy(sz, params["size"].bytes.data(), 8);
  depthType = get<int32_t>("channel.depth", VRTX_DATA_TYPE, VRTX_UNKNOWN);
  primType = get<int32_t>("channel.primitiveId", VRTX_DATA_TYPE, VRTX_UNKNOWN);
  objType = get<int32_t>("channel.objectId", VRTX_DATA_TYPE, VRTX_UNKNOWN);
  instType = get<int32_t>("channel.instanceId", VRTX_DATA_TYPE, VRTX_UNKNOWN);
  albedoType = get<int32_t>("channel.albedo", VRTX_DATA_TYPE, VRTX_UNKNOWN);
  normalType = get<int32_t>("channel.normal", VRTX_DATA_TYPE, VRTX_UNKNOWN);
  size[0] = sz[0];
  size[1] = sz[1];
  // frame buffers (Frame::finalize, Frame.cu:96-161)
  if (!Object::dev->initOk)
    return;
  wait();
  freeBuffers();
  const size_t n = (size_t)size[0] * size[1];
  const bool useFloat = colorType == VRTX_FLOAT32_VEC4;
  fb.format = useFloat
      ? FORMAT_FLOAT
      : (colorType == VRTX_UFIXED8_RGBA_SRGB ? FORMAT_SRGB : FORMAT_UINT);
  fb.w = size[0];
  fb.h = size[1];
  fb.invW = 1.f / float(size[0]);
  fb.invH = 1.f / float(size[1]);
  const bool cPrim = primType == VRTX_UINT32, cObj = objType == VRTX_UINT32,
             cInst = instType == VRTX_UINT32;
  const bool cDepth = depthType == VRTX_FLOAT32 || cPrim || cObj || cInst;
  if (cDepth)
    depthType = VRTX_FLOAT32;
  cudaStream_t s = Object::dev->stream;
  // one failed allocation leaves the frame without buffers: render then
  // skips it with an error instead of writing to a missing buffer
  bool failed = false;
  auto alloc = [&](int slot, size_t bytes) -> void * {
    if (!bytes)
      return nullptr;
    if (frameAlloc(&buffers[slot], bytes, s) != cudaSuccess) {
      buffers[slot] = nullptr;
      failed = true;
    }
    return buffers[slot];
  };
  fb.accum = (float4 *)alloc(0, n * sizeof(float4));
  if (useFloat)
    fb.outColorF = (float4 *)alloc(1, n * sizeof(float4));
  else
    fb.outColorU = (uint32_t *)alloc(1, n * sizeof(uint32_t));
  fb.depth = cDepth ? (float *)alloc(2, n * 4) : nullptr;
  fb.primID = cPrim ? (uint32_t *)alloc(3, n * 4) : nullptr;
  fb.objID = cObj ? (uint32_t *)alloc(4, n * 4) : nullptr;
  fb.instID = cInst ? (uint32_t *)alloc(5, n * 4) : nullptr;
  // The reference enables these accumulations for ANARI_FLOAT32
  // (Frame.cu:116-117); FLOAT32_VEC3, the channel's element type, is
  // accepted too. Slots 8/9 hold the averaged copies that map returns.
  const bool wantAlbedo = albedoType == VRTX_FLOAT32 || albedoType == VRTX_FLOAT32_VEC3;
  const bool wantNormal = normalType == VRTX_FLOAT32 || normalType == VRTX_FLOAT32_VEC3;
  fb.albedo = wantAlbedo ? (f3 *)alloc(6, n * 12) : nullptr;
  fb.normal = wantNormal ? (f3 *)alloc(7, n * 12) : nullptr;
  if (wantAlbedo)
    alloc(8, n * 12);
  if (wantNormal)
    alloc(9, n * 12);
  if (!workCounter && frameAlloc((void **)&workCounter, 16, s) != cudaSuccess) {
    workCounter = nullptr;
    failed = true;
  }
  // error flags collect over the frames rendered since the last commit
  if (!errorFlag && frameAlloc((void **)&errorFlag, 16, s) != cudaSuccess) {
    errorFlag = nullptr;
    failed = true;
  }
  if (errorFlag)
    cudaMemsetAsync(errorFlag, 0, 16, s);
  if (!stats) {
    if (frameAlloc((void **)&stats, 16 * sizeof(unsigned long long), s) == cudaSuccess)
      cudaMemsetAsync(stats, 0, 16 * sizeof(unsigned long long), s);
    else {
      stats = nullptr;
      failed = true;
    }
  }
  if (failed) {
    report(VRTX_SEVERITY_ERROR, "frame buffer allocation failed");
    freeBuffers();
  }
  countTraversal = get<int32_t>("vrtx.countTraversal", VRTX_BOOL, 0) != 0;
  // the traversal loop bound per ray; lowering it makes the device guard
  // end traversals early and report bit 1 of "error_flags" (no GPU fault)
  {
    const int32_t m = get<int32_t>("vrtx.maxTraversalSteps", VRTX_INT32, 1 << 22);
    maxTraversalSteps = m > 0 ? (uint32_t)m : 1u;
  }
  forceMegakernel = get<int32_t>("vrtx.megakernel", VRTX_BOOL, 0) != 0;
  for (cudaEvent_t *e : {&evStart, &evEnd, &evKStart, &evKEnd})
    if (!*e)
      cudaEventCreate(e);
  nextFrameReset = true;
  rendered = false;
}

bool Frame::isValid() const
{
  return renderer && camera && world && renderer->isValid();
}

void Frame::wait()
{
  if (rendered && evEnd)
    cudaEventSynchronize(evEnd);
}

bool Frame::ready()
{
  if (!rendered || !evEnd)
    return true;
  return cudaEventQuery(evEnd) == cudaSuccess;
}

void Frame::render()
{
  NvtxRange frameRange("Frame::renderFrame()");
  Device *d = Object::dev;
  wait();
  launches = 0;
  if (!d->initOk) {
    report(VRTX_SEVERITY_ERROR, "skipping render: no CUDA device");
    return;
  }
  if (!isValid() || !fb.accum || !workCounter || !errorFlag || !stats) {
    const char *why = !renderer ? "missing ANARIRenderer"
        : !camera                ? "missing ANARICamera"
        : !world                 ? "missing ANARIWorld"
                                 : "invalid frame buffers";
    report(VRTX_SEVERITY_ERROR,
        "skipping render of incomplete or invalid frame object -- issue: %s",
        why);
    return;
  }
  cudaStream_t s = d->stream;
  if (world->builtStamp == 0 || world->deepStamp() > world->builtStamp) {
    NvtxRange updateRange("update scene");
    NvtxRange bvhRange("rebuild BVHs");
    if (!world->rebuild())
      return;
    d->markChanged();
  }
  // checkAccumulationReset (Frame.cu:574-588)
  const uint64_t change = d->lastChange.load();
  if (change > lastSeenStamp) {
    lastSeenStamp = change;
    nextFrameReset = true;
  }
  if (!nextFrameReset && renderer->sampleLimit > 0
      && fb.frameID >= renderer->sampleLimit)
    return;
  cudaEventRecord(evStart, s);
  NvtxRange renderRange("render all frames");
  // newFrame (Frame.cu:590-660)
  nvtxRangePushA("Frame::newFrame()");
  if (nextFrameReset) {
    fb.frameID = 0;
    fb.checkerboardID = renderer->checkerboard ? 0 : -1;
    nextFrameReset = false;
    launchClearFrame(fb, s);
    launches++;
  } else {
    if (renderer->checkerboard)
      fb.frameID += int(fb.checkerboardID == 3);
    else
      fb.frameID += renderer->spp;
    fb.checkerboardID = renderer->checkerboard ? ((fb.checkerboardID + 1) & 0x3) : -1;
  }
  nvtxRangePop(); // Frame::newFrame()
  FrameParams P{};
  P.world = world->gpu;
  P.world.maxTraversalSteps = maxTraversalSteps;
  P.camera = camera->gpu;
  renderer->ensureBackground();
  P.renderer = renderer->gpu;
  P.fb = fb;
  P.workCounter = workCounter;
  P.errorFlag = errorFlag;
  P.launchW = renderer->checkerboard ? (fb.w + 1) / 2 : fb.w;
  P.launchH = renderer->checkerboard ? (fb.h + 1) / 2 : fb.h;
  P.numTilesX = (P.launchW + 7) / 8;
  P.numTilesY = (P.launchH + 3) / 4;
  P.stats = stats;
  cudaMemsetAsync(workCounter, 0, 4, s);
  cudaMemsetAsync(stats, 0, 16 * sizeof(unsigned long long), s);
  // Wavefront forms (per sample a primary / any-hit / resolve kernel, or
  // one kernel for raycast) where the frame's path has no volume and no
  // translucent surface: "ao", "default" over matte surfaces, "raycast".
  // Everything else runs the per-pixel integrator kernel. ("ao" and
  // "default" read a background image at each sample's jittered screen
  // position, which their resolve does not keep: such frames run per
  // pixel.)
  const bool plainSurfaces =
      P.world.allOpaque && P.world.numVolumes == 0 && !forceMegakernel;
  const bool aoWave = P.renderer.type == RENDERER_AO && plainSurfaces
      && !P.renderer.backgroundTex;
  const bool dlWave = P.renderer.type == RENDERER_DIRECT_LIGHT && plainSurfaces
      && P.world.allMatte && !P.renderer.backgroundTex;
  const bool rcWave = P.renderer.type == RENDERER_RAYCAST && plainSurfaces;
  const bool wavefront = aoWave || dlWave;
  cudaError_t err = cudaSuccess;
  // the one range not named as the reference's ("optixLaunch()"): the
  // integrator kernels replace the OptiX launch
  NvtxRange launchRange("render kernels");
  cudaEventRecord(evKStart, s);
  if (rcWave) {
    tracePairs = 0;
    err = launchRaycastWavefront(P, countTraversal, s);
    launches++;
  } else if (wavefront) {
    const size_t need = aoWave
        ? aoWavefrontBytes(fb.w, fb.h, P.renderer.aoSamples)
        : dlWavefrontBytes(fb.w, fb.h, P.renderer.aoSamples, P.world.numLights);
    if (need > scratchBytes) {
      if (scratch)
        cudaFreeAsync(scratch, s);
      scratch = nullptr;
      scratchBytes = 0;
      err = cudaMallocAsync(&scratch, need, s);
      if (err == cudaSuccess)
        scratchBytes = need;
    }
    const int n = std::max(P.renderer.numIterations, 1);
    while ((int)traceEvents.size() < 2 * n) {
      cudaEvent_t e = nullptr;
      if (cudaEventCreate(&e) != cudaSuccess)
        break;
      traceEvents.push_back(e);
    }
    const bool timed = (int)traceEvents.size() >= 2 * n;
    tracePairs = timed ? n : 0;
    if (err == cudaSuccess)
      err = aoWave ? launchAOWavefront(P, d->numSMs, countTraversal, scratch, s,
                         timed ? traceEvents.data() : nullptr)
                   : launchDLWavefront(P, d->numSMs, countTraversal, scratch, s,
                         timed ? traceEvents.data() : nullptr);
    launches += 3 * std::max(P.renderer.numIterations, 1);
  } else {
    tracePairs = 0;
    const int blocks =
        d->numSMs
        * renderOccupancyBlocks(P.renderer.type,
            countTraversal,
            P.world.numInstances > 0,
            P.world.hasNanovdb != 0);
    err = launchRender(P, blocks, countTraversal, s);
    launches++;
  }
  cudaEventRecord(evKEnd, s);
  if (err != cudaSuccess)
    report(VRTX_SEVERITY_ERROR, "render launch failed: %s", cudaGetErrorString(err));
  if (callback) {
    cudaLaunchHostFunc(
        s,
        [](void *p) {
          auto *f = (Frame *)p;
          f->callback(f->callbackPtr,
              reinterpret_cast<VRTXDevice>(f->Object::dev),
              reinterpret_cast<VRTXFrame>(f));
        },
        this);
  }
  cudaEventRecord(evEnd, s);
  rendered = true;
}

const void *Frame::map(
    const std::string &channel, uint32_t *w, uint32_t *h, int *pixelType)
{
  wait();
  int t = VRTX_UNKNOWN;
  const void *ret = nullptr;
  const size_t n = (size_t)fb.w * fb.h;
  const bool cuda = channel.size() > 4
      && channel.compare(channel.size() - 4, 4, "CUDA") == 0;
  const std::string base = cuda ? channel.substr(0, channel.size() - 4) : channel;
  void *src = nullptr;
  size_t bytes = 0;
  std::vector<uint8_t> *host = nullptr;
  if (base == "channel.color" && fb.accum) {
    t = colorType;
    src = fb.format == FORMAT_FLOAT ? (void *)fb.outColorF : (void *)fb.outColorU;
    bytes = n * (fb.format == FORMAT_FLOAT ? 16 : 4);
    host = &hostColor;
  } else if (base == "channel.depth" && fb.depth) {
    t = VRTX_FLOAT32;
    src = fb.depth;
    bytes = n * 4;
    host = &hostDepth;
  } else if (base == "channel.primitiveId" && fb.primID) {
    t = VRTX_UINT32;
    src = fb.primID;
    bytes = n * 4;
    host = &hostPrim;
  } else if (base == "channel.objectId" && fb.objID) {
    t = VRTX_UINT32;
    src = fb.objID;
    bytes = n * 4;
    host = &hostObj;
  } else if (base == "channel.instanceId" && fb.instID) {
    t = VRTX_UINT32;
    src = fb.instID;
    bytes = n * 4;
    host = &hostInst;
  } else if ((base == "channel.albedo" && fb.albedo && buffers[8])
      || (base == "channel.normal" && fb.normal && buffers[9])) {
    // mapAlbedoBuffer / mapNormalBuffer (Frame.cu:518-557): the
    // accumulation times 1 / (frameID + 1), into a separate buffer
    const bool alb = base == "channel.albedo";
    t = VRTX_FLOAT32_VEC3;
    src = buffers[alb ? 8 : 9];
    bytes = n * 12;
    host = alb ? &hostAlbedo : &hostNormal;
    launchScale3(alb ? fb.albedo : fb.normal,
        (f3 *)src,
        n,
        1.f / float(fb.frameID + 1),
        Object::dev->stream);
    cudaStreamSynchronize(Object::dev->stream);
  }
  if (t == VRTX_UNKNOWN || !src) {
    *w = *h = 0;
    *pixelType = VRTX_UNKNOWN;
    return nullptr;
  }
  // the buffers are stream-ordered allocations of the device stream: the
  // mapped pointer (or the host copy) is only handed out once the stream has
  // reached them, so any stream or the host may read it
  cudaStreamSynchronize(Object::dev->stream);
  if (cuda)
    ret = src;
  else {
    host->resize(bytes);
    NvtxRange copyRange("copy to host");
    cudaMemcpy(host->data(), src, bytes, cudaMemcpyDeviceToHost);
    ret = host->data();
  }
  *w = fb.w;
  *h = fb.h;
  *pixelType = t;
  return ret;
}

bool Frame::getProperty(
    const std::string &name, int t, void *mem, uint64_t size, uint32_t mask)
{
  if (name == "duration" && t == VRTX_FLOAT32 && size >= 4) {
    if (mask & VRTX_WAIT)
      wait();
    float ms = 0.f;
    if (rendered)
      cudaEventElapsedTime(&ms, evStart, evEnd);
    const float sec = ms / 1000.f;
    std::memcpy(mem, &sec, 4);
    return true;
  }
  if (name == "numSamples" && t == VRTX_INT32 && size >= 4) {
    if (mask & VRTX_WAIT)
      wait();
    int32_t v = fb.frameID;
    std::memcpy(mem, &v, 4);
    return true;
  }
  // libvrtx extension (no reference counterpart): counters of the last
  // render: rays traced; with "vrtx.countTraversal" set also BVH8 nodes
  // visited, triangle tests, sphere tests, BLAS entries; volume march
  // positions and fetched samples; then the traversal error flags (bit 0:
  // stack overflow, bit 1: iteration bound).
  if (name == "vrtx.stats" && t == VRTX_UINT64 && size >= 64 && stats) {
    wait();
    unsigned long long v[8] = {};
    cudaMemcpy(v, stats, 7 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    uint32_t flags = 0;
    cudaMemcpy(&flags, errorFlag, 4, cudaMemcpyDeviceToHost);
    v[7] = flags;
    std::memcpy(mem, v, sizeof(v));
    return true;
  }
  // libvrtx extension: the AO any-hit kernel alone (wavefront path): its
  // counters [rays, nodes, tri tests, sphere tests, BLAS entries] and the
  // summed device time of its launches in the last render (ms, 0 when the
  // frame ran the per-pixel kernel).
  if (name == "vrtx.aoTraceStats" && t == VRTX_UINT64 && size >= 40 && stats) {
    wait();
    unsigned long long v[5] = {};
    cudaMemcpy(v, stats + 8, sizeof(v), cudaMemcpyDeviceToHost);
    std::memcpy(mem, v, sizeof(v));
    return true;
  }
  if (name == "vrtx.aoTraceMilliseconds" && t == VRTX_FLOAT32 && size >= 4) {
    wait();
    float total = 0.f;
    for (int i = 0; i < tracePairs; i++) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, traceEvents[2 * i], traceEvents[2 * i + 1]) == cudaSuccess)
        total += ms;
    }
    std::memcpy(mem, &total, 4);
    return true;
  }
  if (name == "nextFrameReset" && t == VRTX_BOOL && size >= 4) {
    if (mask & VRTX_WAIT)
      wait();
    const bool reset = nextFrameReset || Object::dev->lastChange.load() > lastSeenStamp;
    int32_t v = reset ? 1 : 0;
    std::memcpy(mem, &v, 4);
    return true;
  }
  return Object::getProperty(name, t, mem, size, mask);
}

} // namespace vrtx

// ===========================================================================
// C ABI
// ===========================================================================

using namespace vrtx;

#define VRTX_GUARD_BEGIN try {
#define VRTX_GUARD_END(dev, ret)                                               \
  }                                                                            \
  catch (const std::exception &e)                                              \
  {                                                                            \
    if (dev)                                                                   \
      reinterpret_cast<Device *>(dev)->report(                                 \
          nullptr, VRTX_SEVERITY_FATAL_ERROR, e.what());                       \
    return ret;                                                                \
  }                                                                            \
  catch (...)                                                                  \
  {                                                                            \
    return ret;                                                                \
  }

static Device *D(VRTXDevice d)
{
  return reinterpret_cast<Device *>(d);
}
static Object *O(VRTXObject o)
{
  return reinterpret_cast<Object *>(o);
}

// Every API call runs on the device's GPU and leaves the calling thread's
// current device as it found it (CUDADeviceScope, VisRTXDevice.cpp:790-814).
// A call that initialises the device (init() selects its GPU) is restored
// the same way. Devices without a usable GPU make no CUDA call here.
struct DeviceScope
{
  int prev = -1;
  explicit DeviceScope(Device *dev)
  {
    if (!dev || (dev->initTried && !dev->initOk))
      return;
    if (cudaGetDevice(&prev) != cudaSuccess) {
      cudaGetLastError();
      prev = -1;
      return;
    }
    if (dev->initOk && prev != dev->cudaDevice)
      cudaSetDevice(dev->cudaDevice);
  }
  ~DeviceScope()
  {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev)
      cudaSetDevice(prev);
  }
  DeviceScope(const DeviceScope &) = delete;
  DeviceScope &operator=(const DeviceScope &) = delete;
};

// The GPU is chosen once, by init(); a later "cudaDevice" is reported and
// ignored, as VisRTXDevice::deviceCommitParameters does
// (VisRTXDevice.cpp:464-470), so every object stays on the GPU that owns its
// memory and the device's stream.
static void warnDeviceChange(Device *dev)
{
  if (dev->initTried && dev->desiredDevice != dev->cudaDevice) {
    char msg[160];
    std::snprintf(msg,
        sizeof(msg),
        "libvrtx was already initialised to use GPU %d: new device number %d is "
        "ignored",
        dev->cudaDevice,
        dev->desiredDevice);
    dev->report(nullptr, VRTX_SEVERITY_WARNING, msg);
  }
}

template <typename T>
static VRTXObject newObj(VRTXDevice d, int type, const char *subtype)
{
  Device *dev = D(d);
  if (!dev)
    return nullptr;
  std::lock_guard<std::recursive_mutex> lock(dev->mutex);
  if (!dev->init())
    return nullptr; // factory calls return null when init failed
  Object *o = new T(dev, type, subtype ? subtype : "");
  dev->live.push_back(o);
  return reinterpret_cast<VRTXObject>(o);
}

extern "C" {

VRTX_API VRTXDevice vrtxNewDevice(VRTXStatusCallback cb, const void *ptr)
{
  try {
    Device *d = new Device();
    d->cb = cb;
    d->cbPtr = ptr;
    return reinterpret_cast<VRTXDevice>(d);
  } catch (...) {
    return nullptr;
  }
}

VRTX_API void vrtxDeviceSetParameter(
    VRTXDevice d, const char *name, int type, const void *mem)
{
  if (!d || !name)
    return;
  std::string n(name);
  Device *dev = D(d);
  if (n == "cudaDevice" && type == VRTX_INT32 && mem) {
    std::lock_guard<std::recursive_mutex> lock(dev->mutex);
    dev->desiredDevice = *(const int32_t *)mem;
    warnDeviceChange(dev);
  } else if (n == "forceInit" && type == VRTX_BOOL && mem)
    dev->forceInit = *(const int32_t *)mem != 0;
  else if (n == "vrtx.failFrameAllocations" && type == VRTX_INT32 && mem)
    dev->failFrameAllocs = std::max(0, *(const int32_t *)mem);
  else if (n == "statusCallback" && mem)
    D(d)->cb = *(const VRTXStatusCallback *)mem;
  else if (n == "statusCallbackUserData")
    D(d)->cbPtr = mem ? *(const void *const *)mem : nullptr;
}

// deviceCommitParameters (VisRTXDevice.cpp:460-478): "forceInit" initialises
// CUDA now instead of at the first object creation.
VRTX_API void vrtxDeviceCommitParameters(VRTXDevice d)
{
  Device *dev = D(d);
  if (!dev)
    return;
  std::lock_guard<std::recursive_mutex> lock(dev->mutex);
  if (dev->forceInit && !dev->initTried) {
    DeviceScope scope(dev);
    dev->init();
  }
}

VRTX_API void vrtxDeviceRelease(VRTXDevice d)
{
  DeviceScope scope(D(d));
  if (!d)
    return;
  Device *dev = D(d);
  if (dev->initOk)
    cudaStreamSynchronize(dev->stream);
  // objects still alive are released in reverse creation order
  while (!dev->live.empty()) {
    Object *o = dev->live.back();
    dev->live.pop_back();
    o->refs = 1 << 20; // detach from app references
    for (auto &p : o->params)
      p.second.obj = nullptr;
    for (auto &p : o->pending)
      p.second.obj = nullptr;
    if (o->type == VRTX_ARRAY1D || o->type == VRTX_ARRAY2D
        || o->type == VRTX_ARRAY3D)
      static_cast<Array *>(o)->handles.clear();
    if (o->type == VRTX_WORLD) {
      auto *w = static_cast<World *>(o);
      w->zeroGroup = nullptr;
      w->zeroInstance = nullptr;
    }
    delete o;
  }
  if (dev->initOk)
    cudaStreamDestroy(dev->stream);
  delete dev;
}

// The extensions this library implements, named as the reference's device
// declares them (visrtx_device.json "dependencies", upper-cased with the
// ANARI_ prefix). Left out: array regions, compressed samplers, instance and
// face-varying attributes, MDL materials, neural geometry.
static const char *const kDeviceExtensions[] = {"ANARI_KHR_CAMERA_DEPTH_OF_FIELD",
    "ANARI_KHR_CAMERA_ORTHOGRAPHIC",
    "ANARI_KHR_CAMERA_PERSPECTIVE",
    "ANARI_KHR_DEVICE_SYNCHRONIZATION",
    "ANARI_KHR_FRAME_ACCUMULATION",
    "ANARI_KHR_FRAME_CHANNEL_PRIMITIVE_ID",
    "ANARI_KHR_FRAME_CHANNEL_OBJECT_ID",
    "ANARI_KHR_FRAME_CHANNEL_INSTANCE_ID",
    "ANARI_KHR_FRAME_COMPLETION_CALLBACK",
    "ANARI_KHR_GEOMETRY_CONE",
    "ANARI_KHR_GEOMETRY_CURVE",
    "ANARI_KHR_GEOMETRY_CYLINDER",
    "ANARI_KHR_GEOMETRY_QUAD",
    "ANARI_KHR_GEOMETRY_SPHERE",
    "ANARI_KHR_GEOMETRY_TRIANGLE",
    "ANARI_KHR_INSTANCE_TRANSFORM",
    "ANARI_KHR_INSTANCE_TRANSFORM_ARRAY",
    "ANARI_KHR_LIGHT_DIRECTIONAL",
    "ANARI_KHR_LIGHT_HDRI",
    "ANARI_KHR_LIGHT_POINT",
    "ANARI_KHR_LIGHT_SPOT",
    "ANARI_KHR_MATERIAL_MATTE",
    "ANARI_KHR_MATERIAL_PHYSICALLY_BASED",
    "ANARI_KHR_RENDERER_AMBIENT_LIGHT",
    "ANARI_KHR_RENDERER_BACKGROUND_COLOR",
    "ANARI_KHR_RENDERER_BACKGROUND_IMAGE",
    "ANARI_KHR_SAMPLER_IMAGE1D",
    "ANARI_KHR_SAMPLER_IMAGE2D",
    "ANARI_KHR_SAMPLER_IMAGE3D",
    "ANARI_KHR_SAMPLER_PRIMITIVE",
    "ANARI_KHR_SAMPLER_TRANSFORM",
    "ANARI_KHR_SPATIAL_FIELD_NANOVDB",
    "ANARI_KHR_SPATIAL_FIELD_STRUCTURED_REGULAR",
    "ANARI_KHR_VOLUME_TRANSFER_FUNCTION1D",
    "ANARI_NV_ARRAY_CUDA",
    "ANARI_NV_FRAME_BUFFERS_CUDA",
    "ANARI_VISRTX_TRIANGLE_BACK_FACE_CULLING",
    nullptr};

VRTX_API int vrtxDeviceGetProperty(VRTXDevice d,
    const char *name,
    int type,
    void *mem,
    uint64_t size,
    uint32_t)
{
  DeviceScope scope(D(d));
  if (!d || !name || !mem)
    return 0;
  std::string n(name);
  if (n == "version" && type == VRTX_INT32 && size >= 4) {
    int32_t v = 13; // VisRTX 0.13.0 device surface
    std::memcpy(mem, &v, 4);
    return 1;
  }
  if (n == "visrtx" && type == VRTX_BOOL && size >= 4) {
    int32_t v = 1;
    std::memcpy(mem, &v, 4);
    return 1;
  }
  if (n == "numSMs" && type == VRTX_INT32 && size >= 4) {
    D(d)->init();
    int32_t v = D(d)->numSMs;
    std::memcpy(mem, &v, 4);
    return 1;
  }
  if (n == "extension" && type == VRTX_STRING_LIST && size >= sizeof(void *)) {
    const char *const *list = kDeviceExtensions;
    std::memcpy(mem, &list, sizeof(list));
    return 1;
  }
  return 0;
}

// Subtype lists per object type: what the constructors above accept (the
// reference's generated query_object_types lists, VisRTXDevice.cpp:80-92,
// for the subtypes this library implements).
static const char *const kCameraSubtypes[] = {"perspective", "orthographic", nullptr};
static const char *const kGeometrySubtypes[] = {
    "triangle", "quad", "sphere", "cylinder", "cone", "curve", nullptr};
static const char *const kLightSubtypes[] = {"directional", "point", "spot", "hdri", nullptr};
static const char *const kMaterialSubtypes[] = {"matte", "physicallyBased", nullptr};
static const char *const kRendererSubtypes[] = {
    "default", "directLight", "raycast", "ao", "dpt", "diffuse_pathtracer", nullptr};
static const char *const kSamplerSubtypes[] = {
    "image1D", "image2D", "image3D", "primitive", "transform", nullptr};
static const char *const kFieldSubtypes[] = {"structuredRegular", "nanovdb", nullptr};
static const char *const kVolumeSubtypes[] = {"transferFunction1D", "scivis", nullptr};
static const char *const kInstanceSubtypes[] = {"transform", nullptr};

VRTX_API const char *const *vrtxGetObjectSubtypes(VRTXDevice, int objectType)
{
  switch (objectType) {
  case VRTX_CAMERA:
    return kCameraSubtypes;
  case VRTX_GEOMETRY:
    return kGeometrySubtypes;
  case VRTX_LIGHT:
    return kLightSubtypes;
  case VRTX_MATERIAL:
    return kMaterialSubtypes;
  case VRTX_RENDERER:
    return kRendererSubtypes;
  case VRTX_SAMPLER:
    return kSamplerSubtypes;
  case VRTX_SPATIAL_FIELD:
    return kFieldSubtypes;
  case VRTX_VOLUME:
    return kVolumeSubtypes;
  case VRTX_INSTANCE:
    return kInstanceSubtypes;
  default:
    return nullptr;
  }
}

static bool inList(const char *const *list, const char *s)
{
  for (; list && *list; ++list)
    if (std::strcmp(*list, s) == 0)
      return true;
  return false;
}

// Sets the flags named by a feature list, as fillExtensionStruct does
// (VisRTXFeatureUtility.cpp:39-64). The reference's flags spell three
// features with a VISRTX prefix that its device declares under their ANARI
// names (NV_ARRAY_CUDA, NV_FRAME_BUFFERS_CUDA, KHR_SPATIAL_FIELD_NANOVDB):
// both spellings set the flag. MDL is never available here.
static void fillExtensions(VRTXExtensions *ext, const char *const *list)
{
  std::memset(ext, 0, sizeof(*ext));
  auto has = [&](const char *a, const char *b) {
    return inList(list, a) || (b && inList(list, b));
  };
  ext->VISRTX_ARRAY_CUDA = has("ANARI_VISRTX_ARRAY_CUDA", "ANARI_NV_ARRAY_CUDA");
  ext->VISRTX_CUDA_OUTPUT_BUFFERS =
      has("ANARI_VISRTX_CUDA_OUTPUT_BUFFERS", "ANARI_NV_FRAME_BUFFERS_CUDA");
  ext->VISRTX_INSTANCE_ATTRIBUTES = has("ANARI_VISRTX_INSTANCE_ATTRIBUTES", nullptr);
  ext->VISRTX_SPATIAL_FIELD_NANOVDB =
      has("ANARI_VISRTX_SPATIAL_FIELD_NANOVDB", "ANARI_KHR_SPATIAL_FIELD_NANOVDB");
  ext->VISRTX_TRIANGLE_BACK_FACE_CULLING =
      has("ANARI_VISRTX_TRIANGLE_BACK_FACE_CULLING", nullptr);
  ext->VISRTX_TRIANGLE_FACE_VARYING_ATTRIBUTES =
      has("ANARI_VISRTX_TRIANGLE_FACE_VARYING_ATTRIBUTES", nullptr);
  ext->VISRTX_MATERIAL_MDL = 0;
}

// Per-subtype features: the device's whole list for the objects that
// declare extensions in the reference (the triangle's back-face culling, the
// NanoVDB field, the device-pointer arrays and frame channels), else an
// empty list.
static const char *const kTriangleFeatures[] = {
    "ANARI_KHR_GEOMETRY_TRIANGLE", "ANARI_VISRTX_TRIANGLE_BACK_FACE_CULLING", nullptr};
static const char *const kNanovdbFeatures[] = {"ANARI_KHR_SPATIAL_FIELD_NANOVDB", nullptr};
static const char *const kNoFeatures[] = {nullptr};

VRTX_API int vrtxGetObjectExtensions(
    VRTXExtensions *ext, VRTXDevice d, int objectType, const char *subtype)
{
  if (!ext || !subtype)
    return 0;
  const char *const *list = nullptr;
  if (objectType == VRTX_DEVICE)
    list = kDeviceExtensions;
  else if (inList(vrtxGetObjectSubtypes(d, objectType), subtype)) {
    if (objectType == VRTX_GEOMETRY && std::strcmp(subtype, "triangle") == 0)
      list = kTriangleFeatures;
    else if (objectType == VRTX_SPATIAL_FIELD && std::strcmp(subtype, "nanovdb") == 0)
      list = kNanovdbFeatures;
    else
      list = kNoFeatures;
  }
  if (!list)
    return 0;
  fillExtensions(ext, list);
  return 1;
}

VRTX_API int vrtxGetInstanceExtensions(VRTXExtensions *ext, VRTXDevice d, VRTXObject o)
{
  if (!ext || !d || o)
    return 0; // only the device carries an "extension" property
  const char *const *list = nullptr;
  if (!vrtxDeviceGetProperty(d, "extension", VRTX_STRING_LIST, &list, sizeof(list), 1))
    return 0;
  fillExtensions(ext, list);
  return 1;
}

VRTX_API int vrtxDeviceIsValid(VRTXDevice d)
{
  DeviceScope scope(D(d));
  return d && D(d)->init() ? 1 : 0;
}

static VRTXArray newArray(VRTXDevice d,
    int dims,
    const void *mem,
    VRTXMemoryDeleter del,
    const void *ud,
    int et,
    uint64_t n1,
    uint64_t n2,
    uint64_t n3)
{
  Device *dev = D(d);
  if (!dev)
    return nullptr;
  VRTX_GUARD_BEGIN
  std::lock_guard<std::recursive_mutex> lock(dev->mutex);
  if (!dev->init())
    return nullptr;
  if (sizeOfType(et) == 0 && !isObjectType(et)) {
    dev->report(nullptr, VRTX_SEVERITY_ERROR, "array element type not supported");
    return nullptr;
  }
  auto *a = new Array(dev, dims, mem, del, ud, et, n1, n2, n3);
  if (isObjectType(et) && (a->appIsDevice || a->appIsForeign)) {
    // Array.cpp:78-81
    a->appMem = nullptr; // not the library's to release or delete
    a->deleter = nullptr;
    delete a;
    dev->report(nullptr,
        VRTX_SEVERITY_ERROR,
        "illegal operation: cannot create object arrays from GPU memory");
    return nullptr;
  }
  dev->live.push_back(a);
  dev->markChanged();
  return reinterpret_cast<VRTXArray>(a);
  VRTX_GUARD_END(d, nullptr)
}

VRTX_API VRTXArray vrtxNewArray1D(VRTXDevice d,
    const void *mem,
    VRTXMemoryDeleter del,
    const void *ud,
    int et,
    uint64_t n1)
{
  DeviceScope scope(D(d));
  return newArray(d, 1, mem, del, ud, et, n1, 1, 1);
}

VRTX_API VRTXArray vrtxNewArray2D(VRTXDevice d,
    const void *mem,
    VRTXMemoryDeleter del,
    const void *ud,
    int et,
    uint64_t n1,
    uint64_t n2)
{
  DeviceScope scope(D(d));
  return newArray(d, 2, mem, del, ud, et, n1, n2, 1);
}

VRTX_API VRTXArray vrtxNewArray3D(VRTXDevice d,
    const void *mem,
    VRTXMemoryDeleter del,
    const void *ud,
    int et,
    uint64_t n1,
    uint64_t n2,
    uint64_t n3)
{
  DeviceScope scope(D(d));
  return newArray(d, 3, mem, del, ud, et, n1, n2, n3);
}

VRTX_API void *vrtxMapArray(VRTXDevice d, VRTXArray a)
{
  DeviceScope scope(D(d));
  if (!d || !a)
    return nullptr;
  return static_cast<Array *>(O(a))->map();
}

VRTX_API void vrtxUnmapArray(VRTXDevice d, VRTXArray a)
{
  DeviceScope scope(D(d));
  if (!d || !a)
    return;
  std::lock_guard<std::recursive_mutex> lock(D(d)->mutex);
  static_cast<Array *>(O(a))->unmap();
}

VRTX_API VRTXObject vrtxNewCamera(VRTXDevice d, const char *st)
{
  DeviceScope scope(D(d));
  return newObj<Camera>(d, VRTX_CAMERA, st);
}
VRTX_API VRTXObject vrtxNewGeometry(VRTXDevice d, const char *st)
{
  DeviceScope scope(D(d));
  return newObj<Geometry>(d, VRTX_GEOMETRY, st);
}
VRTX_API VRTXObject vrtxNewLight(VRTXDevice d, const char *st)
{
  DeviceScope scope(D(d));
  return newObj<Light>(d, VRTX_LIGHT, st);
}
VRTX_API VRTXObject vrtxNewMaterial(VRTXDevice d, const char *st)
{
  DeviceScope scope(D(d));
  return newObj<Material>(d, VRTX_MATERIAL, st);
}
VRTX_API VRTXObject vrtxNewRenderer(VRTXDevice d, const char *st)
{
  DeviceScope scope(D(d));
  VRTXObject o = newObj<Renderer>(d, VRTX_RENDERER, st);
  if (o) // renderers are usable with defaults before any commit
    static_cast<Renderer *>(O(o))->commit();
  return o;
}
VRTX_API VRTXObject vrtxNewSampler(VRTXDevice d, const char *st)
{
  DeviceScope scope(D(d));
  return newObj<Sampler>(d, VRTX_SAMPLER, st);
}
VRTX_API VRTXObject vrtxNewSpatialField(VRTXDevice d, const char *st)
{
  DeviceScope scope(D(d));
  return newObj<SpatialField>(d, VRTX_SPATIAL_FIELD, st);
}
VRTX_API VRTXObject vrtxNewVolume(VRTXDevice d, const char *st)
{
  DeviceScope scope(D(d));
  return newObj<Volume>(d, VRTX_VOLUME, st);
}
VRTX_API VRTXObject vrtxNewSurface(VRTXDevice d)
{
  DeviceScope scope(D(d));
  return newObj<Surface>(d, VRTX_SURFACE, "");
}
VRTX_API VRTXObject vrtxNewGroup(VRTXDevice d)
{
  DeviceScope scope(D(d));
  return newObj<Group>(d, VRTX_GROUP, "");
}
VRTX_API VRTXObject vrtxNewInstance(VRTXDevice d, const char *st)
{
  DeviceScope scope(D(d));
  VRTXObject o = newObj<Instance>(d, VRTX_INSTANCE, st ? st : "transform");
  if (o)
    static_cast<Instance *>(O(o))->commit();
  return o;
}
VRTX_API VRTXObject vrtxNewWorld(VRTXDevice d)
{
  DeviceScope scope(D(d));
  VRTXObject o = newObj<World>(d, VRTX_WORLD, "");
  if (o)
    static_cast<World *>(O(o))->commit();
  return o;
}
VRTX_API VRTXFrame vrtxNewFrame(VRTXDevice d)
{
  DeviceScope scope(D(d));
  return newObj<Frame>(d, VRTX_FRAME, "");
}

VRTX_API void vrtxSetParameter(
    VRTXDevice d, VRTXObject o, const char *name, int type, const void *mem)
{
  DeviceScope scope(D(d));
  if (!d || !o || !name)
    return;
  VRTX_GUARD_BEGIN
  std::lock_guard<std::recursive_mutex> lock(D(d)->mutex);
  O(o)->setParam(name, type, mem);
  VRTX_GUARD_END(d, )
}

VRTX_API void vrtxUnsetParameter(VRTXDevice d, VRTXObject o, const char *name)
{
  DeviceScope scope(D(d));
  if (!d || !o || !name)
    return;
  std::lock_guard<std::recursive_mutex> lock(D(d)->mutex);
  O(o)->unsetParam(name);
}

VRTX_API void vrtxUnsetAllParameters(VRTXDevice d, VRTXObject o)
{
  DeviceScope scope(D(d));
  if (!d || !o)
    return;
  std::lock_guard<std::recursive_mutex> lock(D(d)->mutex);
  O(o)->unsetAll();
}

VRTX_API void vrtxCommitParameters(VRTXDevice d, VRTXObject o)
{
  DeviceScope scope(D(d));
  if (!d || !o)
    return;
  VRTX_GUARD_BEGIN
  std::lock_guard<std::recursive_mutex> lock(D(d)->mutex);
  O(o)->commitParams();
  VRTX_GUARD_END(d, )
}

VRTX_API void vrtxRelease(VRTXDevice d, VRTXObject o)
{
  DeviceScope scope(D(d));
  if (!d || !o)
    return;
  std::lock_guard<std::recursive_mutex> lock(D(d)->mutex);
  Object *obj = O(o);
  if (--obj->publicRefs <= 0 && obj->refs > 1
      && (obj->type == VRTX_ARRAY1D || obj->type == VRTX_ARRAY2D
          || obj->type == VRTX_ARRAY3D))
    static_cast<Array *>(obj)->privatize();
  releaseObj(obj);
}

VRTX_API void vrtxRetain(VRTXDevice d, VRTXObject o)
{
  DeviceScope scope(D(d));
  if (!d || !o)
    return;
  O(o)->publicRefs++;
  retainObj(O(o));
}

VRTX_API int vrtxGetProperty(VRTXDevice d,
    VRTXObject o,
    const char *name,
    int type,
    void *mem,
    uint64_t size,
    uint32_t mask)
{
  DeviceScope scope(D(d));
  if (!d || !o || !name || !mem)
    return 0;
  VRTX_GUARD_BEGIN
  std::lock_guard<std::recursive_mutex> lock(D(d)->mutex);
  return O(o)->getProperty(name, type, mem, size, mask) ? 1 : 0;
  VRTX_GUARD_END(d, 0)
}

VRTX_API void vrtxRenderFrame(VRTXDevice d, VRTXFrame f)
{
  DeviceScope scope(D(d));
  if (!d || !f)
    return;
  VRTX_GUARD_BEGIN
  std::lock_guard<std::recursive_mutex> lock(D(d)->mutex);
  Object *o = O(f);
  if (o->type != VRTX_FRAME)
    return;
  static_cast<Frame *>(o)->render();
  VRTX_GUARD_END(d, )
}

VRTX_API int vrtxFrameReady(VRTXDevice d, VRTXFrame f, uint32_t waitMask)
{
  DeviceScope scope(D(d));
  if (!d || !f)
    return 1;
  auto *fr = static_cast<Frame *>(O(f));
  if (waitMask & VRTX_WAIT) {
    fr->wait();
    return 1;
  }
  return fr->ready() ? 1 : 0;
}

VRTX_API void vrtxDiscardFrame(VRTXDevice, VRTXFrame) {}

VRTX_API const void *vrtxMapFrame(VRTXDevice d,
    VRTXFrame f,
    const char *channel,
    uint32_t *width,
    uint32_t *height,
    int *pixelType)
{
  DeviceScope scope(D(d));
  uint32_t w0, h0;
  int t0;
  if (!width)
    width = &w0;
  if (!height)
    height = &h0;
  if (!pixelType)
    pixelType = &t0;
  *width = *height = 0;
  *pixelType = VRTX_UNKNOWN;
  if (!d || !f || !channel)
    return nullptr;
  VRTX_GUARD_BEGIN
  std::lock_guard<std::recursive_mutex> lock(D(d)->mutex);
  return static_cast<Frame *>(O(f))->map(channel, width, height, pixelType);
  VRTX_GUARD_END(d, nullptr)
}

VRTX_API void vrtxUnmapFrame(VRTXDevice, VRTXFrame, const char *) {}

VRTX_API int vrtxDebugDiscretizeTF(const float *color,
    int numColor,
    int colorComponents,
    const float *opacity,
    int numOpacity,
    float valueLo,
    float valueHi,
    const float *uniformColor,
    float uniformOpacity,
    float *out)
{
  if (!out || !uniformColor || (color && (numColor < 2 || (colorComponents != 3 && colorComponents != 4)))
      || (opacity && numOpacity < 2))
    return -1;
  discretizeTF(color,
      numColor,
      colorComponents,
      opacity,
      numOpacity,
      valueLo,
      valueHi,
      uniformColor,
      uniformOpacity,
      256,
      out);
  return 0;
}

VRTX_API int vrtxDebugStageImage(int elementType,
    int background,
    const void *texels,
    uint64_t n,
    float *outFloat,
    uint8_t *outBytes)
{
  if (background) {
    const int nc = backgroundChannels(elementType);
    if (!nc || (n && (!texels || !outBytes)))
      return -1;
    stageBackgroundImage(elementType, nc, (const uint8_t *)texels, n, outBytes);
    return 0;
  }
  const uint32_t ch = attrChannels(elementType);
  if (!ch || (n && !texels))
    return -1;
  std::vector<float> f4;
  std::vector<uint8_t> u8;
  const bool isFloat = stageSamplerImage(elementType, ch, (const uint8_t *)texels, n, f4, u8);
  if (isFloat ? !outFloat : !outBytes)
    return -1;
  if (isFloat)
    std::memcpy(outFloat, f4.data(), f4.size() * sizeof(float));
  else
    std::memcpy(outBytes, u8.data(), u8.size());
  return isFloat ? 1 : 0;
}

VRTX_API int vrtxDebugWriteColors(VRTXDevice d,
    const float *accum,
    uint32_t n,
    int frameID,
    int format,
    uint32_t *out)
{
  DeviceScope scope(D(d));
  Device *dev = D(d);
  if (!dev || !dev->init())
    return -1;
  if ((n && (!accum || !out)) || frameID < 0 || (format != 0 && format != 1)) {
    dev->report(nullptr, VRTX_SEVERITY_ERROR, "vrtxDebugWriteColors: invalid arguments");
    return -2;
  }
  if (n == 0)
    return 0;
  cudaStream_t s = dev->stream;
  float4 *dAcc = nullptr;
  uint32_t *dOut = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&dAcc, sizeof(float4) * n, s);
  if (e == cudaSuccess)
    e = cudaMallocAsync((void **)&dOut, sizeof(uint32_t) * n, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dAcc, accum, sizeof(float4) * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    FramebufferGPU fb{};
    fb.frameID = frameID;
    fb.format = format == 0 ? FORMAT_SRGB : FORMAT_UINT;
    fb.outColorU = dOut;
    e = launchWriteColors(fb, dAcc, n, s);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, dOut, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s);
  if (dAcc)
    cudaFreeAsync(dAcc, s);
  if (dOut)
    cudaFreeAsync(dOut, s);
  const cudaError_t es = cudaStreamSynchronize(s);
  if (e == cudaSuccess)
    e = es;
  if (e != cudaSuccess) {
    cudaGetLastError();
    dev->report(nullptr, VRTX_SEVERITY_ERROR, cudaGetErrorString(e));
    return -3;
  }
  return 0;
}

VRTX_API int vrtxDebugRadixSort(
    VRTXDevice d, uint64_t *keys, uint32_t *vals, uint32_t n, int bits)
{
  DeviceScope scope(D(d));
  Device *dev = D(d);
  if (!dev || !dev->init())
    return -1;
  if ((n && (!keys || !vals)) || bits < 1 || bits > 64) {
    dev->report(nullptr, VRTX_SEVERITY_ERROR, "vrtxDebugRadixSort: invalid arguments");
    return -2;
  }
  if (n == 0)
    return 0;
  cudaStream_t s = dev->stream;
  uint64_t *k[2] = {nullptr, nullptr};
  uint32_t *v[2] = {nullptr, nullptr};
  void *scratch = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&k[0], sizeof(uint64_t) * n, s);
  if (e == cudaSuccess)
    e = cudaMallocAsync((void **)&k[1], sizeof(uint64_t) * n, s);
  if (e == cudaSuccess)
    e = cudaMallocAsync((void **)&v[0], sizeof(uint32_t) * n, s);
  if (e == cudaSuccess)
    e = cudaMallocAsync((void **)&v[1], sizeof(uint32_t) * n, s);
  if (e == cudaSuccess)
    e = cudaMallocAsync(&scratch, radixSortScratchBytes(n), s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(k[0], keys, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(v[0], vals, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s);
  uint64_t *ko = nullptr;
  uint32_t *vo = nullptr;
  if (e == cudaSuccess)
    e = radixSortPairs64(k[0], v[0], k[1], v[1], n, bits, scratch, s, &ko, &vo);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(keys, ko, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(vals, vo, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s);
  for (void *p : {(void *)k[0], (void *)k[1], (void *)v[0], (void *)v[1], scratch})
    if (p)
      cudaFreeAsync(p, s);
  const cudaError_t se = cudaStreamSynchronize(s);
  if (e == cudaSuccess)
    e = se;
  if (e != cudaSuccess) {
    cudaGetLastError();
    dev->report(nullptr, VRTX_SEVERITY_ERROR, cudaGetErrorString(e));
    return -3;
  }
  return 0;
}

VRTX_API uint64_t vrtxDebugCopyAccel(
    VRTXDevice d, VRTXObject world, int kind, void *dst, uint64_t capacity)
{
  DeviceScope scope(D(d));
  if (!d || !world || O(world)->type != VRTX_WORLD)
    return 0;
  std::lock_guard<std::recursive_mutex> lock(D(d)->mutex);
  auto *w = static_cast<World *>(O(world));
  cudaStream_t s = D(d)->stream;
  cudaStreamSynchronize(s);
  std::vector<std::pair<const void *, size_t>> parts;
  if (kind == 0 && w->tlas.nodes)
    parts.push_back({w->tlas.nodes, w->tlas.numNodes * sizeof(BVH8Node)});
  else if (kind == 1)
    for (auto &b : w->blases)
      parts.push_back({b.bvh.nodes, b.bvh.numNodes * sizeof(BVH8Node)});
  else if (kind == 2)
    for (auto &b : w->blases) {
      if (b.type == GEOM_TRIANGLE)
        parts.push_back({b.records, b.bvh.numPrims * sizeof(TriRecord)});
    }
  else if (kind == 3 && w->gpu.instances)
    parts.push_back({w->gpu.instances, w->gpu.numInstances * sizeof(InstanceRecord)});
  else if (kind == 4)
    for (auto &b : w->blases) {
      if (b.type == GEOM_SPHERE)
        parts.push_back({b.records, b.bvh.numPrims * sizeof(SphereRecord)});
    }
  else if (kind == 5) {
    // host-side table: per BLAS {type, numNodes, numPrims, pad}
    uint64_t total = w->blases.size() * 16;
    if (dst && capacity >= total)
      for (size_t i = 0; i < w->blases.size(); i++) {
        uint32_t row[4] = {w->blases[i].type,
            w->blases[i].bvh.numNodes,
            w->blases[i].bvh.numPrims,
            0};
        std::memcpy((uint8_t *)dst + 16 * i, row, 16);
      }
    return total;
  }
  uint64_t total = 0;
  for (auto &p : parts)
    total += p.second;
  if (!dst)
    return total;
  if (capacity < total)
    return 0;
  uint64_t off = 0;
  for (auto &p : parts) {
    cudaMemcpy((uint8_t *)dst + off, p.first, p.second, cudaMemcpyDeviceToHost);
    off += p.second;
  }
  return total;
}

VRTX_API float vrtxWorldBuildMilliseconds(VRTXDevice d, VRTXObject world)
{
  DeviceScope scope(D(d));
  if (!d || !world || O(world)->type != VRTX_WORLD)
    return 0.f;
  return static_cast<World *>(O(world))->buildMs;
}

VRTX_API float vrtxFrameKernelMilliseconds(VRTXDevice d, VRTXFrame f)
{
  DeviceScope scope(D(d));
  if (!d || !f)
    return 0.f;
  auto *fr = static_cast<Frame *>(O(f));
  if (!fr->rendered)
    return 0.f;
  fr->wait();
  float ms = 0.f;
  cudaEventElapsedTime(&ms, fr->evKStart, fr->evKEnd);
  return ms;
}

VRTX_API int vrtxFrameKernelLaunches(VRTXDevice d, VRTXFrame f)
{
  DeviceScope scope(D(d));
  if (!d || !f)
    return 0;
  return static_cast<Frame *>(O(f))->launches;
}

void vrtxInternalReport(VRTXDevice d, int severity, const char *msg)
{
  if (d)
    D(d)->report(nullptr, severity, msg);
}

VRTX_API void *vrtxDeviceStream(VRTXDevice d)
{
  DeviceScope scope(D(d));
  if (!d || !D(d)->init())
    return nullptr;
  return D(d)->stream;
}

} // extern "C"
