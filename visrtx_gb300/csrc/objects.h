// Host object model of libvrtx: the ANARI objects of the VisRTX device
// (devices/rtx/{array,camera,frame,renderer,scene}) reduced to what the hot
// path reads, with helium's parameter/commit/refcount semantics.
#pragma once

#include <atomic>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/vrtx.h"
#include "bvh.h"
#include "render.h"

namespace vrtx {

struct Device;
struct Object;

uint64_t newStamp();
size_t sizeOfType(int t);
bool isObjectType(int t);
const char *typeName(int t);

struct Param
{
  int type = VRTX_UNKNOWN;
  std::vector<uint8_t> bytes;
  std::string str;
  Object *obj = nullptr;
};

struct Object
{
  Device *dev;
  int type;
  std::string subtype;
  std::atomic<int> refs{1}; // internal + public references
  std::atomic<int> publicRefs{1}; // references held by the application
  std::map<std::string, Param> pending;
  std::map<std::string, Param> params; // committed
  uint64_t commitStamp = 0;

  Object(Device *d, int t, const std::string &st = "");
  virtual ~Object();

  void setParam(const std::string &name, int type, const void *mem);
  void unsetParam(const std::string &name);
  void unsetAll();
  void commitParams();
  virtual void commit() {}
  virtual bool isValid() const
  {
    return true;
  }
  virtual bool getProperty(
      const std::string &name, int type, void *mem, uint64_t size, uint32_t mask);
  // newest stamp of this object and everything it references
  virtual uint64_t deepStamp() const
  {
    return commitStamp;
  }

  bool has(const std::string &name, int type) const;
  template <typename T>
  T get(const std::string &name, int type, T def) const
  {
    auto it = params.find(name);
    if (it == params.end() || it->second.type != type
        || it->second.bytes.size() < sizeof(T))
      return def;
    T v;
    std::memcpy(&v, it->second.bytes.data(), sizeof(T));
    return v;
  }
  Object *getObject(const std::string &name, int type) const;
  std::string getString(const std::string &name, const std::string &def) const;

  void report(int severity, const char *fmt, ...) const;
};

void retainObj(Object *o);
void releaseObj(Object *o);

// ---------------------------------------------------------------------------

struct Array : Object
{
  int elemType;
  uint64_t n[3];
  const void *appMem = nullptr;
  VRTXMemoryDeleter deleter = nullptr;
  const void *deleterPtr = nullptr;
  std::vector<uint8_t> owned; // managed arrays / privatised copies
  bool appIsDevice = false; // application memory on this device's GPU
  // application memory on another GPU (the reference's FOREIGN address
  // space, Array.cpp:50-53): copied to this GPU at upload, never read in
  // place
  bool appIsForeign = false;
  void *dptr = nullptr;
  size_t devBytes = 0;
  uint64_t dataStamp = 0;
  uint64_t devStamp = 0;
  // an asynchronous copy reading the application's host memory has been
  // queued on the device stream since the last synchronisation: the stream
  // is synchronised before that memory is given back (privatisation,
  // destruction)
  bool hostReadQueued = false;
  std::vector<Object *> handles; // object arrays: retained elements

  Array(Device *d,
      int dims,
      const void *mem,
      VRTXMemoryDeleter del,
      const void *delPtr,
      int et,
      uint64_t n1,
      uint64_t n2,
      uint64_t n3);
  ~Array() override;
  uint64_t count() const
  {
    return n[0] * n[1] * n[2];
  }
  size_t bytes() const
  {
    return count() * sizeOfType(elemType);
  }
  const void *hostData() const;
  // waits for queued copies that read the application's host memory
  void settleHostReads();
  // device copy (uploads on first use after a data change)
  const void *deviceData();
  void *map();
  void unmap();
  void refreshHandles();
  // shared app memory -> owned copy, once the app no longer holds the array
  // (Array.cpp:164-182)
  void privatize();
  uint64_t deepStamp() const override
  {
    return dataStamp > commitStamp ? dataStamp : commitStamp;
  }
};

struct Camera : Object
{
  CameraGPU gpu{};
  using Object::Object;
  void commit() override;
};

struct Geometry : Object
{
  using Object::Object;
  ~Geometry() override;
  Array *vertex = nullptr, *index = nullptr, *normal = nullptr,
        *normalFV = nullptr, *primId = nullptr, *radius = nullptr;
  float globalRadius = 0.01f;
  bool cull = false;
  bool caps = false;
  uint32_t numPrims = 0;
  Array *vattr[NUM_ATTRS] = {}, *pattr[NUM_ATTRS] = {};
  float4 uattr[NUM_ATTRS] = {};
  // quads: generated triangle indices (2 per quad) on the device
  uint32_t *quadIndices = nullptr;
  uint64_t quadStamp = 0;
  void commit() override;
  bool isValid() const override;
  uint64_t deepStamp() const override;
  int geomClass() const;
  uint32_t kind() const;
  GeometryGPU gpuData();
};

// Material samplers (scene/surface/material/sampler/*.cpp): image1D /
// image2D / image3D (float4 texture from the image array), transform,
// primitive.
struct Sampler : Object
{
  using Object::Object;
  ~Sampler() override;
  Array *image = nullptr, *primArray = nullptr;
  std::string filter = "linear";
  std::string wrap[3] = {"clampToEdge", "clampToEdge", "clampToEdge"};
  uint32_t attribute = 0;
  float inT[16], outT[16];
  float4 inO{0.f, 0.f, 0.f, 0.f}, outO{0.f, 0.f, 0.f, 0.f};
  uint32_t primOffset = 0;
  cudaArray_t cuArray = nullptr;
  cudaTextureObject_t tex = 0;
  uint64_t builtStamp = 0;
  void commit() override;
  bool isValid() const override;
  uint64_t deepStamp() const override;
  void cleanup();
  bool ensureBuilt();
  SamplerGPU gpuData() const;
  uint32_t type() const;
};

struct Material : Object
{
  using Object::Object;
  MaterialGPU gpu{};
  Sampler *samplers[MP_COUNT] = {nullptr, nullptr, nullptr, nullptr};
  void commit() override;
  uint64_t deepStamp() const override;
};

struct Light : Object
{
  using Object::Object;
  LightGPU gpu{};
  // hdri (HDRI.cu): the radiance image, its texture and CDF tables
  Array *radiance = nullptr;
  f3 hdriDirection{1.f, 0.f, 0.f}, hdriUp{0.f, 0.f, 1.f};
  cudaArray_t cuArray = nullptr;
  float *cdfs = nullptr; // marginal (H) then conditional (H x W)
  uint64_t builtStamp = 0;
  ~Light() override;
  void commit() override;
  bool isValid() const override;
  uint64_t deepStamp() const override;
  void cleanup();
  bool ensureBuilt();
};

struct Surface : Object
{
  using Object::Object;
  Geometry *geometry = nullptr;
  Material *material = nullptr;
  uint32_t id = ~0u;
  void commit() override;
  bool isValid() const override;
  uint64_t deepStamp() const override;
};

struct SpatialField : Object
{
  using Object::Object;
  bool nanovdb = false; // subtype "nanovdb" (NvdbRegularField.cpp)
  uint8_t *gridDev = nullptr; // device copy of the NanoVDB grid buffer
  float *bricks = nullptr; // NanoVDB brick cache (9^3 floats per leaf)
  int32_t *brickTable = nullptr; // block -> brick slot, or -2: constant
  float *blockFill = nullptr; // the value of constant blocks
  bool useBricks = true; // "vrtx.brickCache"
  NvdbGPU nvdbGPU{};
  box3 gridBounds{{0.f, 0.f, 0.f}, {1.f, 1.f, 1.f}};
  f3 gridVoxel{1.f, 1.f, 1.f};
  Array *data = nullptr;
  f3 origin{0.f, 0.f, 0.f}, spacing{1.f, 1.f, 1.f};
  std::string filter = "linear";
  cudaArray_t cuArray = nullptr;
  cudaTextureObject_t tex = 0, pointTex = 0;
  int dims[3] = {0, 0, 0};
  int mcDims[3] = {0, 0, 0};
  float *ranges = nullptr; // 2 floats per macrocell
  float *refRanges = nullptr; // delta-tracking grid ranges (reference rule)
  uint64_t builtStamp = 0;
  ~SpatialField() override;
  void commit() override;
  bool isValid() const override;
  uint64_t deepStamp() const override;
  void cleanup();
  bool ensureBuilt();
  bool buildNanovdb();
  void buildNanovdbBricks(const std::vector<int32_t> &leafOrigins);
  box3 bounds() const;
  float stepSize() const;
};

struct Volume : Object
{
  using Object::Object;
  SpatialField *field = nullptr;
  Array *color = nullptr, *opacity = nullptr;
  float valueRange[2] = {0.f, 1.f};
  float unitDistance = 1.f;
  f3 uniformColor{1.f, 1.f, 1.f};
  float uniformColorW = 1.f;
  float uniformOpacity = 1.f;
  uint32_t id = ~0u;
  std::vector<float> tf; // 256 x RGBA
  cudaArray_t tfArray = nullptr;
  cudaTextureObject_t tfTex = 0;
  float4 *tfDev = nullptr;
  float *majorants = nullptr;
  float *dptMajorants = nullptr; // delta-tracking majorants (reference rule)
  bool hasEmptyCells = false; // some skipping-grid cell has majorant 0
  bool emptySpaceSkipping = true; // "vrtx.emptySpaceSkipping"
  uint64_t builtStamp = 0;
  ~Volume() override;
  void commit() override;
  bool isValid() const override;
  uint64_t deepStamp() const override;
  void cleanup();
  bool ensureBuilt();
  void discretize();
};

struct Group : Object
{
  using Object::Object;
  Array *surfaces = nullptr, *volumes = nullptr, *lights = nullptr;
  void commit() override;
  uint64_t deepStamp() const override;
  std::vector<Surface *> validSurfaces() const;
  std::vector<Volume *> validVolumes() const;
  std::vector<Light *> validLights() const;
  bool getProperty(const std::string &name,
      int type,
      void *mem,
      uint64_t size,
      uint32_t mask) override;
};

struct Instance : Object
{
  using Object::Object;
  Group *group = nullptr;
  Array *xfmArray = nullptr, *idArray = nullptr;
  float xfm[12]; // 3 rows x 4
  uint32_t id = ~0u;
  void commit() override;
  bool isValid() const override
  {
    return group != nullptr;
  }
  uint64_t deepStamp() const override;
  size_t numTransforms() const;
  void transform(size_t i, float out[12]) const;
  uint32_t userID(size_t i) const;
};

struct BLASBuild
{
  BVH8Build bvh;
  void *records = nullptr;
  uint32_t type = 0;
  uint32_t numPrims = 0;
};

struct World : Object
{
  using Object::Object;
  Array *instances = nullptr;
  Array *zeroSurfaces = nullptr, *zeroVolumes = nullptr, *zeroLights = nullptr;
  uint32_t id = ~0u;
  Group *zeroGroup = nullptr;
  int maxLeaf[GEOM_NUM_TYPES] = {1, 1, 1, 1, 1}; // single-primitive leaves
  Instance *zeroInstance = nullptr;

  // built state
  uint64_t builtStamp = 0;
  WorldGPU gpu{};
  std::vector<BLASBuild> blases;
  BVH8Build tlas;
  std::vector<void *> allocations;
  box3 worldBounds = emptyBox();
  float buildMs = 0.f;

  ~World() override;
  void commit() override;
  uint64_t deepStamp() const override;
  bool rebuild();
  void freeBuilt();
  std::vector<Instance *> instanceList() const;
  bool getProperty(const std::string &name,
      int type,
      void *mem,
      uint64_t size,
      uint32_t mask) override;
};

struct Renderer : Object
{
  using Object::Object;
  RendererGPU gpu{};
  int spp = 1;
  int sampleLimit = 128;
  bool checkerboard = false;
  // "background" given as an Array2D image (Renderer.cpp:152-175)
  Array *bgImage = nullptr;
  cudaArray_t bgArray = nullptr;
  uint64_t bgStamp = 0;
  ~Renderer() override;
  void commit() override;
  bool isValid() const override;
  uint64_t deepStamp() const override;
  bool ensureBackground();
};

struct Frame : Object
{
  using Object::Object;
  Renderer *renderer = nullptr;
  Camera *camera = nullptr;
  World *world = nullptr;
  uint32_t size[2] = {10, 10};
  int colorType = VRTX_UFIXED8_RGBA_SRGB;
  int depthType = VRTX_UNKNOWN, primType = VRTX_UNKNOWN,
      objType = VRTX_UNKNOWN, instType = VRTX_UNKNOWN,
      albedoType = VRTX_UNKNOWN, normalType = VRTX_UNKNOWN;
  VRTXFrameCompletionCallback callback = nullptr;
  const void *callbackPtr = nullptr;

  FramebufferGPU fb{};
  void *buffers[10] = {};
  uint32_t *workCounter = nullptr;
  uint32_t *errorFlag = nullptr;
  unsigned long long *stats = nullptr; // see FrameParams::stats
  bool countTraversal = false; // "vrtx.countTraversal": counting build
  uint32_t maxTraversalSteps = 1u << 22; // "vrtx.maxTraversalSteps"
  bool forceMegakernel = false; // "vrtx.megakernel": per-pixel kernel only
  void *scratch = nullptr; // wavefront queues (stream-ordered allocation)
  size_t scratchBytes = 0;
  bool nextFrameReset = true;
  uint64_t lastSeenStamp = 0;
  cudaEvent_t evStart = nullptr, evEnd = nullptr, evKStart = nullptr,
              evKEnd = nullptr;
  std::vector<cudaEvent_t> traceEvents; // around each AO any-hit launch
  int tracePairs = 0; // pairs recorded by the last render
  bool rendered = false;
  int launches = 0;
  std::vector<uint8_t> hostColor, hostDepth, hostPrim, hostObj, hostInst,
      hostAlbedo, hostNormal;

  ~Frame() override;
  void commit() override;
  bool isValid() const override;
  void freeBuffers();
  cudaError_t frameAlloc(void **p, size_t bytes, cudaStream_t s);
  void render();
  void wait();
  bool ready();
  const void *map(const std::string &channel,
      uint32_t *w,
      uint32_t *h,
      int *pixelType);
  bool getProperty(const std::string &name,
      int type,
      void *mem,
      uint64_t size,
      uint32_t mask) override;
};

struct Device
{
  VRTXStatusCallback cb = nullptr;
  const void *cbPtr = nullptr;
  // the GPU requested through "cudaDevice", and the one init() chose; a
  // request after init is reported and ignored (VisRTXDevice.cpp:464-470)
  int desiredDevice = 0;
  int cudaDevice = 0;
  bool forceInit = false;
  // devices made through the ANARI entry points report ANARI codes:
  // reportMap(0, objectType) and reportMap(1, severity)
  int (*reportMap)(int kind, int value) = nullptr;
  std::recursive_mutex mutex;
  // written once under the mutex by init(); read without it by the
  // per-call device scope
  std::atomic<bool> initTried{false};
  std::atomic<bool> initOk{false};
  cudaStream_t stream = nullptr;
  int numSMs = 0;
  // host-side fault injection: the next N frame allocations fail without a
  // CUDA call ("vrtx.failFrameAllocations")
  std::atomic<int> failFrameAllocs{0};
  std::atomic<uint64_t> lastChange{0};
  std::vector<Object *> live; // every object ever created and not destroyed

  bool init();
  void report(const Object *src, int severity, const char *msg);
  void markChanged()
  {
    lastChange = newStamp();
  }
};

} // namespace vrtx
