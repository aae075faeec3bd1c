// The wavefront kernels and their launchers: "ao" (primary, any-hit queue,
// resolve), "default" (primary, the same any-hit queue with shadow rays,
// resolve) and "raycast" (one kernel); shared device code in
// render_impl.cuh.
#include "render_impl.cuh"

namespace vrtx {

namespace {

// ---------------------------------------------------------------------------
// Wavefront form of the "ao" renderer (opaque materials, no volumes).
//
// The reference runs one raygen per pixel that loops over pixelSamples and,
// per hit, traces ambientSamples any-hit rays inline
// (AmbientOcclusion_ptx.cu:86-220, computeAO.h:38-60). Inline, lanes whose
// camera ray missed sit idle while their neighbours trace 16 occlusion rays,
// and the warp runs at a fraction of its width. Here every sample is three
// kernels:
//   k_aoPrimary  camera ray + closest hit; draws the AO directions and
//                appends the rays to a compacted queue (16 slots per hit
//                pixel, reserved with one atomic per warp);
//   k_aoTrace    one thread per queued ray, any-hit traversal only (a
//                small kernel with room for many warps per SM);
//   k_aoResolve  sums weight * attenuation in ray order, shades, and
//                accumulates exactly as accumResults does.
// Each pixel's Philox stream is re-entered at its consumed offset
// (curand_init(seed, 0, frameID*512 + consumed)), which is the position the
// reference's single long-lived state has reached at that point, so every
// random number lands where the reference draws it.
// ---------------------------------------------------------------------------

struct AOPixel
{
  float depth;
  uint32_t prim, obj, inst;
  f3 base; // matte colour of the hit (unused on a miss)
  float weights; // sum of AO weights; < 0 marks a miss
  f3 normal; // outputNormal (Ng of the hit, or the ray direction)
  uint32_t rayBase;
};

struct AORay
{
  float4 orgTmax; // org.xyz, tmax (< 0: weight 0, not traced)
  float4 dirWeight; // dir.xyz, weight
};

// Queue slots for the whole warp at once (all 32 lanes call it; the full
// mask makes them converge): one atomic, each lane's slots after the lanes
// below it, so the warp's rays form one contiguous block.
__device__ __forceinline__ uint32_t warpAppendAll(uint32_t *counter, uint32_t n)
{
  const uint32_t full = 0xffffffffu;
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t incl = n;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t v = __shfl_up_sync(full, incl, d);
    if ((int)lane >= d)
      incl += v;
  }
  const uint32_t total = __shfl_sync(full, incl, 31);
  uint32_t base = 0;
  if (lane == 31 && total)
    base = atomicAdd(counter, total);
  base = __shfl_sync(full, base, 31);
  return base + incl - n;
}

template <bool STATS, bool SEG>
__global__ void __launch_bounds__(128, VRTX_PRIMARY_MIN_BLOCKS) k_aoPrimary(const FrameParams P,
    int sampleIdx,
    uint32_t *consumed,
    AOPixel *pixels,
    AORay *rays,
    uint32_t *rayCount)
{
  const uint32_t lx = blockIdx.x * 8 + (threadIdx.x & 7);
  const uint32_t ly = blockIdx.y * 16 + (threadIdx.x >> 3);
  const FramebufferGPU &fb = P.fb;
  const int x = computePixelX((int)lx, fb.checkerboardID);
  const int y = computePixelY((int)ly, fb.checkerboardID);
  const bool valid = lx < P.launchW && ly < P.launchH && x < (int)fb.w && y < (int)fb.h;
  TravStats st{0u, 0u, 0u, 0u, 0u, 0u, 0u};
  uint32_t nRays = 0;
  RandState rs;
  AOPixel px;
  px.weights = -1.f;
  f3 org = mk3(0.f, 0.f, 0.f), Ns = mk3(0.f, 0.f, 1.f);
  uint32_t idx = 0;
  if (valid) {
    idx = (uint32_t)x + (uint32_t)y * fb.w;
    const uint32_t used = sampleIdx ? consumed[idx] : 0u;
    curand_init((unsigned long long)(y * (int)fb.w + x),
        0ull,
        (unsigned long long)fb.frameID * 512ull + used,
        &rs);
    float sx, sy;
    Ray ray = makePrimaryRay(P, rs, x, y, false, sx, sy);
    Hit h;
    float unused;
    const bool found = traverse<0, STATS, SEG>(P.world,
        ray.org,
        ray.dir,
        ray.tmin,
        ray.tmax,
        P.renderer.cullTriangleBF != 0,
        true,
        h,
        unused,
        P.errorFlag,
        st);
    uint32_t draws = 4;
    if (found) {
      SurfaceHit sh;
      populateSurfaceHit(P.world, ray, h, sh);
      px.depth = sh.t;
      px.prim = geometryPrimId(P.world, sh);
      px.obj = P.world.surfaces[sh.surface].id;
      px.inst = sh.instUserId;
      px.base = matteInit(P.world, sh).baseColor;
      px.normal = sh.Ng;
      px.weights = 0.f;
      org = sh.hitpoint + (sh.epsilon * sh.Ng);
      Ns = sh.Ns;
      nRays = (uint32_t)max(P.renderer.aoSamples, 0);
      draws += 4 * nRays;
    } else {
      px.depth = fminf(1e30f, ray.tmax);
      px.prim = 0u;
      px.obj = ~0u;
      px.inst = ~0u;
      px.normal = ray.dir;
    }
    consumed[idx] = used + draws;
  }
  const uint32_t base = warpAppendAll(rayCount, nRays);
  if (valid) {
    px.rayBase = base;
    for (uint32_t i = 0; i < nRays; i++) {
      const f3 dir = randomDir(rs, Ns);
      const float weight = fmaxf(0.f, dot(dir, Ns));
      px.weights += weight;
      AORay r;
      r.orgTmax = make_float4(
          org.x, org.y, org.z, weight != 0.f ? P.renderer.occlusionDistance : -1.f);
      r.dirWeight = make_float4(dir.x, dir.y, dir.z, weight);
      rays[base + i] = r;
    }
    pixels[idx] = px;
  }
  if (STATS || true) {
    const unsigned long long r = warpSum(valid ? st.rays : 0u);
    if ((threadIdx.x & 31) == 0)
      atomicAdd(P.stats + 0, r);
  }
  if (STATS) {
    const unsigned long long n = warpSum(st.nodes), t = warpSum(st.tris),
                             sp = warpSum(st.spheres), in = warpSum(st.instances);
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(P.stats + 1, n);
      atomicAdd(P.stats + 2, t);
      atomicAdd(P.stats + 3, sp);
      atomicAdd(P.stats + 4, in);
    }
  }
}

// Any-hit pass over the compacted AO ray queue. Persistent: every lane
// holds one ray; a lane whose ray has ended takes the next one from the
// queue (one atomic per warp, once at least VRTX_AO_REFILL lanes wait, or
// when the warp has no live ray), so a warp keeps most lanes busy instead
// of waiting for its slowest ray. Between refill checks each lane takes up
// to VRTX_AO_STEPS traversal steps; the warp votes each time whether this
// is a leaf turn (leaf postponement, occlusionStep). Each ray's result
// depends on that ray alone: neither the queue order in which lanes take
// rays nor the order of its tests changes it.
template <bool STATS, bool SEG>
__global__ void __launch_bounds__(128, VRTX_TRACE_MIN_BLOCKS) k_aoTrace(const FrameParams P,
    const AORay *rays,
    const uint32_t *rayCount,
    uint32_t *fetchCounter,
    float *weighted)
{
  const uint32_t n = *rayCount;
  const uint32_t lane = threadIdx.x & 31u;
  TravStats st{0u, 0u, 0u, 0u, 0u, 0u, 0u};
#if VRTX_AO_SHARED_STACK > 0
  __shared__ uint2 shStack[VRTX_AO_SHARED_STACK * 128];
  SplitStack<VRTX_TRAVERSAL_STACK, VRTX_AO_SHARED_STACK, 128> stack;
  stack.sh = shStack + threadIdx.x;
#else
  LocalStack<VRTX_TRAVERSAL_STACK> stack;
#endif
  OccState s;
  uint32_t idx = 0;
  bool live = false, exhausted = false;
  while (true) {
    const uint32_t want = __ballot_sync(0xffffffffu, !live && !exhausted);
    const uint32_t busy = __ballot_sync(0xffffffffu, live);
#if VRTX_AO_LEAF_TURN > 0
    // leaf tests run once this share (percent) of the live lanes hold a
    // leaf group, or all of them do; until then those lanes keep to nodes
    const uint32_t pend = __ballot_sync(0xffffffffu, live && s.tri.y != 0u);
    const bool leafTurn =
        pend == busy || __popc(pend) * 100u >= __popc(busy) * (uint32_t)VRTX_AO_LEAF_TURN;
#else
    const bool leafTurn = true;
#endif
    if (want && (__popc(want) >= VRTX_AO_REFILL || busy == 0u)) {
      const uint32_t leader = __ffs(want) - 1;
      uint32_t base = 0;
      if (lane == leader)
        base = atomicAdd(fetchCounter, (uint32_t)__popc(want));
      base = __shfl_sync(0xffffffffu, base, leader);
      if ((want >> lane) & 1u) {
        idx = base + __popc(want & ((1u << lane) - 1u));
        if (idx >= n) {
          exhausted = true;
        } else {
          const float4 o = __ldg(&rays[idx].orgTmax);
          if (o.w < 0.f) {
            weighted[idx] = 0.f; // zero weight: not traced
          } else {
            const float4 d = __ldg(&rays[idx].dirWeight);
            st.rays++;
            live = occlusionBegin(
                P.world, s, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), o.w);
            if (!live)
              weighted[idx] = 0.f;
          }
        }
      }
    }
    if (__all_sync(0xffffffffu, exhausted))
      break;
#pragma unroll 1
    for (int k = 0; k < VRTX_AO_STEPS && live; k++) {
      const int r = occlusionStep<STATS, VRTX_TRAVERSAL_STACK, decltype(stack), SEG>(P.world,
          s,
          stack,
          reinterpret_cast<const float4 *>(rays + idx),
          P.errorFlag,
          st,
          leafTurn && k == 0);
      if (r != OCC_CONTINUE) {
        weighted[idx] = r == OCC_HIT ? __ldg(&rays[idx].dirWeight.w) : 0.f;
        live = false;
      }
    }
  }
  // the frame totals, and the same counts for this kernel alone ([8..12])
  const unsigned long long rs = warpSum(st.rays);
  if (lane == 0) {
    atomicAdd(P.stats + 0, rs);
    atomicAdd(P.stats + 8, rs);
  }
  if (STATS) {
    const unsigned long long nn = warpSum(st.nodes), t = warpSum(st.tris),
                             sp = warpSum(st.spheres), in = warpSum(st.instances);
    if (lane == 0) {
      atomicAdd(P.stats + 1, nn);
      atomicAdd(P.stats + 2, t);
      atomicAdd(P.stats + 3, sp);
      atomicAdd(P.stats + 4, in);
      atomicAdd(P.stats + 9, nn);
      atomicAdd(P.stats + 10, t);
      atomicAdd(P.stats + 11, sp);
      atomicAdd(P.stats + 12, in);
    }
  }
}

// One sample of a wavefront pixel into the frame, as renderPixel and
// accumResults do it (gpu_util.h:393-443): tonemapped accumulation, the
// albedo and normal channels, depth-tested ids, and on the last sample the
// output colour with the first-frame 2x2 splat.
__device__ __forceinline__ void accumulateSample(const FrameParams &P,
    uint32_t idx,
    int x,
    int y,
    int sampleIdx,
    int numSamples,
    f3 outputColor,
    float outputOpacity,
    f3 normal,
    float depth,
    uint32_t prim,
    uint32_t obj,
    uint32_t inst)
{
  const FramebufferGPU &fb = P.fb;
  float4 acc = fb.accum[idx];
  const float4 tm = tonemap(make_float4(
      outputColor.x, outputColor.y, outputColor.z, outputOpacity));
  acc.x += tm.x;
  acc.y += tm.y;
  acc.z += tm.z;
  acc.w += tm.w;
  fb.accum[idx] = acc;
  if (fb.albedo)
    fb.albedo[idx] += outputColor;
  if (fb.normal)
    fb.normal[idx] += normal;
  if (!fb.depth || depth < fb.depth[idx]) {
    if (fb.depth)
      fb.depth[idx] = depth;
    if (fb.primID)
      fb.primID[idx] = prim;
    if (fb.objID)
      fb.objID[idx] = obj;
    if (fb.instID)
      fb.instID[idx] = inst;
  }
  if (sampleIdx == numSamples - 1) {
    writeOutputColor(fb, acc, idx, sampleIdx);
    if (fb.checkerboardID == 0 && fb.frameID + sampleIdx == 0) {
      if (x + 1 < (int)fb.w)
        writeOutputColor(fb, acc, idx + 1, sampleIdx);
      if (y + 1 < (int)fb.h)
        writeOutputColor(fb, acc, idx + fb.w, sampleIdx);
      if (x + 1 < (int)fb.w && y + 1 < (int)fb.h)
        writeOutputColor(fb, acc, idx + fb.w + 1, sampleIdx);
    }
  }
}

// the colour of a miss: the background along the ray, at screen position
// (sx, sy) for a background image
__device__ __forceinline__ void missColor(
    const FrameParams &P, f3 dir, float sx, float sy, f3 &outputColor, float &outputOpacity)
{
  f3 color = mk3(0.f, 0.f, 0.f);
  float opacity = 0.f;
  color *= opacity;
  const float4 bg = backgroundOf(P, dir, sx, sy);
  color += mk3(bg.x, bg.y, bg.z) * (1.f - opacity);
  opacity += bg.w * (1.f - opacity);
  outputColor = mk3(0.f, 0.f, 0.f) + color * (1.f - 0.f);
  outputOpacity = 0.f + opacity * (1.f - 0.f);
}

__global__ void __launch_bounds__(128) k_aoResolve(const FrameParams P,
    int sampleIdx,
    int numSamples,
    const AOPixel *pixels,
    const float *weighted)
{
  const uint32_t lx = blockIdx.x * 8 + (threadIdx.x & 7);
  const uint32_t ly = blockIdx.y * 16 + (threadIdx.x >> 3);
  const FramebufferGPU &fb = P.fb;
  const int x = computePixelX((int)lx, fb.checkerboardID);
  const int y = computePixelY((int)ly, fb.checkerboardID);
  if (lx >= P.launchW || ly >= P.launchH || x >= (int)fb.w || y >= (int)fb.h)
    return;
  const RendererGPU &rp = P.renderer;
  const uint32_t idx = (uint32_t)x + (uint32_t)y * fb.w;
  const AOPixel px = pixels[idx];
  f3 outputColor;
  float outputOpacity;
  if (px.weights >= 0.f) {
    float hits = 0.f;
    const int n = max(rp.aoSamples, 0);
    for (int i = 0; i < n; i++)
      hits += weighted[px.rayBase + i];
    const float aoFactor =
        n > 0 ? (px.weights > 0.f ? 1.f - hits / px.weights : 0.f) : 1.f;
    const f3 lighting = aoFactor * rp.ambientIntensity * rp.ambientColor;
    f3 color = mk3(0.f, 0.f, 0.f);
    float opacity = 0.f;
    color += (px.base * lighting) * (1.f - opacity);
    opacity += 1.f * (1.f - opacity);
    color *= opacity;
    outputColor = mk3(0.f, 0.f, 0.f) + color * (1.f - 0.f);
    outputOpacity = 0.f + opacity * (1.f - 0.f);
  } else {
    // a miss keeps the ray direction (frames with a background image do
    // not take this path)
    missColor(P, px.normal, 0.f, 0.f, outputColor, outputOpacity);
  }
  accumulateSample(P, idx, x, y, sampleIdx, numSamples, outputColor, outputOpacity, px.normal,
      px.depth, px.prim, px.obj, px.inst);
}

// ---------------------------------------------------------------------------
// Wavefront form of the "default" (directLight) renderer over opaque matte
// surfaces without volumes, and of "raycast" over opaque surfaces without
// volumes.
//
// The reference's directLight raygen shades each hit inline
// (DirectLight_ptx.cu:73-224,294-418): computeAO's occlusion rays, then per
// light a sample and a shadow any-hit ray (attenuation 1 - opacity along it),
// the contributions summed in light order and scaled by the AO factor; matte
// surfaces give no bounce ray. Inline, lanes whose camera ray missed idle
// while their neighbours trace shadow rays. Here each sample is three
// kernels:
//   k_dlPrimary  camera ray, closest hit, the AO directions and the light
//                samples in the reference's draw order; appends the AO rays
//                and one shadow ray per light (its shaded contribution kept
//                beside it) to the queue that k_aoTrace consumes;
//   k_aoTrace    the any-hit pass, unchanged (a shadow ray has weight 1, so
//                its result is the surface opacity along it);
//   k_dlResolve  AO factor, the lights' contributions times (1 - opacity)
//                in light order, then the compositing and accumulation of
//                the per-pixel kernel.
// "raycast" traces no secondary rays: one kernel shades and accumulates in
// place.
// ---------------------------------------------------------------------------

struct DLPixel
{
  float depth;
  uint32_t prim, obj, inst;
  f3 normal; // outputNormal (Ns of the hit, or the ray direction)
  f3 ambient; // the shaded colour's ambient term
  float opacity; // the material's opacity; < 0 marks a miss
  float weights; // sum of the AO weights
  uint32_t rayBase; // AO rays, then one shadow ray per light
};

template <bool STATS>
__global__ void __launch_bounds__(128, VRTX_PRIMARY_MIN_BLOCKS) k_dlPrimary(const FrameParams P,
    int sampleIdx,
    uint32_t *consumed,
    DLPixel *pixels,
    AORay *rays,
    float4 *payload,
    uint32_t *rayCount)
{
  const uint32_t lx = blockIdx.x * 8 + (threadIdx.x & 7);
  const uint32_t ly = blockIdx.y * 16 + (threadIdx.x >> 3);
  const FramebufferGPU &fb = P.fb;
  const RendererGPU &rp = P.renderer;
  const int x = computePixelX((int)lx, fb.checkerboardID);
  const int y = computePixelY((int)ly, fb.checkerboardID);
  const bool valid = lx < P.launchW && ly < P.launchH && x < (int)fb.w && y < (int)fb.h;
  TravStats st{0u, 0u, 0u, 0u, 0u, 0u, 0u};
  RandState rs;
  DLPixel px;
  px.opacity = -1.f;
  px.weights = 0.f;
  px.rayBase = 0u;
  px.ambient = mk3(0.f, 0.f, 0.f);
  SurfaceHit sh;
  Ray ray;
  bool found = false;
  uint32_t idx = 0, used = 0;
  if (valid) {
    idx = (uint32_t)x + (uint32_t)y * fb.w;
    used = sampleIdx ? consumed[idx] : 0u;
    curand_init((unsigned long long)(y * (int)fb.w + x),
        0ull,
        (unsigned long long)fb.frameID * 512ull + used,
        &rs);
    float sx, sy;
    ray = makePrimaryRay(P, rs, x, y, false, sx, sy);
    Hit h;
    float unused;
    found = traverse<0, STATS, true>(P.world,
        ray.org,
        ray.dir,
        ray.tmin,
        ray.tmax,
        rp.cullTriangleBF != 0,
        true,
        h,
        unused,
        P.errorFlag,
        st);
    if (found) {
      populateSurfaceHit(P.world, ray, h, sh);
      px.depth = sh.t;
      px.prim = geometryPrimId(P.world, sh);
      px.obj = P.world.surfaces[sh.surface].id;
      px.inst = sh.instUserId;
      px.normal = sh.Ns;
    } else {
      px.depth = fminf(1e30f, ray.tmax);
      px.prim = 0u;
      px.obj = ~0u;
      px.inst = ~0u;
      px.normal = ray.dir;
    }
  }
  const uint32_t nAO = (uint32_t)max(rp.aoSamples, 0);
  const uint32_t nL = P.world.numLights;
  const uint32_t base = warpAppendAll(rayCount, valid && found ? nAO + nL : 0u);
  if (valid) {
    uint32_t draws = 4;
    if (found) {
      px.rayBase = base;
      // computeAO first (shadeSurface, DirectLight_ptx.cu:84-90)
      const f3 aoOrg = sh.hitpoint + (sh.epsilon * sh.Ng);
      for (uint32_t i = 0; i < nAO; i++) {
        const f3 dir = randomDir(rs, sh.Ns);
        const float weight = fmaxf(0.f, dot(dir, sh.Ns));
        px.weights += weight;
        AORay r;
        r.orgTmax = make_float4(
            aoOrg.x, aoOrg.y, aoOrg.z, weight != 0.f ? rp.occlusionDistance : -1.f);
        r.dirWeight = make_float4(dir.x, dir.y, dir.z, weight);
        rays[base + i] = r;
      }
      draws += 4 * nAO;
      const MatteState ms = matteInit(P.world, sh);
      px.opacity = ms.opacity;
      if (rp.ambientIntensity > 0.f)
        px.ambient = rp.ambientColor * rp.ambientIntensity * ms.baseColor;
      const f3 shadePoint = sh.hitpoint + (sh.epsilon * sh.Ns);
      for (uint32_t l = 0; l < nL; l++) {
        const LightGPU &L = P.world.lights[l];
        if (L.type != LIGHT_DIRECTIONAL && L.type != LIGHT_POINT && L.type != LIGHT_SPOT)
          draws += 2; // sampleHDRILight's two uniforms
        const LightSample ls = sampleLight(L, sh.hitpoint, rs);
        AORay r;
        float4 pl = make_float4(0.f, 0.f, 0.f, 0.f);
        if (ls.pdf == 0.f) {
          r.orgTmax = make_float4(0.f, 0.f, 0.f, -1.f); // no shadow ray
          r.dirWeight = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
          const f3 thisLight = shadeMaterial(ms, sh.Ns, ls, -ray.dir);
          r.orgTmax = make_float4(shadePoint.x, shadePoint.y, shadePoint.z, ls.dist);
          r.dirWeight = make_float4(ls.dir.x, ls.dir.y, ls.dir.z, 1.f);
          pl = make_float4(thisLight.x, thisLight.y, thisLight.z, anyNan(thisLight) ? 0.f : 1.f);
        }
        rays[base + nAO + l] = r;
        payload[base + nAO + l] = pl;
      }
    }
    consumed[idx] = used + draws;
    pixels[idx] = px;
  }
  const unsigned long long r = warpSum(valid ? st.rays : 0u);
  if ((threadIdx.x & 31) == 0)
    atomicAdd(P.stats + 0, r);
  if (STATS) {
    const unsigned long long n = warpSum(st.nodes), t = warpSum(st.tris),
                             sp = warpSum(st.spheres), in = warpSum(st.instances);
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(P.stats + 1, n);
      atomicAdd(P.stats + 2, t);
      atomicAdd(P.stats + 3, sp);
      atomicAdd(P.stats + 4, in);
    }
  }
}

__global__ void __launch_bounds__(128) k_dlResolve(const FrameParams P,
    int sampleIdx,
    int numSamples,
    const DLPixel *pixels,
    const float *weighted,
    const float4 *payload)
{
  const uint32_t lx = blockIdx.x * 8 + (threadIdx.x & 7);
  const uint32_t ly = blockIdx.y * 16 + (threadIdx.x >> 3);
  const FramebufferGPU &fb = P.fb;
  const int x = computePixelX((int)lx, fb.checkerboardID);
  const int y = computePixelY((int)ly, fb.checkerboardID);
  if (lx >= P.launchW || ly >= P.launchH || x >= (int)fb.w || y >= (int)fb.h)
    return;
  const RendererGPU &rp = P.renderer;
  const uint32_t idx = (uint32_t)x + (uint32_t)y * fb.w;
  const DLPixel px = pixels[idx];
  f3 outputColor;
  float outputOpacity;
  if (px.opacity >= 0.f) {
    const int nAO = max(rp.aoSamples, 0);
    float aoFactor = 1.f;
    if (nAO > 0) {
      float hits = 0.f;
      for (int i = 0; i < nAO; i++)
        hits += weighted[px.rayBase + i];
      aoFactor = px.weights > 0.f ? 1.f - hits / px.weights : 0.f;
    }
    f3 contrib = px.ambient;
    for (uint32_t l = 0; l < P.world.numLights; l++) {
      const uint32_t j = px.rayBase + (uint32_t)nAO + l;
      const float4 pl = payload[j];
      if (pl.w == 0.f)
        continue;
      // surface_o * volume_o, with no volume on the path
      const float attenuation = (1.f - weighted[j]) * 1.f;
      contrib += mk3(pl.x, pl.y, pl.z) * attenuation;
    }
    contrib *= aoFactor;
    // the compositing of the per-pixel kernel (DirectLight_ptx.cu:362-373)
    const f3 srgb = contrib;
    f3 color;
    float opacity;
    if (anyNan(srgb)) {
      color = mk3(0.f, 0.f, 0.f);
      opacity = 0.f;
    } else {
      color = srgb;
      opacity = px.opacity;
    }
    color += srgb * (1.f - opacity);
    opacity += px.opacity * (1.f - opacity);
    color *= opacity;
    outputColor = mk3(0.f, 0.f, 0.f) + color * (1.f - 0.f);
    outputOpacity = 0.f + opacity * (1.f - 0.f);
  } else {
    missColor(P, px.normal, 0.f, 0.f, outputColor, outputOpacity);
  }
  accumulateSample(P, idx, x, y, sampleIdx, numSamples, outputColor, outputOpacity, px.normal,
      px.depth, px.prim, px.obj, px.inst);
}

// "raycast" over opaque surfaces: pixel-corner camera ray, closest hit,
// |dir . Ns| * ambientColor * baseColor (Raycast_ptx.cu:60-179), shaded and
// accumulated in place.
template <bool STATS>
__global__ void __launch_bounds__(128, VRTX_PRIMARY_MIN_BLOCKS) k_raycastWave(const FrameParams P)
{
  const uint32_t lx = blockIdx.x * 8 + (threadIdx.x & 7);
  const uint32_t ly = blockIdx.y * 16 + (threadIdx.x >> 3);
  const FramebufferGPU &fb = P.fb;
  const RendererGPU &rp = P.renderer;
  const int x = computePixelX((int)lx, fb.checkerboardID);
  const int y = computePixelY((int)ly, fb.checkerboardID);
  const bool valid = lx < P.launchW && ly < P.launchH && x < (int)fb.w && y < (int)fb.h;
  TravStats st{0u, 0u, 0u, 0u, 0u, 0u, 0u};
  if (valid) {
    RandState rs;
    curand_init((unsigned long long)(y * (int)fb.w + x),
        0ull,
        (unsigned long long)fb.frameID * 512ull,
        &rs);
    float sx, sy;
    const Ray ray = makePrimaryRay(P, rs, x, y, true, sx, sy);
    Hit h;
    float unused;
    const bool found = traverse<0, STATS, true>(P.world,
        ray.org,
        ray.dir,
        ray.tmin,
        ray.tmax,
        rp.cullTriangleBF != 0,
        true,
        h,
        unused,
        P.errorFlag,
        st);
    const uint32_t idx = (uint32_t)x + (uint32_t)y * fb.w;
    f3 outputColor;
    float outputOpacity;
    if (found) {
      SurfaceHit sh;
      populateSurfaceHit(P.world, ray, h, sh);
      const MatteState ms = matteInit(P.world, sh);
      const f3 lighting = fabsf(dot(ray.dir, sh.Ns)) * rp.ambientColor;
      f3 color = mk3(0.f, 0.f, 0.f);
      float opacity = 0.f;
      color += (ms.baseColor * lighting) * (1.f - opacity);
      opacity += ms.opacity * (1.f - opacity);
      color *= opacity;
      outputColor = mk3(0.f, 0.f, 0.f) + color * (1.f - 0.f);
      outputOpacity = 0.f + opacity * (1.f - 0.f);
      accumulateSample(P, idx, x, y, 0, 1, outputColor, outputOpacity, sh.Ng, sh.t,
          geometryPrimId(P.world, sh), P.world.surfaces[sh.surface].id, sh.instUserId);
    } else {
      missColor(P, ray.dir, sx, sy, outputColor, outputOpacity);
      accumulateSample(P, idx, x, y, 0, 1, outputColor, outputOpacity, ray.dir,
          fminf(1e30f, ray.tmax), 0u, ~0u, ~0u);
    }
  }
  const unsigned long long r = warpSum(valid ? st.rays : 0u);
  if ((threadIdx.x & 31) == 0)
    atomicAdd(P.stats + 0, r);
  if (STATS) {
    const unsigned long long n = warpSum(st.nodes), t = warpSum(st.tris),
                             sp = warpSum(st.spheres), in = warpSum(st.instances);
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(P.stats + 1, n);
      atomicAdd(P.stats + 2, t);
      atomicAdd(P.stats + 3, sp);
      atomicAdd(P.stats + 4, in);
    }
  }
}

} // namespace

size_t aoWavefrontBytes(uint32_t w, uint32_t h, int aoSamples)
{
  const size_t px = (size_t)w * h;
  const size_t rays = px * (size_t)max(aoSamples, 0);
  return px * (sizeof(AOPixel) + sizeof(uint32_t)) + rays * (sizeof(AORay) + 4) + 1024;
}

// The per-sample launches of the wavefront AO renderer for one (stats,
// segment primitives) combination.
template <bool STATS, bool SEG>
static void aoSamples(const FrameParams &P,
    dim3 grid,
    int numSMs,
    uint32_t *consumed,
    AOPixel *pixels,
    AORay *rays,
    uint32_t *rayCount,
    float *weighted,
    cudaStream_t s,
    cudaEvent_t *traceEvents)
{
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_aoTrace<STATS, SEG>, 128, 0);
  const int traceGrid = numSMs * (occ > 0 ? occ : 1);
  const int n = max(P.renderer.numIterations, 1);
  for (int i = 0; i < n; i++) {
    cudaMemsetAsync(rayCount, 0, 8, s); // queue length, fetch counter
    // the primary pass keeps the general traversal (the per-pixel kernel's),
    // so both forms of the renderer produce the same hits bit for bit
    k_aoPrimary<STATS, true><<<grid, 128, 0, s>>>(P, i, consumed, pixels, rays, rayCount);
    if (traceEvents)
      cudaEventRecord(traceEvents[2 * i], s);
    k_aoTrace<STATS, SEG><<<traceGrid, 128, 0, s>>>(P, rays, rayCount, rayCount + 1, weighted);
    if (traceEvents)
      cudaEventRecord(traceEvents[2 * i + 1], s);
    k_aoResolve<<<grid, 128, 0, s>>>(P, i, n, pixels, weighted);
  }
}

size_t dlWavefrontBytes(uint32_t w, uint32_t h, int aoSamples, uint32_t numLights)
{
  const size_t px = (size_t)w * h;
  const size_t rays = px * ((size_t)max(aoSamples, 0) + numLights);
  return px * (sizeof(DLPixel) + sizeof(uint32_t)) + rays * (sizeof(AORay) + 4 + 16) + 1536;
}

template <bool STATS, bool SEG>
static void dlSamples(const FrameParams &P,
    dim3 grid,
    int numSMs,
    uint32_t *consumed,
    DLPixel *pixels,
    AORay *rays,
    float4 *payload,
    uint32_t *rayCount,
    float *weighted,
    cudaStream_t s,
    cudaEvent_t *traceEvents)
{
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_aoTrace<STATS, SEG>, 128, 0);
  const int traceGrid = numSMs * (occ > 0 ? occ : 1);
  const int n = max(P.renderer.numIterations, 1);
  for (int i = 0; i < n; i++) {
    cudaMemsetAsync(rayCount, 0, 8, s); // queue length, fetch counter
    k_dlPrimary<STATS><<<grid, 128, 0, s>>>(P, i, consumed, pixels, rays, payload, rayCount);
    if (traceEvents)
      cudaEventRecord(traceEvents[2 * i], s);
    k_aoTrace<STATS, SEG><<<traceGrid, 128, 0, s>>>(P, rays, rayCount, rayCount + 1, weighted);
    if (traceEvents)
      cudaEventRecord(traceEvents[2 * i + 1], s);
    k_dlResolve<<<grid, 128, 0, s>>>(P, i, n, pixels, weighted, payload);
  }
}

cudaError_t launchDLWavefront(const FrameParams &P,
    int numSMs,
    bool stats,
    void *scratch,
    cudaStream_t s,
    cudaEvent_t *traceEvents)
{
  const size_t px = (size_t)P.fb.w * P.fb.h;
  const size_t nr = px * ((size_t)max(P.renderer.aoSamples, 0) + P.world.numLights);
  uint8_t *p = (uint8_t *)scratch;
  uint32_t *rayCount = (uint32_t *)p;
  p += 256;
  uint32_t *consumed = (uint32_t *)p;
  p += ((px * 4 + 255) / 256) * 256;
  DLPixel *pixels = (DLPixel *)p;
  p += ((px * sizeof(DLPixel) + 255) / 256) * 256;
  AORay *rays = (AORay *)p;
  p += ((nr * sizeof(AORay) + 255) / 256) * 256;
  float4 *payload = (float4 *)p;
  p += ((nr * sizeof(float4) + 255) / 256) * 256;
  float *weighted = (float *)p;
  const dim3 grid((P.launchW + 7) / 8, (P.launchH + 15) / 16);
  const bool seg = P.world.hasSegments != 0;
  if (stats) {
    if (seg)
      dlSamples<true, true>(P, grid, numSMs, consumed, pixels, rays, payload, rayCount, weighted, s, traceEvents);
    else
      dlSamples<true, false>(P, grid, numSMs, consumed, pixels, rays, payload, rayCount, weighted, s, traceEvents);
  } else {
    if (seg)
      dlSamples<false, true>(P, grid, numSMs, consumed, pixels, rays, payload, rayCount, weighted, s, traceEvents);
    else
      dlSamples<false, false>(P, grid, numSMs, consumed, pixels, rays, payload, rayCount, weighted, s, traceEvents);
  }
  return cudaGetLastError();
}

cudaError_t launchRaycastWavefront(const FrameParams &P, bool stats, cudaStream_t s)
{
  const dim3 grid((P.launchW + 7) / 8, (P.launchH + 15) / 16);
  if (stats)
    k_raycastWave<true><<<grid, 128, 0, s>>>(P);
  else
    k_raycastWave<false><<<grid, 128, 0, s>>>(P);
  return cudaGetLastError();
}

cudaError_t launchAOWavefront(const FrameParams &P,
    int numSMs,
    bool stats,
    void *scratch,
    cudaStream_t s,
    cudaEvent_t *traceEvents)
{
  const size_t px = (size_t)P.fb.w * P.fb.h;
  const size_t nr = px * (size_t)max(P.renderer.aoSamples, 0);
  uint8_t *p = (uint8_t *)scratch;
  uint32_t *rayCount = (uint32_t *)p;
  p += 256;
  uint32_t *consumed = (uint32_t *)p;
  p += ((px * 4 + 255) / 256) * 256;
  AOPixel *pixels = (AOPixel *)p;
  p += ((px * sizeof(AOPixel) + 255) / 256) * 256;
  AORay *rays = (AORay *)p;
  p += ((nr * sizeof(AORay) + 255) / 256) * 256;
  float *weighted = (float *)p;
  const dim3 grid((P.launchW + 7) / 8, (P.launchH + 15) / 16);
  const bool seg = P.world.hasSegments != 0;
  if (stats) {
    if (seg)
      aoSamples<true, true>(P, grid, numSMs, consumed, pixels, rays, rayCount, weighted, s, traceEvents);
    else
      aoSamples<true, false>(P, grid, numSMs, consumed, pixels, rays, rayCount, weighted, s, traceEvents);
  } else {
    if (seg)
      aoSamples<false, true>(P, grid, numSMs, consumed, pixels, rays, rayCount, weighted, s, traceEvents);
    else
      aoSamples<false, false>(P, grid, numSMs, consumed, pixels, rays, rayCount, weighted, s, traceEvents);
  }
  return cudaGetLastError();
}

} // namespace vrtx
