// Differentiable emission-absorption marcher (forward + adjoint), batched
// over many views of many volumes in one persistent launch.
//
// The model is the one stated in include/vrtx.h next to vrtxDMForward. Its
// classification and compositing are the reference scivis marcher's
// (devices/rtx/gpu/volumeIntegration.h:46-103: TF lookup, alpha ->
// 1 - (1 - alpha)^(step/unit), front-to-back accumulation), written in the
// log-transmittance form so that
//   * the forward sums sigma_k = (step/unit) * log(1 - alpha_k) with Kahan
//     compensation (long rays keep T accurate), and
//   * the adjoint walks the same samples in reverse from the end state
//     (log T_end, sample count: stored by the forward kernel, or still in
//     registers in the fused L2 training step), recovering log T_k =
//     log T_{k+1} - sigma_k without storing any per-sample state, and
//     building the suffix radiance S_k = S_{k+1} + T_k a_k c_k from
//     S_K = T_end * background, so dL/dsigma_k = g . (S_{k+1} - T_{k+1} c_k)
//     needs no division.
// Density is read as fp32, fp16 or bf16 and interpolated in fp32; TF
// gradients are staged per thread and per warp in shared memory; density
// gradients are staged per thread and go to fp32 global memory as vector
// reductions.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/vrtx.h"
#include "vmath.h"

namespace vrtx {
namespace {

constexpr float kAlphaMax = 0.999f;
constexpr float kLogTStop = -6.90775527898f; // log(1e-3)
constexpr int kMaxSamples = 1 << 20; // per ray (the host also bounds step)

struct DMVol
{
  const void *density;
  int type;
  int dims[3];
  const void *tf; // tfSize x RGBA, fp32 (float4) or fp16 / bf16 (4 x 16 bit)
  int tfType; // 0 fp32, 1 fp16, 2 bf16
  int tfSize;
  float scale, step, ratio, lo, hi, invRange;
  int sx, sy, sz; // index strides to the +1 neighbour (0 on a 1-voxel axis)
  float *gD;
  float *gTF;
  float *gS;
  const float *scalePtr; // device scalar overriding `scale`
  int flags; // VRTX_DM_PLAIN: one atomic per gradient term
};

struct DMViewG
{
  int vol, w, h, tilesX;
  f3 eye, d00, du, dv, bg;
  long long pixOff;
  unsigned tileStart;
};

template <typename T>
__device__ __forceinline__ float ld(const T *p, size_t i);
template <>
__device__ __forceinline__ float ld<float>(const float *p, size_t i)
{
  return __ldg(p + i);
}
template <>
__device__ __forceinline__ float ld<__half>(const __half *p, size_t i)
{
  return __half2float(__ldg(p + i));
}
template <>
__device__ __forceinline__ float ld<__nv_bfloat16>(const __nv_bfloat16 *p, size_t i)
{
  return __bfloat162float(__ldg(p + i));
}

// a * s + b per component, one rounding each (the file is compiled
// without implicit contraction, so every kernel rounds alike)
__device__ __forceinline__ f3 fma3(float s, f3 a, f3 b)
{
  return mk3(fmaf(s, a.x, b.x), fmaf(s, a.y, b.y), fmaf(s, a.z, b.z));
}

// A trilinear cell: the index of its lowest corner and the fractions.
struct Tri
{
  size_t base;
  float fx, fy, fz;
};

__device__ __forceinline__ void axis(float p, int n, int &i0, float &f)
{
  if (n < 2) {
    i0 = 0;
    f = 0.f;
    return;
  }
  const float c = fminf(fmaxf(p, 0.f), float(n - 1));
  i0 = min((int)floorf(c), n - 2);
  f = c - float(i0);
}

__device__ __forceinline__ Tri triSetup(const DMVol &v, f3 p)
{
  int ix, iy, iz;
  Tri t;
  axis(p.x, v.dims[0], ix, t.fx);
  axis(p.y, v.dims[1], iy, t.fy);
  axis(p.z, v.dims[2], iz, t.fz);
  const size_t X = v.dims[0], XY = (size_t)v.dims[0] * v.dims[1];
  t.base = (size_t)iz * XY + (size_t)iy * X + ix;
  return t;
}

template <typename T>
__device__ __forceinline__ float trilinear(const DMVol &v, const Tri &t)
{
  const T *D = reinterpret_cast<const T *>(v.density);
  const size_t b = t.base;
  const float c000 = ld(D, b), c100 = ld(D, b + v.sx);
  const float c010 = ld(D, b + v.sy), c110 = ld(D, b + v.sy + v.sx);
  const float c001 = ld(D, b + v.sz), c101 = ld(D, b + v.sz + v.sx);
  const float c011 = ld(D, b + v.sz + v.sy), c111 = ld(D, b + v.sz + v.sy + v.sx);
  const float c00 = fmaf(t.fx, c100 - c000, c000);
  const float c10 = fmaf(t.fx, c110 - c010, c010);
  const float c01 = fmaf(t.fx, c101 - c001, c001);
  const float c11 = fmaf(t.fx, c111 - c011, c011);
  const float c0 = fmaf(t.fy, c10 - c00, c00);
  const float c1 = fmaf(t.fy, c11 - c01, c01);
  return fmaf(t.fz, c1 - c0, c0);
}

// One TF entry in fp32 whatever the storage type (uniform per volume).
__device__ __forceinline__ float4 tfEntry(const DMVol &v, int i)
{
  if (v.tfType == 0)
    return __ldg(reinterpret_cast<const float4 *>(v.tf) + i);
  const uint2 raw = __ldg(reinterpret_cast<const uint2 *>(v.tf) + i);
  float2 lo, hi;
  if (v.tfType == 1) {
    lo = __half22float2(*reinterpret_cast<const __half2 *>(&raw.x));
    hi = __half22float2(*reinterpret_cast<const __half2 *>(&raw.y));
  } else {
    lo = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&raw.x));
    hi = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&raw.y));
  }
  return make_float4(lo.x, lo.y, hi.x, hi.y);
}

struct Classified
{
  float4 c; // rgb + raw TF alpha
  float4 ea, eb; // the two TF entries interpolated
  int i0;
  float f;
  float dxds; // d(x)/d(s), 0 where the value range clamps
};

__device__ __forceinline__ Classified classify(const DMVol &v, float s)
{
  Classified r;
  float u = (s - v.lo) * v.invRange;
  r.dxds = (u > 0.f && u < 1.f) ? float(v.tfSize - 1) * v.invRange : 0.f;
  u = fminf(fmaxf(u, 0.f), 1.f);
  const float x = u * float(v.tfSize - 1);
  r.i0 = min((int)floorf(x), v.tfSize - 2);
  r.f = x - float(r.i0);
  r.ea = tfEntry(v, r.i0);
  r.eb = tfEntry(v, r.i0 + 1);
  r.c = make_float4(fmaf(r.f, r.eb.x - r.ea.x, r.ea.x),
      fmaf(r.f, r.eb.y - r.ea.y, r.ea.y),
      fmaf(r.f, r.eb.z - r.ea.z, r.ea.z),
      fmaf(r.f, r.eb.w - r.ea.w, r.ea.w));
  return r;
}

__device__ __forceinline__ bool rayBox(
    f3 o, f3 d, const int dims[3], float &t0, float &t1)
{
  const f3 inv = mk3(1.f / d.x, 1.f / d.y, 1.f / d.z);
  const f3 hi = mk3(float(dims[0] - 1), float(dims[1] - 1), float(dims[2] - 1));
  const f3 a = (mk3(0.f, 0.f, 0.f) - o) * inv;
  const f3 b = (hi - o) * inv;
  t0 = fmaxf(compMax(fmin3(a, b)), 0.f);
  t1 = compMin(fmax3(a, b));
  return t0 < t1;
}

__device__ __forceinline__ int findView(const DMViewG *views, int n, unsigned item)
{
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (views[mid].tileStart <= item)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ f3 viewRay(const DMViewG &vw, int px, int py)
{
  return normalize(fma3(float(py) + 0.5f, vw.dv, fma3(float(px) + 0.5f, vw.du, vw.d00)));
}

// One ray's forward march: premultiplied colour (background not added),
// final log-transmittance and sample count.
template <typename T>
__device__ __forceinline__ void forwardRay(
    const DMVol &v, f3 eye, f3 d, f3 &C, float &logT, int &k)
{
  C = mk3(0.f, 0.f, 0.f);
  logT = 0.f;
  k = 0;
  float comp = 0.f, t0, t1;
  if (!rayBox(eye, d, v.dims, t0, t1))
    return;
  while (k < kMaxSamples) {
    const float t = fmaf(float(k) + 0.5f, v.step, t0);
    if (t > t1)
      break;
    const f3 p = fma3(t, d, eye);
    const float s = trilinear<T>(v, triSetup(v, p));
    const Classified cl = classify(v, s);
    const float alpha = fminf(cl.c.w * v.scale, kAlphaMax);
    const float sigma = v.ratio * log1pf(-alpha);
    const float T0 = __expf(logT);
    const float a = -expm1f(sigma);
    C = fma3(T0 * a, mk3(cl.c.x, cl.c.y, cl.c.z), C);
    // Kahan: logT += sigma
    const float y = sigma - comp;
    const float nt = logT + y;
    comp = (nt - logT) - y;
    logT = nt;
    k++;
    if (logT < kLogTStop)
      break;
  }
}

// The pixel value: marched colour plus the background seen through T_end.
__device__ __forceinline__ f3 pixelValue(f3 C, float logT, f3 bg)
{
  const float Tend = __expf(logT);
  return fma3(Tend, bg, C);
}

template <typename T>
__global__ void __launch_bounds__(256) k_dmForward(const DMVol *vols,
    const DMViewG *views,
    int numViews,
    unsigned numItems,
    unsigned *counter,
    int tileW,
    int tileH,
    unsigned fetch,
    float *image,
    float *state)
{
  // work items come from the queue `fetch` consecutive tiles at a time
  __shared__ unsigned item;
  unsigned next = 0, left = 0;
  while (true) {
    if (left == 0) {
      __syncthreads();
      if (threadIdx.x == 0)
        item = atomicAdd(counter, fetch);
      __syncthreads();
      next = item;
      left = fetch;
    }
    const unsigned it = next++;
    left--;
    if (it >= numItems)
      break;
    const DMViewG vw = views[findView(views, numViews, it)];
    const unsigned tile = it - vw.tileStart;
    const int px = (int)(tile % vw.tilesX) * tileW + (int)threadIdx.x % tileW;
    const int py = (int)(tile / vw.tilesX) * tileH + (int)threadIdx.x / tileW;
    if (px >= vw.w || py >= vw.h)
      continue;
    DMVol v = vols[vw.vol];
    if (v.scalePtr)
      v.scale = __ldg(v.scalePtr);
    f3 C;
    float logT;
    int k;
    forwardRay<T>(v, vw.eye, viewRay(vw, px, py), C, logT, k);
    const f3 img = pixelValue(C, logT, vw.bg);
    const size_t pix = (size_t)vw.pixOff + (size_t)py * vw.w + px;
    image[3 * pix + 0] = img.x;
    image[3 * pix + 1] = img.y;
    image[3 * pix + 2] = img.z;
    state[2 * pix + 0] = logT;
    state[2 * pix + 1] = __int_as_float(k);
  }
}

// Vector reduction of 4 consecutive floats (16-byte aligned), one L2 atomic
// operation instead of four.
__device__ __forceinline__ void redAddV4(float *p, float a, float b, float c, float d)
{
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(
                   __cvta_generic_to_global(p)),
               "f"(a),
               "f"(b),
               "f"(c),
               "f"(d)
               : "memory");
}

// Adds (a, b) at p[0] and p[dx] (dx 0 or 1). With `vec` (16-byte aligned
// array) the pair goes out as one vector reduction on the aligned float4
// holding p[0], plus a second on the next float4 when p[0] is its last
// element.
__device__ __forceinline__ void redPair(float *p, float a, float b, int dx, bool vec)
{
  if (a == 0.f && b == 0.f)
    return;
  if (dx == 0) {
    atomicAdd(p, a + b);
    return;
  }
  if (!vec) {
    if (a != 0.f)
      atomicAdd(p, a);
    if (b != 0.f)
      atomicAdd(p + 1, b);
    return;
  }
  const unsigned lane = (unsigned)(reinterpret_cast<uintptr_t>(p) >> 2) & 3u;
  float *q = p - lane;
  redAddV4(q,
      lane == 0u ? a : 0.f,
      lane == 0u ? b : (lane == 1u ? a : 0.f),
      lane == 1u ? b : (lane == 2u ? a : 0.f),
      lane == 2u ? b : (lane == 3u ? a : 0.f));
  if (lane == 3u)
    redAddV4(q + 4, b, 0.f, 0.f, 0.f);
}

// Commits a trilinear cell's 8 corner accumulators: the x-pairs of its four
// (y, z) rows go out as one 16-byte vector reduction each when the pair
// sits inside an aligned float4 (`vec`: the gradient array is 16-byte
// aligned), else as scalar atomics.
__device__ __forceinline__ void flushCell(
    const DMVol &v, size_t base, float acc[8], bool vec)
{
  if (base == ~size_t(0))
    return;
  float *g = v.gD + base;
  redPair(g, acc[0], acc[1], v.sx, vec);
  redPair(g + v.sy, acc[2], acc[3], v.sx, vec);
  redPair(g + v.sz, acc[4], acc[5], v.sx, vec);
  redPair(g + v.sz + v.sy, acc[6], acc[7], v.sx, vec);
#pragma unroll
  for (int q = 0; q < 8; q++)
    acc[q] = 0.f;
}

// TF gradients live in one shared-memory copy per warp (float4 per entry).
// Lanes that add to the same entry at the same time are grouped with
// match.any; each group's leader sums its peers' values with shuffles and
// does one plain read-modify-write of the float4, so no shared-memory
// atomics are needed (float atomics on shared memory are much slower than
// this on the hardware measured).
__device__ __forceinline__ void addEntry(float4 *wTF, int e, float4 v, unsigned mask)
{
  const unsigned lane = threadIdx.x & 31u;
  const unsigned peers = __match_any_sync(mask, e);
  const unsigned leader = __ffs(peers) - 1;
  if (peers != (1u << lane)) {
    float4 tot = make_float4(0.f, 0.f, 0.f, 0.f);
    for (unsigned rest = peers; rest; rest &= rest - 1) {
      const int l = __ffs(rest) - 1;
      tot.x += __shfl_sync(peers, v.x, l);
      tot.y += __shfl_sync(peers, v.y, l);
      tot.z += __shfl_sync(peers, v.z, l);
      tot.w += __shfl_sync(peers, v.w, l);
    }
    v = tot;
  }
  if (lane == leader && e >= 0) {
    float4 o = wTF[e];
    o.x += v.x;
    o.y += v.y;
    o.z += v.z;
    o.w += v.w;
    wTF[e] = o;
  }
}

// Adds a segment's 8 accumulators to entries seg and seg + 1 of this warp's
// copy (entries seg in one pass, seg + 1 in the next, so that one lane's
// seg + 1 and another's seg never race) and clears them.
__device__ __forceinline__ void flushTF(float4 *wTF, int seg, float acc[8])
{
  const unsigned mask = __activemask();
  const bool has = seg >= 0;
  addEntry(wTF, has ? seg : -1, make_float4(acc[0], acc[1], acc[2], acc[3]), mask);
  __syncwarp(mask);
  addEntry(wTF, has ? seg + 1 : -2, make_float4(acc[4], acc[5], acc[6], acc[7]), mask);
  __syncwarp(mask);
#pragma unroll
  for (int q = 0; q < 8; q++)
    acc[q] = 0.f;
}

// With VRTX_DM_TF_SLIDE 1 (the default) a run that moves to a neighbouring
// TF segment keeps the entry the two segments share staged (measured
// 28.0 ms against 31.0 ms for committing both entries at every change,
// backward of 32 views of 512^2 at 256^3; shared-memory float atomics
// instead of match.any groups measured 36.6 ms staged and 62.1 ms per term).
#ifndef VRTX_DM_TF_SLIDE
#define VRTX_DM_TF_SLIDE 1
#endif

// Moves a lane's TF staging (the terms of entries seg and seg + 1) to the
// segment `to`. When `to` is a neighbour the shared entry stays staged and
// only the other entry is committed, so a ray crossing segments one by one
// commits one entry per crossing instead of two.
__device__ __forceinline__ void slideTF(float4 *wTF, int &seg, float acc[8], int to)
{
#if VRTX_DM_TF_SLIDE
  const unsigned mask = __activemask();
  int e0 = -1, e1 = -2;
  float4 v0 = make_float4(0.f, 0.f, 0.f, 0.f), v1 = v0;
  if (seg >= 0) {
    if (to == seg + 1) {
      e0 = seg;
      v0 = make_float4(acc[0], acc[1], acc[2], acc[3]);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        acc[q] = acc[q + 4];
        acc[q + 4] = 0.f;
      }
    } else if (to == seg - 1) {
      e0 = seg + 1;
      v0 = make_float4(acc[4], acc[5], acc[6], acc[7]);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        acc[q + 4] = acc[q];
        acc[q] = 0.f;
      }
    } else {
      e0 = seg;
      v0 = make_float4(acc[0], acc[1], acc[2], acc[3]);
      e1 = seg + 1;
      v1 = make_float4(acc[4], acc[5], acc[6], acc[7]);
#pragma unroll
      for (int q = 0; q < 8; q++)
        acc[q] = 0.f;
    }
  }
  addEntry(wTF, e0, v0, mask);
  __syncwarp(mask);
  if (__any_sync(mask, e1 >= 0)) {
    addEntry(wTF, e1, v1, mask);
    __syncwarp(mask);
  }
#else
  flushTF(wTF, seg, acc);
#endif
  seg = to;
}

// Commits a block's TF gradient (the sum of its warps' shared-memory
// copies; one vector reduction per entry when gTF is 16-byte aligned) and
// its opacity-scale gradient (block reduction, one atomic). All threads of
// the block call it; it synchronises the block.
__device__ __forceinline__ void commitBlockGrads(
    const DMVol &v, const float4 *sTF, int tfStride, float *sScale, float gScale)
{
  for (int o = 16; o > 0; o >>= 1)
    gScale += __shfl_xor_sync(0xffffffffu, gScale, o);
  __syncthreads(); // sTF complete; sScale free
  if ((threadIdx.x & 31) == 0)
    sScale[threadIdx.x >> 5] = gScale;
  __syncthreads();
  const int warps = (int)(blockDim.x >> 5);
  if (threadIdx.x == 0 && v.gS) {
    float sum = 0.f;
    for (int i = 0; i < warps; i++)
      sum += sScale[i];
    atomicAdd(v.gS, sum);
  }
  if (v.gTF) {
    const bool vec = (reinterpret_cast<uintptr_t>(v.gTF) & 15u) == 0;
    for (int e = threadIdx.x; e < v.tfSize; e += blockDim.x) {
      float4 t = sTF[e];
      for (int w = 1; w < warps; w++) {
        const float4 u = sTF[w * tfStride + e];
        t.x += u.x;
        t.y += u.y;
        t.z += u.z;
        t.w += u.w;
      }
      if (t.x == 0.f && t.y == 0.f && t.z == 0.f && t.w == 0.f)
        continue;
      if (vec) {
        redAddV4(v.gTF + 4 * e, t.x, t.y, t.z, t.w);
      } else {
        atomicAdd(v.gTF + 4 * e, t.x);
        atomicAdd(v.gTF + 4 * e + 1, t.y);
        atomicAdd(v.gTF + 4 * e + 2, t.z);
        atomicAdd(v.gTF + 4 * e + 3, t.w);
      }
    }
  }
  __syncthreads(); // sTF may be cleared next
}

#ifndef VRTX_DM_BWD_MIN_BLOCKS
#define VRTX_DM_BWD_MIN_BLOCKS 3
#endif

// Per-thread gradient staging of the backward march: the trilinear cell and
// the TF segment the ray is in, with the terms accumulated there since it
// entered them.
struct Stage
{
  size_t cell; // lowest-corner index of the staged trilinear cell
  float dacc[8];
  int tfSeg;
  float tacc[8];
};

__device__ __forceinline__ void stageReset(Stage &st)
{
  st.cell = ~size_t(0);
  st.tfSeg = -1;
#pragma unroll
  for (int q = 0; q < 8; q++) {
    st.dacc[q] = 0.f;
    st.tacc[q] = 0.f;
  }
}

// Commits what a work item left staged. Every lane of the warp calls it.
__device__ __forceinline__ void stageFlush(
    const DMVol &v, bool plain, bool vecD, float4 *wTF, Stage &st)
{
  if (plain)
    return;
  if (v.gTF)
    flushTF(wTF, st.tfSeg, st.tacc);
  if (v.gD)
    flushCell(v, st.cell, st.dacc, vecD);
}

// One ray's adjoint: walks its K samples in reverse from the end state
// (log T_end) with the pixel's loss gradient g, adding the density and TF
// terms to the staging (or straight to memory when `plain`) and the
// opacity-scale term to gScale.
template <typename T>
__device__ __forceinline__ void backwardRay(const DMVol &v,
    f3 eye,
    f3 d,
    f3 bg,
    int K,
    float logT,
    f3 g,
    bool plain,
    bool vecD,
    float4 *wTF,
    Stage &st,
    float &gScale)
{
  float t0 = 0.f, t1 = 0.f;
  if (K <= 0 || !rayBox(eye, d, v.dims, t0, t1))
    return;
  float Tnext = __expf(logT);
  f3 S = Tnext * bg;
  float comp = 0.f;
  for (int k = K - 1; k >= 0; k--) {
    const float t = fmaf(float(k) + 0.5f, v.step, t0);
    const f3 p = fma3(t, d, eye);
    const Tri tr = triSetup(v, p);
    const float s = trilinear<T>(v, tr);
    const Classified cl = classify(v, s);
    const float araw = cl.c.w * v.scale;
    const float alpha = fminf(araw, kAlphaMax);
    const float sigma = v.ratio * log1pf(-alpha);
    // Kahan: logT -= sigma
    const float y = -sigma - comp;
    const float nt = logT + y;
    comp = (nt - logT) - y;
    logT = nt;
    const float Tk = __expf(logT);
    const float a = -expm1f(sigma);
    const float w = Tk * a;
    const f3 c = mk3(cl.c.x, cl.c.y, cl.c.z);
    const f3 dc = w * g;
    const f3 r = fma3(-Tnext, c, S);
    const float dSigma = fmaf(g.z, r.z, fmaf(g.y, r.y, g.x * r.x));
    S = fma3(w, c, S);
    Tnext = Tk;
    // d sigma / d alpha = -ratio / (1 - alpha), with 1 - alpha >= 1e-3
    const float dAlpha =
        araw < kAlphaMax ? dSigma * __fdividef(-v.ratio, 1.f - alpha) : 0.f;
    const float dA = dAlpha * v.scale;
    gScale = fmaf(dAlpha, cl.c.w, gScale);
    const float f0 = 1.f - cl.f, f1 = cl.f;
    if (v.gTF) {
      if (plain) {
        float *e0 = reinterpret_cast<float *>(wTF + cl.i0);
        atomicAdd(e0 + 0, f0 * dc.x);
        atomicAdd(e0 + 1, f0 * dc.y);
        atomicAdd(e0 + 2, f0 * dc.z);
        atomicAdd(e0 + 3, f0 * dA);
        atomicAdd(e0 + 4, f1 * dc.x);
        atomicAdd(e0 + 5, f1 * dc.y);
        atomicAdd(e0 + 6, f1 * dc.z);
        atomicAdd(e0 + 7, f1 * dA);
      } else {
        if (cl.i0 != st.tfSeg)
          slideTF(wTF, st.tfSeg, st.tacc, cl.i0);
        st.tacc[0] = fmaf(f0, dc.x, st.tacc[0]);
        st.tacc[1] = fmaf(f0, dc.y, st.tacc[1]);
        st.tacc[2] = fmaf(f0, dc.z, st.tacc[2]);
        st.tacc[3] = fmaf(f0, dA, st.tacc[3]);
        st.tacc[4] = fmaf(f1, dc.x, st.tacc[4]);
        st.tacc[5] = fmaf(f1, dc.y, st.tacc[5]);
        st.tacc[6] = fmaf(f1, dc.z, st.tacc[6]);
        st.tacc[7] = fmaf(f1, dA, st.tacc[7]);
      }
    }
    if (v.gD && cl.dxds != 0.f) {
      const float dval = fmaf(dA, cl.eb.w - cl.ea.w,
          fmaf(dc.z, cl.eb.z - cl.ea.z, fmaf(dc.y, cl.eb.y - cl.ea.y, dc.x * (cl.eb.x - cl.ea.x))));
      const float ds = dval * cl.dxds;
      if (ds != 0.f) {
        const float gx0 = 1.f - tr.fx, gy0 = 1.f - tr.fy, gz0 = 1.f - tr.fz;
        const float wt[8] = {gx0 * gy0 * gz0,
            tr.fx * gy0 * gz0,
            gx0 * tr.fy * gz0,
            tr.fx * tr.fy * gz0,
            gx0 * gy0 * tr.fz,
            tr.fx * gy0 * tr.fz,
            gx0 * tr.fy * tr.fz,
            tr.fx * tr.fy * tr.fz};
        if (plain) {
          float *G = v.gD + tr.base;
          atomicAdd(G, ds * wt[0]);
          atomicAdd(G + v.sx, ds * wt[1]);
          atomicAdd(G + v.sy, ds * wt[2]);
          atomicAdd(G + v.sy + v.sx, ds * wt[3]);
          atomicAdd(G + v.sz, ds * wt[4]);
          atomicAdd(G + v.sz + v.sx, ds * wt[5]);
          atomicAdd(G + v.sz + v.sy, ds * wt[6]);
          atomicAdd(G + v.sz + v.sy + v.sx, ds * wt[7]);
        } else {
          // consecutive samples mostly stay in one trilinear cell:
          // accumulate there and commit when the ray leaves it
          if (tr.base != st.cell) {
            flushCell(v, st.cell, st.dacc, vecD);
            st.cell = tr.base;
          }
#pragma unroll
          for (int q = 0; q < 8; q++)
            st.dacc[q] = fmaf(ds, wt[q], st.dacc[q]);
        }
      }
    }
  }
}

// The backward pass (FUSED false): each pixel's end state and loss gradient
// come from memory (the forward's state, the caller's gradImage).
// The training step (FUSED true): each pixel is marched forward first, its
// L2 loss gradient lossGrad * (pixel - target) formed in registers, and the
// same thread then runs the adjoint, so one launch does forward, loss and
// backward; `image` (optional) receives the pixels and `loss` (optional)
// has lossScale * sum((pixel - target)^2) added to it.
template <typename T, bool FUSED>
__global__ void __launch_bounds__(256, VRTX_DM_BWD_MIN_BLOCKS) k_dmBackward(const DMVol *vols,
    const DMViewG *views,
    int numViews,
    unsigned numItems,
    unsigned *counter,
    int tileW,
    int tileH,
    unsigned fetch,
    int tfMax,
    const float *state,
    const float *gradImage,
    const float *target,
    float lossGrad,
    float lossScale,
    float *image,
    float *loss)
{
  // TF gradient of one volume: one copy of tfStride float4 entries per warp
  extern __shared__ float4 sTF[];
  const int tfStride = tfMax;
  float4 *wTF = sTF + (threadIdx.x >> 5) * tfStride;
  __shared__ unsigned item;
  __shared__ float sScale[8];
  // The block's TF and opacity-scale gradients stay in shared memory and
  // registers across consecutive work items of the same volume and are
  // committed when the volume changes and at exit.
  int curVol = -1;
  float gScale = 0.f;
  float lossAcc = 0.f;
  // work items come from the queue `fetch` consecutive tiles at a time
  unsigned next = 0, left = 0;
  while (true) {
    __syncthreads();
    if (left == 0) {
      if (threadIdx.x == 0)
        item = atomicAdd(counter, fetch);
      __syncthreads();
      next = item;
      left = fetch;
    }
    const unsigned it = next++;
    left--;
    const int nextVol =
        it < numItems ? views[findView(views, numViews, it)].vol : -1;
    if (nextVol != curVol) {
      if (curVol >= 0)
        commitBlockGrads(vols[curVol], sTF, tfStride, sScale, gScale);
      gScale = 0.f;
      curVol = nextVol;
      if (curVol >= 0)
        for (int i = threadIdx.x; i < (int)(blockDim.x >> 5) * tfStride; i += blockDim.x)
          sTF[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      __syncthreads();
    }
    if (it >= numItems)
      break;
    const DMViewG vw = views[findView(views, numViews, it)];
    DMVol v = vols[vw.vol];
    if (v.scalePtr)
      v.scale = __ldg(v.scalePtr);
    const unsigned tile = it - vw.tileStart;
    const int px = (int)(tile % vw.tilesX) * tileW + (int)threadIdx.x % tileW;
    const int py = (int)(tile / vw.tilesX) * tileH + (int)threadIdx.x / tileW;
    const bool plain = (v.flags & VRTX_DM_PLAIN) != 0;
    const bool vecD = (reinterpret_cast<uintptr_t>(v.gD) & 15u) == 0;
    Stage st;
    stageReset(st);
    if (px < vw.w && py < vw.h) {
      const size_t pix = (size_t)vw.pixOff + (size_t)py * vw.w + px;
      const f3 d = viewRay(vw, px, py);
      int K;
      float logT;
      f3 g;
      if (FUSED) {
        f3 C;
        forwardRay<T>(v, vw.eye, d, C, logT, K);
        const f3 img = pixelValue(C, logT, vw.bg);
        if (image) {
          image[3 * pix + 0] = img.x;
          image[3 * pix + 1] = img.y;
          image[3 * pix + 2] = img.z;
        }
        const f3 diff = mk3(img.x - __ldg(target + 3 * pix),
            img.y - __ldg(target + 3 * pix + 1),
            img.z - __ldg(target + 3 * pix + 2));
        lossAcc += diff.x * diff.x + diff.y * diff.y + diff.z * diff.z;
        g = lossGrad * diff;
      } else {
        K = __float_as_int(state[2 * pix + 1]);
        logT = state[2 * pix + 0];
        g = mk3(gradImage[3 * pix], gradImage[3 * pix + 1], gradImage[3 * pix + 2]);
      }
      backwardRay<T>(v, vw.eye, d, vw.bg, K, logT, g, plain, vecD, wTF, st, gScale);
    }
    // every lane of the warp reaches this point each item; reconverge so
    // that no lane still inside its sample loop (committing TF entries of
    // the warp's shared copy) runs beside this final commit
    __syncwarp();
    stageFlush(v, plain, vecD, wTF, st);
  }
  if (FUSED && loss) {
    for (int o = 16; o > 0; o >>= 1)
      lossAcc += __shfl_xor_sync(0xffffffffu, lossAcc, o);
    if ((threadIdx.x & 31) == 0 && lossAcc != 0.f)
      atomicAdd(loss, lossScale * lossAcc);
  }
}

// --- host side ----------------------------------------------------------------

// Descriptors of one launch, validated and laid out for the device:
// [counter (256 B) | DMVol x numVolumes | DMViewG x numViews].
struct Layout
{
  std::vector<uint8_t> bytes;
  size_t offVols = 256, offViews = 0;
  unsigned numItems = 0;
  int type = 0;
  int maxTf = 0;
  int numViews = 0;
  int tileW = 0, tileH = 0;
  // launch shape: resident blocks per SM (0: as many as fit) and work items
  // per queue fetch
  int blocksPerSM = 0;
  unsigned fetch = 1;
};

int layout(const VRTXDMVolume *volumes,
    int numVolumes,
    const VRTXDMView *views,
    int numViews,
    int tileW,
    int tileH,
    Layout &L,
    const char **err)
{
  if (!volumes || numVolumes <= 0 || !views || numViews <= 0) {
    *err = "no volumes or no views";
    return -1;
  }
  if (tileW <= 0 || tileH <= 0 || (tileW * tileH) % 32 != 0 || tileW * tileH > 256) {
    *err = "tileW * tileH must be a positive multiple of 32, at most 256";
    return -2;
  }
  std::vector<DMVol> hv(numVolumes);
  for (int i = 0; i < numVolumes; i++) {
    const VRTXDMVolume &v = volumes[i];
    if (!v.density || !v.tf || v.tfSize < 2 || v.tfSize > 256 || v.dims[0] < 1
        || v.dims[1] < 1 || v.dims[2] < 1 || !(v.step >= 1e-3f)
        || !(v.unitDistance > 0.f) || !(v.valueHi != v.valueLo)) {
      *err = "invalid volume description";
      return -3;
    }
    if (v.densityType != VRTX_FLOAT32 && v.densityType != VRTX_FLOAT16
        && v.densityType != VRTX_BFLOAT16) {
      *err = "density must be FLOAT32, FLOAT16 or BFLOAT16";
      return -4;
    }
    const int tfType = v.tfType == 0 || v.tfType == VRTX_FLOAT32 ? 0
        : v.tfType == VRTX_FLOAT16                              ? 1
        : v.tfType == VRTX_BFLOAT16                             ? 2
                                                                : -1;
    if (tfType < 0) {
      *err = "tf must be FLOAT32, FLOAT16 or BFLOAT16";
      return -4;
    }
    const size_t elemAlign = tfType == 0 ? 16 : 8;
    if ((reinterpret_cast<uintptr_t>(v.tf) % elemAlign) != 0) {
      *err = "tf must be aligned to one entry (16 bytes fp32, 8 bytes fp16 / bf16)";
      return -4;
    }
    if (i == 0)
      L.type = v.densityType;
    else if (v.densityType != L.type) {
      *err = "all volumes of one launch must share the density type";
      return -5;
    }
    L.maxTf = v.tfSize > L.maxTf ? v.tfSize : L.maxTf;
    DMVol &o = hv[i];
    o.density = v.density;
    o.type = v.densityType;
    for (int k = 0; k < 3; k++)
      o.dims[k] = v.dims[k];
    o.tf = v.tf;
    o.tfType = tfType;
    o.tfSize = v.tfSize;
    o.scale = v.opacityScale;
    o.step = v.step;
    o.ratio = v.step / v.unitDistance;
    o.lo = v.valueLo;
    o.hi = v.valueHi;
    o.invRange = 1.f / (v.valueHi - v.valueLo);
    o.sx = v.dims[0] > 1 ? 1 : 0;
    o.sy = v.dims[1] > 1 ? v.dims[0] : 0;
    o.sz = v.dims[2] > 1 ? v.dims[0] * v.dims[1] : 0;
    o.gD = v.gradDensity;
    o.gTF = v.gradTf;
    o.gS = v.gradOpacityScale;
    o.scalePtr = v.opacityScaleDevice;
    o.flags = v.flags;
  }
  std::vector<DMViewG> hw(numViews);
  unsigned items = 0;
  for (int i = 0; i < numViews; i++) {
    const VRTXDMView &w = views[i];
    if (w.volume < 0 || w.volume >= numVolumes || w.width <= 0 || w.height <= 0
        || w.pixelOffset < 0) {
      *err = "invalid view description";
      return -6;
    }
    DMViewG &o = hw[i];
    o.vol = w.volume;
    o.w = w.width;
    o.h = w.height;
    o.tilesX = (w.width + tileW - 1) / tileW;
    const int tilesY = (w.height + tileH - 1) / tileH;
    o.eye = mk3(w.eye[0], w.eye[1], w.eye[2]);
    o.d00 = mk3(w.d00[0], w.d00[1], w.d00[2]);
    o.du = mk3(w.du[0], w.du[1], w.du[2]);
    o.dv = mk3(w.dv[0], w.dv[1], w.dv[2]);
    o.bg = mk3(w.background[0], w.background[1], w.background[2]);
    o.pixOff = w.pixelOffset;
    o.tileStart = items;
    items += (unsigned)(o.tilesX * tilesY);
  }
  L.numItems = items;
  L.numViews = numViews;
  L.tileW = tileW;
  L.tileH = tileH;
  L.offViews = L.offVols + ((sizeof(DMVol) * numVolumes + 255) / 256) * 256;
  L.bytes.assign(L.offViews + sizeof(DMViewG) * numViews, 0);
  std::memcpy(L.bytes.data() + L.offVols, hv.data(), sizeof(DMVol) * numVolumes);
  std::memcpy(L.bytes.data() + L.offViews, hw.data(), sizeof(DMViewG) * numViews);
  return 0;
}

int gridFor(const void *kernel, int threads, size_t smem, int blocksPerSM)
{
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem);
  per = per > 0 ? per : 1;
  if (blocksPerSM > 0 && blocksPerSM < per)
    per = blocksPerSM;
  return sms * per;
}

// The forward kernel over a descriptor block already on the device.
cudaError_t launchForward(const Layout &L, uint8_t *block, float *image, float *state,
    cudaStream_t s)
{
  unsigned *counter = reinterpret_cast<unsigned *>(block);
  const DMVol *vols = reinterpret_cast<const DMVol *>(block + L.offVols);
  const DMViewG *views = reinterpret_cast<const DMViewG *>(block + L.offViews);
  cudaMemsetAsync(counter, 0, 4, s);
  const int threads = L.tileW * L.tileH;
  switch (L.type) {
  case VRTX_FLOAT16:
    k_dmForward<__half><<<gridFor((const void *)k_dmForward<__half>, threads, 0, L.blocksPerSM), threads, 0, s>>>(
        vols, views, L.numViews, L.numItems, counter, L.tileW, L.tileH, L.fetch, image, state);
    break;
  case VRTX_BFLOAT16:
    k_dmForward<__nv_bfloat16><<<gridFor((const void *)k_dmForward<__nv_bfloat16>, threads, 0, L.blocksPerSM), threads, 0, s>>>(
        vols, views, L.numViews, L.numItems, counter, L.tileW, L.tileH, L.fetch, image, state);
    break;
  default:
    k_dmForward<float><<<gridFor((const void *)k_dmForward<float>, threads, 0, L.blocksPerSM), threads, 0, s>>>(
        vols, views, L.numViews, L.numItems, counter, L.tileW, L.tileH, L.fetch, image, state);
    break;
  }
  return cudaGetLastError();
}

// The adjoint over a descriptor block already on the device: the backward
// pass (state, gradImage) or, with `target`, the fused training step.
struct AdjointArgs
{
  const float *state = nullptr, *gradImage = nullptr;
  const float *target = nullptr;
  float lossGrad = 0.f, lossScale = 0.f;
  float *image = nullptr, *loss = nullptr;
};

template <typename T, bool FUSED>
void launchAdjointT(const Layout &L, uint8_t *block, const AdjointArgs &a, cudaStream_t s)
{
  unsigned *counter = reinterpret_cast<unsigned *>(block);
  const DMVol *vols = reinterpret_cast<const DMVol *>(block + L.offVols);
  const DMViewG *views = reinterpret_cast<const DMViewG *>(block + L.offViews);
  cudaMemsetAsync(counter, 0, 4, s);
  const int threads = L.tileW * L.tileH;
  // one float4 TF-gradient copy per warp
  const size_t smem = sizeof(float4) * (size_t)(threads / 32) * L.maxTf;
  const void *k = (const void *)k_dmBackward<T, FUSED>;
  k_dmBackward<T, FUSED><<<gridFor(k, threads, smem, L.blocksPerSM), threads, smem, s>>>(vols,
      views,
      L.numViews,
      L.numItems,
      counter,
      L.tileW,
      L.tileH,
      L.fetch,
      L.maxTf,
      a.state,
      a.gradImage,
      a.target,
      a.lossGrad,
      a.lossScale,
      a.image,
      a.loss);
}

template <bool FUSED>
cudaError_t launchAdjoint(const Layout &L, uint8_t *block, const AdjointArgs &a, cudaStream_t s)
{
  switch (L.type) {
  case VRTX_FLOAT16:
    launchAdjointT<__half, FUSED>(L, block, a, s);
    break;
  case VRTX_BFLOAT16:
    launchAdjointT<__nv_bfloat16, FUSED>(L, block, a, s);
    break;
  default:
    launchAdjointT<float, FUSED>(L, block, a, s);
    break;
  }
  return cudaGetLastError();
}

cudaError_t launchBackward(const Layout &L, uint8_t *block, const float *state,
    const float *gradImage, cudaStream_t s)
{
  AdjointArgs a;
  a.state = state;
  a.gradImage = gradImage;
  return launchAdjoint<false>(L, block, a, s);
}

// Stream-ordered device copy of a layout (freed by the caller).
uint8_t *upload(const Layout &L, cudaStream_t s)
{
  uint8_t *blk = nullptr;
  if (cudaMallocAsync((void **)&blk, L.bytes.size(), s) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  cudaMemcpyAsync(blk, L.bytes.data(), L.bytes.size(), cudaMemcpyHostToDevice, s);
  return blk;
}

} // namespace
} // namespace vrtx

// status reporting lives in device.cpp
extern "C" void vrtxInternalReport(VRTXDevice d, int severity, const char *msg);

struct VRTXDMPlan_st
{
  VRTXDevice dev;
  vrtx::Layout L;
  uint8_t *block = nullptr;
};

using namespace vrtx;

static int fail(VRTXDevice d, const char *msg, int rc)
{
  vrtxInternalReport(d, VRTX_SEVERITY_ERROR, msg);
  return rc;
}

extern "C" {

VRTX_API int vrtxDMForward(VRTXDevice d,
    const VRTXDMVolume *volumes,
    int numVolumes,
    const VRTXDMView *views,
    int numViews,
    float *image,
    float *state,
    int tileW,
    int tileH,
    void *stream)
{
  cudaStream_t s = (cudaStream_t)stream;
  if (!image || !state)
    return fail(d, "vrtxDMForward: image and state are required", -1);
  Layout L;
  const char *err = nullptr;
  const int rc = layout(volumes, numVolumes, views, numViews, tileW, tileH, L, &err);
  if (rc)
    return fail(d, err, rc);
  uint8_t *blk = upload(L, s);
  if (!blk)
    return fail(d, "vrtxDMForward: device allocation failed", -7);
  const cudaError_t e = launchForward(L, blk, image, state, s);
  cudaFreeAsync(blk, s);
  if (e != cudaSuccess)
    return fail(d, cudaGetErrorString(e), -8);
  return 0;
}

VRTX_API int vrtxDMBackward(VRTXDevice d,
    const VRTXDMVolume *volumes,
    int numVolumes,
    const VRTXDMView *views,
    int numViews,
    const float *image,
    const float *state,
    const float *gradImage,
    int tileW,
    int tileH,
    void *stream)
{
  (void)image;
  cudaStream_t s = (cudaStream_t)stream;
  if (!state || !gradImage)
    return fail(d, "vrtxDMBackward: state and gradImage are required", -1);
  Layout L;
  const char *err = nullptr;
  const int rc = layout(volumes, numVolumes, views, numViews, tileW, tileH, L, &err);
  if (rc)
    return fail(d, err, rc);
  uint8_t *blk = upload(L, s);
  if (!blk)
    return fail(d, "vrtxDMBackward: device allocation failed", -7);
  const cudaError_t e = launchBackward(L, blk, state, gradImage, s);
  cudaFreeAsync(blk, s);
  if (e != cudaSuccess)
    return fail(d, cudaGetErrorString(e), -8);
  return 0;
}

VRTX_API VRTXDMPlan vrtxDMPlanCreate(VRTXDevice d,
    const VRTXDMVolume *volumes,
    int numVolumes,
    const VRTXDMView *views,
    int numViews,
    int tileW,
    int tileH,
    void *stream)
{
  auto *p = new VRTXDMPlan_st();
  p->dev = d;
  const char *err = nullptr;
  if (layout(volumes, numVolumes, views, numViews, tileW, tileH, p->L, &err)) {
    fail(d, err, -1);
    delete p;
    return nullptr;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMalloc((void **)&p->block, p->L.bytes.size()) != cudaSuccess) {
    cudaGetLastError();
    fail(d, "vrtxDMPlanCreate: device allocation failed", -7);
    delete p;
    return nullptr;
  }
  cudaMemcpyAsync(
      p->block, p->L.bytes.data(), p->L.bytes.size(), cudaMemcpyHostToDevice, s);
  cudaStreamSynchronize(s);
  return p;
}

VRTX_API int vrtxDMPlanForward(
    VRTXDMPlan plan, float *image, float *state, void *stream)
{
  if (!plan || !image || !state)
    return -1;
  const cudaError_t e =
      launchForward(plan->L, plan->block, image, state, (cudaStream_t)stream);
  return e == cudaSuccess ? 0 : fail(plan->dev, cudaGetErrorString(e), -8);
}

VRTX_API int vrtxDMPlanBackward(
    VRTXDMPlan plan, const float *state, const float *gradImage, void *stream)
{
  if (!plan || !state || !gradImage)
    return -1;
  const cudaError_t e =
      launchBackward(plan->L, plan->block, state, gradImage, (cudaStream_t)stream);
  return e == cudaSuccess ? 0 : fail(plan->dev, cudaGetErrorString(e), -8);
}

VRTX_API int vrtxDMPlanStepL2(VRTXDMPlan plan,
    const float *target,
    float lossScale,
    float *image,
    float *loss,
    void *stream)
{
  if (!plan || !target)
    return plan ? fail(plan->dev, "vrtxDMPlanStepL2: target is required", -1) : -1;
  if (!std::isfinite(lossScale))
    return fail(plan->dev, "vrtxDMPlanStepL2: lossScale must be finite", -2);
  AdjointArgs a;
  a.target = target;
  a.lossScale = lossScale;
  a.lossGrad = 2.f * lossScale;
  a.image = image;
  a.loss = loss;
  const cudaError_t e = launchAdjoint<true>(plan->L, plan->block, a, (cudaStream_t)stream);
  return e == cudaSuccess ? 0 : fail(plan->dev, cudaGetErrorString(e), -8);
}

VRTX_API int vrtxDMPlanSetLaunch(VRTXDMPlan plan, int blocksPerSM, int tilesPerFetch)
{
  if (!plan)
    return -1;
  if (blocksPerSM < 0 || blocksPerSM > 64 || tilesPerFetch < 1 || tilesPerFetch > 64)
    return fail(plan->dev,
        "vrtxDMPlanSetLaunch: blocksPerSM must be 0..64, tilesPerFetch 1..64",
        -2);
  plan->L.blocksPerSM = blocksPerSM;
  plan->L.fetch = (unsigned)tilesPerFetch;
  return 0;
}

VRTX_API void vrtxDMPlanRelease(VRTXDMPlan plan)
{
  if (!plan)
    return;
  if (plan->block)
    cudaFree(plan->block);
  delete plan;
}

} // extern "C"

// ---------------------------------------------------------------------------
// vrtxDMForwardNoAlloc: the forward pass for callers that cannot allocate
// device memory (a host whose allocator is not CUDA's, code running where
// cudaMalloc is not allowed).
//
// Its scratch -- the launch counter and the volume/view descriptors that
// vrtxDMForward puts in a stream-ordered allocation -- lives in one
// file-scope device array of fixed size instead. Every GPU that loads the
// library holds that array until the process exits. Every call reuses it:
// the counter is cleared and the descriptors are rewritten on each call, so
// two calls that overlap on the GPU (different streams, no ordering) race
// on it.
// ---------------------------------------------------------------------------

namespace {

constexpr int kNoAllocMaxVolumes = 64;
constexpr int kNoAllocMaxViews = 4096;
constexpr size_t kNoAllocBytes = 256
    + ((sizeof(vrtx::DMVol) * kNoAllocMaxVolumes + 255) / 256) * 256
    + sizeof(vrtx::DMViewG) * kNoAllocMaxViews;

__device__ __align__(256) uint8_t g_dmNoAllocScratch[kNoAllocBytes];

// Device address of g_dmNoAllocScratch per device ordinal. The symbol's name
// in host code is only a host-side stand-in; kernels need this address. It
// is looked up once per device and kept for the life of the process, so it
// does not survive a cudaDeviceReset (or a primary-context re-creation) of
// that device.
std::mutex g_noAllocMutex;
uint8_t *g_noAllocAddr[64] = {};

uint8_t *noAllocScratch(VRTXDevice d)
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    fail(d, "vrtxDMForwardNoAlloc: no current CUDA device", -9);
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(g_noAllocMutex);
  if (!g_noAllocAddr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_dmNoAllocScratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      fail(d, "vrtxDMForwardNoAlloc: cudaGetSymbolAddress failed", -9);
      return nullptr;
    }
    g_noAllocAddr[dev] = (uint8_t *)p;
  }
  return g_noAllocAddr[dev];
}

} // namespace

extern "C" VRTX_API int vrtxDMForwardNoAlloc(VRTXDevice d,
    const VRTXDMVolume *volumes,
    int numVolumes,
    const VRTXDMView *views,
    int numViews,
    float *image,
    float *state,
    int tileW,
    int tileH,
    void *stream)
{
  cudaStream_t s = (cudaStream_t)stream;
  // The descriptors are copied from host memory that this call frees when
  // it returns; a captured copy would read freed memory at every replay.
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &capture) != cudaSuccess) {
    cudaGetLastError();
    return fail(d, "vrtxDMForwardNoAlloc: cannot query the stream's capture state", -12);
  }
  if (capture != cudaStreamCaptureStatusNone)
    return fail(d,
        "vrtxDMForwardNoAlloc: the stream is capturing; this entry point copies its "
        "descriptors from host memory on every call",
        -12);
  if (!image || !state)
    return fail(d, "vrtxDMForwardNoAlloc: image and state are required", -1);
  if (numVolumes > kNoAllocMaxVolumes || numViews > kNoAllocMaxViews)
    return fail(d,
        "vrtxDMForwardNoAlloc: at most 64 volumes and 4096 views per call",
        -10);
  Layout L;
  const char *err = nullptr;
  const int rc = layout(volumes, numVolumes, views, numViews, tileW, tileH, L, &err);
  if (rc)
    return fail(d, err, rc);
  uint8_t *blk = noAllocScratch(d);
  if (!blk)
    return -9;
  // the counter is zeroed by launchForward; descriptors overwrite the rest
  if (cudaMemcpyAsync(blk, L.bytes.data(), L.bytes.size(), cudaMemcpyHostToDevice, s)
      != cudaSuccess) {
    cudaGetLastError();
    return fail(d, "vrtxDMForwardNoAlloc: descriptor copy failed", -11);
  }
  const cudaError_t e = launchForward(L, blk, image, state, s);
  if (e != cudaSuccess)
    return fail(d, cudaGetErrorString(e), -8);
  return 0;
}
