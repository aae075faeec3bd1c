// GPU BVH8 builder. See bvh.h for the pipeline.
//
// Design notes:
//  * The binary tree is the Karras (HPG 2012) radix tree over 63-bit Morton
//    codes; equal codes are disambiguated by the sorted index, so the tree is
//    well formed for any input.
//  * Before the collapse, a bottom-up pass solves the SAH-optimal collapse
//    of the binary tree into 8-wide nodes (Ylitie, Karras and Laine, HPG
//    2017): C(n, i), the cost of representing subtree n by at most i
//    children of a wide node, from C(n, 1) = a leaf (<= maxLeafPrims
//    primitives: A(n) * count * C_PRIM) or a wide node (A(n) * C_NODE +
//    D(n, 8)), and C(n, i) = min(C(n, i - 1), D(n, i)) with the distribution
//    D(n, j) = min_k C(left, k) + C(right, j - k); each node keeps its
//    choices (the split k per i, and whether D is taken) in one word.
//  * The collapse runs level by level: every thread takes one task (a binary
//    subtree root and the BVH8 slot it fills), takes its children from the
//    SAH choices (or, with VRTX_BVH_SAH 0, opens up to 8 children by
//    repeatedly splitting the child with the largest surface area), turns
//    subtrees of <= maxLeafPrims primitives into leaves, assigns children to
//    slots so that the slot index XOR the ray octant gives a near-to-far
//    order, quantises child boxes outward, and appends one task per internal
//    child. Node and primitive ranges are claimed with atomics, so a node's
//    internal children are contiguous and its leaf primitives are contiguous.
#include <utility>

#include "bvh.h"
#include "radix_sort.h"

namespace vrtx {
namespace {

constexpr uint32_t LEAF_BIT = 0x80000000u;
constexpr uint32_t NONE = 0xFFFFFFFFu;

// --- bounds reduction -------------------------------------------------------

__global__ void k_boundsPartial(
    const box3 *boxes, uint32_t n, box3 *partialCent, box3 *partialAll)
{
  __shared__ box3 sc[256];
  __shared__ box3 sa[256];
  box3 c = emptyBox(), a = emptyBox();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const box3 b = boxes[i];
    extend(a, b);
    extend(c, (b.lo + b.hi) * 0.5f);
  }
  sc[threadIdx.x] = c;
  sa[threadIdx.x] = a;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      extend(sc[threadIdx.x], sc[threadIdx.x + s]);
      extend(sa[threadIdx.x], sa[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partialCent[blockIdx.x] = sc[0];
    partialAll[blockIdx.x] = sa[0];
  }
}

// the partial boxes of k_boundsPartial's blocks reduced by one block of
// 256 threads (one partial per thread, then a shared-memory tree)
__global__ void k_boundsFinal(box3 *partialCent, box3 *partialAll, int nb)
{
  __shared__ box3 sc[256];
  __shared__ box3 sa[256];
  box3 c = emptyBox(), a = emptyBox();
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    extend(c, partialCent[i]);
    extend(a, partialAll[i]);
  }
  sc[threadIdx.x] = c;
  sa[threadIdx.x] = a;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      extend(sc[threadIdx.x], sc[threadIdx.x + s]);
      extend(sa[threadIdx.x], sa[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partialCent[0] = sc[0];
    partialAll[0] = sa[0];
  }
}

// --- Morton codes -----------------------------------------------------------

__device__ __forceinline__ uint64_t spread21(uint32_t v)
{
  uint64_t x = v & 0x1fffffu;
  x = (x | x << 32) & 0x1f00000000ffffull;
  x = (x | x << 16) & 0x1f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}

__device__ __forceinline__ uint32_t quant21(float v, float lo, float ext)
{
  float u = ext > 0.f ? (v - lo) / ext : 0.5f;
  u = fminf(fmaxf(u * 2097152.f, 0.f), 2097151.f);
  return (uint32_t)u;
}

__global__ void k_morton(const box3 *boxes,
    uint32_t n,
    const box3 *centBounds,
    uint64_t *keys,
    uint32_t *vals)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const box3 cb = centBounds[0];
  const box3 b = boxes[i];
  const f3 c = (b.lo + b.hi) * 0.5f;
  const f3 e = cb.hi - cb.lo;
  const uint32_t qx = quant21(c.x, cb.lo.x, e.x);
  const uint32_t qy = quant21(c.y, cb.lo.y, e.y);
  const uint32_t qz = quant21(c.z, cb.lo.z, e.z);
  keys[i] = (spread21(qx) << 2) | (spread21(qy) << 1) | spread21(qz);
  vals[i] = i;
}

// --- Karras radix tree --------------------------------------------------------

__device__ __forceinline__ int delta(
    const uint64_t *keys, int n, int i, int j)
{
  if (j < 0 || j >= n)
    return -1;
  const uint64_t ki = keys[i], kj = keys[j];
  if (ki == kj)
    return 64 + __clz((uint32_t)(i ^ j));
  return __clzll(ki ^ kj);
}

__global__ void k_karras(const uint64_t *keys,
    int n,
    uint32_t *left,
    uint32_t *right,
    uint32_t *parentInternal,
    uint32_t *parentLeaf)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1)
    return;
  const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = delta(keys, n, i, i - d);
  int lmax = 2;
  while (delta(keys, n, i, i + lmax * d) > dmin)
    lmax *= 2;
  int l = 0;
  for (int t = lmax / 2; t >= 1; t /= 2)
    if (delta(keys, n, i, i + (l + t) * d) > dmin)
      l += t;
  const int j = i + l * d;
  const int dnode = delta(keys, n, i, j);
  int s = 0;
  int div = 2;
  int t = (l + div - 1) / div;
  while (true) {
    if (delta(keys, n, i, i + (s + t) * d) > dnode)
      s += t;
    if (t <= 1)
      break;
    div *= 2;
    t = (l + div - 1) / div;
  }
  const int gamma = i + s * d + min(d, 0);
  const int lo = min(i, j), hi = max(i, j);
  uint32_t L, R;
  if (lo == gamma) {
    L = LEAF_BIT | (uint32_t)gamma;
    parentLeaf[gamma] = i;
  } else {
    L = (uint32_t)gamma;
    parentInternal[gamma] = i;
  }
  if (hi == gamma + 1) {
    R = LEAF_BIT | (uint32_t)(gamma + 1);
    parentLeaf[gamma + 1] = i;
  } else {
    R = (uint32_t)(gamma + 1);
    parentInternal[gamma + 1] = i;
  }
  left[i] = L;
  right[i] = R;
  if (i == 0)
    parentInternal[0] = NONE;
}

// --- bottom-up refit ----------------------------------------------------------

__device__ __forceinline__ box3 loadBoxL2(const box3 *p)
{
  const float *f = reinterpret_cast<const float *>(p);
  box3 b;
  b.lo.x = __ldcg(f + 0);
  b.lo.y = __ldcg(f + 1);
  b.lo.z = __ldcg(f + 2);
  b.hi.x = __ldcg(f + 3);
  b.hi.y = __ldcg(f + 4);
  b.hi.z = __ldcg(f + 5);
  return b;
}

__global__ void k_refit(int n,
    const uint32_t *sortedIdx,
    const box3 *boxes,
    const uint32_t *left,
    const uint32_t *right,
    const uint32_t *parentInternal,
    const uint32_t *parentLeaf,
    box3 *internalBoxes,
    uint32_t *internalCount,
    uint32_t *flags)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || n < 2)
    return;
  uint32_t p = parentLeaf[i];
  while (p != NONE) {
    __threadfence();
    if (atomicAdd(&flags[p], 1u) == 0)
      return;
    __threadfence();
    box3 b = emptyBox();
    uint32_t cnt = 0;
    const uint32_t kids[2] = {left[p], right[p]};
    for (int k = 0; k < 2; k++) {
      const uint32_t r = kids[k];
      if (r & LEAF_BIT) {
        extend(b, boxes[sortedIdx[r & ~LEAF_BIT]]);
        cnt += 1;
      } else {
        extend(b, loadBoxL2(internalBoxes + r));
        cnt += __ldcg(internalCount + r);
      }
    }
    internalBoxes[p] = b;
    internalCount[p] = cnt;
    p = parentInternal[p];
  }
}

// --- SAH-optimal collapse costs ---------------------------------------------

#ifndef VRTX_BVH_SAH
#define VRTX_BVH_SAH 1
#endif

#ifndef VRTX_SAH_PRIM_COST
#define VRTX_SAH_PRIM_COST 0.3f
#endif
constexpr float kCostNode = 1.0f; // a wide-node test
constexpr float kCostPrim = VRTX_SAH_PRIM_COST; // a primitive test

// decision word: 4 bits per i = 2..8 at bit 4 (i - 2): the split k (1..7)
// of D(n, i) in bits 0-2, bit 3 set when C(n, i) takes D(n, i) (else it is
// C(n, i - 1)); i = 8 is the wide-node distribution of C(n, 1)
__device__ __forceinline__ uint32_t decSplit(uint32_t d, int i)
{
  return (d >> (4 * (i - 2))) & 7u;
}

__device__ __forceinline__ bool decTakesD(uint32_t d, int i)
{
  return (d >> (4 * (i - 2) + 3)) & 1u;
}

__global__ void k_sahCosts(int n,
    const uint32_t *sortedIdx,
    const box3 *boxes,
    const uint32_t *left,
    const uint32_t *right,
    const uint32_t *parentInternal,
    const uint32_t *parentLeaf,
    const box3 *internalBoxes,
    const uint32_t *internalCount,
    int maxLeaf,
    float *cost, // 7 per internal node: C(n, 1..7)
    uint32_t *dec,
    uint32_t *flags)
{
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (i0 >= n || n < 2)
    return;
  uint32_t p = parentLeaf[i0];
  while (p != NONE) {
    __threadfence();
    if (atomicAdd(&flags[p], 1u) == 0)
      return;
    __threadfence();
    float cc[2][8];
    const uint32_t kids[2] = {left[p], right[p]};
    for (int k = 0; k < 2; k++) {
      const uint32_t r = kids[k];
      if (r & LEAF_BIT) {
        const float c = halfArea(boxes[sortedIdx[r & ~LEAF_BIT]]) * kCostPrim;
        for (int i = 1; i < 8; i++)
          cc[k][i] = c;
      } else {
        for (int i = 1; i < 8; i++)
          cc[k][i] = __ldcg(cost + (size_t)r * 7 + (i - 1));
      }
    }
    float D[9];
    uint32_t kBest[9];
    for (int j = 2; j <= 8; j++) {
      float best = 3.4e38f;
      uint32_t bk = 1;
      for (int k = 1; k < j; k++) {
        const float c = cc[0][min(k, 7)] + cc[1][min(j - k, 7)];
        if (c < best) {
          best = c;
          bk = (uint32_t)k;
        }
      }
      D[j] = best;
      kBest[j] = bk;
    }
    const float area = halfArea(loadBoxL2(internalBoxes + p));
    const uint32_t cnt = __ldcg(internalCount + p);
    float C = cnt <= (uint32_t)maxLeaf ? area * (float)cnt * kCostPrim
                                       : area * kCostNode + D[8];
    uint32_t d = (kBest[8] | 8u) << (4 * 6);
    cost[(size_t)p * 7] = C;
    for (int i = 2; i <= 7; i++) {
      const bool takeD = D[i] < C;
      if (takeD)
        C = D[i];
      d |= (kBest[i] | (takeD ? 8u : 0u)) << (4 * (i - 2));
      cost[(size_t)p * 7 + (i - 1)] = C;
    }
    dec[p] = d;
    p = parentInternal[p];
  }
}

// --- collapse to BVH8 -------------------------------------------------------

struct CollapseArgs
{
  const uint32_t *left;
  const uint32_t *right;
  const uint32_t *internalCount;
  const box3 *internalBoxes;
  const box3 *boxes;
  const uint32_t *sortedIdx;
  BVH8Node *nodes;
  uint32_t *primOrder;
  uint32_t *counters; // [0] nodes, [1] prims, [2] out tasks
  const uint2 *tasksIn;
  const uint32_t *numTasks; // this level's task count (device)
  uint32_t capacity; // tasks a level can hold
  uint2 *tasksOut;
  uint32_t *numTasksOut; // the next level's task count (device)
  int maxLeaf;
  const uint32_t *dec; // SAH choices (null: largest-area opening)
};

__device__ __forceinline__ box3 refBox(const CollapseArgs &a, uint32_t r)
{
  return (r & LEAF_BIT) ? a.boxes[a.sortedIdx[r & ~LEAF_BIT]]
                        : a.internalBoxes[r];
}

__device__ __forceinline__ uint32_t refCount(const CollapseArgs &a, uint32_t r)
{
  return (r & LEAF_BIT) ? 1u : a.internalCount[r];
}

// Smallest power of two s with 255 * s >= extent, as a biased exponent.
__device__ __forceinline__ uint32_t quantExp(float lo, float hi)
{
  const float d = __fsub_ru(hi, lo);
  const float ext = __fdiv_ru(d, 255.f);
  if (!(ext > 0.f))
    return 1u; // 2^-126: degenerate axis
  const uint32_t bits = __float_as_uint(ext);
  uint32_t e = bits >> 23;
  if (bits & 0x7fffffu)
    e += 1;
  return min(max(e, 1u), 254u);
}

__device__ __forceinline__ void collapseTask(const CollapseArgs &a, uint32_t tid)
{
  const uint2 task = a.tasksIn[tid];
  const uint32_t nodeIdx = task.y;

  uint32_t c[8];
  int nc;
  if (task.x & LEAF_BIT) {
    c[0] = task.x;
    nc = 1;
  } else if (a.dec) {
    // the SAH choices: distribute 8 slots over the subtree; a binary node
    // given j >= 2 slots splits per its decision for j (falling back to
    // fewer slots where that is cheaper), given 1 it becomes one child
    uint32_t ref[8];
    int slots[8];
    int sp = 0;
    nc = 0;
    const uint32_t k8 = decSplit(a.dec[task.x], 8);
    ref[sp] = a.right[task.x];
    slots[sp++] = 8 - (int)k8;
    ref[sp] = a.left[task.x];
    slots[sp++] = (int)k8;
    while (sp > 0 && nc < 8) {
      const uint32_t m = ref[--sp];
      int j = slots[sp];
      if (!(m & LEAF_BIT)) {
        const uint32_t dm = a.dec[m];
        while (j >= 2 && !decTakesD(dm, j))
          j--;
        if (j >= 2 && sp + 2 <= 8) {
          const int kk = (int)decSplit(dm, j);
          ref[sp] = a.right[m];
          slots[sp++] = j - kk;
          ref[sp] = a.left[m];
          slots[sp++] = kk;
          continue;
        }
      }
      c[nc++] = m;
    }
  } else {
    c[0] = a.left[task.x];
    c[1] = a.right[task.x];
    nc = 2;
  }
  while (!a.dec && nc < 8) {
    int best = -1;
    float bestA = -1.f;
    for (int i = 0; i < nc; i++) {
      const uint32_t r = c[i];
      if (!(r & LEAF_BIT) && a.internalCount[r] > (uint32_t)a.maxLeaf) {
        const float ar = halfArea(a.internalBoxes[r]);
        if (ar > bestA) {
          bestA = ar;
          best = i;
        }
      }
    }
    if (best < 0)
      break;
    const uint32_t r = c[best];
    c[best] = a.left[r];
    c[nc++] = a.right[r];
  }

  box3 b[8];
  box3 nb = emptyBox();
  for (int i = 0; i < nc; i++) {
    b[i] = refBox(a, c[i]);
    extend(nb, b[i]);
  }

  // slot assignment: slot s is visited first by rays whose octant is s
  const f3 pc = (nb.lo + nb.hi) * 0.5f;
  float cost[8][8];
  for (int i = 0; i < nc; i++) {
    const f3 d = (b[i].lo + b[i].hi) * 0.5f - pc;
    for (int s = 0; s < 8; s++)
      cost[i][s] = ((s & 1) ? -d.x : d.x) + ((s & 2) ? -d.y : d.y)
          + ((s & 4) ? -d.z : d.z);
  }
  int childAt[8];
  for (int s = 0; s < 8; s++)
    childAt[s] = -1;
  uint32_t assigned = 0;
  for (int k = 0; k < nc; k++) {
    float bc = 3.4e38f;
    int bi = -1, bs = -1;
    for (int i = 0; i < nc; i++) {
      if (assigned & (1u << i))
        continue;
      for (int s = 0; s < 8; s++) {
        if (childAt[s] >= 0)
          continue;
        if (cost[i][s] < bc || bi < 0) {
          bc = cost[i][s];
          bi = i;
          bs = s;
        }
      }
    }
    assigned |= 1u << bi;
    childAt[bs] = bi;
  }

  int numInternal = 0;
  int numLeafPrims = 0;
  for (int i = 0; i < nc; i++) {
    const uint32_t cnt = refCount(a, c[i]);
    if (!(c[i] & LEAF_BIT) && cnt > (uint32_t)a.maxLeaf)
      numInternal++;
    else
      numLeafPrims += (int)cnt;
  }

  const uint32_t childBase =
      numInternal ? atomicAdd(&a.counters[0], (uint32_t)numInternal) : 0u;
  const uint32_t primBase =
      numLeafPrims ? atomicAdd(&a.counters[1], (uint32_t)numLeafPrims) : 0u;
  const uint32_t taskBase =
      numInternal ? atomicAdd(a.numTasksOut, (uint32_t)numInternal) : 0u;

  BVH8Node node;
  node.px = nb.lo.x;
  node.py = nb.lo.y;
  node.pz = nb.lo.z;
  const uint32_t ex = quantExp(nb.lo.x, nb.hi.x);
  const uint32_t ey = quantExp(nb.lo.y, nb.hi.y);
  const uint32_t ez = quantExp(nb.lo.z, nb.hi.z);
  node.ex = (uint8_t)ex;
  node.ey = (uint8_t)ey;
  node.ez = (uint8_t)ez;
  // 1 / 2^e, exact as long as 254 - e >= 1
  const float isx = __uint_as_float((254u - ex) << 23);
  const float isy = __uint_as_float((254u - ey) << 23);
  const float isz = __uint_as_float((254u - ez) << 23);
  node.childBase = childBase;
  node.primBase = primBase;
  uint8_t imask = 0;
  int k = 0;
  int off = 0;
  for (int s = 0; s < 8; s++) {
    const int i = childAt[s];
    if (i < 0) {
      node.meta[s] = 0;
      node.qlox[s] = node.qloy[s] = node.qloz[s] = 0;
      node.qhix[s] = node.qhiy[s] = node.qhiz[s] = 0;
      continue;
    }
    const box3 cb = b[i];
    node.qlox[s] = (uint8_t)fminf(fmaxf(floorf(__fsub_rd(cb.lo.x, nb.lo.x) * isx), 0.f), 255.f);
    node.qloy[s] = (uint8_t)fminf(fmaxf(floorf(__fsub_rd(cb.lo.y, nb.lo.y) * isy), 0.f), 255.f);
    node.qloz[s] = (uint8_t)fminf(fmaxf(floorf(__fsub_rd(cb.lo.z, nb.lo.z) * isz), 0.f), 255.f);
    node.qhix[s] = (uint8_t)fminf(fmaxf(ceilf(__fsub_ru(cb.hi.x, nb.lo.x) * isx), 0.f), 255.f);
    node.qhiy[s] = (uint8_t)fminf(fmaxf(ceilf(__fsub_ru(cb.hi.y, nb.lo.y) * isy), 0.f), 255.f);
    node.qhiz[s] = (uint8_t)fminf(fmaxf(ceilf(__fsub_ru(cb.hi.z, nb.lo.z) * isz), 0.f), 255.f);
    const uint32_t r = c[i];
    const uint32_t cnt = refCount(a, r);
    if (!(r & LEAF_BIT) && cnt > (uint32_t)a.maxLeaf) {
      node.meta[s] = (uint8_t)(0x20u | (24u + s));
      imask |= (uint8_t)(1u << s);
      a.tasksOut[taskBase + k] = make_uint2(r, childBase + k);
      k++;
    } else {
      node.meta[s] = (uint8_t)((((1u << cnt) - 1u) << 5) | (uint32_t)off);
      // gather the (<= 3) primitives of this subtree in order
      uint32_t stack[4];
      int sp = 0;
      stack[sp++] = r;
      int w = 0;
      while (sp > 0) {
        const uint32_t q = stack[--sp];
        if (q & LEAF_BIT) {
          a.primOrder[primBase + off + w] = a.sortedIdx[q & ~LEAF_BIT];
          w++;
        } else {
          stack[sp++] = a.right[q];
          stack[sp++] = a.left[q];
        }
      }
      off += (int)cnt;
    }
  }
  node.imask = imask;
  a.nodes[nodeIdx] = node;
}

// One level of the collapse: the task count comes from the device, so levels
// are queued without a host round trip (grid-stride over the tasks).
__global__ void k_collapse(CollapseArgs a)
{
  const uint32_t num = min(*a.numTasks, a.capacity);
  for (uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x; tid < num;
       tid += gridDim.x * blockDim.x)
    collapseTask(a, tid);
}

__global__ void k_iota(uint32_t *v, uint32_t n)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    v[i] = i;
}

template <typename T>
cudaError_t dalloc(T **p, size_t count, cudaStream_t s)
{
  return cudaMallocAsync((void **)p, sizeof(T) * (count ? count : 1), s);
}

} // namespace

cudaError_t buildBVH8(const box3 *d_boxes,
    uint32_t n,
    cudaStream_t stream,
    BVH8Build &out,
    int maxLeafPrims)
{
  out = BVH8Build{};
  if (n == 0)
    return cudaSuccess;
  maxLeafPrims = maxLeafPrims < 1 ? 1 : (maxLeafPrims > 3 ? 3 : maxLeafPrims);
  cudaError_t err = cudaSuccess;
#define VRTX_TRY(x)                                                            \
  do {                                                                         \
    err = (x);                                                                 \
    if (err != cudaSuccess)                                                    \
      goto fail;                                                               \
  } while (0)

  const int T = 256;
  const int nbPartial = 256;
  box3 *pCent = nullptr, *pAll = nullptr;
  uint64_t *keys = nullptr, *keysSorted = nullptr;
  uint32_t *vals = nullptr, *valsSorted = nullptr;
  void *tmp = nullptr;
  uint32_t *left = nullptr, *right = nullptr, *parI = nullptr, *parL = nullptr;
  box3 *iBoxes = nullptr;
  uint32_t *iCount = nullptr, *flags = nullptr, *counters = nullptr;
  float *sahCost = nullptr;
  uint32_t *sahDec = nullptr;
  uint2 *tasksA = nullptr, *tasksB = nullptr;
  box3 hostAll;
  uint32_t hostCounters[4];

  VRTX_TRY(dalloc(&pCent, nbPartial, stream));
  VRTX_TRY(dalloc(&pAll, nbPartial, stream));
  k_boundsPartial<<<nbPartial, 256, 0, stream>>>(d_boxes, n, pCent, pAll);
  k_boundsFinal<<<1, 256, 0, stream>>>(pCent, pAll, nbPartial);

  VRTX_TRY(dalloc(&keys, n, stream));
  VRTX_TRY(dalloc(&keysSorted, n, stream));
  VRTX_TRY(dalloc(&vals, n, stream));
  VRTX_TRY(dalloc(&valsSorted, n, stream));
  k_morton<<<(n + T - 1) / T, T, 0, stream>>>(d_boxes, n, pCent, keys, vals);
  VRTX_TRY(cudaMallocAsync(&tmp, radixSortScratchBytes(n), stream));
  {
    uint64_t *kSorted = nullptr;
    uint32_t *vSorted = nullptr;
    VRTX_TRY(radixSortPairs64(
        keys, vals, keysSorted, valsSorted, n, 63, tmp, stream, &kSorted, &vSorted));
    if (kSorted != keysSorted) {
      std::swap(keys, keysSorted);
      std::swap(vals, valsSorted);
    }
  }

  VRTX_TRY(dalloc(&left, n, stream));
  VRTX_TRY(dalloc(&right, n, stream));
  VRTX_TRY(dalloc(&parI, n, stream));
  VRTX_TRY(dalloc(&parL, n, stream));
  VRTX_TRY(dalloc(&iBoxes, n, stream));
  VRTX_TRY(dalloc(&iCount, n, stream));
  VRTX_TRY(dalloc(&flags, n, stream));
  VRTX_TRY(cudaMemsetAsync(flags, 0, sizeof(uint32_t) * n, stream));
  if (n > 1) {
    k_karras<<<(n - 1 + T - 1) / T, T, 0, stream>>>(
        keysSorted, (int)n, left, right, parI, parL);
    k_refit<<<(n + T - 1) / T, T, 0, stream>>>((int)n,
        valsSorted,
        d_boxes,
        left,
        right,
        parI,
        parL,
        iBoxes,
        iCount,
        flags);
    if (VRTX_BVH_SAH) {
      VRTX_TRY(dalloc(&sahCost, (size_t)n * 7, stream));
      VRTX_TRY(dalloc(&sahDec, n, stream));
      VRTX_TRY(cudaMemsetAsync(flags, 0, sizeof(uint32_t) * n, stream));
      k_sahCosts<<<(n + T - 1) / T, T, 0, stream>>>((int)n,
          valsSorted,
          d_boxes,
          left,
          right,
          parI,
          parL,
          iBoxes,
          iCount,
          maxLeafPrims,
          sahCost,
          sahDec,
          flags);
    }
  }

  VRTX_TRY(dalloc(&out.nodes, n, stream));
  VRTX_TRY(dalloc(&out.primOrder, n, stream));
  VRTX_TRY(dalloc(&counters, 4, stream));
  VRTX_TRY(dalloc(&tasksA, n, stream));
  VRTX_TRY(dalloc(&tasksB, n, stream));
  {
    // root task: binary root -> BVH8 node 0; counters: [0] nodes, [1] prims,
    // [2] and [3] the task counts of alternate levels
    const uint2 root = make_uint2(n > 1 ? 0u : LEAF_BIT, 0u);
    const uint32_t init[4] = {1u, 0u, 1u, 0u};
    VRTX_TRY(cudaMemcpyAsync(
        tasksA, &root, sizeof(uint2), cudaMemcpyHostToDevice, stream));
    VRTX_TRY(cudaMemcpyAsync(
        counters, init, sizeof(init), cudaMemcpyHostToDevice, stream));
  }
  {
    // levels in batches of 8 between host checks of the task count
    const uint32_t grid = (uint32_t)std::min<size_t>((n + 127) / 128, 2048);
    int level = 0;
    while (true) {
      for (int b = 0; b < 8; b++, level++) {
        uint32_t *in = counters + 2 + (level & 1);
        uint32_t *outCount = counters + 2 + ((level + 1) & 1);
        VRTX_TRY(cudaMemsetAsync(outCount, 0, sizeof(uint32_t), stream));
        CollapseArgs ca;
        ca.left = left;
        ca.right = right;
        ca.internalCount = iCount;
        ca.internalBoxes = iBoxes;
        ca.boxes = d_boxes;
        ca.sortedIdx = valsSorted;
        ca.nodes = out.nodes;
        ca.primOrder = out.primOrder;
        ca.counters = counters;
        ca.tasksIn = tasksA;
        ca.numTasks = in;
        ca.capacity = (uint32_t)n;
        ca.tasksOut = tasksB;
        ca.numTasksOut = outCount;
        ca.maxLeaf = maxLeafPrims;
        ca.dec = sahDec;
        k_collapse<<<grid, 128, 0, stream>>>(ca);
        uint2 *t = tasksA;
        tasksA = tasksB;
        tasksB = t;
      }
      VRTX_TRY(cudaMemcpyAsync(hostCounters,
          counters,
          sizeof(uint32_t) * 4,
          cudaMemcpyDeviceToHost,
          stream));
      VRTX_TRY(cudaStreamSynchronize(stream));
      const uint32_t pending = hostCounters[2 + (level & 1)];
      if (pending == 0)
        break;
      if (level > 512 || pending > n) {
        err = cudaErrorUnknown; // a radix tree over n keys is shallower
        goto fail;
      }
    }
  }
  VRTX_TRY(cudaMemcpyAsync(
      &hostAll, pAll, sizeof(box3), cudaMemcpyDeviceToHost, stream));
  VRTX_TRY(cudaStreamSynchronize(stream));
  out.numNodes = hostCounters[0];
  out.numPrims = hostCounters[1];
  out.bounds = hostAll;

fail:
  cudaFreeAsync(pCent, stream);
  cudaFreeAsync(pAll, stream);
  cudaFreeAsync(keys, stream);
  cudaFreeAsync(keysSorted, stream);
  cudaFreeAsync(vals, stream);
  cudaFreeAsync(valsSorted, stream);
  cudaFreeAsync(tmp, stream);
  cudaFreeAsync(left, stream);
  cudaFreeAsync(right, stream);
  cudaFreeAsync(parI, stream);
  cudaFreeAsync(parL, stream);
  cudaFreeAsync(iBoxes, stream);
  cudaFreeAsync(iCount, stream);
  cudaFreeAsync(flags, stream);
  cudaFreeAsync(sahCost, stream);
  cudaFreeAsync(sahDec, stream);
  cudaFreeAsync(counters, stream);
  cudaFreeAsync(tasksA, stream);
  cudaFreeAsync(tasksB, stream);
  if (err != cudaSuccess) {
    cudaFreeAsync(out.nodes, stream);
    cudaFreeAsync(out.primOrder, stream);
    out = BVH8Build{};
  }
#undef VRTX_TRY
  return err;
}

void freeBVH8(BVH8Build &b, cudaStream_t stream)
{
  if (b.nodes)
    cudaFreeAsync(b.nodes, stream);
  if (b.primOrder)
    cudaFreeAsync(b.primOrder, stream);
  b = BVH8Build{};
}

} // namespace vrtx
