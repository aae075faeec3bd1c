// CPU oracle for the VisRTX hot path -- TEST INFRASTRUCTURE ONLY (see
// oracle.h). Plain C++17, built with -ffp-contract=off so x86 and Arm hosts
// produce the same bits. Each function names the reference code it
// restates (paths within the VisRTX project).
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// small vector math (float; the reference computes in fp32 via glm)
// ---------------------------------------------------------------------------

struct V3
{
  float x, y, z;
};
inline V3 v3(float x, float y, float z)
{
  return V3{x, y, z};
}
inline V3 operator+(V3 a, V3 b)
{
  return {a.x + b.x, a.y + b.y, a.z + b.z};
}
inline V3 operator-(V3 a, V3 b)
{
  return {a.x - b.x, a.y - b.y, a.z - b.z};
}
inline V3 operator-(V3 a)
{
  return {-a.x, -a.y, -a.z};
}
inline V3 operator*(V3 a, float s)
{
  return {a.x * s, a.y * s, a.z * s};
}
inline V3 operator*(float s, V3 a)
{
  return {a.x * s, a.y * s, a.z * s};
}
inline V3 operator*(V3 a, V3 b)
{
  return {a.x * b.x, a.y * b.y, a.z * b.z};
}
inline V3 operator/(V3 a, float s)
{
  return {a.x / s, a.y / s, a.z / s};
}
inline float dot(V3 a, V3 b)
{
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
inline V3 cross(V3 a, V3 b)
{
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 normalize(V3 v)
{
  const float inv = 1.f / std::sqrt(dot(v, v));
  return v * inv;
}
inline float comp(V3 v, int i)
{
  return i == 0 ? v.x : (i == 1 ? v.y : v.z);
}
inline V3 ld3(const float *p, size_t i)
{
  return {p[3 * i], p[3 * i + 1], p[3 * i + 2]};
}
inline float cmax(V3 v)
{
  return std::max(v.x, std::max(v.y, v.z));
}
inline V3 vabs(V3 v)
{
  return {std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)};
}

struct X34
{
  float m[12];
};
inline V3 xPoint(const X34 &t, V3 p)
{
  const float *m = t.m;
  return {m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3],
      m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
      m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]};
}
inline V3 xVec(const X34 &t, V3 p)
{
  const float *m = t.m;
  return {m[0] * p.x + m[1] * p.y + m[2] * p.z,
      m[4] * p.x + m[5] * p.y + m[6] * p.z,
      m[8] * p.x + m[9] * p.y + m[10] * p.z};
}
inline V3 xNormalT(const X34 &w2o, V3 n)
{
  const float *m = w2o.m;
  return {m[0] * n.x + m[4] * n.y + m[8] * n.z,
      m[1] * n.x + m[5] * n.y + m[9] * n.z,
      m[2] * n.x + m[6] * n.y + m[10] * n.z};
}

// Affine inverse in double, rounded to float.
X34 invert(const float *m)
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
  X34 o;
  for (int r = 0; r < 3; r++) {
    for (int cc = 0; cc < 3; cc++)
      o.m[r * 4 + cc] = (float)inv[r][cc];
    o.m[r * 4 + 3] =
        (float)(-(inv[r][0] * t[0] + inv[r][1] * t[1] + inv[r][2] * t[2]));
  }
  return o;
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and the curand-style
// stream the reference draws from (gpu/createScreenSample.h:58,
// cameraCreateRay.h:76, volumeIntegration.h:83,120, gpu_util.h:199).
// ---------------------------------------------------------------------------

const uint32_t PH_M0 = 0xD2511F53u, PH_M1 = 0xCD9E8D57u;
const uint32_t PH_W0 = 0x9E3779B9u, PH_W1 = 0xBB67AE85u;

void philox(const uint32_t in[4], const uint32_t key[2], uint32_t out[4])
{
  uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    if (r > 0) {
      k0 += PH_W0;
      k1 += PH_W1;
    }
    const uint64_t p0 = (uint64_t)PH_M0 * c0;
    const uint64_t p1 = (uint64_t)PH_M1 * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

// Stream state: a 128-bit counter (word 0 least significant), the 64-bit
// seed as key, the current 4-word block and the next word's index in it.
// init(seed, subsequence, offset): the subsequence selects the counter's
// upper 64 bits, the offset skips `offset` words of the stream.
struct Stream
{
  uint32_t ctr[4];
  uint32_t key[2];
  uint32_t blk[4];
  int idx;

  void add(uint64_t n)
  {
    uint64_t lo = (uint64_t)ctr[0] | ((uint64_t)ctr[1] << 32);
    const uint64_t nlo = lo + n;
    const uint64_t carry = nlo < lo ? 1 : 0;
    ctr[0] = (uint32_t)nlo;
    ctr[1] = (uint32_t)(nlo >> 32);
    uint64_t hi = (uint64_t)ctr[2] | ((uint64_t)ctr[3] << 32);
    hi += carry;
    ctr[2] = (uint32_t)hi;
    ctr[3] = (uint32_t)(hi >> 32);
  }
  void addHi(uint64_t n)
  {
    uint64_t hi = (uint64_t)ctr[2] | ((uint64_t)ctr[3] << 32);
    hi += n;
    ctr[2] = (uint32_t)hi;
    ctr[3] = (uint32_t)(hi >> 32);
  }
  void init(uint64_t seed, uint64_t subsequence, uint64_t offset)
  {
    ctr[0] = ctr[1] = ctr[2] = ctr[3] = 0;
    key[0] = (uint32_t)seed;
    key[1] = (uint32_t)(seed >> 32);
    idx = 0;
    addHi(subsequence);
    idx += (int)(offset & 3);
    add(offset >> 2);
    philox(ctr, key, blk);
  }
  uint32_t next()
  {
    const uint32_t r = blk[idx++];
    if (idx == 4) {
      add(1);
      philox(ctr, key, blk);
      idx = 0;
    }
    return r;
  }
  void next4(uint32_t r[4])
  {
    uint32_t cur[4];
    std::memcpy(cur, blk, sizeof(cur));
    add(1);
    philox(ctr, key, blk);
    for (int i = 0; i < 4; i++) {
      const int j = idx + i;
      r[i] = j < 4 ? cur[j] : blk[j - 4];
    }
  }
};

// (x + 1/2) * 2^-32, evaluated as the float expression x * 2^-32 + 2^-33
inline float u01(uint32_t x)
{
  const float inv = 2.3283064365386963e-10f;
  return (float)x * inv + inv * 0.5f;
}

inline float uniform(Stream &s)
{
  return u01(s.next());
}
inline void uniform4(Stream &s, float r[4])
{
  uint32_t v[4];
  s.next4(v);
  for (int i = 0; i < 4; i++)
    r[i] = u01(v[i]);
}

// ---------------------------------------------------------------------------
// texture filtering (parity mode): the texture unit's linear filter on a
// clamped, normalised-coordinate float texture, as the reference samples
// its field (sampleSpatialField.h:66-71) and TF (volumeIntegration.h:53).
//
// The rule was recovered from GPU-captured sweeps (axis ramps of sizes
// 2..512 on each axis, one-hot 2x2x2 corners, random volumes, a 256-entry
// float4 table) and reproduces every captured value bit for bit:
//  1. the normalised coordinate is truncated to 21 fractional bits;
//  2. x = u * n - 0.5 exactly, clamped to [0, n - 1]; i = floor(x); the
//     fraction is rounded half up to an 8-bit weight w (0..256 / 256);
//  3. 3D: the eight corner weights are integers summing to 256, split in
//     the order z, x, y: the z1 slice gets wz, the z0 slice 256 - wz; in a
//     slice of budget B the x1 column gets round-half-up(wx * B / 256); in
//     a column of budget C the y1 corner gets wy * C / 256 rounded half
//     down in the x0 column and half up in the x1 column;
//  4. the value is the exact sum of weight * texel / 256, rounded to float
//     with ties away from zero.
// mode 0 instead gives the textbook form (FP32 lerps with weights rounded
// to 8 bits), kept to measure how far that form is from the texture unit.
// ---------------------------------------------------------------------------

// Exact sum of doubles as a nonoverlapping expansion (Shewchuk, "Adaptive
// precision floating-point arithmetic", 1997: Two-Sum and grow-expansion
// with zero elimination), rounded once to float, ties away from zero.
struct ExactSum
{
  double c[24];
  int n = 0;
  void add(double b)
  {
    double q = b;
    int m = 0;
    for (int i = 0; i < n; i++) {
      const double s = q + c[i];
      const double bv = s - q;
      const double e = (q - (s - bv)) + (c[i] - bv);
      if (e != 0.0)
        c[m++] = e;
      q = s;
    }
    if (q != 0.0)
      c[m++] = q;
    n = m;
  }
  float toFloatTiesAway() const
  {
    double h = 0.0;
    for (int i = 0; i < n; i++)
      h += c[i];
    // sign of the exact residual (sum - h): the top component of the
    // expansion of sum - h
    ExactSum r = *this;
    r.add(-h);
    const int rs = r.n ? (r.c[r.n - 1] > 0.0 ? 1 : -1) : 0;
    const float f = (float)h;
    if ((double)f == h)
      return f;
    const float a = (double)f < h ? f : std::nextafter(f, -INFINITY);
    const float b = std::nextafter(a, INFINITY);
    const double mid = 0.5 * ((double)a + (double)b);
    if (h < mid)
      return a;
    if (h > mid)
      return b;
    if (rs > 0)
      return b;
    if (rs < 0)
      return a;
    return std::fabs(a) > std::fabs(b) ? a : b;
  }
};

// one axis: texel pair and the 8-bit weight of the upper texel
inline void hwAxis(float coord, int n, int &i0, int &i1, int &w)
{
  double u = std::isfinite(coord) ? std::floor((double)coord * 2097152.0) / 2097152.0 : 0.0;
  double x = u * (double)n - 0.5;
  x = std::min(std::max(x, 0.0), (double)(n - 1));
  const double fl = std::floor(x);
  int i = (int)fl;
  w = (int)std::floor((x - fl) * 256.0 + 0.5);
  if (w >= 256) {
    w = 0;
    i++;
  }
  i0 = i;
  i1 = std::min(i + 1, n - 1);
}

inline float quantW(float a, int round = 1)
{
  return round ? std::nearbyint(a * 256.f) * (1.f / 256.f)
               : std::floor(a * 256.f) * (1.f / 256.f);
}

inline void axisTap(float coord, int n, int &i0, int &i1, float &w)
{
  const float x = coord * (float)n - 0.5f;
  const float fl = std::floor(x);
  w = quantW(x - fl);
  const int i = (int)fl;
  i0 = std::min(std::max(i, 0), n - 1);
  i1 = std::min(std::max(i + 1, 0), n - 1);
}

float tex3dLinear(const float *v, const int d[3], float cx, float cy, float cz, int mode)
{
  auto at = [&](int x, int y, int z) {
    return v[((size_t)z * d[1] + y) * d[0] + x];
  };
  if (mode == 0) {
    int x0, x1, y0, y1, z0, z1;
    float a, b, c;
    axisTap(cx, d[0], x0, x1, a);
    axisTap(cy, d[1], y0, y1, b);
    axisTap(cz, d[2], z0, z1, c);
    const float c00 = (1.f - a) * at(x0, y0, z0) + a * at(x1, y0, z0);
    const float c10 = (1.f - a) * at(x0, y1, z0) + a * at(x1, y1, z0);
    const float c01 = (1.f - a) * at(x0, y0, z1) + a * at(x1, y0, z1);
    const float c11 = (1.f - a) * at(x0, y1, z1) + a * at(x1, y1, z1);
    const float c0 = (1.f - b) * c00 + b * c10;
    const float c1 = (1.f - b) * c01 + b * c11;
    return (1.f - c) * c0 + c * c1;
  }
  int xi[2], yi[2], zi[2], wx, wy, wz;
  hwAxis(cx, d[0], xi[0], xi[1], wx);
  hwAxis(cy, d[1], yi[0], yi[1], wy);
  hwAxis(cz, d[2], zi[0], zi[1], wz);
  ExactSum sum;
  for (int z = 0; z < 2; z++) {
    const int B = z ? wz : 256 - wz;
    const int x1 = (wx * B + 128) >> 8;
    for (int x = 0; x < 2; x++) {
      const int C = x ? x1 : B - x1;
      const int y1 = (wy * C + (x ? 128 : 127)) >> 8;
      const int wcorner[2] = {C - y1, y1};
      for (int y = 0; y < 2; y++)
        if (wcorner[y])
          sum.add((double)wcorner[y] * (1.0 / 256.0) * (double)at(xi[x], yi[y], zi[z]));
    }
  }
  return sum.toFloatTiesAway();
}

// nearest filtering: the coordinate truncated to 21 fractional bits, then
// floor(u * n) clamped (as the texture unit; see texSample)
float tex3dPoint(const float *v, const int d[3], float cx, float cy, float cz)
{
  auto idx = [](float c, int n) {
    const double u = std::isfinite(c) ? std::floor((double)c * 2097152.0) / 2097152.0 : 0.0;
    const double x = std::min(std::max(std::floor(u * n), 0.0), (double)(n - 1));
    return (int)x;
  };
  return v[((size_t)idx(cz, d[2]) * d[1] + idx(cy, d[1])) * d[0] + idx(cx, d[0])];
}

// exact (FP64) trilinear at the same texel convention
double tex3dExact(const float *v, const int d[3], double cx, double cy, double cz)
{
  int i0[3], i1[3];
  double w[3];
  const double c[3] = {cx, cy, cz};
  for (int k = 0; k < 3; k++) {
    const double x = c[k] * d[k] - 0.5;
    const double fl = std::floor(x);
    w[k] = x - fl;
    i0[k] = std::min(std::max((int)fl, 0), d[k] - 1);
    i1[k] = std::min(std::max((int)fl + 1, 0), d[k] - 1);
  }
  double s = 0.0;
  for (int q = 0; q < 8; q++) {
    const int ix = (q & 1) ? i1[0] : i0[0], iy = (q & 2) ? i1[1] : i0[1],
              iz = (q & 4) ? i1[2] : i0[2];
    const double ww = ((q & 1) ? w[0] : 1 - w[0]) * ((q & 2) ? w[1] : 1 - w[1])
        * ((q & 4) ? w[2] : 1 - w[2]);
    s += ww * v[((size_t)iz * d[1] + iy) * d[0] + ix];
  }
  return s;
}

void tex1dLinear(const float *t, int n, int comps, float coord, int mode, float *out)
{
  if (mode == 0) {
    int i0, i1;
    float a;
    axisTap(coord, n, i0, i1, a);
    for (int c = 0; c < comps; c++)
      out[c] = (1.f - a) * t[i0 * comps + c] + a * t[i1 * comps + c];
    return;
  }
  int i0, i1, w;
  hwAxis(coord, n, i0, i1, w);
  for (int c = 0; c < comps; c++) {
    ExactSum sum;
    sum.add((double)(256 - w) * (1.0 / 256.0) * (double)t[i0 * comps + c]);
    sum.add((double)w * (1.0 / 256.0) * (double)t[i1 * comps + c]);
    out[c] = sum.toFloatTiesAway();
  }
}

void tex1dExact(const float *t, int n, double coord, double *out)
{
  const double x = coord * n - 0.5;
  const double fl = std::floor(x);
  const double a = x - fl;
  const int i0 = std::min(std::max((int)fl, 0), n - 1);
  const int i1 = std::min(std::max((int)fl + 1, 0), n - 1);
  for (int c = 0; c < 4; c++)
    out[c] = (1 - a) * t[i0 * 4 + c] + a * t[i1 * 4 + c];
}

// ---------------------------------------------------------------------------
// oracle BVH: binned SAH binary tree per instance, object space
// ---------------------------------------------------------------------------

struct Box
{
  V3 lo{FLT_MAX, FLT_MAX, FLT_MAX}, hi{-FLT_MAX, -FLT_MAX, -FLT_MAX};
  void ext(V3 p)
  {
    lo = {std::min(lo.x, p.x), std::min(lo.y, p.y), std::min(lo.z, p.z)};
    hi = {std::max(hi.x, p.x), std::max(hi.y, p.y), std::max(hi.z, p.z)};
  }
  void ext(const Box &b)
  {
    ext(b.lo);
    ext(b.hi);
  }
  float area() const
  {
    const V3 d = hi - lo;
    if (d.x < 0)
      return 0.f;
    return 2.f * (d.x * d.y + d.y * d.z + d.z * d.x);
  }
};

struct Prim
{
  int surface; // index into scene surfaces
  uint32_t prim;
};

struct BNode
{
  Box box;
  int left; // internal: child index; leaf: first prim
  int count; // 0 = internal
};

struct InstBVH
{
  std::vector<BNode> nodes;
  std::vector<Prim> prims;
};

// HDRI::finalize / generateCDFTables (scene/light/HDRI.cu:98-170,218-319):
// luminance weighted by the row's sin(theta), row sums, marginal and
// conditional inclusive scans (in order), normalised by their last entries,
// pdf weight total / (2 pi^2 W H), and the rotation rows (right, forward, up)
struct HdriPre
{
  std::vector<float> marginal, conditional;
  float pdfWeight = 0.f;
  float rot[9];
};

struct SceneCtx
{
  const OrcScene *sc;
  std::vector<HdriPre> hdri; // per light (filled for hdri lights)
  int hdriIndex = -1; // the first hdri light
  std::vector<InstBVH> unique; // one per distinct surface range
  std::vector<const InstBVH *> bvh; // per instance
  std::vector<X34> w2o, o2w;
  std::vector<Box> worldBox;
  bool allOpaque = true;
};

// Quad.cpp:115-141: quad (x, y, z, w) becomes triangles (x, y, w) and
// (z, w, y); without an index quad q uses vertices 4q .. 4q + 3
void quadTri(const OrcSurface &s, uint32_t k, uint32_t &i0, uint32_t &i1, uint32_t &i2)
{
  const uint32_t q = k / 2;
  uint32_t x, y, z, w;
  if (s.indices) {
    x = s.indices[4 * q];
    y = s.indices[4 * q + 1];
    z = s.indices[4 * q + 2];
    w = s.indices[4 * q + 3];
  } else {
    x = 4 * q;
    y = x + 1;
    z = x + 2;
    w = x + 3;
  }
  if (k % 2 == 0) {
    i0 = x;
    i1 = y;
    i2 = w;
  } else {
    i0 = z;
    i1 = w;
    i2 = y;
  }
}

void triVerts(const OrcSurface &s, uint32_t p, V3 &a, V3 &b, V3 &c)
{
  uint32_t i0, i1, i2;
  if (s.type == 2) {
    quadTri(s, p, i0, i1, i2);
  } else if (s.indices) {
    i0 = s.indices[3 * p];
    i1 = s.indices[3 * p + 1];
    i2 = s.indices[3 * p + 2];
  } else {
    i0 = 3 * p;
    i1 = i0 + 1;
    i2 = i0 + 2;
  }
  a = ld3(s.vertices, i0);
  b = ld3(s.vertices, i1);
  c = ld3(s.vertices, i2);
}

void sphereOf(const OrcSurface &s, uint32_t p, V3 &c, float &r)
{
  const uint32_t i = s.indices ? s.indices[p] : p;
  c = ld3(s.vertices, i);
  r = s.radii ? s.radii[i] : s.radius;
}

// The segment of a cylinder (3), cone (4) or curve (5) primitive
// (Intersectors_ptx.cu:100-246, populateHit.h:292-303, Curve.cpp:88-113)
void segmentOf(const OrcSurface &s, uint32_t p, V3 &p0, float &r0, V3 &p1, float &r1)
{
  uint32_t i0, i1;
  if (s.type == 5) {
    i0 = s.indices ? s.indices[p] : p;
    i1 = i0 + 1;
  } else {
    i0 = s.indices ? s.indices[2 * p] : 2 * p;
    i1 = s.indices ? s.indices[2 * p + 1] : 2 * p + 1;
  }
  p0 = ld3(s.vertices, i0);
  p1 = ld3(s.vertices, i1);
  if (s.type == 3) {
    r0 = r1 = std::fabs(s.radii ? s.radii[p] : s.radius);
  } else if (s.type == 4) {
    r0 = s.radii[i0];
    r1 = s.radii[i1];
  } else {
    r0 = s.radii ? s.radii[i0] : s.radius;
    r1 = s.radii ? s.radii[i1] : s.radius;
  }
}

Box primBox(const OrcScene *sc, const Prim &pr)
{
  const OrcSurface &s = sc->surfaces[pr.surface];
  Box b;
  if (s.type >= 3) {
    V3 p0, p1;
    float r0, r1;
    segmentOf(s, pr.prim, p0, r0, p1, r1);
    if (s.type == 5) {
      b.ext(p0 - v3(r0, r0, r0));
      b.ext(p0 + v3(r0, r0, r0));
      b.ext(p1 - v3(r1, r1, r1));
      b.ext(p1 + v3(r1, r1, r1));
    } else {
      const float m = std::max(r0, r1);
      b.ext(p0 - v3(m, m, m));
      b.ext(p0 + v3(m, m, m));
      b.ext(p1 - v3(m, m, m));
      b.ext(p1 + v3(m, m, m));
    }
    return b;
  }
  if (s.type == 0 || s.type == 2) {
    V3 a, bb, c;
    triVerts(s, pr.prim, a, bb, c);
    b.ext(a);
    b.ext(bb);
    b.ext(c);
  } else {
    V3 c;
    float r;
    sphereOf(s, pr.prim, c, r);
    b.ext(c - v3(r, r, r));
    b.ext(c + v3(r, r, r));
  }
  return b;
}

void buildBVH(const OrcScene *sc, InstBVH &b)
{
  const int n = (int)b.prims.size();
  if (n == 0)
    return;
  std::vector<Box> boxes(n);
  std::vector<V3> cent(n);
  for (int i = 0; i < n; i++) {
    boxes[i] = primBox(sc, b.prims[i]);
    cent[i] = (boxes[i].lo + boxes[i].hi) * 0.5f;
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; i++)
    idx[i] = i;
  struct Task
  {
    int node, begin, end;
  };
  b.nodes.reserve(2 * n);
  b.nodes.push_back(BNode{});
  std::vector<Task> st{{0, 0, n}};
  const int NB = 16;
  while (!st.empty()) {
    Task t = st.back();
    st.pop_back();
    Box bb, cb;
    for (int i = t.begin; i < t.end; i++) {
      bb.ext(boxes[idx[i]]);
      cb.ext(cent[idx[i]]);
    }
    BNode &nd = b.nodes[t.node];
    nd.box = bb;
    const int cnt = t.end - t.begin;
    if (cnt <= 4) {
      nd.left = t.begin;
      nd.count = cnt;
      continue;
    }
    int bestAxis = -1, bestBin = -1;
    float bestCost = FLT_MAX;
    for (int ax = 0; ax < 3; ax++) {
      const float lo = comp(cb.lo, ax), hi = comp(cb.hi, ax);
      if (!(hi > lo))
        continue;
      Box bins[NB];
      int counts[NB] = {0};
      const float sc2 = NB / (hi - lo);
      for (int i = t.begin; i < t.end; i++) {
        int k = (int)((comp(cent[idx[i]], ax) - lo) * sc2);
        k = std::min(std::max(k, 0), NB - 1);
        bins[k].ext(boxes[idx[i]]);
        counts[k]++;
      }
      float la[NB], ra[NB];
      int lc[NB], rc[NB];
      Box acc;
      int c = 0;
      for (int k = 0; k < NB; k++) {
        acc.ext(bins[k]);
        c += counts[k];
        la[k] = acc.area();
        lc[k] = c;
      }
      acc = Box();
      c = 0;
      for (int k = NB - 1; k >= 0; k--) {
        acc.ext(bins[k]);
        c += counts[k];
        ra[k] = acc.area();
        rc[k] = c;
      }
      for (int k = 0; k < NB - 1; k++) {
        if (lc[k] == 0 || rc[k + 1] == 0)
          continue;
        const float cost = la[k] * lc[k] + ra[k + 1] * rc[k + 1];
        if (cost < bestCost) {
          bestCost = cost;
          bestAxis = ax;
          bestBin = k;
        }
      }
    }
    int mid;
    if (bestAxis < 0) {
      mid = (t.begin + t.end) / 2;
    } else {
      const float lo = comp(cb.lo, bestAxis), hi = comp(cb.hi, bestAxis);
      const float sc2 = NB / (hi - lo);
      auto it = std::partition(idx.begin() + t.begin, idx.begin() + t.end, [&](int i) {
        int k = (int)((comp(cent[i], bestAxis) - lo) * sc2);
        k = std::min(std::max(k, 0), NB - 1);
        return k <= bestBin;
      });
      mid = (int)(it - idx.begin());
      if (mid == t.begin || mid == t.end)
        mid = (t.begin + t.end) / 2;
    }
    const int l = (int)b.nodes.size();
    b.nodes.push_back(BNode{});
    b.nodes.push_back(BNode{});
    b.nodes[t.node].left = l;
    b.nodes[t.node].count = 0;
    st.push_back({l + 1, mid, t.end});
    st.push_back({l, t.begin, mid});
  }
  std::vector<Prim> sorted(n);
  for (int i = 0; i < n; i++)
    sorted[i] = b.prims[idx[i]];
  b.prims.swap(sorted);
}

// ---------------------------------------------------------------------------
// ray/primitive tests
// ---------------------------------------------------------------------------

struct RayPre
{
  V3 o, d, inv;
  int kx, ky, kz;
  float Sx, Sy, Sz;
};

RayPre prep(V3 o, V3 d)
{
  RayPre r;
  r.o = o;
  r.d = d;
  r.inv = v3(1.f / d.x, 1.f / d.y, 1.f / d.z);
  const float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
  int kz = 0;
  if (ay > ax)
    kz = 1;
  if (az > std::max(ax, ay))
    kz = 2;
  int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
  if (comp(d, kz) < 0.f)
    std::swap(kx, ky);
  r.kx = kx;
  r.ky = ky;
  r.kz = kz;
  r.Sx = comp(d, kx) / comp(d, kz);
  r.Sy = comp(d, ky) / comp(d, kz);
  r.Sz = 1.f / comp(d, kz);
  return r;
}

// Watertight ray/triangle intersection (Woop, Benthin, Wald, JCGT 2013),
// standing in for OptiX's built-in triangle test. u, v are the weights of
// v1 and v2 (OptiX barycentrics, populateHit.h:144-148); front face when the
// vertices wind counter-clockwise seen from the ray origin.
bool hitTriangle(const RayPre &r, V3 a, V3 b, V3 c, float tmin, float tmax,
    float &t, float &u, float &v, bool &front)
{
  const V3 A = a - r.o, B = b - r.o, C = c - r.o;
  const float Ax = comp(A, r.kx) - r.Sx * comp(A, r.kz);
  const float Ay = comp(A, r.ky) - r.Sy * comp(A, r.kz);
  const float Bx = comp(B, r.kx) - r.Sx * comp(B, r.kz);
  const float By = comp(B, r.ky) - r.Sy * comp(B, r.kz);
  const float Cx = comp(C, r.kx) - r.Sx * comp(C, r.kz);
  const float Cy = comp(C, r.ky) - r.Sy * comp(C, r.kz);
  float U = Cx * By - Cy * Bx;
  float V = Ax * Cy - Ay * Cx;
  float W = Bx * Ay - By * Ax;
  if (U == 0.f || V == 0.f || W == 0.f) {
    U = (float)((double)Cx * By - (double)Cy * Bx);
    V = (float)((double)Ax * Cy - (double)Ay * Cx);
    W = (float)((double)Bx * Ay - (double)By * Ax);
  }
  if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f))
    return false;
  const float det = U + V + W;
  if (det == 0.f)
    return false;
  const float T = U * (r.Sz * comp(A, r.kz)) + V * (r.Sz * comp(B, r.kz))
      + W * (r.Sz * comp(C, r.kz));
  const float rcp = 1.f / det;
  const float tt = T * rcp;
  if (!(tt >= tmin && tt < tmax))
    return false;
  t = tt;
  u = V * rcp;
  v = W * rcp;
  front = dot(r.d, cross(b - a, c - a)) < 0.f;
  return true;
}

// intersectSphere (scene/Intersectors_ptx.cu:74-99): object space, non-unit
// direction, near root only; OptiX drops t outside the ray interval.
bool hitSphere(const RayPre &r, V3 center, float radius, float tmin, float tmax, float &t)
{
  const V3 d = r.d;
  const float rd2 = 1.f / dot(d, d);
  const V3 CO = center - r.o;
  const float projCO = dot(CO, d) * rd2;
  const V3 perp = CO - projCO * d;
  const float l2 = dot(perp, perp);
  const float r2 = radius * radius;
  if (l2 > r2)
    return false;
  const float td = std::sqrt((r2 - l2) * rd2);
  const float tt = projCO - td;
  if (!(tt >= tmin && tt < tmax))
    return false;
  t = tt;
  return true;
}

// intersectCylinder (scene/Intersectors_ptx.cu:100-175): reports side
// entry, side exit (between the end planes), then the nearer cap disk
template <typename F>
void cylinderReports(const RayPre &r, V3 p0, V3 p1, float radius, bool caps, F &&report)
{
  const V3 ro = r.o, rd = r.d;
  const V3 sv = p1 - p0;
  const V3 sxd = cross(sv, rd);
  const float a = dot(sxd, sxd);
  if (a == 0.f)
    return;
  const V3 f = p0 - ro;
  const V3 sxf = cross(sv, f);
  const float ra = 1.f / a;
  const float ts = dot(sxd, sxf) * ra;
  const V3 fp = f - ts * rd;
  const float s2 = dot(sv, sv);
  const V3 perp = cross(sv, fp);
  const float c = (radius * radius) * s2 - dot(perp, perp);
  if (c < 0.f)
    return;
  const float td = std::sqrt(c * ra);
  const float tin = ts - td, tout = ts + td;
  const float sf = dot(sv, f), sd = dot(sv, rd);
  const float u_in = (tin * sd - sf) * (1.f / s2);
  const V3 N_in = -td * rd - fp - u_in * sv;
  const float u_out = (tout * sd - sf) * (1.f / s2);
  const V3 N_out = td * rd - fp - u_out * sv;
  if (sd != 0.f) {
    const float rsd = 1.f / sd;
    const float tA = sf * rsd;
    const float tB = tA + s2 * rsd;
    const float capIn = std::min(tA, tB), capOut = std::max(tA, tB);
    if (tin > capIn && tin < capOut)
      report(tin, N_in, u_in);
    if (tout > capIn && tout < capOut)
      report(tout, N_out, u_out);
  } else if (sf <= 0.f && sf >= -s2) {
    report(tin, N_in, u_in);
    report(tout, N_out, u_out);
  }
  if (caps) {
    const float ca = s2 - sd * sd;
    const float cb = s2 * dot(-f, rd) + (sf * sd);
    const float cc = s2 * dot(-f, -f) - (sf * sf) - (radius * radius * s2);
    float h = cb * cb - ca * cc;
    if (h < 0.f)
      return;
    h = std::sqrt(h);
    const float y = ((-cb - h) / ca) * sd - sf;
    const float d = ((y < 0.f ? 0.f : s2) + sf) / sd;
    if (std::fabs(cb + ca * d) < h) {
      const float sg = y > 0.f ? 1.f : (y < 0.f ? -1.f : 0.f);
      report(d, sv * sg / s2, y < 0.f ? 0.f : 1.f);
    }
  }
}

// intersectCone (scene/Intersectors_ptx.cu:177-246)
template <typename F>
void coneReports(const RayPre &r, V3 p0, float ra, V3 p1, float rb, F &&report)
{
  const V3 ro = r.o, rd = r.d;
  const V3 ba = p1 - p0, oa = ro - p0, ob = ro - p1;
  const float m0 = dot(ba, ba), m1 = dot(oa, ba), m2 = dot(ob, ba), m3 = dot(rd, ba);
  if (m1 < 0.f) {
    const V3 q = oa * m3 - rd * m1;
    if (dot(q, q) < (ra * ra * m3 * m3))
      report(-m1 / m3, -ba * (1.f / std::sqrt(m0)), 0.f);
  } else if (m2 > 0.f) {
    const V3 q = ob * m3 - rd * m2;
    if (dot(q, q) < (rb * rb * m3 * m3))
      report(-m2 / m3, ba * (1.f / std::sqrt(m0)), 1.f);
  }
  const float m4 = dot(rd, oa), m5 = dot(oa, oa);
  const float rr = ra - rb;
  const float hy = m0 + rr * rr;
  const float k2 = m0 * m0 - m3 * m3 * hy;
  const float k1 = m0 * m0 * m4 - m1 * m3 * hy + m0 * ra * (rr * m3 * 1.0f);
  const float k0 = m0 * m0 * m5 - m1 * m1 * hy + m0 * ra * (rr * m1 * 2.0f - m0 * ra);
  const float h = k1 * k1 - k2 * k0;
  if (h < 0.f)
    return;
  const float t = (-k1 - std::sqrt(h)) / k2;
  const float y = m1 + t * m3;
  if (y > 0.f && y < m0)
    report(t, normalize(m0 * (m0 * (oa + t * rd) + rr * ba * ra) - ba * hy * y), y / m0);
}

// Round linear curve segment: the libvrtx definition (OptiX's own test is
// closed) -- the union of the two end balls and their tangent cone, entered
// at the smallest entry root of its convex parts; a ray starting inside
// reports nothing. Same arithmetic as the GPU test.
template <typename F>
void curveReports(const RayPre &r, V3 pa, float ra, V3 pb, float rb, float tmin, F &&report)
{
  const V3 d = r.d;
  const float dd = dot(d, d);
  const float shift = dot(pa - r.o, d) / dd;
  const V3 o = r.o + d * shift;
  const V3 ba = pb - pa;
  const float L2 = dot(ba, ba);
  const V3 oa = o - pa, ob = o - pb;
  float best = 3.0e38f, bestU = 0.f;
  {
    const V3 oa0 = r.o - pa, ob0 = r.o - pb;
    if (dot(oa0, oa0) < ra * ra || dot(ob0, ob0) < rb * rb)
      return;
    const float Lq = std::sqrt(L2);
    if (L2 > 0.f) {
      const float sn = (ra - rb) / Lq;
      const float c2 = 1.f - sn * sn;
      const V3 w0 = ba / Lq;
      const float z = dot(oa0, w0);
      const V3 q = oa0 - w0 * z;
      const float A = ra - sn * z;
      if (c2 > 0.f && z >= ra * sn && z <= Lq + rb * sn && A >= 0.f && c2 * dot(q, q) < A * A)
        return;
    }
  }
  // end balls, each from the ray point closest to its own centre
  auto ball = [&](V3 c, float rad, float u) {
    const float sc = dot(c - r.o, d) / dd;
    const V3 oc = (r.o + d * sc) - c;
    const float bq = dot(oc, d), cq = dot(oc, oc) - rad * rad;
    const float disc = bq * bq - dd * cq;
    if (disc < 0.f)
      return;
    const float t = sc + (-bq - std::sqrt(disc)) / dd;
    if (t < best && t >= tmin) {
      best = t;
      bestU = u;
    }
  };
  ball(pa, ra, 0.f);
  ball(pb, rb, 1.f);
  const float L = std::sqrt(L2);
  const float sinp = (ra - rb) / L;
  const float cos2 = 1.f - sinp * sinp;
  if (L2 > 0.f && cos2 > 0.f) {
    const V3 w = ba / L;
    const float z0 = dot(oa, w), dz = dot(d, w);
    const V3 q0 = oa - z0 * w, dq = d - dz * w;
    const float zA = ra * sinp, zB = L + rb * sinp;
    const float A0 = ra - sinp * z0, A1 = -sinp * dz;
    const float qq = dot(q0, q0);
    const float a = cos2 * dot(dq, dq) - A1 * A1;
    const float b = cos2 * dot(q0, dq) - A0 * A1;
    const float c = cos2 * qq - A0 * A0;
    const float disc = b * b - a * c;
    if (a != 0.f && disc >= 0.f) {
      const float sq = std::sqrt(disc);
      const float t0 = (-b - sq) / a, t1 = (-b + sq) / a;
      for (int k = 0; k < 2; k++) {
        const float t = k == 0 ? std::min(t0, t1) : std::max(t0, t1);
        const float z = z0 + t * dz;
        const float tg = shift + t;
        if (a * t + b < 0.f && z >= zA && z <= zB && A0 + A1 * t >= 0.f && tg < best
            && tg >= tmin) {
          best = tg;
          bestU = (z - zA) / (zB - zA);
        }
      }
    }
  }
  if (best < 3.0e38f)
    report(best, v3(0, 0, 0), bestU);
}

template <typename F>
void segmentReports(const RayPre &r, const OrcSurface &s, uint32_t prim, float tmin, F &&report)
{
  V3 p0, p1;
  float r0, r1;
  segmentOf(s, prim, p0, r0, p1, r1);
  if (s.type == 3)
    cylinderReports(r, p0, p1, r0, s.caps != 0, report);
  else if (s.type == 4)
    coneReports(r, p0, r0, p1, r1, report);
  else
    curveReports(r, p0, r0, p1, r1, tmin, report);
}

bool hitBox(const Box &b, const RayPre &r, float tmin, float tmax)
{
  float t0 = tmin, t1 = tmax;
  for (int a = 0; a < 3; a++) {
    const float inv = comp(r.inv, a), o = comp(r.o, a);
    float tn = (comp(b.lo, a) - o) * inv, tf = (comp(b.hi, a) - o) * inv;
    if (tn > tf)
      std::swap(tn, tf);
    if (!(tn <= tf))
      continue; // NaN from 0 * inf on a degenerate axis: keep
    t0 = std::max(t0, tn);
    t1 = std::min(t1, tf * 1.0000004f);
  }
  return t0 <= t1;
}

struct HitRec
{
  float t, u, v;
  int inst;
  int surface;
  uint32_t prim;
  bool front;
  V3 n; // cylinder / cone: the reported object-space normal
};

float surfOpacity(const OrcSurface &s)
{
  if (s.alphaMode == 0)
    return 1.f;
  if (s.alphaMode == 1)
    return s.opacity;
  return s.opacity < s.cutoff ? 0.f : 1.f;
}

// MODE 0 closest hit (cull per flags); MODE 1 any-hit opacity accumulation
// (DirectLight_ptx.cu:233-256, AmbientOcclusion_ptx.cu:53-69).
template <int MODE>
bool trace(const SceneCtx &S, V3 org, V3 dir, float tmin, float tmax, bool cullRay,
    bool geomCull, HitRec &hit, float &opacity)
{
  bool found = false;
  opacity = 0.f;
  const RayPre wr = prep(org, dir);
  for (int ii = 0; ii < S.sc->numInstances; ii++) {
    if (!hitBox(S.worldBox[ii], wr, tmin, tmax))
      continue;
    const InstBVH &B = *S.bvh[ii];
    if (B.nodes.empty())
      continue;
    const RayPre r = prep(xPoint(S.w2o[ii], org), xVec(S.w2o[ii], dir));
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
      const BNode &n = B.nodes[stack[--sp]];
      if (!hitBox(n.box, r, tmin, tmax))
        continue;
      if (n.count == 0) {
        stack[sp++] = n.left + 1;
        stack[sp++] = n.left;
        continue;
      }
      for (int k = 0; k < n.count; k++) {
        const Prim &p = B.prims[n.left + k];
        const OrcSurface &s = S.sc->surfaces[p.surface];
        float t, u = 0.f, v = 0.f;
        bool front = false, ok;
        if (s.type >= 3) {
          // every report inside [tmin, tmax) is an intersection
          bool done = false;
          segmentReports(r, s, p.prim, tmin, [&](float tt, V3 nn, float uu) {
            if (done || !(tt >= tmin && tt <= tmax))
              return;
            if (tt == tmax) {
              // exact ties within one instance go to the lower (surface,
              // primitive), as the GPU traversal decides them
              if (MODE != 0 || !found || hit.inst != ii)
                return;
              // (the GPU keeps one structure per primitive class)
              const OrcSurface &hs = S.sc->surfaces[hit.surface];
              if (hs.type != s.type)
                return;
              if (!(p.surface < hit.surface || (p.surface == hit.surface && p.prim < hit.prim)))
                return;
            }
            if (MODE == 0) {
              tmax = tt;
              hit = HitRec{tt, uu, 0.f, ii, p.surface, p.prim, true, nn};
              found = true;
            } else {
              opacity += surfOpacity(s) * (1.f - opacity);
              if (opacity >= 0.99f)
                done = true;
            }
          });
          if (MODE == 1 && done)
            return true;
          continue;
        }
        if (s.type == 0 || s.type == 2) {
          V3 a, b, c;
          triVerts(s, p.prim, a, b, c);
          ok = hitTriangle(r, a, b, c, tmin, tmax, t, u, v, front);
          if (ok && MODE == 0 && !front && (cullRay || (geomCull && s.cullBackfaces)))
            ok = false;
        } else {
          V3 c;
          float rad;
          sphereOf(s, p.prim, c, rad);
          ok = hitSphere(r, c, rad, tmin, tmax, t);
        }
        if (!ok)
          continue;
        if (MODE == 0) {
          tmax = t;
          hit = HitRec{t, u, v, ii, p.surface, p.prim, front, v3(0, 0, 0)};
          found = true;
        } else {
          opacity += surfOpacity(s) * (1.f - opacity);
          if (opacity >= 0.99f)
            return true;
        }
      }
    }
  }
  return found;
}

// ---------------------------------------------------------------------------
// integrators
// ---------------------------------------------------------------------------

struct Ray
{
  V3 org, dir;
  float tmin, tmax;
};

struct CamPre
{
  int type;
  float region[4];
  V3 pos, dir, d00, du, dv, p00, pdu, pdv;
  float aperture, aspect;
};

// Camera::readBaseParameters + Perspective/Orthographic::commitParameters
// (camera/Camera.cpp:68-76, Perspective.cpp:40-72, Orthographic.cpp:38-52)
CamPre camSetup(const OrcCamera &c)
{
  CamPre p{};
  p.type = c.type;
  for (int i = 0; i < 4; i++)
    p.region[i] = c.imageRegion[i];
  p.pos = ld3(c.position, 0);
  p.dir = normalize(ld3(c.direction, 0));
  const V3 up = normalize(ld3(c.up, 0));
  if (c.type == 1) {
    const float sx = c.height * c.aspect, sy = c.height;
    p.pdu = normalize(cross(p.dir, up)) * sx;
    p.pdv = normalize(cross(p.pdu, p.dir)) * sy;
    p.p00 = p.pos - 0.5f * p.pdu - 0.5f * p.pdv;
  } else {
    const float ipy = 2.f * std::tan(0.5f * c.fovy);
    const float ipx = ipy * c.aspect;
    V3 du = normalize(cross(p.dir, up)) * ipx;
    V3 dv = normalize(cross(du, p.dir)) * ipy;
    V3 d00 = p.dir - .5f * du - .5f * dv;
    const float ap = c.apertureRadius / (ipx * c.focusDistance);
    if (ap > 0.f) {
      du = du * c.focusDistance;
      dv = dv * c.focusDistance;
      d00 = d00 * c.focusDistance;
    }
    p.du = du;
    p.dv = dv;
    p.d00 = d00;
    p.aperture = ap;
    p.aspect = c.aspect;
  }
  return p;
}

inline float mixf(float a, float b, float t)
{
  return a * (1.f - t) + b * t;
}

// makePrimaryRay + cameraCreateRay (gpu/cameraCreateRay.h:38-81)
// uniformSampleDisk (gpu/gpu_math.h:292-297): the thin-lens aperture sample
void uniformSampleDisk(float radius, float s0, float s1, float &x, float &y)
{
  const float r = std::sqrt(s0) * radius;
  const float phi = 2.f * (float)M_PI * s1;
  x = r * std::cos(phi);
  y = r * std::sin(phi);
}

// uniformSampleCone (gpu/gpu_math.h:299-312): the physically based
// material's next-ray sample (2 * M_PI * s0 is a double product there, as
// here)
V3 uniformSampleCone(float cosThetaMax, float s0, float s1, float s2)
{
  const float phi = (float)(2.0 * M_PI * (double)s0);
  const float cosTheta = (1.f - s1) + s1 * cosThetaMax;
  const float sinTheta = std::sqrt(1.f - cosTheta * cosTheta);
  const float d = std::pow(s2, 1.f / 3.f);
  return v3(d * sinTheta * std::cos(phi), d * sinTheta * std::sin(phi), d * cosTheta);
}

// sphericalCoordsFromDirection (gpu/gpu_math.h:254-261): the HDRI lookup
void sphericalCoordsFromDirection(V3 d, float &theta, float &phi)
{
  theta = std::acos(std::min(std::max(d.z, -1.f), 1.f));
  const float p = std::atan2(d.y, d.x);
  phi = p < 0.f ? p + 2.f * (float)M_PI : p;
}

// The ray of pixel (px, py) from one uniform4 draw r: r[0..1] the
// sub-pixel offset, r[2..3] the aperture sample.
Ray primaryRayFrom(const CamPre &c, const float r[4], int px, int py, float invW, float invH,
    bool centerPixel, float *screen)
{
  const float sx0 = (centerPixel ? (float)px : (float)px + r[0]) * invW;
  const float sy0 = (centerPixel ? (float)py : (float)py + r[1]) * invH;
  if (screen) {
    screen[0] = sx0;
    screen[1] = sy0;
  }
  const float sx = mixf(c.region[0], c.region[2], sx0);
  const float sy = mixf(c.region[1], c.region[3], sy0);
  Ray ray;
  ray.tmin = 0.f;
  ray.tmax = FLT_MAX;
  if (c.type == 0) {
    ray.org = c.pos;
    V3 d = c.d00 + sx * c.du + sy * c.dv;
    if (c.aperture > 0.f) {
      float lx, ly;
      uniformSampleDisk(c.aperture, r[2], r[3], lx, ly);
      const V3 lp = lx * c.du + (ly * c.aspect) * c.dv;
      ray.org = ray.org + lp;
      d = d - lp;
    }
    ray.dir = normalize(d);
  } else {
    ray.dir = c.dir;
    ray.org = c.p00 + sx * c.pdu + sy * c.pdv;
  }
  return ray;
}

Ray primaryRay(const CamPre &c, Stream &rs, int px, int py, float invW, float invH,
    bool centerPixel, float *screen = nullptr)
{
  float r[4];
  uniform4(rs, r);
  return primaryRayFrom(c, r, px, py, invW, invH, centerPixel, screen);
}

struct SHit
{
  float t;
  V3 P, Ng, Ns;
  float eps;
  uint32_t primId, objId, instId;
  int surface;
  uint32_t prim; // geometry-local primitive index
  float u, v; // triangle barycentrics; segments: u
};

// epsilonFrom (gpu/gpu_util.h:245-250)
float epsilonFrom(V3 P, V3 d, float t)
{
  return std::max(cmax(vabs(P)), cmax(vabs(d)) * t) * 0x1.fp-21f;
}

// populateSurfaceHit + computeTangentSpace (gpu/populateHit.h:200-368);
// primitive ids per computeGeometryPrimId (gpu_util.h:309-315)
SHit populate(const SceneCtx &S, const Ray &ray, const HitRec &h)
{
  const OrcSurface &s = S.sc->surfaces[h.surface];
  const OrcInstance &in = S.sc->instances[h.inst];
  SHit sh;
  sh.t = h.t;
  sh.P = ray.org + h.t * ray.dir;
  sh.eps = epsilonFrom(sh.P, ray.dir, h.t);
  sh.surface = h.surface;
  sh.prim = h.prim;
  sh.u = h.u;
  sh.v = h.v;
  sh.primId = s.primIds ? s.primIds[h.prim] : h.prim;
  sh.objId = s.id;
  sh.instId = in.userId;
  V3 Ng, Ns;
  if (s.type == 2) {
    // QUAD case (populateHit.h:267-279)
    V3 a, b, c;
    triVerts(s, h.prim, a, b, c);
    Ng = cross(b - a, c - a);
    if (!h.front)
      Ng = -Ng;
    Ns = Ng;
  } else if (s.type == 3 || s.type == 4) {
    Ng = Ns = h.n;
  } else if (s.type == 5) {
    // CURVE case with curveSurfaceNormal (curveHelpers.h:91-107)
    V3 p0, p1;
    float r0, r1;
    segmentOf(s, h.prim, p0, r0, p1, r1);
    const V3 dv = p1 - p0;
    const float rad = r0 + (r1 - r0) * h.u;
    const V3 ps = xPoint(S.w2o[h.inst], sh.P);
    V3 o1 = ps - (p0 + h.u * dv);
    o1 = o1 - (dot(o1, dv) / dot(dv, dv)) * dv;
    o1 = o1 * (rad / std::sqrt(dot(o1, o1)));
    Ng = Ns = normalize(o1);
  } else if (s.type == 0) {
    V3 a, b, c;
    triVerts(s, h.prim, a, b, c);
    Ng = normalize(cross(b - a, c - a));
    if (!h.front)
      Ng = -Ng;
    if (s.normals) {
      uint32_t i0, i1, i2;
      if (s.indices) {
        i0 = s.indices[3 * h.prim];
        i1 = s.indices[3 * h.prim + 1];
        i2 = s.indices[3 * h.prim + 2];
      } else {
        i0 = 3 * h.prim;
        i1 = i0 + 1;
        i2 = i0 + 2;
      }
      const float b0 = 1.f - h.u - h.v;
      Ns = b0 * ld3(s.normals, i0) + h.u * ld3(s.normals, i1) + h.v * ld3(s.normals, i2);
    } else
      Ns = Ng;
    Ns = normalize(Ns);
    if (dot(Ng, Ns) < 0.f)
      Ns = -Ns;
  } else {
    V3 c;
    float r;
    sphereOf(s, h.prim, c, r);
    const V3 lo = xPoint(S.w2o[h.inst], ray.org);
    const V3 ld = xVec(S.w2o[h.inst], ray.dir);
    Ng = Ns = (lo + h.t * ld) - c;
  }
  sh.Ng = normalize(xNormalT(S.w2o[h.inst], Ng));
  sh.Ns = normalize(xNormalT(S.w2o[h.inst], Ns));
  return sh;
}

// randomDir(rs, normal) (gpu/gpu_util.h:190-208)
V3 randomDir(Stream &rs, V3 n)
{
  float r[4];
  uniform4(rs, r);
  const V3 d = normalize(v3(2.f * r[0] - 1.f, 2.f * r[1] - 1.f, 2.f * r[2] - 1.f));
  return dot(d, n) > 0.f ? d : -d;
}

struct Ctx
{
  const SceneCtx *S;
  const OrcRenderer *R;
  int volMode;
  int texRound;
  uint64_t rays = 0;
  uint64_t samples = 0; // volume march positions
  // per volume: the reference's delta-tracking majorants (dpt only)
  const std::vector<std::vector<float>> *dptMaj = nullptr;
};

float surfaceAttenuation(Ctx &C, V3 o, V3 d, float tmin, float tmax)
{
  HitRec h;
  float op;
  C.rays++;
  trace<1>(*C.S, o, d, tmin, tmax, false, false, h, op);
  return op;
}

// computeAO (gpu/computeAO.h:38-60)
float computeAO(Ctx &C, Stream &rs, const SHit &hit, float dist, int n)
{
  float weights = 0.f, hits = 0.f;
  const V3 org = hit.P + (hit.eps * hit.Ng);
  for (int i = 0; i < n; i++) {
    const V3 dir = randomDir(rs, hit.Ns);
    const float w = std::max(0.f, dot(dir, hit.Ns));
    weights += w;
    if (w != 0.f)
      hits += w * surfaceAttenuation(C, org, dir, 0.f, dist);
  }
  return weights > 0.f ? 1.f - hits / weights : 0.f;
}

// --- volumes (gpu/volumeIntegration.h, sampleSpatialField.h) ----------------

struct VolHit
{
  int entry;
  V3 lo, ld;
  float t0, t1;
};

void volBounds(const OrcVolume &v, V3 &lo, V3 &hi);
void gridDims(const OrcVolume &v, int d[3]);

// glm::min / glm::max on floats (glm/detail/func_common.inl): the first
// operand where either is NaN
inline float glmMin(float a, float b)
{
  return (b < a) ? b : a;
}
inline float glmMax(float a, float b)
{
  return (a < b) ? b : a;
}

// intersectVolume (scene/Intersectors_ptx.cu:248-274): the local ray's slab
// interval in the volume's bounds -- glm::min / glm::max per axis, then
// glm::compMax / glm::compMin (left folds), so that a ray parallel to a
// bounding plane with its origin on it (a NaN slab) enters or misses as the
// reference's does -- clamped to [tmin, tmax] (gpu_math.h clamp)
bool volumeInterval(V3 blo, V3 bhi, V3 org, V3 dir, float tmin, float tmax, float &t0, float &t1)
{
  const V3 inv = v3(1.f / dir.x, 1.f / dir.y, 1.f / dir.z);
  const V3 mins = (blo - org) * inv, maxs = (bhi - org) * inv;
  const V3 nr = v3(glmMin(mins.x, maxs.x), glmMin(mins.y, maxs.y), glmMin(mins.z, maxs.z));
  const V3 fr = v3(glmMax(mins.x, maxs.x), glmMax(mins.y, maxs.y), glmMax(mins.z, maxs.z));
  const float tin = glmMax(glmMax(nr.x, nr.y), nr.z);
  const float tout = glmMin(glmMin(fr.x, fr.y), fr.z);
  if (!(tin < tout))
    return false;
  t0 = glmMax(tmin, glmMin(tin, tmax));
  t1 = glmMax(tmin, glmMin(tout, tmax));
  return true;
}

bool volumeSlab(const OrcVolume &v, const X34 &w2o, V3 o, V3 d, float tmin, float tmax,
    VolHit &h)
{
  const V3 lo = xPoint(w2o, o), ld = xVec(w2o, d);
  V3 blo, bhi;
  volBounds(v, blo, bhi);
  float t0, t1;
  if (!volumeInterval(blo, bhi, lo, ld, tmin, tmax, t0, t1))
    return false;
  h.lo = lo;
  h.ld = ld;
  h.t0 = t0;
  h.t1 = t1;
  return true;
}

struct VolCtx
{
  std::vector<X34> w2o;
};

// ---------------------------------------------------------------------------
// NanoVDB grids (the layout of the NanoVDB version the reference vendors,
// external/nanovdb/include/nanovdb/NanoVDB.h, 32.7): GridData 672 B, then
// TreeData 64 B whose mNodeOffset[3] locates the RootData; RootData 64 B
// (index bbox, tile count, background, stats) followed by 32-byte tiles
// (key, child offset from the RootData, state, value); upper nodes (32^3
// entries: child mask at 4128, table of 8-byte entries at 8256), lower
// nodes (16^3: child mask at 544, table at 1088) whose table entries hold a
// child offset from the node or a tile value; leaves (8^3) whose values
// start at byte 96 (float) or whose codes do (Fp4/Fp8/Fp16/FpN, decoded as
// code * quantum + minimum with the minimum at 80 and the quantum at 84).
// ---------------------------------------------------------------------------

struct Nvdb
{
  const uint8_t *grid = nullptr, *root = nullptr;
  uint32_t type = 0, tiles = 0;
  float background = 0.f;
  float inv[9], vec[3];
  double wlo[3], whi[3], voxel[3];
  int ilo[3], ihi[3];
};

template <typename T>
T rd(const uint8_t *p)
{
  T v;
  std::memcpy(&v, p, sizeof(T));
  return v;
}

bool nvdbOpen(const uint8_t *g, Nvdb &n)
{
  if (!g)
    return false;
  const uint64_t magic = rd<uint64_t>(g);
  if (magic != 0x304244566F6E614EULL && magic != 0x314244566F6E614EULL)
    return false;
  if ((rd<uint32_t>(g + 16) >> 21) != 32u) // major version
    return false;
  n.grid = g;
  n.type = rd<uint32_t>(g + 636);
  if (n.type != 1 && (n.type < 13 || n.type > 16))
    return false;
  for (int k = 0; k < 9; k++)
    n.inv[k] = rd<float>(g + 296 + 36 + 4 * k);
  for (int k = 0; k < 3; k++) {
    n.vec[k] = rd<float>(g + 296 + 72 + 4 * k);
    n.wlo[k] = rd<double>(g + 560 + 8 * k);
    n.whi[k] = rd<double>(g + 584 + 8 * k);
    n.voxel[k] = rd<double>(g + 608 + 8 * k);
  }
  n.root = g + 672 + rd<int64_t>(g + 672 + 24);
  for (int k = 0; k < 3; k++) {
    n.ilo[k] = rd<int32_t>(n.root + 4 * k);
    n.ihi[k] = rd<int32_t>(n.root + 12 + 4 * k);
  }
  n.tiles = rd<uint32_t>(n.root + 24);
  n.background = rd<float>(n.root + 28);
  return true;
}

bool maskBit(const uint8_t *mask, uint32_t i)
{
  return (rd<uint64_t>(mask + 8 * (i >> 6)) >> (i & 63)) & 1u;
}

// LeafData<float / Fp4 / Fp8 / Fp16 / FpN>::getValue (NanoVDB.h:3880-4031)
float nvdbLeafValue(const Nvdb &n, const uint8_t *leaf, uint32_t i, int fused)
{
  if (n.type == 1)
    return rd<float>(leaf + 96 + 4 * i);
  uint32_t code;
  if (n.type == 13)
    code = (leaf[96 + (i >> 1)] >> ((i & 1) << 2)) & 15u;
  else if (n.type == 14)
    code = leaf[96 + i];
  else if (n.type == 15)
    code = rd<uint16_t>(leaf + 96 + 2 * i);
  else {
    const uint32_t b = leaf[15] >> 5; // log2 of the bit width
    const uint32_t w = rd<uint32_t>(leaf + 96 + 4 * (i >> (5 - b)));
    code = (w >> ((i & ((32u >> b) - 1u)) << b)) & ((1u << (1u << b)) - 1u);
  }
  const float mn = rd<float>(leaf + 80), q = rd<float>(leaf + 84);
  return fused ? std::fma((float)code, q, mn) : (float)code * q + mn;
}

// RootNode / InternalNode / LeafNode getValue (NanoVDB.h:2947, 3528)
float nvdbValue(const Nvdb &n, int x, int y, int z, int fused)
{
  const uint64_t key = (uint64_t)((uint32_t)z >> 12) | ((uint64_t)((uint32_t)y >> 12) << 21)
      | ((uint64_t)((uint32_t)x >> 12) << 42);
  const uint8_t *tile = nullptr;
  for (uint32_t t = 0; t < n.tiles; t++) {
    const uint8_t *p = n.root + 64 + 32 * t;
    if (rd<uint64_t>(p) == key) {
      tile = p;
      break;
    }
  }
  if (!tile)
    return n.background;
  const int64_t child = rd<int64_t>(tile + 8);
  if (!child)
    return rd<float>(tile + 20);
  const uint8_t *up = n.root + child;
  const uint32_t nu = (((uint32_t)x & 4095u) >> 7) << 10 | (((uint32_t)y & 4095u) >> 7) << 5
      | (((uint32_t)z & 4095u) >> 7);
  if (!maskBit(up + 4128, nu))
    return rd<float>(up + 8256 + 8 * nu);
  const uint8_t *lo = up + rd<int64_t>(up + 8256 + 8 * nu);
  const uint32_t nl = (((uint32_t)x & 127u) >> 3) << 8 | (((uint32_t)y & 127u) >> 3) << 4
      | (((uint32_t)z & 127u) >> 3);
  if (!maskBit(lo + 544, nl))
    return rd<float>(lo + 1088 + 8 * nl);
  const uint8_t *leaf = lo + rd<int64_t>(lo + 1088 + 8 * nl);
  const uint32_t i = ((uint32_t)x & 7u) << 6 | ((uint32_t)y & 7u) << 3 | ((uint32_t)z & 7u);
  return nvdbLeafValue(n, leaf, i, fused);
}

// SpatialFieldSampler<nanovdb::Grid> (gpu/sampleSpatialField.h:80-109):
// worldToIndexF (Map::applyInverseMapF: the location as double minus the
// float translation, cast to float, then the float inverse matrix through
// fmaf, math/Math.h matMult), then SampleFromVoxels<_, 1>: floor, the
// 2x2x2 stencil, and lerps a + w (b - a) over z, then y, then x
// (math/SampleFromVoxels.h:200-245,400-407).
float nvdbSample(const Nvdb &n, V3 p, int fused)
{
  const float dx = (float)((double)p.x - (double)n.vec[0]);
  const float dy = (float)((double)p.y - (double)n.vec[1]);
  const float dz = (float)((double)p.z - (double)n.vec[2]);
  const float ix = std::fma(dx, n.inv[0], std::fma(dy, n.inv[1], dz * n.inv[2]));
  const float iy = std::fma(dx, n.inv[3], std::fma(dy, n.inv[4], dz * n.inv[5]));
  const float iz = std::fma(dx, n.inv[6], std::fma(dy, n.inv[7], dz * n.inv[8]));
  const double fx = std::floor((double)ix), fy = std::floor((double)iy), fz = std::floor((double)iz);
  const float ux = (float)((double)ix - fx), uy = (float)((double)iy - fy),
              uz = (float)((double)iz - fz);
  const int i = (int32_t)fx, j = (int32_t)fy, k = (int32_t)fz;
  float v[2][2][2];
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++)
      for (int c = 0; c < 2; c++)
        v[a][b][c] = nvdbValue(n, i + a, j + b, k + c, fused);
  auto lerp = [&](float a, float b, float w) {
    return fused ? std::fma(w, b - a, a) : a + w * (b - a);
  };
  return lerp(lerp(lerp(v[0][0][0], v[0][0][1], uz), lerp(v[0][1][0], v[0][1][1], uz), uy),
      lerp(lerp(v[1][0][0], v[1][0][1], uz), lerp(v[1][1][0], v[1][1][1], uz), uy),
      ux);
}

// the same lookup in FP64 (exact weights and interpolation; the clean marcher)
double nvdbSampleExact(const Nvdb &n, double px, double py, double pz)
{
  const double ix = (px - n.vec[0]) * n.inv[0] + (py - n.vec[1]) * n.inv[1]
      + (pz - n.vec[2]) * n.inv[2];
  const double iy = (px - n.vec[0]) * n.inv[3] + (py - n.vec[1]) * n.inv[4]
      + (pz - n.vec[2]) * n.inv[5];
  const double iz = (px - n.vec[0]) * n.inv[6] + (py - n.vec[1]) * n.inv[7]
      + (pz - n.vec[2]) * n.inv[8];
  const double fx = std::floor(ix), fy = std::floor(iy), fz = std::floor(iz);
  const double ux = ix - fx, uy = iy - fy, uz = iz - fz;
  const int i = (int)fx, j = (int)fy, k = (int)fz;
  double r = 0.0;
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++)
      for (int c = 0; c < 2; c++)
        r += (a ? ux : 1.0 - ux) * (b ? uy : 1.0 - uy) * (c ? uz : 1.0 - uz)
            * (double)nvdbValue(n, i + a, j + b, k + c, 1);
  return r;
}

// SpatialFieldSampler<cudaTextureObject_t> (gpu/sampleSpatialField.h:54-78)
// with StructuredRegularField::gpuData's invSpacing
// (StructuredRegularField.cpp:188-189): the normalised texture coordinate of
// world point p
V3 fieldCoord(const float *origin, const float *spacing, const int *dims, V3 p)
{
  const V3 sp = ld3(spacing, 0);
  const V3 inv = v3(1.f / (sp.x * (float)dims[0]), 1.f / (sp.y * (float)dims[1]),
      1.f / (sp.z * (float)dims[2]));
  return ((p - ld3(origin, 0)) + 0.5f * sp) * inv;
}

float sampleFieldParity(const OrcVolume &v, V3 p, int round)
{
  if (v.nvdb) {
    Nvdb n;
    return nvdbOpen(v.nvdb, n) ? nvdbSample(n, p, 1) : 0.f;
  }
  const V3 c = fieldCoord(v.origin, v.spacing, v.dims, p);
  return v.filterLinear ? tex3dLinear(v.field, v.dims, c.x, c.y, c.z, round)
                        : tex3dPoint(v.field, v.dims, c.x, c.y, c.z);
}

void classifyParity(const OrcVolume &v, float s, int round, float out[4])
{
  if (!v.tf) {
    out[0] = v.uniformColor[0];
    out[1] = v.uniformColor[1];
    out[2] = v.uniformColor[2];
    out[3] = v.uniformOpacity;
    return;
  }
  const float lo = v.valueRange[0], hi = v.valueRange[1];
  const float cs = std::max(lo, std::min(s, hi));
  const float coord = (cs - lo) * (1.f / (hi - lo));
  tex1dLinear(v.tf, 256, 4, coord, round, out);
}

float volStep(const OrcVolume &v)
{
  // NvdbRegularField::stepSize (NvdbRegularField.cpp:119-122): min voxel / 2
  Nvdb n;
  if (v.nvdb && nvdbOpen(v.nvdb, n))
    return std::min((float)n.voxel[0], std::min((float)n.voxel[1], (float)n.voxel[2])) / 2.f;
  return std::min(v.spacing[0] / 2.f, std::min(v.spacing[1] / 2.f, v.spacing[2] / 2.f));
}

// rayMarchVolume + _rayMarchVolume (volumeIntegration.h:64-126), in fp32
// with emulated texture filtering (parity mode) or in FP64 with exact
// filtering (clean mode).
float rayMarchVolume(Ctx &C, const OrcVolume &v, const VolHit &h, Stream &rs, V3 *color,
    float &opacity, float invSamplingRate)
{
  float lower = h.t0;
  const float upper = h.t1;
  const float depth = lower;
  const float st0 = volStep(v);
  const float u0 = uniform(rs);
  lower += st0 * u0;
  const float stepSize = st0 * invSamplingRate;
  const float exponent = stepSize * (1.f / v.unitDistance);
  const float u1 = uniform(rs);
  lower += stepSize * u1;
  if (C.volMode == 0) {
    float T = 1.f;
    while (opacity < 0.99f && upper - lower >= 0.f) {
      C.samples++;
      const V3 p = h.lo + h.ld * lower;
      const float s = sampleFieldParity(v, p, C.texRound);
      if (!std::isnan(s)) {
        float co[4];
        classifyParity(v, s, C.texRound, co);
        const float stT = std::pow(1.f - co[3], exponent);
        const float a = T * (1.f - stT);
        if (color)
          *color = *color + a * v3(co[0], co[1], co[2]);
        opacity += a;
        T *= stT;
      }
      lower += stepSize;
    }
    return depth;
  }
  // clean FP64 mode: same jitter draws and sample lattice, exact arithmetic
  double lo = (double)h.t0 + (double)st0 * u0;
  const double step = (double)st0 * invSamplingRate;
  lo += step * u1;
  const double ex = step / v.unitDistance;
  double T = 1.0, op = opacity;
  double col[3] = {0, 0, 0};
  const double sx = v.spacing[0], sy = v.spacing[1], sz = v.spacing[2];
  for (long k = 0; op < 0.99 && (double)upper - lo >= 0.0; k++) {
    C.samples++;
    const double px = (double)h.lo.x + (double)h.ld.x * lo;
    const double py = (double)h.lo.y + (double)h.ld.y * lo;
    const double pz = (double)h.lo.z + (double)h.ld.z * lo;
    double s;
    Nvdb nv;
    if (v.nvdb && nvdbOpen(v.nvdb, nv)) {
      s = nvdbSampleExact(nv, px, py, pz);
    } else {
      const double cx = ((px - v.origin[0]) + 0.5 * sx) / (sx * v.dims[0]);
      const double cy = ((py - v.origin[1]) + 0.5 * sy) / (sy * v.dims[1]);
      const double cz = ((pz - v.origin[2]) + 0.5 * sz) / (sz * v.dims[2]);
      s = v.filterLinear
          ? tex3dExact(v.field, v.dims, cx, cy, cz)
          : (double)tex3dPoint(v.field, v.dims, (float)cx, (float)cy, (float)cz);
    }
    if (!std::isnan(s)) {
      double co[4];
      if (v.tf) {
        const double l = v.valueRange[0], hh = v.valueRange[1];
        const double cs = std::max(l, std::min(s, hh));
        tex1dExact(v.tf, 256, (cs - l) / (hh - l), co);
      } else {
        co[0] = v.uniformColor[0];
        co[1] = v.uniformColor[1];
        co[2] = v.uniformColor[2];
        co[3] = v.uniformOpacity;
      }
      const double stT = std::pow(1.0 - co[3], ex);
      const double a = T * (1.0 - stT);
      for (int c = 0; c < 3; c++)
        col[c] += a * co[c];
      op += a;
      T *= stT;
    }
    lo = (double)h.t0 + (double)st0 * u0 + step * u1 + step * (double)(k + 1);
  }
  opacity = (float)op;
  if (color)
    *color = *color + v3((float)col[0], (float)col[1], (float)col[2]);
  return depth;
}

bool intersectVolumes(const Ctx &C, const VolCtx &VC, V3 o, V3 d, float tmin, float tmax,
    int skip, VolHit &best)
{
  bool found = false;
  for (int i = 0; i < C.S->sc->numVolumes; i++) {
    if (i == skip)
      continue;
    VolHit h;
    if (volumeSlab(C.S->sc->volumes[i], VC.w2o[i], o, d, tmin, tmax, h)) {
      if (!found || h.t0 < best.t0) {
        best = h;
        best.entry = i;
        found = true;
      }
    }
  }
  return found;
}

// rayMarchAllVolumes (volumeIntegration.h:318-350)
float rayMarchAllVolumes(Ctx &C, const VolCtx &VC, Stream &rs, V3 o, V3 d, float tmin,
    float tfar, float invRate, V3 &color, float &opacity, uint32_t &objID,
    uint32_t &instID)
{
  float depth = tfar;
  if (C.S->sc->numVolumes == 0)
    return depth;
  bool first = true;
  int last = -1;
  do {
    VolHit h;
    if (!intersectVolumes(C, VC, o, d, tmin, tfar, last, h))
      break;
    const OrcVolume &v = C.S->sc->volumes[h.entry];
    if (first) {
      objID = v.id;
      instID = v.instId;
      first = false;
    }
    depth = std::min(depth, h.t0);
    h.t1 = std::min(tfar, h.t1);
    rayMarchVolume(C, v, h, rs, &color, opacity, invRate);
    tmin = h.t1 + 1e-3f;
    last = h.entry;
  } while (opacity < 0.99f);
  return depth;
}

float volumeAttenuation(Ctx &C, const VolCtx &VC, Stream &rs, V3 o, V3 d, float tmin,
    float tmax, float invRate)
{
  float a = 0.f;
  for (int i = 0; i < C.S->sc->numVolumes; i++) {
    VolHit h;
    if (!volumeSlab(C.S->sc->volumes[i], VC.w2o[i], o, d, tmin, tmax, h))
      continue;
    h.entry = i;
    rayMarchVolume(C, C.S->sc->volumes[i], h, rs, nullptr, a, invRate);
    if (a >= 0.99f)
      break;
  }
  return a;
}

// ---------------------------------------------------------------------------
// delta tracking for the dpt renderer
// ---------------------------------------------------------------------------

// float -> int32 the way the GPU converts: truncate, saturate, NaN -> 0
int f2iSat(float x)
{
  if (std::isnan(x))
    return 0;
  if (x >= 2147483648.f)
    return INT32_MAX;
  if (x <= -2147483648.f)
    return INT32_MIN;
  return (int)x;
}

// projectOnGrid (gpu/uniformGrid.h:43-50), one axis
int projectAxis(float v, float lo, float hi, int n)
{
  const float v01 = (v - lo) / (hi - lo);
  return std::min(std::max(f2iSat(v01 * (float)n), 0), n - 1);
}

void volBounds(const OrcVolume &v, V3 &lo, V3 &hi)
{
  // NvdbRegularField::bounds: the grid's world bbox as float
  Nvdb n;
  if (v.nvdb && nvdbOpen(v.nvdb, n)) {
    lo = v3((float)n.wlo[0], (float)n.wlo[1], (float)n.wlo[2]);
    hi = v3((float)n.whi[0], (float)n.whi[1], (float)n.whi[2]);
    return;
  }
  lo = ld3(v.origin, 0);
  hi = lo
      + v3((float)(v.dims[0] - 1) * v.spacing[0],
          (float)(v.dims[1] - 1) * v.spacing[1],
          (float)(v.dims[2] - 1) * v.spacing[2]);
}

// UniformGrid::init / buildGridGPU / computeMaxOpacitiesGPU
// (scene/volume/space_skipping/UniformGrid.cu:44-258) as the reference
// drives them (StructuredRegularField.cpp:205-212, TransferFunction1D.cpp:
// 76-77): ceil(dims/16) cells over the field bounds; each cell's 8 taps sit
// at the object-space points (id +- 0.5) / cellDims, go through the field
// sampler, and their max is splatted (min/max) into every cell that the
// cell's bounds project onto; the majorant is the max TF alpha over entries
// [int(lo * 255), int(hi * 255) + 1] of the TF range [0, 1] (the default
// argument), read at entry centres.
// The grid dims are the field's voxel dims, or for a NanoVDB field its index
// bbox extent (NvdbRegularField::buildGrid, NvdbRegularField.cpp:141-149).
void gridDims(const OrcVolume &v, int d[3])
{
  Nvdb n;
  if (v.nvdb && nvdbOpen(v.nvdb, n)) {
    for (int k = 0; k < 3; k++)
      d[k] = n.ihi[k] - n.ilo[k] + 1;
    return;
  }
  for (int k = 0; k < 3; k++)
    d[k] = v.dims[k];
}

void dptMajorants(const OrcVolume &v, int round, std::vector<float> &maj)
{
  int gd[3];
  gridDims(v, gd);
  const int md[3] = {(gd[0] + 15) / 16, (gd[1] + 15) / 16, (gd[2] + 15) / 16};
  const size_t cells = (size_t)md[0] * md[1] * md[2];
  std::vector<float> lo(cells, 1e30f), hi(cells, -1e30f);
  V3 blo, bhi;
  volBounds(v, blo, bhi);
  const float ex = (bhi.x - blo.x) / (float)md[0];
  const float ey = (bhi.y - blo.y) / (float)md[1];
  const float ez = (bhi.z - blo.z) / (float)md[2];
  for (int iz = 0; iz < md[2]; iz++)
    for (int iy = 0; iy < md[1]; iy++)
      for (int ix = 0; ix < md[0]; ix++) {
        const float lx = blo.x + (float)ix * ex, ly = blo.y + (float)iy * ey,
                    lz = blo.z + (float)iz * ez;
        const float ux = lx + ex, uy = ly + ey, uz = lz + ez;
        float value = -1e30f;
        for (int k = 0; k < 8; k++) {
          const float ox = (k == 1 || k == 2 || k == 5 || k == 6) ? 0.5f : -0.5f;
          const float oy = (k == 2 || k == 3 || k == 6 || k == 7) ? 0.5f : -0.5f;
          const float oz = k >= 4 ? 0.5f : -0.5f;
          const V3 p = v3(((float)ix + ox) / (float)md[0], ((float)iy + oy) / (float)md[1],
              ((float)iz + oz) / (float)md[2]);
          value = std::fmax(value, sampleFieldParity(v, p, round));
        }
        const int x0 = projectAxis(lx, blo.x, bhi.x, md[0]);
        const int x1 = projectAxis(ux, blo.x, bhi.x, md[0]);
        const int y0 = projectAxis(ly, blo.y, bhi.y, md[1]);
        const int y1 = projectAxis(uy, blo.y, bhi.y, md[1]);
        const int z0 = projectAxis(lz, blo.z, bhi.z, md[2]);
        const int z1 = projectAxis(uz, blo.z, bhi.z, md[2]);
        for (int z = z0; z <= z1; z++)
          for (int y = y0; y <= y1; y++)
            for (int x = x0; x <= x1; x++) {
              const size_t c = ((size_t)z * md[1] + y) * md[0] + x;
              if (value < lo[c])
                lo[c] = value;
              if (value > hi[c])
                hi[c] = value;
            }
      }
  maj.assign(cells, 0.f);
  for (size_t c = 0; c < cells; c++) {
    if (hi[c] < lo[c])
      continue;
    if (!v.tf) {
      maj[c] = v.uniformOpacity;
      continue;
    }
    const int e0 = std::min(std::max(f2iSat(lo[c] * 255.f), 0), 255);
    const int e1 = std::min(std::max((int)((uint32_t)f2iSat(hi[c] * 255.f) + 1u), 0), 255);
    float m = 0.f;
    for (int i = e0; i <= e1; i++) {
      float co[4];
      tex1dLinear(v.tf, 256, 4, ((float)i + 0.5f) / 256.f, round, co);
      m = std::fmax(m, co[3]);
    }
    maj[c] = m;
  }
}

// dda3 (gpu/dda.h:44-122): cell walk over `dims` cells spanning [blo, bhi];
// the first-boundary distances are fused multiply-adds, as in the GPU code.
template <typename F>
void dda3(V3 org, V3 dir, float tlo, float thi, const int dims[3], V3 blo, V3 bhi, F func)
{
  const V3 rcp = v3(dir.x != 0.f ? 1.f / dir.x : 0.f, dir.y != 0.f ? 1.f / dir.y : 0.f,
      dir.z != 0.f ? 1.f / dir.z : 0.f);
  const V3 lo = (blo - org) * rcp;
  const V3 hi = (bhi - org) * rcp;
  const V3 tnear = v3(std::min(lo.x, hi.x), std::min(lo.y, hi.y), std::min(lo.z, hi.z));
  const V3 tfar = v3(std::max(lo.x, hi.x), std::max(lo.y, hi.y), std::max(lo.z, hi.z));
  int c[3] = {projectAxis(org.x, blo.x, bhi.x, dims[0]), projectAxis(org.y, blo.y, bhi.y, dims[1]),
      projectAxis(org.z, blo.z, bhi.z, dims[2])};
  const float dist[3] = {(tfar.x - tnear.x) / (float)dims[0],
      (tfar.y - tnear.y) / (float)dims[1], (tfar.z - tnear.z) / (float)dims[2]};
  const float dv[3] = {dir.x, dir.y, dir.z};
  const float tn[3] = {tnear.x, tnear.y, tnear.z};
  int step[3], stop[3];
  float tnext[3];
  for (int a = 0; a < 3; a++) {
    step[a] = dv[a] > 0.f ? 1 : -1;
    stop[a] = dv[a] > 0.f ? dims[a] : -1;
    tnext[a] = std::fma((float)(dv[a] > 0.f ? c[a] + 1 : dims[a] - c[a]), dist[a], tn[a]);
  }
  float t0 = std::max(tlo, 0.f);
  for (int guard = 0; guard < 4 * (dims[0] + dims[1] + dims[2]) + 8; guard++) {
    const float tc = std::min(tnext[0], std::min(tnext[1], tnext[2]));
    const float t1 = std::min(tc, thi);
    const size_t cell = ((size_t)c[2] * dims[1] + c[1]) * dims[0] + c[0];
    if (!func(cell, t0, t1))
      return;
    bool stopNow = false;
    for (int a = 0; a < 3 && !stopNow; a++) {
      if (tnext[a] == tc) {
        tnext[a] += dist[a];
        c[a] += step[a];
        if (c[a] == stop[a])
          stopNow = true;
      }
    }
    if (stopNow)
      break;
    t0 = t1;
  }
}

// _sampleDistance (volumeIntegration.h:167-238): Woodcock tracking per DDA
// cell against the cell majorant, t -= log(1-u)/majorant*stepSize (a fused
// multiply-add, as in the GPU code).
float sampleDistance(Ctx &C, const OrcVolume &v, const std::vector<float> &maj,
    const VolHit &h, Stream &rs, V3 &albedo, float &extinction, float &tr)
{
  const float stepSize = volStep(v);
  float t_out = h.t1;
  tr = 1.f;
  const V3 org = v3(std::fma(h.ld.x, h.t0, h.lo.x), std::fma(h.ld.y, h.t0, h.lo.y),
      std::fma(h.ld.z, h.t0, h.lo.z));
  int gd[3];
  gridDims(v, gd);
  const int md[3] = {(gd[0] + 15) / 16, (gd[1] + 15) / 16, (gd[2] + 15) / 16};
  V3 blo, bhi;
  volBounds(v, blo, bhi);
  dda3(org, h.ld, 0.f, h.t1 - h.t0, md, blo, bhi, [&](size_t cell, float t0, float t1) {
    const float majorant = maj[cell];
    float t = t0;
    for (int guard = 0; guard < (1 << 20); guard++) {
      if (majorant <= 0.f)
        break;
      const float lg = std::log(1.f - uniform(rs));
      t = std::fma(-(lg / majorant), stepSize, t);
      if (t >= t1)
        break;
      const float tt = t + h.t0;
      const V3 p = v3(std::fma(h.ld.x, tt, h.lo.x), std::fma(h.ld.y, tt, h.lo.y),
          std::fma(h.ld.z, tt, h.lo.z));
      const float s = sampleFieldParity(v, p, C.texRound);
      if (!std::isnan(s)) {
        float co[4];
        classifyParity(v, s, C.texRound, co);
        albedo = v3(co[0], co[1], co[2]);
        extinction = co[3];
        const float u = uniform(rs);
        if (extinction >= u * majorant) {
          tr = 0.f;
          t_out = t;
          return false;
        }
      }
    }
    return true;
  });
  return t_out + h.t0;
}

// sampleDistanceAllVolumes (volumeIntegration.h:352-389)
float sampleDistanceAllVolumes(Ctx &C, const VolCtx &VC, Stream &rs, V3 o, V3 d, float tmin,
    float tfar, V3 &albedo, float &extinction, float &transmittance, uint32_t &objID,
    uint32_t &instID)
{
  float depth = tfar;
  transmittance = 1.f;
  int last = -1;
  for (int guard = 0; guard <= C.S->sc->numVolumes; guard++) {
    VolHit h;
    if (!intersectVolumes(C, VC, o, d, tmin, tfar, last, h))
      break;
    const OrcVolume &v = C.S->sc->volumes[h.entry];
    h.t1 = std::min(tfar, h.t1);
    V3 alb = v3(0, 0, 0);
    float ext = 0.f, tr = 0.f;
    const float dd = sampleDistance(C, v, (*C.dptMaj)[h.entry], h, rs, alb, ext, tr);
    if (dd < depth) {
      depth = dd;
      albedo = alb;
      extinction = ext;
      transmittance = tr;
      objID = v.id;
      instID = v.instId;
    }
    tmin = h.t1 + 1e-3f;
    last = h.entry;
  }
  return depth;
}

float matteOpacity(const OrcSurface &s)
{
  return surfOpacity(s);
}

// --- geometry attributes and material parameters
// (gpu/evalMaterialParameters.h:60-374, MatteShader_ptx.cu:38-49) ---

struct V4
{
  float x, y, z, w;
};
inline V4 v4add(V4 a, V4 b)
{
  return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w};
}
inline V4 v4sub(V4 a, V4 b)
{
  return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w};
}
inline V4 v4mul(V4 a, float s)
{
  return {a.x * s, a.y * s, a.z * s, a.w * s};
}

float srgbChannel(float c)
{
  const float x = std::min(std::max(c, 0.f), 1.f);
  return x < 0.0031308f ? x * 12.92f : std::pow(x, 0.41666f) * 1.055f - 0.055f;
}

V4 attrValue(const OrcAttr &a, uint32_t offset, V4 uf)
{
  if (!a.data || offset == 0xFFFFFFFFu)
    return uf;
  switch (a.type) {
  case 240:
    return {((const float *)a.data)[offset], 0.f, 0.f, 1.f};
  case 241: {
    const float *p = (const float *)a.data + 2 * (size_t)offset;
    return {p[0], p[1], 0.f, 1.f};
  }
  case 242: {
    const float *p = (const float *)a.data + 3 * (size_t)offset;
    return {p[0], p[1], p[2], 1.f};
  }
  case 243: {
    const float *p = (const float *)a.data + 4 * (size_t)offset;
    return {p[0], p[1], p[2], p[3]};
  }
  case 221:
    return {((const uint8_t *)a.data)[offset] / 255.f, 0.f, 0.f, 1.f};
  case 223:
    return {((const uint16_t *)a.data)[offset] / 65535.f, 0.f, 0.f, 1.f};
  case 260:
  case 261: {
    const uint8_t *p = (const uint8_t *)a.data + 4 * (size_t)offset;
    V4 r{p[0] / 255.f, p[1] / 255.f, p[2] / 255.f, p[3] / 255.f};
    if (a.type == 261)
      r = {srgbChannel(r.x), srgbChannel(r.y), srgbChannel(r.z), r.w};
    return r;
  }
  default:
    return uf;
  }
}

// readAttributeValue: per-vertex values interpolated per subtype, then
// per-primitive values, then the uniform value
V4 readAttribute(const SceneCtx &S, const SHit &sh, int id)
{
  const OrcSurface &s = S.sc->surfaces[sh.surface];
  const V4 uf{s.uattr[id][0], s.uattr[id][1], s.uattr[id][2], s.uattr[id][3]};
  const OrcAttr &ap = s.vattr[id];
  const uint32_t prim = sh.prim;
  if (ap.data) {
    const float b0 = 1.f - sh.u - sh.v, b1 = sh.u, b2 = sh.v;
    if (s.type == 0) {
      uint32_t i0, i1, i2;
      if (s.indices) {
        i0 = s.indices[3 * prim];
        i1 = s.indices[3 * prim + 1];
        i2 = s.indices[3 * prim + 2];
      } else {
        i0 = 3 * prim;
        i1 = i0 + 1;
        i2 = i0 + 2;
      }
      return v4add(v4add(v4mul(attrValue(ap, i0, uf), b0), v4mul(attrValue(ap, i1, uf), b1)),
          v4mul(attrValue(ap, i2, uf), b2));
    }
    if (s.type == 2) {
      const uint32_t pair = prim & ~1u;
      uint32_t x, y, w, z, d0, d1;
      quadTri(s, pair, x, y, w);
      quadTri(s, pair + 1, z, d0, d1);
      const V4 v0 = attrValue(ap, x, uf), v1 = attrValue(ap, y, uf);
      const V4 v2 = attrValue(ap, z, uf), v3 = attrValue(ap, w, uf);
      const float qu = (prim & 1u) ? b1 : 1.f - b1;
      const float qv = (prim & 1u) ? b2 : 1.f - b2;
      const V4 l0 = v4add(v1, v4mul(v4sub(v0, v1), qu));
      const V4 l1 = v4add(v2, v4mul(v4sub(v3, v2), qu));
      return v4add(l1, v4mul(v4sub(l0, l1), qv));
    }
    if (s.type == 3 || s.type == 4) {
      const uint32_t i0 = s.indices ? s.indices[2 * prim] : 2 * prim;
      const uint32_t i1 = s.indices ? s.indices[2 * prim + 1] : 2 * prim + 1;
      return v4add(v4mul(attrValue(ap, i0, uf), 1.f - sh.u), v4mul(attrValue(ap, i1, uf), sh.u));
    }
    if (s.type == 5) {
      const uint32_t i0 = s.indices ? s.indices[prim] : prim;
      return v4add(v4mul(attrValue(ap, i0, uf), 1.f - sh.u), v4mul(attrValue(ap, i0 + 1, uf), sh.u));
    }
    const uint32_t i = s.indices ? s.indices[prim] : prim;
    return attrValue(ap, i, uf);
  }
  const OrcAttr &pp = s.pattr[id];
  if (pp.data)
    return attrValue(pp, s.type == 2 ? prim / 2 : prim, uf);
  return uf;
}

// Texture lookup with normalised coordinates, float4 texels: address modes
// clamp (0) / repeat (1) / mirror (2), point or linear filtering, as the
// texture unit computes them (recovered from GPU-captured sweeps of every
// mode in 1D, 2D and 3D and reproduced bit for bit):
//  * the coordinate is truncated to 21 fractional bits;
//  * point: clamp takes floor(u * n) clamped; repeat the same of u's
//    fraction; mirror folds u into [0, 1] over a period of 2 first;
//  * linear: x = u * n - 0.5 and the fraction rounded half up to 8 bits, as
//    hwAxis; clamp clamps x to [0, n - 1]; repeat takes u's fraction
//    first and wraps the texel indices; mirror mirrors the texel indices
//    (period 2n) of the unfolded x;
//  * the corner weights are integers summing to 256 (hwCornerWeights) and
//    the value is their exact weighted sum rounded once to float.
int wrapIndex(long long i, int n, int mode)
{
  if (mode == 1) {
    long long m = i % n;
    return (int)(m < 0 ? m + n : m);
  }
  if (mode == 2) {
    const long long p = 2LL * n;
    long long m = i % p;
    if (m < 0)
      m += p;
    return (int)(m < n ? m : p - 1 - m);
  }
  return (int)std::min(std::max(i, 0LL), (long long)n - 1);
}

// texel pair (or the single texel, i0 == i1, w == 0) of one axis
void hwTap(float coord, int n, int mode, int linear, int &i0, int &i1, int &w)
{
  double u = std::isfinite(coord) ? std::floor((double)coord * 2097152.0) / 2097152.0 : 0.0;
  if (!linear) {
    double x;
    if (mode == 1)
      x = (u - std::floor(u)) * n;
    else if (mode == 2) {
      const double t = u - 2.0 * std::floor(u * 0.5);
      x = (t > 1.0 ? 2.0 - t : t) * n;
    } else
      x = u * n;
    i0 = i1 = wrapIndex((long long)std::floor(std::min(std::max(x, -1.0), (double)n + 1.0)), n,
        mode == 1 ? 1 : 0);
    w = 0;
    return;
  }
  if (mode == 1)
    u -= std::floor(u);
  double x = u * (double)n - 0.5;
  if (mode == 0)
    x = std::min(std::max(x, 0.0), (double)(n - 1));
  else
    x = std::min(std::max(x, -4.0 * n), 4.0 * n);
  const double fl = std::floor(x);
  long long i = (long long)fl;
  w = (int)std::floor((x - fl) * 256.0 + 0.5);
  if (w >= 256) {
    w = 0;
    i++;
  }
  i0 = wrapIndex(i, n, mode);
  i1 = wrapIndex(i + 1, n, mode);
}

// Integer corner weights (sum 256) of a linear fetch from the per-axis
// 8-bit weights w[]: corner q = x + 2y + 4z. 3D splits z, then x within
// each z slice, then y within each x column; 2D is one slice of budget 256;
// the y split rounds half down in the x0 column and half up in the x1
// column, the x split half up.
void hwCornerWeights(int ndim, const int w[3], int out[8])
{
  for (int q = 0; q < 8; q++)
    out[q] = 0;
  if (ndim == 1) {
    out[0] = 256 - w[0];
    out[1] = w[0];
    return;
  }
  for (int z = 0; z < (ndim == 3 ? 2 : 1); z++) {
    const int B = ndim == 3 ? (z ? w[2] : 256 - w[2]) : 256;
    const int x1 = (w[0] * B + 128) >> 8;
    for (int x = 0; x < 2; x++) {
      const int C = x ? x1 : B - x1;
      const int y1 = (w[1] * C + (x ? 128 : 127)) >> 8;
      out[x + 4 * z] = C - y1;
      out[x + 2 + 4 * z] = y1;
    }
  }
}

// glm::convertSRGBToLinear of one component (gamma 2.4), as the
// reference's image staging calls it
float srgbToLinearGlm(float x)
{
  return x <= 0.04045f ? x * 0.07739938080495356f
                       : std::pow((x + 0.055f) * 0.94786729857819905f, 2.4f);
}

// convertComponentUint8 (utility/CudaImageTexture.cpp:43-57) of component c
// of one texel of element type et: 8-bit values as they are, sRGB bytes
// linearised and truncated to 8 bits, 16-bit values truncated from
// (c / 65535) * 255
uint8_t stageByte(int et, const uint8_t *texel, int c)
{
  if (et == 223) {
    uint16_t v;
    std::memcpy(&v, texel + 2 * c, 2);
    return (uint8_t)((v / 65535.f) * 255.f);
  }
  if (et == 261)
    return (uint8_t)(srgbToLinearGlm(texel[c] / 255.f) * 255.f);
  return texel[c];
}

// the texture unit's normalised-float read of 8-bit texels: point reads
// b / 255; linear filters the bytes as integers, the weighted sum F (weights
// summing to 256) scaled to a 16-bit normalised value
// round-half-up(F * 257 / 256) and read as that / 65535
float unorm8Point(int b)
{
  return (float)((double)b / 255.0);
}

float unorm8Linear(int64_t F)
{
  const int64_t r16 = (F * 257 + 128) >> 8;
  return (float)((double)r16 / 65535.0);
}

V4 texSample(const OrcSampler &sm, int ndim, const float tc[3])
{
  int i0[3] = {0, 0, 0}, i1[3] = {0, 0, 0}, w[3] = {0, 0, 0};
  for (int k = 0; k < ndim; k++)
    hwTap(tc[k], sm.dims[k], sm.wrap[k], sm.filter != 0, i0[k], i1[k], w[k]);
  if (sm.image8) {
    auto at8 = [&](int x, int y, int z, int c) {
      return (int)sm.image8[4 * (((size_t)z * sm.dims[1] + y) * sm.dims[0] + x) + c];
    };
    float out[4];
    if (sm.filter == 0) {
      for (int c = 0; c < 4; c++)
        out[c] = unorm8Point(at8(i0[0], i0[1], i0[2], c));
    } else {
      int cw[8];
      hwCornerWeights(ndim, w, cw);
      for (int c = 0; c < 4; c++) {
        int64_t F = 0;
        for (int q = 0; q < 8; q++)
          if (cw[q])
            F += (int64_t)cw[q]
                * at8((q & 1) ? i1[0] : i0[0], (q & 2) ? i1[1] : i0[1], (q & 4) ? i1[2] : i0[2], c);
        out[c] = unorm8Linear(F);
      }
    }
    return {out[0], out[1], out[2], out[3]};
  }
  auto at = [&](int x, int y, int z, int c) {
    return sm.image[4 * (((size_t)z * sm.dims[1] + y) * sm.dims[0] + x) + c];
  };
  if (sm.filter == 0)
    return {at(i0[0], i0[1], i0[2], 0), at(i0[0], i0[1], i0[2], 1), at(i0[0], i0[1], i0[2], 2),
        at(i0[0], i0[1], i0[2], 3)};
  int cw[8];
  hwCornerWeights(ndim, w, cw);
  float out[4];
  for (int c = 0; c < 4; c++) {
    ExactSum sum;
    for (int q = 0; q < 8; q++)
      if (cw[q])
        sum.add((double)cw[q] * (1.0 / 256.0)
            * (double)at((q & 1) ? i1[0] : i0[0], (q & 2) ? i1[1] : i0[1],
                (q & 4) ? i1[2] : i0[2], c));
    out[c] = sum.toFloatTiesAway();
  }
  return {out[0], out[1], out[2], out[3]};
}

// glm mat4 * vec4 (pairwise sums of the column products) + offset
V4 affine4(const float *m, V4 v, const float *o)
{
  float r[4];
  for (int i = 0; i < 4; i++)
    r[i] = (m[i] * v.x + m[4 + i] * v.y) + (m[8 + i] * v.z + m[12 + i] * v.w);
  return {r[0] + o[0], r[1] + o[1], r[2] + o[2], r[3] + o[3]};
}

// evaluateSampler (gpu/evalMaterialParameters.h:291-334)
V4 evaluateSampler(const SceneCtx &S, const SHit &sh, const OrcSampler &sm)
{
  V4 r{0.f, 0.f, 0.f, 1.f};
  const V4 tc = affine4(sm.inT, readAttribute(S, sh, sm.attribute), sm.inO);
  const float t3[3] = {tc.x, tc.y, tc.z};
  if (sm.type >= 1 && sm.type <= 3 && (sm.image || sm.image8))
    r = texSample(sm, sm.type, t3);
  else if (sm.type == 5)
    r = attrValue(sm.prim, sh.prim + sm.primOffset, r);
  else if (sm.type == 4)
    r = tc;
  return affine4(sm.outT, r, sm.outO);
}

V4 materialParam(const SceneCtx &S, const SHit &sh, int src, V4 value, const OrcSampler *sm)
{
  switch (src) {
  case 0:
    return value;
  case 10:
    return evaluateSampler(S, sh, *sm);
  case 1:
  case 2:
  case 3:
  case 4:
    return readAttribute(S, sh, src - 1);
  case 5:
    return readAttribute(S, sh, 4);
  case 6:
  case 8:
    return {sh.P.x, sh.P.y, sh.P.z, 1.f};
  case 7:
  case 9:
    return {sh.Ns.x, sh.Ns.y, sh.Ns.z, 1.f};
  default:
    return {0.f, 0.f, 0.f, 0.f};
  }
}

struct Matte
{
  V3 base;
  float opacity;
  int type; // 0 matte, 1 physicallyBased
  float metallic, roughness, ior;
};

// the material's init callable (MatteShader_ptx.cu:38-49,
// PhysicallyBasedShader_ptx.cu:41-58)
Matte matteAt(const SceneCtx &S, const SHit &sh)
{
  const OrcSurface &s = S.sc->surfaces[sh.surface];
  Matte m;
  m.type = s.materialType;
  m.ior = s.ior;
  m.metallic = m.roughness = 0.f;
  if (s.materialType == 1) {
    m.metallic = materialParam(S, sh, s.metallicSrc, {s.metallic, 0.f, 0.f, 1.f},
        &s.metallicSampler).x;
    m.roughness = materialParam(S, sh, s.roughnessSrc, {s.roughness, 0.f, 0.f, 1.f},
        &s.roughnessSampler).x;
  }
  float op;
  if (s.colorSrc == 0 && s.opacitySrc == 0) {
    m.base = ld3(s.color, 0);
    op = s.colorW * s.opacity;
  } else {
    const V4 c = materialParam(
        S, sh, s.colorSrc, {s.color[0], s.color[1], s.color[2], s.colorW}, &s.colorSampler);
    const float o =
        materialParam(S, sh, s.opacitySrc, {s.opacity, 0.f, 0.f, 1.f}, &s.opacitySampler).x;
    m.base = v3(c.x, c.y, c.z);
    op = c.w * o;
  }
  m.opacity = s.alphaMode == 0 ? 1.f : (s.alphaMode == 1 ? op : (op < s.cutoff ? 0.f : 1.f));
  return m;
}

// --- lights (gpu/sampleLight.h) and material evaluation ------------------

struct LightSample
{
  V3 radiance, dir;
  float dist, pdf;
};

// the HDRI texture: float4 texels (rgb, 1), linear filtering, normalised
// coordinates, x repeat, y clamp (HDRI.cu:121-122), as the texture unit
// filters (texSample)
V3 hdriTexel(const OrcLight &L, float u, float v)
{
  const int W = L.hdriW, H = L.hdriH;
  int x0, x1, y0, y1, w[3] = {0, 0, 0};
  hwTap(u, W, 1, 1, x0, x1, w[0]);
  hwTap(v, H, 0, 1, y0, y1, w[1]);
  int cw[8];
  hwCornerWeights(2, w, cw);
  float out[3];
  for (int c = 0; c < 3; c++) {
    auto at = [&](int x, int y) { return L.hdri[3 * ((size_t)y * W + x) + c]; };
    ExactSum sum;
    const float t[4] = {at(x0, y0), at(x1, y0), at(x0, y1), at(x1, y1)};
    for (int q = 0; q < 4; q++)
      if (cw[q])
        sum.add((double)cw[q] * (1.0 / 256.0) * (double)t[q]);
    out[c] = sum.toFloatTiesAway();
  }
  return v3(out[0], out[1], out[2]);
}

// sampleHDRI(ld, rayDir) (gpu_util.h:275-288)
V3 hdriRadiance(const SceneCtx &S, int li, V3 dir)
{
  const OrcLight &L = S.sc->lights[li];
  const float *R = S.hdri[li].rot;
  const V3 d = v3(std::fma(R[2], dir.z, std::fma(R[1], dir.y, R[0] * dir.x)),
      std::fma(R[5], dir.z, std::fma(R[4], dir.y, R[3] * dir.x)),
      std::fma(R[8], dir.z, std::fma(R[7], dir.y, R[6] * dir.x)));
  float theta, phi;
  sphericalCoordsFromDirection(d, theta, phi);
  return hdriTexel(L, phi * (1.f / (2.f * (float)M_PI)), theta * (1.f / (float)M_PI));
}

// the background image as the device stages it (acquireCUDAArrayUint8,
// utility/CudaImageTexture.cpp:43-93): RGBA8, float components truncated
// from c * 255 (clamped), sRGB bytes (alpha too) linearised, alpha 255 for
// three channels
uint8_t bgTexel(const OrcRenderer &R, size_t i, int c)
{
  const int nc = R.bgType == 242 ? 3 : 4;
  if (c >= nc)
    return 255;
  if (R.bgType == 242 || R.bgType == 243) {
    const float s = ((const float *)R.bgImage)[i * nc + c] * 255.f;
    return (uint8_t)(s >= 255.f ? 255.f : (s > 0.f ? s : 0.f));
  }
  return stageByte(R.bgType, (const uint8_t *)R.bgImage + i * 4, c);
}

// normalised-float reads of the RGBA8 image: linear, clamped, normalised
// coordinates. The texture unit filters 8-bit normalised texels as
// integers: the weighted sum F of the bytes (weights summing to 256) is
// scaled to a 16-bit normalised value R = round-half-up(F * 257 / 256) and
// read as R / 65535.
V4 bgImageAt(const OrcRenderer &R, float u, float v)
{
  const int W = R.bgW, H = R.bgH;
  int x0, x1, y0, y1, w[3] = {0, 0, 0};
  hwTap(u, W, 0, 1, x0, x1, w[0]);
  hwTap(v, H, 0, 1, y0, y1, w[1]);
  int cw[8];
  hwCornerWeights(2, w, cw);
  float out[4];
  for (int c = 0; c < 4; c++) {
    auto at = [&](int x, int y) { return (int64_t)bgTexel(R, (size_t)y * W + x, c); };
    const int64_t F = cw[0] * at(x0, y0) + cw[1] * at(x1, y0) + cw[2] * at(x0, y1)
        + cw[3] * at(x1, y1);
    out[c] = unorm8Linear(F);
  }
  return {out[0], out[1], out[2], out[3]};
}

// getBackground (gpu_util.h:290-307): a visible HDRI light, else the
// background image at loc, else the colour
V4 backgroundOf(const Ctx &C, V3 dir, float lx, float ly)
{
  const SceneCtx &S = *C.S;
  if (S.hdriIndex >= 0 && S.sc->lights[S.hdriIndex].hdriVisible) {
    const V3 r = hdriRadiance(S, S.hdriIndex, dir);
    return {r.x, r.y, r.z, 1.f};
  }
  if (C.R->bgImage && C.R->bgW > 0 && C.R->bgH > 0)
    return bgImageAt(*C.R, lx, ly);
  return {C.R->background[0], C.R->background[1], C.R->background[2], C.R->background[3]};
}

// cub::LowerBound: the first entry not below u
int lowerBound(const float *cdf, int n, float u)
{
  int lo = 0, count = n;
  while (count > 0) {
    const int half = count >> 1;
    if (cdf[lo + half] < u) {
      lo += half + 1;
      count -= half + 1;
    } else {
      count = half;
    }
  }
  return lo;
}

// sampleHDRILight (sampleLight.h:110-149)
LightSample sampleHDRILight(const SceneCtx &S, int li, Stream &rs)
{
  const OrcLight &L = S.sc->lights[li];
  const HdriPre &hp = S.hdri[li];
  const int W = L.hdriW, H = L.hdriH;
  const int y = lowerBound(hp.marginal.data(), H, uniform(rs));
  const int x = lowerBound(hp.conditional.data() + (size_t)std::min(y, H - 1) * W, W, uniform(rs));
  const float u = std::min(std::max(((float)x + 0.5f) / (float)W, 0.f), 1.f);
  const float v = std::min(std::max(((float)y + 0.5f) / (float)H, 0.f), 1.f);
  const float theta = (float)M_PI * v, phi = (float)M_PI * (2.f * u);
  const V3 rad = hdriTexel(L, u, v);
  LightSample ls;
  ls.pdf = (rad.x * 0.2126f + rad.y * 0.7152f + rad.z * 0.0722f) * hp.pdfWeight;
  const float st = std::sin(theta);
  const V3 sd = v3(st * std::cos(phi), st * std::sin(phi), std::cos(theta));
  const float *R = hp.rot;
  ls.dir = v3(std::fma(sd.z, R[6], std::fma(sd.y, R[3], sd.x * R[0])),
      std::fma(sd.z, R[7], std::fma(sd.y, R[4], sd.x * R[1])),
      std::fma(sd.z, R[8], std::fma(sd.y, R[5], sd.x * R[2])));
  ls.dist = 1e20f;
  ls.radiance = rad * L.hdriScale;
  return ls;
}

// sampleLight (sampleLight.h:60-173); lights are given in world space
LightSample sampleLight(const SceneCtx &S, int li, V3 hitP, Stream &rs)
{
  const OrcLight &L = S.sc->lights[li];
  LightSample ls;
  ls.pdf = 1.f;
  if (L.type == 0) {
    ls.dir = -1.f * normalize(ld3(L.direction, 0));
    ls.dist = INFINITY;
    ls.radiance = ld3(L.radiance, 0);
  } else if (L.type == 1) {
    const V3 d = ld3(L.position, 0) - hitP;
    ls.dist = std::sqrt(dot(d, d));
    ls.dir = normalize(d);
    ls.radiance = ld3(L.radiance, 0);
  } else if (L.type == 2) {
    // the distance is taken of the normalised direction (sampleLight.h:87-88)
    ls.dir = normalize(ld3(L.position, 0) - hitP);
    ls.dist = std::sqrt(dot(ls.dir, ls.dir));
    float spot = dot(normalize(ld3(L.direction, 0)), -1.f * ls.dir);
    if (spot < L.cosOuter)
      spot = 0.f;
    else if (spot > L.cosInner)
      spot = 1.f;
    else {
      spot = (spot - L.cosOuter) / (L.cosInner - L.cosOuter);
      spot = spot * spot * (3.f - 2.f * spot);
    }
    ls.radiance = ld3(L.radiance, 0) * spot;
  } else {
    ls = sampleHDRILight(S, li, rs);
  }
  return ls;
}

inline float heavisideF(float x)
{
  return x < 0.f ? 0.f : 1.f;
}

// shadeSurface (MatteShader_ptx.cu:72-80, PhysicallyBasedShader_ptx.cu:98-149)
V3 shadeMaterial(const Matte &m, V3 Ns, const LightSample &ls, V3 outgoing)
{
  if (m.type != 1) {
    const float NdotL = std::max(0.f, dot(Ns, ls.dir));
    return m.base * (float)M_1_PI * NdotL * ls.radiance / ls.pdf;
  }
  const V3 H = normalize(ls.dir + outgoing);
  const float NdotH = dot(Ns, H), NdotL = dot(Ns, ls.dir), NdotV = dot(Ns, outgoing);
  const float VdotH = dot(outgoing, H), LdotH = dot(ls.dir, H);
  const float q = (1.f - m.ior) / (1.f + m.ior);
  const float f0s = q * q;
  const V3 f0 = v3(f0s, f0s, f0s) * (1.f - m.metallic) + m.base * m.metallic;
  const float e = 1.f - std::fabs(VdotH);
  const float fw = e * e * e * e * e;
  const V3 F = f0 + (v3(1.f, 1.f, 1.f) - f0) * fw;
  const V3 diffuseColor = m.base * (1.f - m.metallic) + v3(0.f, 0.f, 0.f) * m.metallic;
  const V3 diffuseBRDF =
      (v3(1.f, 1.f, 1.f) - F) * (float)M_1_PI * diffuseColor * std::max(0.f, NdotL);
  const float alpha = (m.roughness * m.roughness) * m.opacity;
  const float a2 = alpha * alpha;
  const float dd = NdotH * NdotH * (a2 - 1.f) + 1.f;
  const float D = (a2 * heavisideF(NdotH)) / ((float)M_PI * (dd * dd));
  const float G = ((2.f * std::fabs(NdotL) * heavisideF(LdotH))
                      / (std::fabs(NdotL) + std::sqrt(a2 + (1.f - a2) * NdotL * NdotL)))
      * ((2.f * std::fabs(NdotV) * heavisideF(VdotH))
          / (std::fabs(NdotV) + std::sqrt(a2 + (1.f - a2) * NdotV * NdotV)));
  const float denom = 4.f * std::fabs(NdotV) * std::fabs(NdotL);
  const V3 spec = denom != 0.f ? (F * D * G) / denom : v3(0.f, 0.f, 0.f);
  return (diffuseBRDF + spec) * ls.radiance / ls.pdf;
}

V3 onbMul(V3 n, V3 s);

// nextRay (MatteShader_ptx.cu:51-57: none; PhysicallyBasedShader_ptx.cu:
// 60-84 with uniformSampleCone gpu_math.h:299-312)
bool nextRay(const Matte &m, V3 Ns, V3 rayDir, Stream &rs, V3 &dir, V3 &weight)
{
  if (m.type != 1) {
    dir = v3(0.f, 0.f, 0.f);
    weight = v3(0.f, 0.f, 0.f);
    return false;
  }
  const V3 refl = rayDir - 2.f * dot(rayDir, Ns) * Ns;
  const float cosThetaMax = 1.f - m.roughness * m.roughness;
  const float s0 = uniform(rs), s1 = uniform(rs), s2 = uniform(rs);
  const V3 cone = uniformSampleCone(cosThetaMax, s0, s1, s2);
  dir = onbMul(normalize(refl), cone);
  weight = m.base * m.metallic;
  return true;
}

// shadeSurface (renderer/DirectLight_ptx.cu:73-224): ambient, every light
// (sampleLight.h:60-173) with surface and volume attenuation, AO, then the
// bounce rays of the material's nextRay up to maxRayDepth
void shadeDL(Ctx &C, const VolCtx &VC, Stream &rs, const Ray &ray, const SHit &hit,
    int px, int py, float out[4])
{
  const OrcRenderer &R = *C.R;
  const SceneCtx &S = *C.S;
  V3 shadePoint = hit.P + (hit.eps * hit.Ns);
  const float aoFactor = R.ambientSamples > 0
      ? computeAO(C, rs, hit, R.occlusionDistance, R.ambientSamples)
      : 1.f;
  V3 contrib = v3(0, 0, 0);
  Matte mt = matteAt(S, hit);
  const float opacity = mt.opacity;
  if (R.ambientRadiance > 0.f)
    contrib = ld3(R.ambientColor, 0) * R.ambientRadiance * mt.base;
  const float invRate = 1.f / std::min(std::max(R.volumeSamplingRate, 1e-3f), 10.f);
  for (int l = 0; l < S.sc->numLights; l++) {
    const LightSample ls = sampleLight(S, l, hit.P, rs);
    if (ls.pdf == 0.f)
      continue;
    const float so = 1.f - surfaceAttenuation(C, shadePoint, ls.dir, 0.f, ls.dist);
    const float vo = 1.f
        - volumeAttenuation(C, VC, rs, shadePoint, ls.dir, 0.f, ls.dist, invRate);
    const float att = so * vo;
    const V3 tl = shadeMaterial(mt, hit.Ns, ls, -1.f * ray.dir);
    if (std::isnan(tl.x) || std::isnan(tl.y) || std::isnan(tl.z))
      continue;
    contrib = contrib + tl * att;
  }
  contrib = contrib * aoFactor;
  V3 weight = v3(1.f, 1.f, 1.f);
  V3 bounceDir = ray.dir, Ns = hit.Ns;
  for (int depth = 0; depth < R.maxRayDepth; depth++) {
    V3 nd, nw;
    nextRay(mt, Ns, bounceDir, rs, nd, nw);
    if (!(std::fabs(nd.x) > 1.0e-8f && std::fabs(nd.y) > 1.0e-8f && std::fabs(nd.z) > 1.0e-8f))
      break;
    weight = weight * nw;
    if (weight.x < 1.0e-12f && weight.y < 1.0e-12f && weight.z < 1.0e-12f)
      break;
    Ray br;
    br.org = shadePoint;
    br.dir = normalize(nd);
    br.tmin = 0.f;
    br.tmax = 3.402823466e+38f;
    HitRec h;
    float unused;
    C.rays++;
    const bool found = trace<0>(S, br.org, br.dir, br.tmin, br.tmax,
        R.cullTriangleBackfaces != 0, true, h, unused);
    bounceDir = br.dir;
    if (found) {
      const SHit bh = populate(S, br, h);
      shadePoint = bh.P + (bh.eps * bh.Ns);
      LightSample ls;
      if (S.hdriIndex >= 0 && S.sc->lights[S.hdriIndex].hdriVisible) {
        ls = sampleHDRILight(S, S.hdriIndex, rs);
      } else {
        // the bounce reads the background at the pixel position
        const V4 bg = backgroundOf(C, br.dir, (float)px, (float)py);
        ls.radiance = v3(bg.x, bg.y, bg.z);
        ls.dir = br.dir;
        ls.dist = 1.f;
        ls.pdf = 1.f;
      }
      mt = matteAt(S, bh);
      Ns = bh.Ns;
      const V3 c = shadeMaterial(mt, bh.Ns, ls, -1.f * br.dir);
      if (std::isnan(c.x) || std::isnan(c.y) || std::isnan(c.z))
        break;
      contrib = contrib + c * weight;
    } else {
      const V4 bg = backgroundOf(C, br.dir, (float)px, (float)py);
      contrib = contrib + v3(bg.x, bg.y, bg.z) * weight;
      break;
    }
  }
  out[0] = contrib.x;
  out[1] = contrib.y;
  out[2] = contrib.z;
  out[3] = opacity;
}

struct Sample
{
  V3 color;
  float opacity;
  float depth;
  uint32_t prim, obj, inst;
  V3 albedo, normal; // accumResults' albedo and normal arguments
};

// default/directLight, raycast and ao raygen bodies
// (DirectLight_ptx.cu:294-418, Raycast_ptx.cu:60-179,
// AmbientOcclusion_ptx.cu:86-220)
Sample integrate(Ctx &C, const VolCtx &VC, const CamPre &cam, Stream &rs, int px, int py,
    float invW, float invH)
{
  const OrcRenderer &R = *C.R;
  const int rt = R.type;
  const float invRate = 1.f / std::min(std::max(R.volumeSamplingRate, 1e-3f), 10.f);
  float scr[2];
  Ray ray = primaryRay(cam, rs, px, py, invW, invH, rt == 1, scr);
  const float tmax = ray.tmax;
  V3 outC = v3(0, 0, 0);
  V3 outN = ray.dir; // outputNormal: the ray direction on a miss
  float outO = 0.f, depth = 1e30f;
  uint32_t prim = ~0u, obj = ~0u, inst = ~0u;
  bool first = true;
  while (outO < 0.99f) {
    ray.tmax = tmax;
    HitRec h;
    float unused;
    C.rays++;
    const bool found = trace<0>(*C.S, ray.org, ray.dir, ray.tmin, ray.tmax,
        R.cullTriangleBackfaces != 0, true, h, unused);
    V3 color = v3(0, 0, 0);
    float opacity = 0.f;
    if (found) {
      const SHit sh = populate(*C.S, ray, h);
      uint32_t vo = ~0u, vi = ~0u;
      const float vDepth = rayMarchAllVolumes(
          C, VC, rs, ray.org, ray.dir, ray.tmin, sh.t, invRate, color, opacity, vo, vi);
      if (first) {
        if (vDepth < sh.t) {
          outN = -1.f * ray.dir;
          depth = vDepth;
          prim = 0;
          obj = vo;
          inst = vi;
        } else {
          // directLight reports Ns, raycast and ao Ng
          // (DirectLight_ptx.cu:351, Raycast_ptx.cu:114,
          // AmbientOcclusion_ptx.cu:144)
          outN = rt == 0 ? sh.Ns : sh.Ng;
          depth = sh.t;
          prim = sh.primId;
          obj = sh.objId;
          inst = sh.instId;
        }
        first = false;
      }
      const OrcSurface &s = C.S->sc->surfaces[sh.surface];
      if (rt == 0) {
        float sr[4];
        shadeDL(C, VC, rs, ray, sh, px, py, sr);
        const V3 srgb = v3(sr[0], sr[1], sr[2]);
        if (std::isnan(sr[0]) || std::isnan(sr[1]) || std::isnan(sr[2])) {
          color = v3(0, 0, 0);
          opacity = 0.f;
        } else {
          color = srgb;
          opacity = sr[3];
        }
        color = color + srgb * (1.f - opacity);
        opacity += sr[3] * (1.f - opacity);
      } else if (rt == 1) {
        const V3 lighting = std::fabs(dot(ray.dir, sh.Ns)) * ld3(R.ambientColor, 0);
        const Matte mt = matteAt(*C.S, sh);
        color = color + (mt.base * lighting) * (1.f - opacity);
        opacity += mt.opacity * (1.f - opacity);
      } else {
        const float ao = R.ambientSamples > 0
            ? computeAO(C, rs, sh, R.occlusionDistance, R.ambientSamples)
            : 1.f;
        const V3 lighting = ao * R.ambientRadiance * ld3(R.ambientColor, 0);
        const Matte mt = matteAt(*C.S, sh);
        color = color + (mt.base * lighting) * (1.f - opacity);
        opacity += mt.opacity * (1.f - opacity);
      }
      color = color * opacity;
      outC = outC + color * (1.f - outO);
      outO += opacity * (1.f - outO);
      ray.tmin = sh.t + sh.eps;
    } else {
      uint32_t vo = ~0u, vi = ~0u;
      const float vd = rayMarchAllVolumes(
          C, VC, rs, ray.org, ray.dir, ray.tmin, ray.tmax, invRate, color, opacity, vo, vi);
      if (first) {
        depth = std::min(depth, vd);
        prim = 0;
        obj = vo;
        inst = vi;
      }
      color = color * opacity;
      const V4 bg = backgroundOf(C, ray.dir, scr[0], scr[1]);
      color = color + v3(bg.x, bg.y, bg.z) * (1.f - opacity);
      opacity += bg.w * (1.f - opacity);
      outC = outC + color * (1.f - outO);
      outO += opacity * (1.f - outO);
      break;
    }
  }
  return Sample{outC, outO, depth, prim, obj, inst, outC, outN};
}

// --- output (gpu/gpu_util.h:321-443) ---------------------------------------

inline void tonemap(float v[4])
{
  const float d = 1.f + std::max(0.f, std::max(v[0], std::max(v[1], v[2])));
  v[0] /= d;
  v[1] /= d;
  v[2] /= d;
}

inline float srgb(float c)
{
  const float x = std::min(std::max(c, 0.f), 1.f);
  return x < 0.0031308f ? x * 12.92f : std::pow(x, 0.41666f) * 1.055f - 0.055f;
}

inline uint32_t pack8(float r, float g, float b, float a)
{
  auto q = [](float v) {
    return (uint32_t)std::round(std::min(std::max(v, 0.f), 1.f) * 255.f);
  };
  return q(r) | (q(g) << 8) | (q(b) << 16) | (q(a) << 24);
}

void writeColor(const OrcFrame &F, const float acc[4], size_t idx, int offs)
{
  const float n = (float)(F.frameID + offs + 1);
  float c[4] = {acc[0] / n, acc[1] / n, acc[2] / n, acc[3] / n};
  const float d = std::max(1e-12f, 1.f - std::max(c[0], std::max(c[1], c[2])));
  c[0] /= d;
  c[1] /= d;
  c[2] /= d;
  if (F.colorFormat == 0)
    ((uint32_t *)F.color)[idx] = pack8(srgb(c[0]), srgb(c[1]), srgb(c[2]), c[3]);
  else if (F.colorFormat == 1)
    ((uint32_t *)F.color)[idx] = pack8(c[0], c[1], c[2], c[3]);
  else
    std::memcpy((float *)F.color + 4 * idx, c, 16);
}

// computeOrthonormalBasis (gpu_util.h:210-222) applied to s
V3 onb(V3 n, V3 s)
{
  const float sign = n.z >= 0.f ? 1.f : -1.f;
  const float a = -1.f / (sign + n.z);
  const float b = n.x * n.y * a;
  const V3 u = v3(1.f + sign * n.x * n.x * a, sign * b, -sign * n.x);
  const V3 v = v3(b, sign + n.y * n.y * a, -n.y);
  return u * s.x + v * s.y + n * s.z;
}

// diffuse path tracer raygen (renderer/DiffusePathTracer_ptx.cu:82-215),
// surfaces only; the path state persists across the pixel's samples as in
// the reference
struct PathState
{
  int depth;
  V3 Lw;
};

// computeOrthonormalBasis (gpu/gpu_util.h:210-222, Pixar ONB) applied to s
V3 onbMul(V3 n, V3 s)
{
  const float sign = n.z >= 0.f ? 1.f : -1.f;
  const float a = -1.f / (sign + n.z);
  const float b = n.x * n.y * a;
  const V3 u = v3(1.f + sign * n.x * n.x * a, sign * b, -sign * n.x);
  const V3 w = v3(b, sign + n.y * n.y * a, -n.y);
  return u * s.x + w * s.y + n * s.z;
}

// sampleUnitSphere (gpu/gpu_util.h:234-243)
V3 sampleUnitSphere(Stream &rs, V3 n)
{
  const float cost = 1.f - 2.f * uniform(rs);
  const float sint = std::sqrt(std::max(0.f, 1.f - cost * cost));
  const float phi = 2.f * (float)M_PI * uniform(rs);
  return onbMul(n, v3(sint * std::cos(phi), sint * std::sin(phi), -cost));
}

Sample integrateDPT(Ctx &C, const VolCtx &VC, const CamPre &cam, Stream &rs, int px, int py,
    float invW, float invH, PathState &pd)
{
  const OrcRenderer &R = *C.R;
  float scr[2];
  Ray ray = primaryRay(cam, rs, px, py, invW, invH, false, scr);
  const V4 bg4 = backgroundOf(C, ray.dir, scr[0], scr[1]);
  const V3 bg = v3(bg4.x, bg4.y, bg4.z);
  // outColor (the background) and the primary ray direction go to the
  // albedo and normal channels
  Sample out{bg, 1.f, ray.tmax, ~0u, ~0u, ~0u, bg, ray.dir};
  const bool hasVolumes = C.S->sc->numVolumes > 0;
  while (true) {
    HitRec h;
    float unused;
    C.rays++;
    const bool found = trace<0>(*C.S, ray.org, ray.dir, ray.tmin, ray.tmax,
        R.cullTriangleBackfaces != 0, false, h, unused);
    SHit sh{};
    if (found)
      sh = populate(*C.S, ray, h);
    V3 volumeColor = v3(0, 0, 0);
    float volumeOpacity = 0.f, Tr = 1.f;
    uint32_t vObj = ~0u, vInst = ~0u;
    const float tfar = found ? sh.t : ray.tmax;
    const float volumeDepth = hasVolumes
        ? sampleDistanceAllVolumes(C, VC, rs, ray.org, ray.dir, ray.tmin, tfar, volumeColor,
              volumeOpacity, Tr, vObj, vInst)
        : tfar;
    const bool volumeHit = Tr < 1.f && (!found || volumeDepth < sh.t);
    if (!found && !volumeHit)
      break;
    if (pd.depth++ >= R.maxDepth) {
      pd.Lw = v3(0, 0, 0);
      break;
    }
    V3 pos, albedo;
    if (!volumeHit) {
      pos = sh.P + (sh.eps * sh.Ng);
      albedo = matteAt(*C.S, sh).base;
    } else {
      pos = ray.org + volumeDepth * ray.dir;
      albedo = volumeColor;
    }
    pd.Lw = pd.Lw * albedo;
    const float P = cmax(pd.Lw);
    if (P < .2f) {
      if (uniform(rs) > P) {
        pd.Lw = v3(0, 0, 0);
        break;
      }
      pd.Lw = pd.Lw / P;
    }
    V3 sd;
    if (!volumeHit) {
      sd = randomDir(rs, sh.Ns);
      pd.Lw = pd.Lw * std::max(0.f, dot(sd, sh.Ng));
    } else {
      sd = sampleUnitSphere(rs, -1.f * ray.dir);
    }
    ray.org = pos;
    ray.dir = sd;
    ray.tmin = 0.f;
    ray.tmax = R.occlusionDistance;
  }
  const V3 Ld = v3(R.ambientRadiance, R.ambientRadiance, R.ambientRadiance);
  out.color = pd.depth ? pd.Lw * Ld : bg;
  return out;
}

} // namespace

// ===========================================================================
// C API
// ===========================================================================

extern "C" {

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
  philox(ctr, key, out);
}

void orc_philox_stream(
    uint64_t seed, uint64_t subsequence, uint64_t offset, int kind, int n, void *out)
{
  Stream s;
  s.init(seed, subsequence, offset);
  if (kind == 0) {
    for (int i = 0; i < n; i++)
      ((uint32_t *)out)[i] = s.next();
  } else if (kind == 1) {
    for (int i = 0; i < n; i++)
      ((float *)out)[i] = uniform(s);
  } else {
    for (int i = 0; i + 3 < n; i += 4)
      uniform4(s, (float *)out + i);
  }
}

void orc_tex1d(const float *table, int n, int comps, float coord, int round, float *out)
{
  tex1dLinear(table, n, comps, coord, round, out);
}

float orc_tex3d(const float *vox, const int dims[3], const float coord[3], int round)
{
  return tex3dLinear(vox, dims, coord[0], coord[1], coord[2], round);
}

void orc_tex_float4(const float *texels, int ndim, const int dims[3], int filter,
    const int wrap[3], const float coord[3], float out[4])
{
  OrcSampler sm{};
  sm.image = texels;
  for (int k = 0; k < 3; k++) {
    sm.dims[k] = k < ndim ? dims[k] : 1;
    sm.wrap[k] = k < ndim ? wrap[k] : 0;
  }
  sm.filter = filter;
  const V4 r = texSample(sm, ndim, coord);
  out[0] = r.x;
  out[1] = r.y;
  out[2] = r.z;
  out[3] = r.w;
}

void orc_tex_unorm8(const uint8_t *texels, int ndim, const int dims[3], int filter,
    const int wrap[3], const float coord[3], float out[4])
{
  OrcSampler sm{};
  sm.image8 = texels;
  for (int k = 0; k < 3; k++) {
    sm.dims[k] = k < ndim ? dims[k] : 1;
    sm.wrap[k] = k < ndim ? wrap[k] : 0;
  }
  sm.filter = filter;
  const V4 r = texSample(sm, ndim, coord);
  out[0] = r.x;
  out[1] = r.y;
  out[2] = r.z;
  out[3] = r.w;
}

// The texture unit's linear (or point) read of a single-channel 16-bit
// normalised texture (UFIXED16 scale 65535, FIXED16 scale 32767): the
// integer texels weighted as hwCornerWeights splits them (sum 256), the sum
// F rounded half up to F / 256 and read as that / scale. (The 8-bit rule,
// unorm8Linear, is this rule on the bytes widened to 16 bits as b * 257.)
float orc_tex_norm16(const int32_t *texels, int ndim, const int dims[3], int filter,
    const int wrap[3], const float coord[3], int scale)
{
  int d[3], i0[3] = {0, 0, 0}, i1[3] = {0, 0, 0}, w[3] = {0, 0, 0};
  for (int k = 0; k < 3; k++)
    d[k] = k < ndim ? dims[k] : 1;
  for (int k = 0; k < ndim; k++)
    hwTap(coord[k], d[k], wrap[k], filter != 0, i0[k], i1[k], w[k]);
  auto at = [&](int x, int y, int z) {
    return (int64_t)texels[((size_t)z * d[1] + y) * d[0] + x];
  };
  if (filter == 0)
    return (float)((double)at(i0[0], i0[1], i0[2]) / scale);
  int cw[8];
  hwCornerWeights(ndim, w, cw);
  int64_t F = 0;
  for (int q = 0; q < 8; q++)
    if (cw[q])
      F += cw[q] * at((q & 1) ? i1[0] : i0[0], (q & 2) ? i1[1] : i0[1], (q & 4) ? i1[2] : i0[2]);
  const int64_t r = (F + 128) >> 8; // floor(F / 256 + 1/2), negative F too
  return (float)((double)r / scale);
}

void orc_tex_rgba8(const uint8_t *texels, int w, int h, const float coord[2], float out[4])
{
  OrcRenderer R{};
  R.bgImage = texels;
  R.bgType = 260;
  R.bgW = w;
  R.bgH = h;
  const V4 r = bgImageAt(R, coord[0], coord[1]);
  out[0] = r.x;
  out[1] = r.y;
  out[2] = r.z;
  out[3] = r.w;
}

int orc_nvdb_sample(const uint8_t *grid, const float *xyz, int n, int fused, float *out)
{
  Nvdb g;
  if (!nvdbOpen(grid, g))
    return -1;
  for (int i = 0; i < n; i++)
    out[i] = nvdbSample(g, v3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]), fused);
  return 0;
}

// the two helpers above on n inputs (radius, s0, s1 -> x, y; dir -> theta,
// phi), for checking against the reference's gpu_math.h
void orc_uniform_sample_disk(const float *in3, int n, float *out2)
{
  for (int i = 0; i < n; i++)
    uniformSampleDisk(in3[3 * i], in3[3 * i + 1], in3[3 * i + 2], out2[2 * i], out2[2 * i + 1]);
}

void orc_uniform_sample_cone(const float *in4, int n, float *out3)
{
  for (int i = 0; i < n; i++) {
    const V3 r = uniformSampleCone(in4[4 * i], in4[4 * i + 1], in4[4 * i + 2], in4[4 * i + 3]);
    out3[3 * i] = r.x;
    out3[3 * i + 1] = r.y;
    out3[3 * i + 2] = r.z;
  }
}

// projectOnGrid (gpu/uniformGrid.h:43-50) of n points onto a dims grid
// over the box (lo xyz, hi xyz), axis by axis as the majorant grid builds
// use it
void orc_project_on_grid(const float *p3, int n, const int *dims3, const float *box6, int *out3)
{
  for (int i = 0; i < n; i++)
    for (int a = 0; a < 3; a++)
      out3[3 * i + a] = projectAxis(p3[3 * i + a], box6[a], box6[3 + a], dims3[a]);
}

// the structured field's texture coordinates (fieldCoord) of n points
void orc_field_coords(const float *origin3, const float *spacing3, const int *dims3,
    const float *p3, int n, float *out3)
{
  for (int i = 0; i < n; i++) {
    const V3 c = fieldCoord(origin3, spacing3, dims3, ld3(p3, i));
    out3[3 * i] = c.x;
    out3[3 * i + 1] = c.y;
    out3[3 * i + 2] = c.z;
  }
}

// intersectVolume's interval (scene/Intersectors_ptx.cu:248-274) for n
// local rays (org xyz, dir xyz, tmin, tmax) against box6: hit[i] 1 / 0 and,
// on a hit, the clamped [t0, t1]
void orc_volume_interval(const float *rays8, int n, const float *box6, int *hit, float *t01)
{
  const V3 blo = v3(box6[0], box6[1], box6[2]), bhi = v3(box6[3], box6[4], box6[5]);
  for (int i = 0; i < n; i++) {
    const float *r = rays8 + 8 * i;
    float t0 = 0.f, t1 = 0.f;
    hit[i] = volumeInterval(blo, bhi, v3(r[0], r[1], r[2]), v3(r[3], r[4], r[5]), r[6], r[7], t0, t1)
        ? 1
        : 0;
    t01[2 * i] = hit[i] ? t0 : 0.f;
    t01[2 * i + 1] = hit[i] ? t1 : 0.f;
  }
}

// Image1D/2D/3D::finalize's staging (sampler/Image2D.cpp:70-78 with
// transformToStagingBuffer{Float,Uint8}, utility/CudaImageTexture.cpp:76-111)
int orc_stage_image(int et, const void *texels, uint64_t n, float *outFloat, uint8_t *outBytes)
{
  int ch = 0;
  if (et >= 240 && et <= 243)
    ch = et - 239;
  else if (et == 221 || et == 223)
    ch = 1;
  else if (et == 260 || et == 261)
    ch = 4;
  if (!ch || (n && !texels))
    return -1;
  const uint8_t *src = (const uint8_t *)texels;
  if (et >= 240 && et <= 243) {
    if (!outFloat)
      return -1;
    for (uint64_t i = 0; i < n; i++) {
      float v[4] = {0.f, 0.f, 0.f, 1.f};
      std::memcpy(v, src + i * ch * 4, ch * 4);
      std::memcpy(outFloat + 4 * i, v, 16);
    }
    return 1;
  }
  if (!outBytes)
    return -1;
  const int bytes = et == 223 ? 2 : 1;
  for (uint64_t i = 0; i < n; i++)
    for (int c = 0; c < 4; c++)
      outBytes[4 * i + c] = c < ch ? stageByte(et, src + i * ch * bytes, c) : (c == 3 ? 255 : 0);
  return 0;
}

// Renderer::finalize's background staging (bgTexel) of n texels
int orc_stage_background(int et, const void *texels, uint64_t n, uint8_t *out)
{
  if (et != 242 && et != 243 && et != 260 && et != 261)
    return -1;
  OrcRenderer R{};
  R.bgImage = texels;
  R.bgType = et;
  for (uint64_t i = 0; i < n; i++)
    for (int c = 0; c < 4; c++)
      out[4 * i + c] = bgTexel(R, i, c);
  return 0;
}

// makePrimaryRay + cameraCreateRay (gpu/cameraCreateRay.h:38-81) for n
// samples (pixel x, pixel y, r0..r3) of a camera record (30 floats: region,
// pos, dir, dir_00, dir_du, dir_dv, scaledAperture, aspect, pos_00, pos_du,
// pos_dv; type 0 perspective, 1 orthographic) -> n x (org, dir, screen)
void orc_primary_rays(const float *cam,
    int type,
    const float *samples,
    int n,
    float invW,
    float invH,
    int centerPixel,
    float *out)
{
  CamPre c{};
  c.type = type;
  for (int i = 0; i < 4; i++)
    c.region[i] = cam[i];
  c.pos = ld3(cam + 4, 0);
  c.dir = ld3(cam + 7, 0);
  c.d00 = ld3(cam + 10, 0);
  c.du = ld3(cam + 13, 0);
  c.dv = ld3(cam + 16, 0);
  c.aperture = cam[19];
  c.aspect = cam[20];
  c.p00 = ld3(cam + 21, 0);
  c.pdu = ld3(cam + 24, 0);
  c.pdv = ld3(cam + 27, 0);
  for (int i = 0; i < n; i++) {
    const float *s = samples + 6 * i;
    float *o = out + 8 * i;
    const Ray r = primaryRayFrom(c, s + 2, (int)s[0], (int)s[1], invW, invH, centerPixel != 0, o + 6);
    o[0] = r.org.x;
    o[1] = r.org.y;
    o[2] = r.org.z;
    o[3] = r.dir.x;
    o[4] = r.dir.y;
    o[5] = r.dir.z;
  }
}

// dda3 (gpu/dda.h:43-122), the walk the delta-tracking march takes, for n
// rays (org xyz, dir xyz, tlo, thi) over a dims3 grid spanning box6: per
// visited cell its linear index and [t0, t1], at most maxCells per ray
int orc_dda_walk(const float *rays8,
    int n,
    const int *dims3,
    const float *box6,
    int maxCells,
    int *counts,
    long long *cells,
    float *t01)
{
  const V3 blo = v3(box6[0], box6[1], box6[2]), bhi = v3(box6[3], box6[4], box6[5]);
  int total = 0;
  for (int i = 0; i < n; i++) {
    const float *r = rays8 + 8 * i;
    int k = 0;
    dda3(v3(r[0], r[1], r[2]), v3(r[3], r[4], r[5]), r[6], r[7], dims3, blo, bhi,
        [&](size_t cell, float t0, float t1) {
          const size_t j = (size_t)i * maxCells + k;
          cells[j] = (long long)cell;
          t01[2 * j] = t0;
          t01[2 * j + 1] = t1;
          return ++k < maxCells;
        });
    counts[i] = k;
    total += k;
  }
  return total;
}

void orc_spherical_from_dir(const float *dir3, int n, float *out2)
{
  for (int i = 0; i < n; i++)
    sphericalCoordsFromDirection(
        v3(dir3[3 * i], dir3[3 * i + 1], dir3[3 * i + 2]), out2[2 * i], out2[2 * i + 1]);
}

// writeOutputColor (gpu/gpu_util.h:370-389) on n accumulated colours, as
// the frame writes them (format 0 sRGB rgba8, 1 linear rgba8)
void orc_write_colors(const float *accum, int n, int frameID, int format, uint32_t *out)
{
  OrcFrame F{};
  F.frameID = frameID;
  F.colorFormat = format;
  F.color = out;
  for (int i = 0; i < n; i++)
    writeColor(F, accum + 4 * i, (size_t)i, 0);
}

void orc_dpt_majorants(const OrcVolume *volume, int round, float *out)
{
  std::vector<float> m;
  dptMajorants(*volume, round, m);
  std::memcpy(out, m.data(), m.size() * sizeof(float));
}

// TransferFunction1D::discritizeTFData (TransferFunction1D.cpp:101-150) with
// generateLinearPositions / getInterpolatedValue (colorMapHelpers.h:43-73)
void orc_discretize_tf(const float *color, int nc, int cc, const float *opacity, int no,
    float lo, float hi, const float *uniformColor, float uniformOpacity, float *out)
{
  auto positions = [&](int n) {
    std::vector<float> p(n);
    p.front() = 0.f;
    p.back() = 1.f;
    const float w = 1.f / (float)(n - 1);
    for (int i = 1; i + 1 < n; i++)
      p[i] = p[i - 1] + w;
    for (auto &v : p)
      v = v * (hi - lo) + lo;
    return p;
  };
  auto pos01 = [](float v, float a, float b) {
    v = std::max(a, std::min(v, b));
    return (v - a) * (1.f / (b - a));
  };
  auto interp = [&](const float *vals, int comps, const std::vector<float> &ps, float p,
                    float *o) {
    for (size_t i = 0; i + 1 < ps.size(); i++) {
      const float a = pos01(ps[i], lo, hi), b = pos01(ps[i + 1], lo, hi);
      if (p >= a && p <= b) {
        const float t = pos01(p, a, b);
        for (int c = 0; c < comps; c++)
          o[c] = vals[i * comps + c] * (1.f - t) + vals[(i + 1) * comps + c] * t;
        return;
      }
    }
    const size_t k = p <= pos01(ps[0], lo, hi) ? 0 : ps.size() - 1;
    for (int c = 0; c < comps; c++)
      o[c] = vals[k * comps + c];
  };
  std::vector<float> cp, op;
  if (color && nc >= 2)
    cp = positions(nc);
  if (opacity && no >= 2)
    op = positions(no);
  for (int i = 0; i < 256; i++) {
    const float p = (float)i / 255.f;
    // the volume's uniform colour (TransferFunction1D.cpp:50-54) where no
    // colour array is set
    float c[4] = {1.f, 1.f, 1.f, 1.f};
    if (uniformColor)
      for (int k = 0; k < 4; k++)
        c[k] = uniformColor[k];
    if (!cp.empty()) {
      float v[4] = {0, 0, 0, 1};
      interp(color, cc, cp, p, v);
      c[0] = v[0];
      c[1] = v[1];
      c[2] = v[2];
      c[3] = cc == 4 ? v[3] : 1.f;
    }
    float o = uniformOpacity;
    if (!op.empty())
      interp(opacity, 1, op, p, &o);
    out[4 * i + 0] = c[0];
    out[4 * i + 1] = c[1];
    out[4 * i + 2] = c[2];
    out[4 * i + 3] = c[3] * o;
  }
}

struct OrcPrepared
{
  SceneCtx S;
  VolCtx VC;
};

void *orc_prepare(const OrcScene *scene)
{
  auto *P = new OrcPrepared();
  SceneCtx &S = P->S;
  S.sc = scene;
  const int ni = scene->numInstances;
  S.bvh.resize(ni);
  S.w2o.resize(ni);
  S.o2w.resize(ni);
  S.worldBox.resize(ni);
  // instances that share a surface range share one BVH build
  std::vector<int> which(ni, -1);
  std::vector<std::pair<int, int>> ranges;
  for (int i = 0; i < ni; i++) {
    const OrcInstance &in = scene->instances[i];
    std::memcpy(S.o2w[i].m, in.xfm, sizeof(in.xfm));
    S.w2o[i] = invert(in.xfm);
    const std::pair<int, int> r{in.firstSurface, in.numSurfaces};
    for (size_t j = 0; j < ranges.size(); j++)
      if (ranges[j] == r)
        which[i] = (int)j;
    if (which[i] < 0) {
      which[i] = (int)ranges.size();
      ranges.push_back(r);
    }
  }
  // hdri lights: CDF tables and rotation (HDRI.cu), the first is the world's
  S.hdri.resize(scene->numLights);
  for (int li = 0; li < scene->numLights; li++) {
    const OrcLight &L = scene->lights[li];
    if (L.type != 3 || !L.hdri || L.hdriW < 1 || L.hdriH < 1)
      continue;
    if (S.hdriIndex < 0)
      S.hdriIndex = li;
    HdriPre &hp = S.hdri[li];
    const int W = L.hdriW, H = L.hdriH;
    std::vector<float> lum((size_t)W * H), rowSums(H);
    for (int y = 0; y < H; y++) {
      const float sinTheta = std::sin((float)M_PI * ((float)y + 0.5f) / (float)H);
      for (int x = 0; x < W; x++) {
        const float *c = L.hdri + 3 * ((size_t)y * W + x);
        lum[(size_t)y * W + x] = sinTheta * (c[0] * 0.2126f + c[1] * 0.7152f + c[2] * 0.0722f);
      }
      float sum = 0.f;
      for (int x = 0; x < W; x++)
        sum += lum[(size_t)y * W + x];
      rowSums[y] = sum;
    }
    hp.marginal.resize(H);
    hp.conditional.resize((size_t)W * H);
    float acc = 0.f;
    for (int y = 0; y < H; y++)
      hp.marginal[y] = acc += rowSums[y];
    for (int y = 0; y < H; y++) {
      float r = 0.f;
      for (int x = 0; x < W; x++)
        hp.conditional[(size_t)y * W + x] = r += lum[(size_t)y * W + x];
    }
    const float total = hp.marginal[H - 1];
    hp.pdfWeight = total / (2.0f * (float)M_PI * (float)M_PI * (float)W * (float)H);
    for (int y = 0; y < H; y++)
      hp.marginal[y] = hp.marginal[y] / total;
    for (int y = 0; y < H; y++) {
      const float rt = hp.conditional[(size_t)y * W + W - 1];
      for (int x = 0; x < W; x++)
        hp.conditional[(size_t)y * W + x] = hp.conditional[(size_t)y * W + x] / rt;
    }
    const V3 up = -1.f * normalize(ld3(L.hdriUp, 0));
    const V3 forward = -1.f * normalize(cross(up, ld3(L.hdriDirection, 0)));
    const V3 right = normalize(cross(forward, up));
    const V3 rows[3] = {right, forward, up};
    for (int r = 0; r < 3; r++) {
      hp.rot[3 * r] = rows[r].x;
      hp.rot[3 * r + 1] = rows[r].y;
      hp.rot[3 * r + 2] = rows[r].z;
    }
  }
  S.unique.resize(ranges.size());
  for (size_t j = 0; j < ranges.size(); j++) {
    InstBVH &b = S.unique[j];
    for (int k = 0; k < ranges[j].second; k++) {
      const int si = ranges[j].first + k;
      for (uint32_t p = 0; p < scene->surfaces[si].numPrims; p++)
        b.prims.push_back(Prim{si, p});
    }
    buildBVH(scene, b);
  }
  for (int i = 0; i < ni; i++) {
    S.bvh[i] = &S.unique[which[i]];
    Box wb;
    if (!S.bvh[i]->nodes.empty()) {
      const Box &ob = S.bvh[i]->nodes[0].box;
      for (int c = 0; c < 8; c++)
        wb.ext(xPoint(S.o2w[i],
            v3((c & 1) ? ob.hi.x : ob.lo.x,
                (c & 2) ? ob.hi.y : ob.lo.y,
                (c & 4) ? ob.hi.z : ob.lo.z)));
    }
    S.worldBox[i] = wb;
  }
  for (int i = 0; i < scene->numVolumes; i++)
    P->VC.w2o.push_back(invert(scene->volumes[i].xfm));
  return P;
}

void orc_release(void *prepared)
{
  delete (OrcPrepared *)prepared;
}

int orc_render(const OrcScene *scene, const OrcCamera *camera, const OrcRenderer *renderer,
    OrcFrame *frame, int volumeMode, int texRound, int threads)
{
  void *p = orc_prepare(scene);
  const int rc =
      orc_render_prepared(p, camera, renderer, frame, volumeMode, texRound, threads);
  orc_release(p);
  return rc;
}

int orc_render_prepared(void *prepared, const OrcCamera *camera, const OrcRenderer *renderer,
    OrcFrame *frame, int volumeMode, int texRound, int threads)
{
  const SceneCtx &S = ((OrcPrepared *)prepared)->S;
  const VolCtx &VC = ((OrcPrepared *)prepared)->VC;
  const CamPre cam = camSetup(*camera);
  std::vector<std::vector<float>> dptMaj(S.sc->numVolumes);
  if (renderer->type == 3)
    for (int i = 0; i < S.sc->numVolumes; i++)
      dptMajorants(S.sc->volumes[i], texRound, dptMaj[i]);
  OrcFrame &F = *frame;
  const int W = F.width, H = F.height;
  const float invW = 1.f / (float)W, invH = 1.f / (float)H;
  // checkerboarding (createScreenSample.h:38-46): the launch covers every
  // other pixel in x and y, offset by the checkerboard id
  const int cb = F.checkerboardID;
  const int LW = cb >= 0 ? (W + 1) / 2 : W, LH = cb >= 0 ? (H + 1) / 2 : H;
  const int rb = std::max(0, F.rowBegin), re = std::min(LH, F.rowEnd);
  const int tilesX = (LW + 15) / 16, tilesY = (re - rb + 15) / 16;
  std::atomic<int> next{0};
  std::atomic<uint64_t> rays{0}, samples{0};
  auto worker = [&]() {
    Ctx C{&S, renderer, volumeMode, texRound, 0, 0, &dptMaj};
    while (true) {
      const int t = next.fetch_add(1);
      if (t >= tilesX * tilesY)
        break;
      const int tx = t % tilesX, ty = t / tilesX;
      for (int ly = rb + ty * 16; ly < std::min(re, rb + ty * 16 + 16); ly++)
        for (int lx = tx * 16; lx < std::min(LW, tx * 16 + 16); lx++) {
          const int x = cb < 0 ? lx : lx * 2 + (cb & 1);
          const int y = cb < 0 ? ly : ly * 2 + ((cb >> 1) & 1);
          if (x >= W || y >= H)
            continue;
          Stream rs;
          rs.init((uint64_t)(y * W + x), 0, (uint64_t)F.frameID * 512ull);
          const size_t idx = (size_t)y * W + x;
          float acc[4] = {F.accum[4 * idx], F.accum[4 * idx + 1], F.accum[4 * idx + 2],
              F.accum[4 * idx + 3]};
          float cur = F.depth ? F.depth[idx] : 0.f;
          const int iters = renderer->type == 1 ? 1 : std::max(renderer->pixelSamples, 1);
          PathState pd{0, v3(1, 1, 1)};
          for (int i = 0; i < iters; i++) {
            const Sample s = renderer->type == 3
                ? integrateDPT(C, VC, cam, rs, x, y, invW, invH, pd)
                : integrate(C, VC, cam, rs, x, y, invW, invH);
            float v[4] = {s.color.x, s.color.y, s.color.z, s.opacity};
            tonemap(v);
            for (int c = 0; c < 4; c++)
              acc[c] += v[c];
            if (F.albedo) {
              F.albedo[3 * idx] += s.albedo.x;
              F.albedo[3 * idx + 1] += s.albedo.y;
              F.albedo[3 * idx + 2] += s.albedo.z;
            }
            if (F.normal) {
              F.normal[3 * idx] += s.normal.x;
              F.normal[3 * idx + 1] += s.normal.y;
              F.normal[3 * idx + 2] += s.normal.z;
            }
            if (!F.depth || s.depth < cur) {
              cur = s.depth;
              if (F.depth)
                F.depth[idx] = cur;
              if (F.primId)
                F.primId[idx] = s.prim;
              if (F.objId)
                F.objId[idx] = s.obj;
              if (F.instId)
                F.instId[idx] = s.inst;
            }
            // accumResults (gpu_util.h:393-443): the output is written after
            // every sample; on the first checkerboard pass of a fresh frame
            // (sample frame id 0) it is also splatted to the 2x2 block's
            // three other pixels, which this pass does not render
            if (cb == 0 && F.frameID + i == 0) {
              if (x + 1 < W)
                writeColor(F, acc, idx + 1, i);
              if (y + 1 < H)
                writeColor(F, acc, idx + W, i);
              if (x + 1 < W && y + 1 < H)
                writeColor(F, acc, idx + W + 1, i);
            }
          }
          std::memcpy(F.accum + 4 * idx, acc, 16);
          writeColor(F, acc, idx, iters - 1);
        }
    }
    rays += C.rays;
    samples += C.samples;
  };
  int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
  nt = std::max(1, nt);
  std::vector<std::thread> pool;
  for (int i = 0; i < nt; i++)
    pool.emplace_back(worker);
  for (auto &t : pool)
    t.join();
  F.raysTraced = rays.load();
  F.volumeSamples = samples.load();
  return 0;
}

// ---------------------------------------------------------------------------
// BVH8 visit counter over libvrtx's node layout (80-byte nodes, 48-byte
// triangle records); closest-hit order as in the GPU traversal.
// ---------------------------------------------------------------------------

void orc_bvh8_count(const void *nodesV, const void *trisV, const float *rays, int numRays,
    uint64_t *nodeVisits, uint64_t *primTests, float *tHit)
{
  const uint8_t *nodes = (const uint8_t *)nodesV;
  const float *tris = (const float *)trisV;
  uint64_t nv = 0, pt = 0;
  for (int ri = 0; ri < numRays; ri++) {
    const V3 o = v3(rays[7 * ri], rays[7 * ri + 1], rays[7 * ri + 2]);
    const V3 d = v3(rays[7 * ri + 3], rays[7 * ri + 4], rays[7 * ri + 5]);
    float tmax = rays[7 * ri + 6];
    const RayPre r = prep(o, d);
    const uint32_t oct = (d.x < 0 ? 1u : 0u) | (d.y < 0 ? 2u : 0u) | (d.z < 0 ? 4u : 0u);
    struct G
    {
      uint32_t base, bits;
    };
    std::vector<G> stack;
    G cur{0, 0x80000000u}, tri{0, 0};
    while (true) {
      if (tri.bits) {
        while (tri.bits) {
          const int b = __builtin_ctz(tri.bits);
          tri.bits &= tri.bits - 1;
          const float *t = tris + 12 * (size_t)(tri.base + b);
          float th, u, v;
          bool fr;
          pt++;
          if (hitTriangle(r, v3(t[0], t[1], t[2]), v3(t[4], t[5], t[6]),
                  v3(t[8], t[9], t[10]), 0.f, tmax, th, u, v, fr))
            tmax = th;
        }
        continue;
      }
      if (cur.bits & 0xff000000u) {
        const uint32_t bit = __builtin_ctz(cur.bits >> 24);
        cur.bits &= ~(1u << (24 + bit));
        const uint32_t slot = bit ^ oct;
        const uint32_t idx = cur.base + __builtin_popcount(cur.bits & 0xffu & ((1u << slot) - 1u));
        if (cur.bits & 0xff000000u)
          stack.push_back(cur);
        nv++;
        const uint8_t *n = nodes + 80 * (size_t)idx;
        float p[3];
        std::memcpy(p, n, 12);
        const uint8_t ex = n[12], ey = n[13], ez = n[14], imask = n[15];
        uint32_t childBase, primBase;
        std::memcpy(&childBase, n + 16, 4);
        std::memcpy(&primBase, n + 20, 4);
        const uint8_t *meta = n + 24;
        const uint8_t *q = n + 32; // qlox, qloy, qloz, qhix, qhiy, qhiz
        auto sc = [](uint8_t e) {
          uint32_t b = (uint32_t)e << 23;
          float f;
          std::memcpy(&f, &b, 4);
          return f;
        };
        const float s[3] = {sc(ex), sc(ey), sc(ez)};
        uint32_t hits = 0;
        for (int c = 0; c < 8; c++) {
          if (!meta[c])
            continue;
          Box bb;
          bb.lo = v3(p[0] + q[c] * s[0], p[1] + q[8 + c] * s[1], p[2] + q[16 + c] * s[2]);
          bb.hi = v3(p[0] + q[24 + c] * s[0], p[1] + q[32 + c] * s[1], p[2] + q[40 + c] * s[2]);
          if (!hitBox(bb, r, 0.f, tmax))
            continue;
          if (imask & (1u << c))
            hits |= 1u << (24 + (c ^ oct));
          else
            hits |= (uint32_t)(meta[c] >> 5) << (meta[c] & 31);
        }
        cur = G{childBase, (hits & 0xff000000u) | imask};
        tri = G{primBase, hits & 0x00ffffffu};
        continue;
      }
      if (stack.empty())
        break;
      cur = stack.back();
      stack.pop_back();
    }
    if (tHit)
      tHit[ri] = tmax;
  }
  *nodeVisits = nv;
  *primTests = pt;
}

// ---------------------------------------------------------------------------
// differentiable marcher, FP64 (model stated next to vrtxDMForward)
// ---------------------------------------------------------------------------

void orc_dm(const OrcDMVolume *vol, const OrcDMView *view, double *image,
    const double *gradImage, double *gradDensity, double *gradTf, double *gradScale,
    int threads)
{
  const OrcDMVolume &v = *vol;
  const OrcDMView &w = *view;
  const int N = v.tfSize;
  const double ratio = v.step / v.unitDistance;
  const double logStop = std::log(1e-3);
  const int nt = std::max(1, threads > 0 ? threads : (int)std::thread::hardware_concurrency());
  std::vector<std::vector<double>> gD(gradDensity ? nt : 0), gT(gradTf ? nt : 0);
  std::vector<double> gS(nt, 0.0);
  const size_t nvox = (size_t)v.dims[0] * v.dims[1] * v.dims[2];
  std::atomic<int> nextRow{0};
  auto work = [&](int tid) {
    if (gradDensity)
      gD[tid].assign(nvox, 0.0);
    if (gradTf)
      gT[tid].assign((size_t)N * 4, 0.0);
    struct S
    {
      double s;
      int ix[3], st[3];
      double f[3];
      double c[4];
      int i0;
      double fr;
      double dxds;
    };
    std::vector<S> samples;
    while (true) {
      const int py = nextRow.fetch_add(1);
      if (py >= w.height)
        break;
      for (int px = 0; px < w.width; px++) {
        double d[3];
        for (int k = 0; k < 3; k++)
          d[k] = w.d00[k] + (px + 0.5) * w.du[k] + (py + 0.5) * w.dv[k];
        const double dl = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        for (int k = 0; k < 3; k++)
          d[k] /= dl;
        double t0 = 0.0, t1 = 1e300;
        for (int k = 0; k < 3; k++) {
          const double inv = 1.0 / d[k];
          double a = (0.0 - w.eye[k]) * inv, b = ((v.dims[k] - 1) - w.eye[k]) * inv;
          if (a > b)
            std::swap(a, b);
          t0 = std::max(t0, a);
          t1 = std::min(t1, b);
        }
        samples.clear();
        double logT = 0.0;
        double C[3] = {0, 0, 0};
        if (t0 < t1) {
          for (int k = 0;; k++) {
            const double t = t0 + (k + 0.5) * v.step;
            if (t > t1)
              break;
            S sm;
            size_t base = 0;
            for (int a = 0; a < 3; a++) {
              const int n = v.dims[a];
              const double p = w.eye[a] + t * d[a];
              if (n < 2) {
                sm.ix[a] = 0;
                sm.st[a] = 0;
                sm.f[a] = 0;
                continue;
              }
              const double c = std::min(std::max(p, 0.0), (double)(n - 1));
              sm.ix[a] = std::min((int)std::floor(c), n - 2);
              sm.st[a] = 1;
              sm.f[a] = c - sm.ix[a];
            }
            (void)base;
            double s = 0.0;
            for (int q = 0; q < 8; q++) {
              const int x = sm.ix[0] + ((q & 1) ? sm.st[0] : 0);
              const int y = sm.ix[1] + ((q & 2) ? sm.st[1] : 0);
              const int z = sm.ix[2] + ((q & 4) ? sm.st[2] : 0);
              const double ww = ((q & 1) ? sm.f[0] : 1 - sm.f[0])
                  * ((q & 2) ? sm.f[1] : 1 - sm.f[1]) * ((q & 4) ? sm.f[2] : 1 - sm.f[2]);
              s += ww * v.density[((size_t)z * v.dims[1] + y) * v.dims[0] + x];
            }
            sm.s = s;
            const double range = v.valueHi - v.valueLo;
            double u = (s - v.valueLo) / range;
            sm.dxds = (u > 0 && u < 1) ? (N - 1) / range : 0.0;
            u = std::min(std::max(u, 0.0), 1.0);
            const double x = u * (N - 1);
            sm.i0 = std::min((int)std::floor(x), N - 2);
            sm.fr = x - sm.i0;
            for (int c = 0; c < 4; c++)
              sm.c[c] = v.tf[4 * sm.i0 + c] + sm.fr * (v.tf[4 * (sm.i0 + 1) + c] - v.tf[4 * sm.i0 + c]);
            const double alpha = std::min(sm.c[3] * v.opacityScale, 0.999);
            const double sigma = ratio * std::log1p(-alpha);
            const double T = std::exp(logT);
            const double a = -std::expm1(sigma);
            for (int c = 0; c < 3; c++)
              C[c] += T * a * sm.c[c];
            logT += sigma;
            samples.push_back(sm);
            if (logT < logStop)
              break;
          }
        }
        const double Tend = std::exp(logT);
        const size_t pix = (size_t)py * w.width + px;
        for (int c = 0; c < 3; c++)
          image[3 * pix + c] = C[c] + Tend * w.background[c];
        if (!gradImage)
          continue;
        const double g[3] = {gradImage[3 * pix], gradImage[3 * pix + 1], gradImage[3 * pix + 2]};
        double Snext[3] = {Tend * w.background[0], Tend * w.background[1], Tend * w.background[2]};
        double lt = logT;
        double Tnext = Tend;
        for (int k = (int)samples.size() - 1; k >= 0; k--) {
          const S &sm = samples[k];
          const double araw = sm.c[3] * v.opacityScale;
          const double alpha = std::min(araw, 0.999);
          const double sigma = ratio * std::log1p(-alpha);
          lt -= sigma;
          const double Tk = std::exp(lt);
          const double a = -std::expm1(sigma);
          const double wk = Tk * a;
          double dSigma = 0.0;
          for (int c = 0; c < 3; c++)
            dSigma += g[c] * (Snext[c] - Tnext * sm.c[c]);
          for (int c = 0; c < 3; c++)
            Snext[c] += wk * sm.c[c];
          Tnext = Tk;
          const double dAlpha = araw < 0.999 ? dSigma * (-ratio / (1.0 - alpha)) : 0.0;
          const double dA = dAlpha * v.opacityScale;
          gS[tid] += dAlpha * sm.c[3];
          const double dc[3] = {wk * g[0], wk * g[1], wk * g[2]};
          if (gradTf) {
            double *e0 = gT[tid].data() + 4 * sm.i0;
            for (int c = 0; c < 3; c++) {
              e0[c] += (1 - sm.fr) * dc[c];
              e0[4 + c] += sm.fr * dc[c];
            }
            e0[3] += (1 - sm.fr) * dA;
            e0[7] += sm.fr * dA;
          }
          if (gradDensity && sm.dxds != 0.0) {
            const double *ea = v.tf + 4 * sm.i0, *eb = v.tf + 4 * (sm.i0 + 1);
            const double dval = dc[0] * (eb[0] - ea[0]) + dc[1] * (eb[1] - ea[1])
                + dc[2] * (eb[2] - ea[2]) + dA * (eb[3] - ea[3]);
            const double ds = dval * sm.dxds;
            for (int q = 0; q < 8; q++) {
              const int x = sm.ix[0] + ((q & 1) ? sm.st[0] : 0);
              const int y = sm.ix[1] + ((q & 2) ? sm.st[1] : 0);
              const int z = sm.ix[2] + ((q & 4) ? sm.st[2] : 0);
              const double ww = ((q & 1) ? sm.f[0] : 1 - sm.f[0])
                  * ((q & 2) ? sm.f[1] : 1 - sm.f[1]) * ((q & 4) ? sm.f[2] : 1 - sm.f[2]);
              gD[tid][((size_t)z * v.dims[1] + y) * v.dims[0] + x] += ww * ds;
            }
          }
        }
      }
    }
  };
  std::vector<std::thread> pool;
  for (int i = 0; i < nt; i++)
    pool.emplace_back(work, i);
  for (auto &t : pool)
    t.join();
  if (gradImage) {
    for (int i = 0; i < nt; i++) {
      if (gradDensity)
        for (size_t k = 0; k < nvox; k++)
          gradDensity[k] += gD[i][k];
      if (gradTf)
        for (int k = 0; k < 4 * N; k++)
          gradTf[k] += gT[i][k];
      if (gradScale)
        *gradScale += gS[i];
    }
  }
}

} // extern "C"
