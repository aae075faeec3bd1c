// Small float3 / box math shared by host C++ and device code.
//
// Operations are written out component-wise so the arithmetic a kernel does
// is visible at the call site (the reference gets the same operations from
// glm, e.g. glm::normalize = v * (1 / sqrt(dot(v, v)))).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define VD __host__ __device__ __forceinline__
#else
#define VD inline
#endif

namespace vrtx {

struct f3
{
  float x, y, z;
};

VD f3 mk3(float x, float y, float z)
{
  return f3{x, y, z};
}
VD f3 operator+(f3 a, f3 b)
{
  return {a.x + b.x, a.y + b.y, a.z + b.z};
}
VD f3 operator-(f3 a, f3 b)
{
  return {a.x - b.x, a.y - b.y, a.z - b.z};
}
VD f3 operator-(f3 a)
{
  return {-a.x, -a.y, -a.z};
}
VD f3 operator*(f3 a, f3 b)
{
  return {a.x * b.x, a.y * b.y, a.z * b.z};
}
VD f3 operator*(f3 a, float s)
{
  return {a.x * s, a.y * s, a.z * s};
}
VD f3 operator*(float s, f3 a)
{
  return {a.x * s, a.y * s, a.z * s};
}
VD f3 operator/(f3 a, float s)
{
  return {a.x / s, a.y / s, a.z / s};
}
VD f3 &operator+=(f3 &a, f3 b)
{
  a.x += b.x;
  a.y += b.y;
  a.z += b.z;
  return a;
}
VD f3 &operator*=(f3 &a, float s)
{
  a.x *= s;
  a.y *= s;
  a.z *= s;
  return a;
}
VD f3 &operator*=(f3 &a, f3 b)
{
  a.x *= b.x;
  a.y *= b.y;
  a.z *= b.z;
  return a;
}
VD float dot(f3 a, f3 b)
{
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
VD f3 cross(f3 a, f3 b)
{
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
VD f3 normalize(f3 v)
{
  const float inv = 1.f / sqrtf(dot(v, v));
  return v * inv;
}
VD f3 fmin3(f3 a, f3 b)
{
  return {fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)};
}
VD f3 fmax3(f3 a, f3 b)
{
  return {fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)};
}
VD float compMax(f3 a)
{
  return fmaxf(a.x, fmaxf(a.y, a.z));
}
VD float compMin(f3 a)
{
  return fminf(a.x, fminf(a.y, a.z));
}
VD f3 fabs3(f3 a)
{
  return {fabsf(a.x), fabsf(a.y), fabsf(a.z)};
}
VD float get(const f3 &a, int i)
{
  return i == 0 ? a.x : (i == 1 ? a.y : a.z);
}

struct box3
{
  f3 lo, hi;
};

VD box3 emptyBox()
{
  return {{3.0e38f, 3.0e38f, 3.0e38f}, {-3.0e38f, -3.0e38f, -3.0e38f}};
}
VD void extend(box3 &b, f3 p)
{
  b.lo = fmin3(b.lo, p);
  b.hi = fmax3(b.hi, p);
}
VD void extend(box3 &b, const box3 &o)
{
  b.lo = fmin3(b.lo, o.lo);
  b.hi = fmax3(b.hi, o.hi);
}
VD float halfArea(const box3 &b)
{
  const f3 d = b.hi - b.lo;
  return (d.x + d.y) * d.z + d.x * d.y;
}

// Affine transform stored as 3 rows of (m00 m01 m02 t0): p' = M p + t.
struct xfm34
{
  float r[3][4];
};

VD f3 xfmPoint(const xfm34 &m, f3 p)
{
  return {m.r[0][0] * p.x + m.r[0][1] * p.y + m.r[0][2] * p.z + m.r[0][3],
      m.r[1][0] * p.x + m.r[1][1] * p.y + m.r[1][2] * p.z + m.r[1][3],
      m.r[2][0] * p.x + m.r[2][1] * p.y + m.r[2][2] * p.z + m.r[2][3]};
}
VD f3 xfmVector(const xfm34 &m, f3 v)
{
  return {m.r[0][0] * v.x + m.r[0][1] * v.y + m.r[0][2] * v.z,
      m.r[1][0] * v.x + m.r[1][1] * v.y + m.r[1][2] * v.z,
      m.r[2][0] * v.x + m.r[2][1] * v.y + m.r[2][2] * v.z};
}
// Normal from object to world: transpose of the world->object linear part.
VD f3 xfmNormalTransposed(const xfm34 &worldToObject, f3 n)
{
  const auto &m = worldToObject.r;
  return {m[0][0] * n.x + m[1][0] * n.y + m[2][0] * n.z,
      m[0][1] * n.x + m[1][1] * n.y + m[2][1] * n.z,
      m[0][2] * n.x + m[1][2] * n.y + m[2][2] * n.z};
}

} // namespace vrtx
