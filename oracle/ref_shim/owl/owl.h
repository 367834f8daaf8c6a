// Project-written stand-in for the parts of the OWL math library that the
// owlExaStitcher sampling headers use (Gridlet.h, UElems.h, Plane.h,
// Grid.cuh, common.h).  OWL is an un-vendored submodule of the reference, so
// this file defines each type and operator from its use at those call sites,
// with textbook semantics:
//   vec ops component-wise; dot(a,b) = a.x*b.x + a.y*b.y + a.z*b.z;
//   cross = the usual determinant rows; min/max = (a<b?a:b) / (a>b?a:b);
//   box3f default = empty (+inf / -inf); contains / overlaps inclusive;
//   LinearSpace3f * v = v.x*vx + v.y*vy + v.z*vz.
// It is test infrastructure: only the oracle/_ref build includes it.
#pragma once

#include <cuda_runtime.h>   // float4 (vector_types.h)
#include <cmath>
#include <cstdint>
#include <iostream>
#include <limits>
#include <string>

#ifndef __both__
#define __both__ __host__ __device__
#endif

namespace owl {
namespace common {

  struct vec3i;
  struct vec3f;

  struct vec2f {
    float x, y;
    vec2f() = default;
    __both__ vec2f(float v) : x(v), y(v) {}
    __both__ vec2f(float a, float b) : x(a), y(b) {}
  };

  struct vec3i {
    int x, y, z;
    vec3i() = default;
    __both__ vec3i(int v) : x(v), y(v), z(v) {}
    __both__ vec3i(int a, int b, int c) : x(a), y(b), z(c) {}
    __both__ explicit inline vec3i(const vec3f &v);
  };

  struct vec3f {
    float x, y, z;
    vec3f() = default;
    __both__ vec3f(float v) : x(v), y(v), z(v) {}
    __both__ vec3f(float a, float b, float c) : x(a), y(b), z(c) {}
    __both__ explicit vec3f(const vec3i &v) : x((float)v.x), y((float)v.y), z((float)v.z) {}
    // UElems.h:123 copy-initialises a vec3f from a float4
    __both__ vec3f(const float4 &v) : x(v.x), y(v.y), z(v.z) {}
  };

  inline vec3i::vec3i(const vec3f &v) : x((int)v.x), y((int)v.y), z((int)v.z) {}

  struct vec4f {
    float x, y, z, w;
    vec4f() = default;
    __both__ vec4f(float v) : x(v), y(v), z(v), w(v) {}
    __both__ vec4f(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    __both__ vec4f(const float4 &v) : x(v.x), y(v.y), z(v.z), w(v.w) {}
    __both__ operator float4() const { return make_float4(x, y, z, w); }
  };

  // ---- vec3f arithmetic ----
  inline __both__ vec3f operator+(const vec3f &a, const vec3f &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
  inline __both__ vec3f operator-(const vec3f &a, const vec3f &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
  inline __both__ vec3f operator*(const vec3f &a, const vec3f &b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
  inline __both__ vec3f operator/(const vec3f &a, const vec3f &b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
  inline __both__ vec3f operator+(const vec3f &a, float b) { return {a.x + b, a.y + b, a.z + b}; }
  inline __both__ vec3f operator-(const vec3f &a, float b) { return {a.x - b, a.y - b, a.z - b}; }
  inline __both__ vec3f operator*(const vec3f &a, float b) { return {a.x * b, a.y * b, a.z * b}; }
  inline __both__ vec3f operator*(float a, const vec3f &b) { return {a * b.x, a * b.y, a * b.z}; }
  inline __both__ vec3f operator/(const vec3f &a, float b) { return {a.x / b, a.y / b, a.z / b}; }
  // Gridlet.h:50 divides a vec3f by an int power of two
  inline __both__ vec3f operator/(const vec3f &a, int b) { return a / (float)b; }
  inline __both__ vec3f operator-(const vec3f &a) { return {-a.x, -a.y, -a.z}; }

  // ---- vec3i arithmetic ----
  inline __both__ vec3i operator+(const vec3i &a, const vec3i &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
  inline __both__ vec3i operator-(const vec3i &a, const vec3i &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
  inline __both__ vec3i operator+(const vec3i &a, int b) { return {a.x + b, a.y + b, a.z + b}; }
  inline __both__ vec3i operator-(const vec3i &a, int b) { return {a.x - b, a.y - b, a.z - b}; }
  // Grid.cu:181 multiplies a vec3i by a float cell width
  inline __both__ vec3f operator*(const vec3i &a, float b) { return vec3f(a) * b; }
  inline __both__ bool operator==(const vec3i &a, const vec3i &b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

  inline __both__ vec3i min(const vec3i &a, const vec3i &b) { return {a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z}; }
  inline __both__ vec3i max(const vec3i &a, const vec3i &b) { return {a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z}; }
  inline __both__ vec3i clamp(const vec3i &v, const vec3i &lo, const vec3i &hi) { return min(max(v, lo), hi); }
  inline __both__ vec3f min(const vec3f &a, const vec3f &b) { return {a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z}; }
  inline __both__ vec3f max(const vec3f &a, const vec3f &b) { return {a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z}; }

  inline __both__ float dot(const vec3f &a, const vec3f &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
  inline __both__ vec3f cross(const vec3f &a, const vec3f &b)
  {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
  }

  struct box3f {
    vec3f lower, upper;
    __both__ box3f()
      : lower(std::numeric_limits<float>::infinity()),
        upper(-std::numeric_limits<float>::infinity()) {}
    __both__ box3f(const vec3f &l, const vec3f &u) : lower(l), upper(u) {}
    __both__ bool contains(const vec3f &p) const
    {
      return lower.x <= p.x && lower.y <= p.y && lower.z <= p.z &&
             p.x <= upper.x && p.y <= upper.y && p.z <= upper.z;
    }
    __both__ bool overlaps(const box3f &o) const
    {
      return lower.x <= o.upper.x && lower.y <= o.upper.y && lower.z <= o.upper.z &&
             o.lower.x <= upper.x && o.lower.y <= upper.y && o.lower.z <= upper.z;
    }
    __both__ void extend(const vec3f &p) { lower = min(lower, p); upper = max(upper, p); }
    __both__ vec3f size() const { return upper - lower; }
    __both__ vec3f span() const { return upper - lower; }
  };

  template <typename T>
  struct interval {
    T lower, upper;
  };

  struct LinearSpace3f {
    vec3f vx, vy, vz;
  };

  struct affine3f {
    LinearSpace3f l;
    vec3f p;
  };

  inline std::string prettyNumber(size_t n) { return std::to_string(n); }

  // Gridlet.h:68 and Grid.cu call isnan unqualified (CUDA's global one)
  inline __both__ bool isnan(float f) { return std::isnan(f); }

  // DDA.h:26-113 helpers
  inline __both__ float min(float a, float b) { return a < b ? a : b; }
  inline __both__ float max(float a, float b) { return a > b ? a : b; }
  inline __both__ vec3f rcp(const vec3f &v) { return {1.f / v.x, 1.f / v.y, 1.f / v.z}; }
  inline __both__ float reduce_min(const vec3f &v) { return min(v.x, min(v.y, v.z)); }
  inline __both__ float reduce_max(const vec3f &v) { return max(v.x, max(v.y, v.z)); }

  template <int RT = 0, int NRT = 1>
  struct RayT {
    vec3f origin, direction;
    float tmin = 0.f, tmax = 1e30f;
  };

} // namespace common

  using namespace common;

} // namespace owl
