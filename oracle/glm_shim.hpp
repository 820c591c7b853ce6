// TEST INFRASTRUCTURE (oracle only; never linked into the product library).
//
// A minimal subset of the glm vector library, written for this project from
// the GLSL / glm documented semantics, so that the reference's hot-path
// headers (source/wind.hpp, source/world.hpp, source/cellpool.h,
// source/include/math.h) compile without glm, which is not installed here.
//
// The arithmetic below is the contract that the CPU oracle port
// (oracle/swe_oracle.cpp) and the CUDA kernels both follow, operation by
// operation:
//   dot(a,b)        = (a.x*b.x + a.y*b.y) + a.z*b.z        (left to right)
//   length(v)       = sqrt(dot(v,v))
//   normalize(v)    = v * (1 / sqrt(dot(v,v)))             (glm inversesqrt)
//   cross(a,b)      = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y)
//   mix(x,y,a)      = x*(1-a) + y*a                         (GLSL mix)
//   round(v)        = std::round per component (half away from zero)
//   v *= s (any U)  = each component *= static_cast<float>(s)
// The real glm is not pinned by the reference (no lockfile, README only says
// "glm"), so parity beyond this definition is unpinned.
#pragma once

#include <cmath>

namespace glm {

struct ivec2;

struct vec2 {
  float x, y;
  vec2() : x(0), y(0) {}
  explicit vec2(float s) : x(s), y(s) {}
  template <class X, class Y>
  vec2(X a, Y b) : x(static_cast<float>(a)), y(static_cast<float>(b)) {}
  vec2(const ivec2& v);  // implicit int -> float conversion, as glm allows
};

struct ivec2 {
  int x, y;
  ivec2() : x(0), y(0) {}
  explicit ivec2(int s) : x(s), y(s) {}
  template <class X, class Y>
  ivec2(X a, Y b) : x(static_cast<int>(a)), y(static_cast<int>(b)) {}
  ivec2(const vec2& v) : x(static_cast<int>(v.x)), y(static_cast<int>(v.y)) {}
  ivec2& operator/=(const ivec2& o) { x /= o.x; y /= o.y; return *this; }
};

inline vec2::vec2(const ivec2& v) : x(static_cast<float>(v.x)), y(static_cast<float>(v.y)) {}

struct vec3 {
  float x, y, z;
  vec3() : x(0), y(0), z(0) {}
  explicit vec3(float s) : x(s), y(s), z(s) {}
  template <class X, class Y, class Z>
  vec3(X a, Y b, Z c)
      : x(static_cast<float>(a)), y(static_cast<float>(b)), z(static_cast<float>(c)) {}
  vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
  vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
  template <class U>
  vec3& operator*=(U s) {
    x *= static_cast<float>(s); y *= static_cast<float>(s); z *= static_cast<float>(s);
    return *this;
  }
};

// ---- ivec2 arithmetic (integer, component-wise) ----
inline ivec2 operator+(const ivec2& a, const ivec2& b) { return ivec2(a.x + b.x, a.y + b.y); }
inline ivec2 operator-(const ivec2& a, const ivec2& b) { return ivec2(a.x - b.x, a.y - b.y); }
inline ivec2 operator*(const ivec2& a, const ivec2& b) { return ivec2(a.x * b.x, a.y * b.y); }
inline ivec2 operator*(int s, const ivec2& a) { return ivec2(s * a.x, s * a.y); }
inline ivec2 operator*(const ivec2& a, int s) { return ivec2(a.x * s, a.y * s); }
inline ivec2 operator/(const ivec2& a, const ivec2& b) { return ivec2(a.x / b.x, a.y / b.y); }
inline ivec2 operator/(const ivec2& a, int s) { return ivec2(a.x / s, a.y / s); }

// ---- vec2 arithmetic ----
inline vec2 operator+(const vec2& a, const vec2& b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(const vec2& a, const vec2& b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator/(const vec2& a, const vec2& b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec2 operator/(const vec2& a, float s) { return vec2(a.x / s, a.y / s); }
inline vec2& operator+=(vec2& a, const vec2& b) { a.x += b.x; a.y += b.y; return a; }

// ---- vec3 arithmetic ----
inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator-(const vec3& a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }

// ---- geometric functions ----
inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(const vec2& v) { return std::sqrt(dot(v, v)); }
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline float inversesqrt(float x) { return 1.0f / std::sqrt(x); }
inline vec3 normalize(const vec3& v) { return v * inversesqrt(dot(v, v)); }
inline vec3 cross(const vec3& a, const vec3& b) {
  return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline vec3 mix(const vec3& x, const vec3& y, float a) { return x * (1.0f - a) + y * a; }
inline vec2 round(const vec2& v) { return vec2(std::round(v.x), std::round(v.y)); }

}  // namespace glm
