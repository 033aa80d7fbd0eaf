// Minimal vector-math header that stands in for the glm library when the
// reference svo_builder sources are compiled into the CPU oracle.
//
// This is test infrastructure: it exists only so that the reference's own
// translation units (src/svo_builder/*.cpp) build without glm, which is not
// installed here.  Only the subset those files use is provided, and every
// operation is written from its mathematical definition with a fixed,
// documented evaluation order, because bit-exact FP32 parity with the GPU
// kernels depends on it:
//
//   * component-wise + - * / on vectors, scalar*vector and vector*scalar;
//   * dot(a, b)        = (a.x*b.x + a.y*b.y) + a.z*b.z   (left to right);
//   * cross(a, b)      = (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x);
//   * length(v)        = sqrt(dot(v, v));
//   * normalize(v)     = v * (1 / sqrt(dot(v, v)))   (multiply by reciprocal);
//   * mat3 is stored as three columns; mat3 * v = c0*v.x + c1*v.y + c2*v.z
//     evaluated per row left to right;
//   * inverse(mat3)    = adjugate * (1 / det), det expanded along the first
//     row of the (row, column) matrix.
//
// glm itself is not available to pin these orders against, so parity at this
// boundary is defined by this header (the GPU kernels follow the same orders).
#pragma once

// The real library pulls these standard headers in; the reference relies on
// that (e.g. assert() in OctreeBuilder.cpp), so the stand-in does the same.
#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <type_traits>

namespace glm {

template <typename T>
struct tvec2 {
  T x, y;
  tvec2() : x(T(0)), y(T(0)) {}
  template <typename A, typename B>
  tvec2(A a, B b) : x(static_cast<T>(a)), y(static_cast<T>(b)) {}
  T& operator[](int i) { return i == 0 ? x : y; }
  const T& operator[](int i) const { return i == 0 ? x : y; }
};

template <typename T>
struct tvec3 {
  T x, y, z;
  tvec3() : x(T(0)), y(T(0)), z(T(0)) {}
  template <typename A>
  explicit tvec3(A s) : x(static_cast<T>(s)), y(static_cast<T>(s)), z(static_cast<T>(s)) {}
  template <typename A, typename B, typename C>
  tvec3(A a, B b, C c) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)) {}
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  tvec3& operator+=(const tvec3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
  tvec3& operator-=(const tvec3& o) { x = x - o.x; y = y - o.y; z = z - o.z; return *this; }
};

typedef tvec2<float> vec2;
typedef tvec3<float> vec3;
typedef tvec3<int> ivec3;
typedef tvec3<unsigned int> uvec3;

// ---- vec2 ----
inline vec2 operator+(const vec2& a, const vec2& b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(const vec2& a, const vec2& b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator*(float s, const vec2& v) { return vec2(s * v.x, s * v.y); }
inline vec2 operator*(const vec2& v, float s) { return vec2(v.x * s, v.y * s); }
inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }

// ---- vec3 ----
inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator*(float s, const vec3& v) { return vec3(s * v.x, s * v.y, s * v.z); }
inline vec3 operator*(const vec3& v, float s) { return vec3(v.x * s, v.y * s, v.z * s); }
inline vec3 operator/(const vec3& v, float s) { return vec3(v.x / s, v.y / s, v.z / s); }
inline vec3 operator-(const vec3& v) { return vec3(-v.x, -v.y, -v.z); }
inline bool operator==(const vec3& a, const vec3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool operator!=(const vec3& a, const vec3& b) { return !(a == b); }

inline float dot(const vec3& a, const vec3& b) {
  float px = a.x * b.x;
  float py = a.y * b.y;
  float pz = a.z * b.z;
  return (px + py) + pz;
}
inline vec3 cross(const vec3& a, const vec3& b) {
  return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline vec3 normalize(const vec3& v) {
  float r = 1.0f / std::sqrt(dot(v, v));
  return v * r;
}

// ---- mat3 (column major: c[i] is column i, c[i][j] is row j of column i) ----
struct mat3 {
  vec3 c[3];
  mat3() { c[0] = vec3(1, 0, 0); c[1] = vec3(0, 1, 0); c[2] = vec3(0, 0, 1); }
  mat3(const vec3& c0, const vec3& c1, const vec3& c2) { c[0] = c0; c[1] = c1; c[2] = c2; }
  vec3& operator[](int i) { return c[i]; }
  const vec3& operator[](int i) const { return c[i]; }
};

inline vec3 operator*(const mat3& m, const vec3& v) {
  return vec3(m[0][0] * v.x + m[1][0] * v.y + m[2][0] * v.z,
              m[0][1] * v.x + m[1][1] * v.y + m[2][1] * v.z,
              m[0][2] * v.x + m[1][2] * v.y + m[2][2] * v.z);
}

inline mat3 inverse(const mat3& m) {
  // Rows of the matrix as (r0: a b c, r1: d e f, r2: g h i) with a = m[0][0],
  // b = m[1][0], c = m[2][0], ...  Cofactor Cjk of element (row j, column k).
  const float a = m[0][0], b = m[1][0], c = m[2][0];
  const float d = m[0][1], e = m[1][1], f = m[2][1];
  const float g = m[0][2], h = m[1][2], i = m[2][2];
  const float C00 = e * i - f * h;
  const float C01 = f * g - d * i;
  const float C02 = d * h - e * g;
  const float det = (a * C00 + b * C01) + c * C02;
  const float r = 1.0f / det;
  const float C10 = c * h - b * i;
  const float C11 = a * i - c * g;
  const float C12 = b * g - a * h;
  const float C20 = b * f - c * e;
  const float C21 = c * d - a * f;
  const float C22 = a * e - b * d;
  // inverse(row j, column k) = C(k, j) / det; stored column-major.
  mat3 out;
  out[0] = vec3(C00 * r, C01 * r, C02 * r);  // column 0: rows 0..2 = C00 C01 C02
  out[1] = vec3(C10 * r, C11 * r, C12 * r);
  out[2] = vec3(C20 * r, C21 * r, C22 * r);
  return out;
}

template <typename T>
inline T min(T a, T b) { return b < a ? b : a; }
template <typename T>
inline T max(T a, T b) { return a < b ? b : a; }

}  // namespace glm
