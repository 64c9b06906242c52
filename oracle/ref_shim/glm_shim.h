// glm_shim.h -- a minimal stand-in for the parts of glm 0.9.9.8 that the
// reference's geometry headers use, written here so that those headers
// compile unchanged for the reference pin (oracle/_ref, test infrastructure
// only).  Vectors are plain structs; every operation rounds as glm's scalar
// path does: componentwise operators, dot(a, b) = (a.x*b.x + a.y*b.y) +
// a.z*b.z, cross(x, y) = (x.y*y.z - y.y*x.z, x.z*y.x - y.z*x.x,
// x.x*y.y - y.x*x.y), length = sqrt(dot(v, v)), normalize = v * (1 / length).
#pragma once
#include <cmath>
#include <cstddef>
#include <limits>

namespace glm {

template <typename T> struct tvec1;
template <typename T> struct tvec2;
template <typename T> struct tvec3;
template <typename T> struct tvec4;

template <typename T> struct tvec1 {
  T x;
  tvec1() : x(0) {}
  template <typename U> explicit tvec1(U s) : x(static_cast<T>(s)) {}
  T& operator[](int) { return x; }
  const T& operator[](int) const { return x; }
};

template <typename T> struct tvec2 {
  T x, y;
  tvec2() : x(0), y(0) {}
  template <typename U> explicit tvec2(U s) : x(static_cast<T>(s)), y(static_cast<T>(s)) {}
  template <typename A, typename B> tvec2(A a, B b) : x(static_cast<T>(a)), y(static_cast<T>(b)) {}
  template <typename U> tvec2(const tvec2<U>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)) {}
  T& operator[](int i) { return i == 0 ? x : y; }
  const T& operator[](int i) const { return i == 0 ? x : y; }
};

template <typename T> struct tvec3 {
  T x, y, z;
  tvec3() : x(0), y(0), z(0) {}
  template <typename U> explicit tvec3(U s) : x(static_cast<T>(s)), y(static_cast<T>(s)), z(static_cast<T>(s)) {}
  template <typename A, typename B, typename C>
  tvec3(A a, B b, C c) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)) {}
  template <typename U> tvec3(const tvec3<U>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)) {}
  template <typename U> tvec3(const tvec4<U>& v);
  template <typename U, typename B> tvec3(const tvec2<U>& v, B b) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(b)) {}
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  tvec3& operator+=(const tvec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
  tvec3& operator-=(const tvec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
  tvec3& operator*=(T s) { x *= s; y *= s; z *= s; return *this; }
  tvec3& operator/=(T s) { x /= s; y /= s; z /= s; return *this; }
};

template <typename T> struct tvec4 {
  T x, y, z, w;
  tvec4() : x(0), y(0), z(0), w(0) {}
  template <typename U> explicit tvec4(U s) : x(static_cast<T>(s)), y(static_cast<T>(s)), z(static_cast<T>(s)), w(static_cast<T>(s)) {}
  template <typename A, typename B, typename C, typename D>
  tvec4(A a, B b, C c, D d) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)), w(static_cast<T>(d)) {}
  template <typename U, typename B> tvec4(const tvec3<U>& v, B b) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)), w(static_cast<T>(b)) {}
  template <typename U> tvec4(const tvec4<U>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)), w(static_cast<T>(v.w)) {}
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

template <typename T> template <typename U>
tvec3<T>::tvec3(const tvec4<U>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)) {}

// componentwise arithmetic (vector-vector, vector-scalar, scalar-vector)
#define VFREF_OPS(V, OP)                                                                   \
  template <typename T> V<T> operator OP(const V<T>& a, const V<T>& b) { V<T> r; for (int i = 0; i < (int)(sizeof(V<T>) / sizeof(T)); ++i) r[i] = a[i] OP b[i]; return r; } \
  template <typename T> V<T> operator OP(const V<T>& a, T s) { V<T> r; for (int i = 0; i < (int)(sizeof(V<T>) / sizeof(T)); ++i) r[i] = a[i] OP s; return r; } \
  template <typename T> V<T> operator OP(T s, const V<T>& a) { V<T> r; for (int i = 0; i < (int)(sizeof(V<T>) / sizeof(T)); ++i) r[i] = s OP a[i]; return r; }
VFREF_OPS(tvec2, +) VFREF_OPS(tvec2, -) VFREF_OPS(tvec2, *) VFREF_OPS(tvec2, /)
VFREF_OPS(tvec3, +) VFREF_OPS(tvec3, -) VFREF_OPS(tvec3, *) VFREF_OPS(tvec3, /)
VFREF_OPS(tvec4, +) VFREF_OPS(tvec4, -) VFREF_OPS(tvec4, *) VFREF_OPS(tvec4, /)
#undef VFREF_OPS
template <typename T> tvec3<T> operator-(const tvec3<T>& a) { return tvec3<T>(-a.x, -a.y, -a.z); }
template <typename T> bool operator==(const tvec3<T>& a, const tvec3<T>& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
template <typename T> bool operator!=(const tvec3<T>& a, const tvec3<T>& b) { return !(a == b); }

typedef tvec1<float> vec1; typedef tvec2<float> vec2; typedef tvec3<float> vec3; typedef tvec4<float> vec4;
typedef tvec1<int> ivec1; typedef tvec2<int> ivec2; typedef tvec3<int> ivec3; typedef tvec4<int> ivec4;
typedef tvec1<unsigned> uvec1; typedef tvec2<unsigned> uvec2; typedef tvec3<unsigned> uvec3; typedef tvec4<unsigned> uvec4;

// column-major 3x3 and 4x4 matrices (only what the parsed headers name)
struct mat3 { vec3 c[3]; };
struct mat4 {
  vec4 c[4];
  mat4() {}
  explicit mat4(float s) { for (int i = 0; i < 4; ++i) { c[i] = vec4(0.0f); c[i][i] = s; } }
};
inline vec4 operator*(const mat4& m, const vec4& v) {
  vec4 r;
  for (int i = 0; i < 4; ++i)
    r[i] = ((m.c[0][i] * v.x + m.c[1][i] * v.y) + m.c[2][i] * v.z) + m.c[3][i] * v.w;
  return r;
}

template <typename T> T dot(const tvec3<T>& a, const tvec3<T>& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <typename T> T dot(const tvec2<T>& a, const tvec2<T>& b) { return a.x * b.x + a.y * b.y; }
template <typename T> T dot(const tvec4<T>& a, const tvec4<T>& b) { return (a.x * b.x + a.y * b.y) + (a.z * b.z + a.w * b.w); }
template <typename T> tvec3<T> cross(const tvec3<T>& x, const tvec3<T>& y) {
  return tvec3<T>(x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y);
}
template <typename V> float length(const V& v) { return std::sqrt(dot(v, v)); }
template <typename V> float length2(const V& v) { return dot(v, v); }  // gtx/norm
template <typename V> float distance(const V& p0, const V& p1) { return length(p1 - p0); }
template <typename V> V normalize(const V& v) { return v * (1.0f / std::sqrt(dot(v, v))); }
template <typename T> T abs(T v) { return v < T(0) ? -v : v; }
template <typename T> T min(T a, T b) { return b < a ? b : a; }
template <typename T> T max(T a, T b) { return a < b ? b : a; }
template <typename T> T clamp(T v, T lo, T hi) { return min(max(v, lo), hi); }
template <typename T> T epsilon() { return std::numeric_limits<T>::epsilon(); }
template <typename T> T pi() { return static_cast<T>(3.14159265358979323846264338327950288); }

}  // namespace glm
