// TEST INFRASTRUCTURE ONLY.  A compile shim standing in for glm (the
// reference's vector-math dependency, not vendored and not installed here) so
// that the reference's own hot-path headers and sources compile where they lie
// (oracle/build_ref.sh).  It is not glm: it restates, for float only, the
// arithmetic of the few glm operations those files use, in the operation
// order glm 0.9.x documents and implements:
//   * vector operators are component-wise (v / s divides, it does not
//     multiply by a reciprocal);
//   * dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z;
//   * cross(a, b) = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y);
//   * normalize(v) = v * inversesqrt(dot(v, v)), inversesqrt(x) = 1 / sqrt(x);
//   * min(x, y) = (y < x) ? y : x, max(x, y) = (x < y) ? y : x,
//     clamp(x, lo, hi) = min(max(x, lo), hi);
//   * mat3 is three columns; (m * v)[i] = (m[0][i]*v.x + m[1][i]*v.y) + m[2][i]*v.z;
//   * sqrt, pow, cos, sin, abs forward to the float overloads of <cmath>;
//   * radians(x) = x * T(0.01745329251994329576923690768489) in x's type;
//   * vec4 names its components x y z w or r g b a;
//   * mat4 is four vec4 columns, mat4(s) the diagonal s, mat4() the identity;
//   * (m * v) = (m[0]*v.x + m[1]*v.y) + (m[2]*v.z + m[3]*v.w), the pairwise
//     sum glm has evaluated mat4 * vec4 with since 0.9.5 (type_mat4x4.inl);
//   * translate(m, v)[3] = ((m[0]*v.x + m[1]*v.y) + m[2]*v.z) + m[3];
//     scale(m, v)[i] = m[i] * v[i] (i < 3); rotate(m, a, v) builds R from
//     c = cos(a), s = sin(a), axis = normalize(v), temp = (1 - c) * axis as
//     glm's matrix_transform.inl does and returns
//     [i] = (m[0]*R[i][0] + m[1]*R[i][1]) + m[2]*R[i][2], [3] = m[3].
// mat4 * mat4, which the compiled headers name but the oracle never reaches,
// aborts.
#pragma once

#include <cmath>
#include <cstdlib>

namespace glm {

struct vec2 {
  float x, y;
  vec2() : x(0), y(0) {}
  vec2(float a, float b) : x(a), y(b) {}
  float& operator[](int i) { return i == 0 ? x : y; }
  float operator[](int i) const { return i == 0 ? x : y; }
};

struct vec4;

struct vec3 {
  float x, y, z;
  vec3() : x(0), y(0), z(0) {}
  explicit vec3(float s) : x(s), y(s), z(s) {}
  vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  explicit vec3(const vec4& v);
  float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
  vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
  vec3& operator*=(const vec3& o) { x *= o.x; y *= o.y; z *= o.z; return *this; }
  vec3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
  vec3& operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
};

struct vec4 {
  union { float x, r; };
  union { float y, g; };
  union { float z, b; };
  union { float w, a; };
  vec4() : x(0), y(0), z(0), w(0) {}
  vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
  float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

struct ivec3 {
  int x, y, z;
  ivec3() : x(0), y(0), z(0) {}
  ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
  int& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  int operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator+(const vec3& a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator-(const vec3& a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
inline vec3 operator+(float s, const vec3& a) { return vec3(s + a.x, s + a.y, s + a.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator/(float s, const vec3& a) { return vec3(s / a.x, s / a.y, s / a.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline bool operator==(const vec3& a, const vec3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool operator!=(const vec3& a, const vec3& b) { return !(a == b); }

inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline vec3 cross(const vec3& a, const vec3& b) {
  return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float sqrt(float x) { return std::sqrt(x); }
inline vec3 sqrt(const vec3& v) { return vec3(std::sqrt(v.x), std::sqrt(v.y), std::sqrt(v.z)); }
inline float inversesqrt(float x) { return 1.0f / std::sqrt(x); }
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline vec3 normalize(const vec3& v) { return v * inversesqrt(dot(v, v)); }
inline float min(float x, float y) { return (y < x) ? y : x; }
inline float max(float x, float y) { return (x < y) ? y : x; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float abs(float x) { return std::fabs(x); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline float cos(float x) { return std::cos(x); }
inline float sin(float x) { return std::sin(x); }
template <typename T>
inline T radians(T deg) {
  return deg * static_cast<T>(0.01745329251994329576923690768489);
}

struct mat3 {
  vec3 c[3];
  mat3() { c[0] = vec3(1, 0, 0); c[1] = vec3(0, 1, 0); c[2] = vec3(0, 0, 1); }
  mat3(const vec3& a, const vec3& b, const vec3& d) { c[0] = a; c[1] = b; c[2] = d; }
  vec3& operator[](int i) { return c[i]; }
  const vec3& operator[](int i) const { return c[i]; }
};

inline vec3 operator*(const mat3& m, const vec3& v) {
  return vec3(m[0][0] * v.x + m[1][0] * v.y + m[2][0] * v.z,
              m[0][1] * v.x + m[1][1] * v.y + m[2][1] * v.z,
              m[0][2] * v.x + m[1][2] * v.y + m[2][2] * v.z);
}

inline vec4 operator+(const vec4& a, const vec4& b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator*(const vec4& a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }

struct mat4 {
  vec4 c[4];
  mat4() : mat4(1.0f) {}
  explicit mat4(float s) {
    c[0] = vec4(s, 0, 0, 0);
    c[1] = vec4(0, s, 0, 0);
    c[2] = vec4(0, 0, s, 0);
    c[3] = vec4(0, 0, 0, s);
  }
  vec4& operator[](int i) { return c[i]; }
  const vec4& operator[](int i) const { return c[i]; }
};

inline vec4 operator*(const mat4& m, const vec4& v) {
  const vec4 add0 = m[0] * v.x + m[1] * v.y;
  const vec4 add1 = m[2] * v.z + m[3] * v.w;
  return add0 + add1;
}
inline mat4 operator*(const mat4&, const mat4&) { std::abort(); }

}  // namespace glm
