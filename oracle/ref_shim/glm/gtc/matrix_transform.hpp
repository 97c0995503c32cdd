// TEST INFRASTRUCTURE ONLY.  Compile shim for glm's matrix_transform header:
// translate, scale and rotate of a mat4 by a vec3, in the operation order of
// glm's matrix_transform.inl (restated in glm/glm.hpp's header comment).
#pragma once

#include "glm/glm.hpp"

namespace glm {

inline mat4 translate(const mat4& m, const vec3& v) {
  mat4 r = m;
  r[3] = m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3];
  return r;
}

inline mat4 scale(const mat4& m, const vec3& v) {
  mat4 r;
  r[0] = m[0] * v.x;
  r[1] = m[1] * v.y;
  r[2] = m[2] * v.z;
  r[3] = m[3];
  return r;
}

inline mat4 rotate(const mat4& m, float angle, const vec3& v) {
  const float c = cos(angle);
  const float s = sin(angle);
  const vec3 axis = normalize(v);
  const vec3 temp = (1.0f - c) * axis;
  float R[3][3];
  R[0][0] = c + temp[0] * axis[0];
  R[0][1] = temp[0] * axis[1] + s * axis[2];
  R[0][2] = temp[0] * axis[2] - s * axis[1];
  R[1][0] = temp[1] * axis[0] - s * axis[2];
  R[1][1] = c + temp[1] * axis[1];
  R[1][2] = temp[1] * axis[2] + s * axis[0];
  R[2][0] = temp[2] * axis[0] + s * axis[1];
  R[2][1] = temp[2] * axis[1] - s * axis[0];
  R[2][2] = c + temp[2] * axis[2];
  mat4 r;
  for (int i = 0; i < 3; ++i) r[i] = m[0] * R[i][0] + m[1] * R[i][1] + m[2] * R[i][2];
  r[3] = m[3];
  return r;
}

}  // namespace glm
