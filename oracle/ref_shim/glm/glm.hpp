// Compile shim for building a reference header that names glm::vec2 in a
// helper this oracle never calls (TEST INFRASTRUCTURE ONLY).  It is not glm:
// it only lets the header parse.
#pragma once
namespace glm {
struct vec2 {
  float x, y;
  vec2(float a, float b) : x(a), y(b) {}
};
}  // namespace glm
