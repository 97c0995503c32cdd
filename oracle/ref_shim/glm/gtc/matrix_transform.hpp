// TEST INFRASTRUCTURE ONLY.  Compile shim for glm's matrix_transform header:
// the reference's camera header names glm::rotate in Camera::rotate, which
// the oracle never calls; reaching it aborts.
#pragma once

#include <cstdlib>

#include "glm/glm.hpp"

namespace glm {
inline mat4 rotate(const mat4&, float, const vec3&) { std::abort(); }
}  // namespace glm
