// Test infrastructure only: GLM-compatible length2 (dot(v, v)) for the
// headless oracle build of the reference CPU path.
#pragma once
#include "../glm.hpp"

namespace glm {
inline float length2(const vec3 &v) { return dot(v, v); }
}  // namespace glm
