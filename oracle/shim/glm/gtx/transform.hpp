// Test infrastructure only: GLM-compatible translate(v) and scale(v) for the
// headless oracle build of the reference CPU path.  Both start from the
// identity matrix as GLM's gtx/transform overloads do:
//   translate: column 3 = col0*v.x + col1*v.y + col2*v.z + col3;
//   scale:     column k = colk * v[k] for k < 3, column 3 unchanged.
#pragma once
#include "../glm.hpp"

namespace glm {
inline mat4 translate(const vec3 &v) {
    mat4 m(1.f);
    m[3] = m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3];
    return m;
}
inline mat4 scale(const vec3 &v) {
    mat4 m(1.f);
    m[0] = m[0] * v.x;
    m[1] = m[1] * v.y;
    m[2] = m[2] * v.z;
    return m;
}
}  // namespace glm
