// Test infrastructure only (oracle build of the reference CPU path).
//
// A minimal GLM-compatible vector/matrix shim, written for this project from
// the public GLM API semantics, so that the reference's own CPU hot path
// (src/sph.cpp, src/neighborTable.cpp, src/timer.cpp) compiles headless in a
// container without GLM.  Only what those files use is provided, and each
// operation follows the arithmetic order GLM documents for its pure-C++ path:
//   * vec op vec / vec op scalar / scalar op vec: component-wise, one rounding
//     per component (GLM's operator overloads in type_vec3.inl);
//   * compound ops with a scalar of another type (vec3 *= double) convert the
//     scalar to the component type first (GLM: static_cast<T>(scalar));
//   * ivec3 from floats truncates toward zero (static_cast<int>);
//   * dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z;
//   * normalize(v) = v * (1 / sqrt(dot(v, v)))  (GLM's inversesqrt);
//   * mat4 * mat4 = sum over k of column A[k] * B[j][k], k ascending;
//   * glm::pow is std::pow (GLM brings std::pow into its namespace).
// No GLM source is reproduced here.
#pragma once

#include <cmath>
#include <cstdint>

namespace glm {

using std::pow;
using std::sqrt;

struct vec4;

struct vec3 {
    float x, y, z;
    vec3() : x(0.f), y(0.f), z(0.f) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    template <class X, class Y, class Z>
    vec3(X a, Y b, Z c)
        : x(static_cast<float>(a)), y(static_cast<float>(b)),
          z(static_cast<float>(c)) {}
    float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const float &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }

    vec3 &operator+=(const vec3 &o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    vec3 &operator-=(const vec3 &o) { x = x - o.x; y = y - o.y; z = z - o.z; return *this; }
    template <class U>
    vec3 &operator*=(U s) {
        const float f = static_cast<float>(s);
        x = x * f; y = y * f; z = z * f;
        return *this;
    }
    template <class U>
    vec3 &operator/=(U s) {
        const float f = static_cast<float>(s);
        x = x / f; y = y / f; z = z / f;
        return *this;
    }
};

inline vec3 operator-(const vec3 &v) { return vec3(-v.x, -v.y, -v.z); }
inline vec3 operator+(const vec3 &a, const vec3 &b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3 &a, const vec3 &b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3 &a, const vec3 &b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator*(const vec3 &v, float s) { return vec3(v.x * s, v.y * s, v.z * s); }
inline vec3 operator*(float s, const vec3 &v) { return vec3(s * v.x, s * v.y, s * v.z); }
inline vec3 operator/(const vec3 &v, float s) { return vec3(v.x / s, v.y / s, v.z / s); }

struct ivec3 {
    int x, y, z;
    ivec3() : x(0), y(0), z(0) {}
    explicit ivec3(int s) : x(s), y(s), z(s) {}
    template <class X, class Y, class Z>
    ivec3(X a, Y b, Z c)
        : x(static_cast<int>(a)), y(static_cast<int>(b)), z(static_cast<int>(c)) {}
};
inline ivec3 operator+(const ivec3 &a, const ivec3 &b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }

struct uvec3 {
    unsigned x, y, z;
    uvec3() : x(0), y(0), z(0) {}
    template <class X, class Y, class Z>
    uvec3(X a, Y b, Z c)
        : x(static_cast<unsigned>(a)), y(static_cast<unsigned>(b)),
          z(static_cast<unsigned>(c)) {}
};

struct vec4 {
    float x, y, z, w;
    vec4() : x(0.f), y(0.f), z(0.f), w(0.f) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    template <class X, class Y, class Z, class W>
    vec4(X a, Y b, Z c, W d)
        : x(static_cast<float>(a)), y(static_cast<float>(b)),
          z(static_cast<float>(c)), w(static_cast<float>(d)) {}
    float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    const float &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};
inline vec4 operator+(const vec4 &a, const vec4 &b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator*(const vec4 &v, float s) { return vec4(v.x * s, v.y * s, v.z * s, v.w * s); }

// Column-major 4x4 matrix, as GLM stores it (m[c] is column c).
struct mat4 {
    vec4 c[4];
    mat4() : mat4(1.f) {}
    explicit mat4(float d) {
        c[0] = vec4(d, 0, 0, 0);
        c[1] = vec4(0, d, 0, 0);
        c[2] = vec4(0, 0, d, 0);
        c[3] = vec4(0, 0, 0, d);
    }
    vec4 &operator[](int i) { return c[i]; }
    const vec4 &operator[](int i) const { return c[i]; }
};

inline mat4 operator*(const mat4 &a, const mat4 &b) {
    mat4 r;
    for (int j = 0; j < 4; ++j) {
        r[j] = a[0] * b[j][0] + a[1] * b[j][1] + a[2] * b[j][2] + a[3] * b[j][3];
    }
    return r;
}

inline float dot(const vec3 &a, const vec3 &b) {
    const vec3 t = a * b;
    return t.x + t.y + t.z;
}
inline float length(const vec3 &v) { return std::sqrt(dot(v, v)); }
inline float inversesqrt(float x) { return 1.f / std::sqrt(x); }
inline vec3 normalize(const vec3 &v) { return v * inversesqrt(dot(v, v)); }

}  // namespace glm
