// Stand-in for the subset of GLM 0.9.9.8 (g-truc/glm, commit bf71a834) that the
// VISGSim hot-path sources use.  GLM is a git submodule of the reference that is
// not vendored, so this header restates the library's documented semantics:
//
//   * vec2/vec3/vec4 of float, component-wise + - * / with vectors and scalars,
//     compound assignment, explicit scalar-broadcast and vec4 -> vec3 conversion;
//     a defaulted default constructor (value-initialisation gives zeros).
//   * dot(a, b)      = (a.x*b.x + a.y*b.y) + a.z*b.z   (products first, summed left to right)
//   * cross(a, b)    = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y)
//   * length(v)      = sqrt(dot(v, v))
//   * distance(a, b) = length(b - a)
//   * normalize(v)   = v * inversesqrt(dot(v, v)),  inversesqrt(x) = 1 / sqrt(x)
//   * vector / scalar divides each component (no reciprocal multiply).
//
// Every operation is one IEEE-754 single-precision operation; the refkern cubin is
// compiled with --fmad=false so that none of them are contracted.  This is test
// infrastructure for the oracle, not part of the shipped library.
#pragma once
#include <cmath>
#include <cuda_runtime.h>

#define GLMSTUB_FN __host__ __device__ inline

namespace glm {

struct vec2 {
    float x, y;
    vec2() = default;
    template <typename U> GLMSTUB_FN explicit vec2(U s) : x((float)s), y((float)s) {}
    template <typename A, typename B> GLMSTUB_FN vec2(A a, B b) : x((float)a), y((float)b) {}
};

struct vec4;

struct vec3 {
    float x, y, z;
    vec3() = default;
    template <typename U> GLMSTUB_FN explicit vec3(U s) : x((float)s), y((float)s), z((float)s) {}
    template <typename A, typename B, typename C>
    GLMSTUB_FN vec3(A a, B b, C c) : x((float)a), y((float)b), z((float)c) {}
    GLMSTUB_FN explicit vec3(const vec4& v);

    GLMSTUB_FN float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    GLMSTUB_FN const float& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }

    GLMSTUB_FN vec3& operator+=(const vec3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    GLMSTUB_FN vec3& operator-=(const vec3& o) { x = x - o.x; y = y - o.y; z = z - o.z; return *this; }
    GLMSTUB_FN vec3& operator*=(const vec3& o) { x = x * o.x; y = y * o.y; z = z * o.z; return *this; }
    GLMSTUB_FN vec3& operator/=(const vec3& o) { x = x / o.x; y = y / o.y; z = z / o.z; return *this; }
    template <typename U> GLMSTUB_FN vec3& operator+=(U s) { float f = (float)s; x = x + f; y = y + f; z = z + f; return *this; }
    template <typename U> GLMSTUB_FN vec3& operator-=(U s) { float f = (float)s; x = x - f; y = y - f; z = z - f; return *this; }
    template <typename U> GLMSTUB_FN vec3& operator*=(U s) { float f = (float)s; x = x * f; y = y * f; z = z * f; return *this; }
    template <typename U> GLMSTUB_FN vec3& operator/=(U s) { float f = (float)s; x = x / f; y = y / f; z = z / f; return *this; }
};

struct vec4 {
    float x, y, z, w;
    vec4() = default;
    template <typename U> GLMSTUB_FN explicit vec4(U s) : x((float)s), y((float)s), z((float)s), w((float)s) {}
    template <typename A, typename B, typename C, typename D>
    GLMSTUB_FN vec4(A a, B b, C c, D d) : x((float)a), y((float)b), z((float)c), w((float)d) {}
    template <typename D>
    GLMSTUB_FN vec4(const vec3& v, D d) : x(v.x), y(v.y), z(v.z), w((float)d) {}
    GLMSTUB_FN vec4& operator+=(const vec4& o) { x = x + o.x; y = y + o.y; z = z + o.z; w = w + o.w; return *this; }
    GLMSTUB_FN vec4& operator-=(const vec4& o) { x = x - o.x; y = y - o.y; z = z - o.z; w = w - o.w; return *this; }
};

GLMSTUB_FN vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

// vec3 binary operators
GLMSTUB_FN vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
GLMSTUB_FN vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
GLMSTUB_FN vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
GLMSTUB_FN vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
GLMSTUB_FN vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
GLMSTUB_FN vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
GLMSTUB_FN vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
GLMSTUB_FN vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
GLMSTUB_FN vec3 operator+(const vec3& a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
GLMSTUB_FN vec3 operator-(const vec3& a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }

// vec4 binary operators used by the mesh helpers
GLMSTUB_FN vec4 operator+(const vec4& a, const vec4& b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
GLMSTUB_FN vec4 operator-(const vec4& a, const vec4& b) { return vec4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
GLMSTUB_FN vec4 operator*(float s, const vec4& a) { return vec4(s * a.x, s * a.y, s * a.z, s * a.w); }
GLMSTUB_FN vec4 operator*(const vec4& a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }

// geometric functions
GLMSTUB_FN float dot(const vec3& a, const vec3& b) {
    float px = a.x * b.x;
    float py = a.y * b.y;
    float pz = a.z * b.z;
    return (px + py) + pz;
}
GLMSTUB_FN float dot(const vec4& a, const vec4& b) {
    float px = a.x * b.x;
    float py = a.y * b.y;
    float pz = a.z * b.z;
    float pw = a.w * b.w;
    return ((px + py) + pz) + pw;
}
GLMSTUB_FN vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
GLMSTUB_FN float inversesqrt(float v) { return 1.0f / sqrtf(v); }
GLMSTUB_FN float length(const vec3& v) { return sqrtf(dot(v, v)); }
GLMSTUB_FN float length(const vec4& v) { return sqrtf(dot(v, v)); }
GLMSTUB_FN float distance(const vec3& a, const vec3& b) { return length(b - a); }
GLMSTUB_FN float distance(const vec4& a, const vec4& b) { return length(b - a); }
GLMSTUB_FN vec3 normalize(const vec3& v) { return v * inversesqrt(dot(v, v)); }
GLMSTUB_FN float abs(float v) { return fabsf(v); }
GLMSTUB_FN float sqrt(float v) { return sqrtf(v); }
GLMSTUB_FN float acos(float v) { return acosf(v); }
GLMSTUB_FN float cos(float v) { return cosf(v); }

}  // namespace glm
