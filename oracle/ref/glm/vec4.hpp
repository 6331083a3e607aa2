// Minimal GLM-compatible vec4 for compiling the reference's device code (the reference
// includes <glm/vec4.hpp>; GLM is not installed here).  Project-written from GLM's documented
// semantics: four packed floats x, y, z, w (16 bytes, 4-byte alignment like GLM's default
// packed types), component access by operator[], component-wise arithmetic.
#pragma once

#ifndef GLM_SHIM_HD
#ifdef __CUDACC__
#define GLM_SHIM_HD __host__ __device__
#else
#define GLM_SHIM_HD
#endif
#endif

namespace glm
{
struct vec4
{
    float x, y, z, w;

    vec4() = default;
    GLM_SHIM_HD constexpr vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    GLM_SHIM_HD explicit constexpr vec4(float s) : x(s), y(s), z(s), w(s) {}

    GLM_SHIM_HD float& operator[](int i) { return i == 0 ? x : i == 1 ? y : i == 2 ? z : w; }
    GLM_SHIM_HD const float& operator[](int i) const { return i == 0 ? x : i == 1 ? y : i == 2 ? z : w; }
};

GLM_SHIM_HD inline vec4 operator+(const vec4& a, const vec4& b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
GLM_SHIM_HD inline vec4 operator*(const vec4& a, const vec4& b) { return vec4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
GLM_SHIM_HD inline bool operator==(const vec4& a, const vec4& b)
{
    return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w;
}
GLM_SHIM_HD inline bool operator!=(const vec4& a, const vec4& b) { return !(a == b); }
}  // namespace glm

static_assert(sizeof(glm::vec4) == 16, "glm::vec4 is four packed floats");
