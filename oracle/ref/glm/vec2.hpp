// Minimal GLM-compatible vec2 for compiling the reference's demo evaluator (its simulator.h
// includes <glm/glm.hpp> and stores vehicle positions and velocities as glm::vec2).
// Project-written from GLM's documented semantics: two packed floats, operator[], component-wise
// addition and scaling by a float.
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
struct vec2
{
    float x, y;

    vec2() = default;
    GLM_SHIM_HD constexpr vec2(float a, float b) : x(a), y(b) {}

    GLM_SHIM_HD float& operator[](int i) { return i == 0 ? x : y; }
    GLM_SHIM_HD const float& operator[](int i) const { return i == 0 ? x : y; }
    GLM_SHIM_HD vec2& operator+=(const vec2& o)
    {
        x += o.x;
        y += o.y;
        return *this;
    }
};

GLM_SHIM_HD inline vec2 operator+(const vec2& a, const vec2& b) { return vec2(a.x + b.x, a.y + b.y); }
GLM_SHIM_HD inline vec2 operator*(const vec2& a, float s) { return vec2(a.x * s, a.y * s); }
}  // namespace glm

static_assert(sizeof(glm::vec2) == 8, "glm::vec2 is two packed floats");
