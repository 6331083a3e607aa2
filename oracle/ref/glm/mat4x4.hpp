// Minimal GLM-compatible mat4x4 (see vec4.hpp).  GLM stores four column vectors; the
// 16-scalar constructor takes them column by column; m * v is the linear combination of the
// columns, formed as (c0 v0 + c1 v1) + (c2 v2 + c3 v3) -- the pairwise grouping GLM's
// matrix-vector product uses.  With the reference's transition matrix (entries 0, 1 and dt)
// this gives x' = x + dt * vx with one rounding of the product and one of the sum, whatever
// the compiler contracts.
#pragma once

#include "vec4.hpp"

namespace glm
{
struct mat4x4
{
    vec4 value[4];  // columns

    mat4x4() = default;
    GLM_SHIM_HD constexpr mat4x4(float x0, float y0, float z0, float w0, float x1, float y1, float z1, float w1,
                                 float x2, float y2, float z2, float w2, float x3, float y3, float z3, float w3)
        : value{vec4(x0, y0, z0, w0), vec4(x1, y1, z1, w1), vec4(x2, y2, z2, w2), vec4(x3, y3, z3, w3)}
    {
    }
    GLM_SHIM_HD vec4& operator[](int i) { return value[i]; }
    GLM_SHIM_HD const vec4& operator[](int i) const { return value[i]; }
};
typedef mat4x4 mat4;

GLM_SHIM_HD inline vec4 operator*(const mat4x4& m, const vec4& v)
{
    const vec4 mul0 = m[0] * vec4(v[0]);
    const vec4 mul1 = m[1] * vec4(v[1]);
    const vec4 mul2 = m[2] * vec4(v[2]);
    const vec4 mul3 = m[3] * vec4(v[3]);
    const vec4 add0 = mul0 + mul1;
    const vec4 add1 = mul2 + mul3;
    return add0 + add1;
}

GLM_SHIM_HD inline mat4x4 transpose(const mat4x4& m)
{
    return mat4x4(m[0][0], m[1][0], m[2][0], m[3][0], m[0][1], m[1][1], m[2][1], m[3][1], m[0][2], m[1][2], m[2][2],
                  m[3][2], m[0][3], m[1][3], m[2][3], m[3][3]);
}
}  // namespace glm

static_assert(sizeof(glm::mat4x4) == 64, "glm::mat4x4 is 16 packed floats");
