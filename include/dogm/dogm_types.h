// Host-side data types of the dogm::DOGM drop-in, layout-compatible with the reference's
// dogm/include/dogm/dogm_types.h:13-144 (GridCell 64 B, MeasurementCell 16 B, Particle,
// ParticlesSoA).  GLM is not required: vec4 is a 16-byte {x, y, z, w} POD with the
// glm::vec4 members this API uses (x, y, z, w, operator[], ==, +, scalar *).
#pragma once

#include <cstddef>
#include <cstdlib>
#include <cstring>

#include "../dogm_gb300.h"

namespace dogm
{

struct vec4
{
    float x, y, z, w;

    vec4() : x(0.f), y(0.f), z(0.f), w(0.f) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    float& operator[](int i) { return (&x)[i]; }
    const float& operator[](int i) const { return (&x)[i]; }
    bool operator==(const vec4& o) const { return x == o.x && y == o.y && z == o.z && w == o.w; }
    bool operator!=(const vec4& o) const { return !(*this == o); }
    vec4 operator+(const vec4& o) const { return vec4(x + o.x, y + o.y, z + o.z, w + o.w); }
};
inline vec4 operator*(float s, const vec4& v) { return vec4(s * v.x, s * v.y, s * v.z, s * v.w); }

struct vec2
{
    float x, y;
};

// dogm_types.h:13-33
struct GridCell
{
    int start_idx;
    int end_idx;
    float new_born_occ_mass;
    float pers_occ_mass;
    float free_mass;
    float occ_mass;
    float pred_occ_mass;
    float mu_A;
    float mu_UA;

    float w_A;
    float w_UA;

    float mean_x_vel;
    float mean_y_vel;
    float var_x_vel;
    float var_y_vel;
    float covar_xy_vel;
};

// dogm_types.h:35-41
struct MeasurementCell
{
    float free_mass;
    float occ_mass;
    float likelihood;
    float p_A;
};

// dogm_types.h:43-49
struct Particle
{
    int grid_cell_idx;
    float weight;
    bool associated;
    vec4 state;
};

static_assert(sizeof(GridCell) == sizeof(dogm_grid_cell), "GridCell layout");
static_assert(sizeof(MeasurementCell) == sizeof(dogm_measurement_cell), "MeasurementCell layout");
static_assert(sizeof(vec4) == 16, "vec4 layout");

// dogm_types.h:51-144: one memory block split as state | grid_cell_idx | weight | associated.
// Only host blocks are produced by this API (getParticles); the caller releases them with
// free(), as in the reference (dogm/test/dogm_spec.cpp:62-65).
struct ParticlesSoA
{
    vec4* state;
    int* grid_cell_idx;
    float* weight;
    bool* associated;

    void* memory_block;
    int size;
    bool device;

    ParticlesSoA() : state(nullptr), grid_cell_idx(nullptr), weight(nullptr), associated(nullptr),
                     memory_block(nullptr), size(0), device(false) {}

    ParticlesSoA(int new_size, bool is_device) { init(new_size, is_device); }

    void init(int new_size, bool is_device)
    {
        size = new_size;
        device = is_device;
        const size_t num_bytes = static_cast<size_t>(size) * sizeof(Particle);
        if (device)
        {
            memory_block = nullptr;
            dogm_device_alloc(&memory_block, num_bytes);
        }
        else
        {
            memory_block = std::malloc(num_bytes);
        }
        assignPointers();
    }

    void free()
    {
        if (device)
        {
            dogm_device_free(memory_block);
        }
        else
        {
            std::free(memory_block);
        }
        memory_block = nullptr;
        size = 0;
    }

private:
    void assignPointers()
    {
        state = reinterpret_cast<vec4*>(memory_block);
        grid_cell_idx = reinterpret_cast<int*>(state + size);
        weight = reinterpret_cast<float*>(grid_cell_idx + size);
        associated = reinterpret_cast<bool*>(weight + size);
    }
};

} /* namespace dogm */
