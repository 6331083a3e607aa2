// Measurement-grid generation from a lidar scan: the inverse sensor model in polar
// coordinates and the polar -> cartesian warp, as two CUDA kernels and no graphics API.
//
// The reference builds the grid in three steps (dogm/demo/simulator/mapping/
// laser_to_meas_grid.cu:25-70): a CUDA kernel writes the inverse sensor model of every
// (beam, range bin) into a float2 polar texture (kernel/measurement_grid.cu:73-89); OpenGL
// draws a triangle fan over the sensor's field of view whose fragment shader maps each pixel
// to polar texture coordinates and samples the texture (opengl/renderer.cpp:11-31,66-84,
// shader.cpp:22-35, texture.cpp:11-38); a CUDA kernel turns the framebuffer into
// MeasurementCells (measurement_grid.cu:115-132).  Here:
//   k_polar_ism   the inverse sensor model (measurement_grid.cu:33-71), or its Dempster-Shafer
//                 combination with the previous polar grid (fusePolarGridTextureKernel, :91-113);
//   k_polar_warp  the fan rasterised per cell: the fan triangle that covers the cell centre is
//                 found with exact integer edge functions (vertices snapped to 1/256 pixel, a
//                 top-left rule on shared edges), the texture coordinates are interpolated
//                 barycentrically, uv = (1 - s / (t + 1e-10), t) as in the fragment shader, and
//                 the polar grid is sampled bilinearly with border (0, 0).  The reference's
//                 mipmapped, 16x anisotropic texture fetch depends on the graphics driver and
//                 is not reproduced: level-0 bilinear filtering is used.
// The output rows are flipped as in cartesianGridToMeasurementGridKernel: the sensor sits at
// the centre of the last row, looking towards row 0.
#include <cmath>
#include <string>
#include <vector>

#include "dogm_internal.h"

namespace dogm_gb300 {
namespace {

constexpr float kMassEps = 0.00001f;  // measurement_grid.cu:79

__device__ __forceinline__ float clamp_mass(float m) { return fmaxf(kMassEps, fminf(1.0f - kMassEps, m)); }

// inverse_sensor_model (measurement_grid.cu:33-71) for range bin i of a beam that measured zk
__device__ __forceinline__ float2 inverse_sensor_model(int i, float resolution, float zk, int r_max, float sigma) {
    const float p_min = 0.15f, p_max = 1.0f;
    const float free = __fadd_rn(p_min, __fdiv_rn(__fmul_rn((float)i, __fsub_rn(p_max, p_min)), (float)r_max));
    if (isfinite(zk)) {
        const int r = (int)__fdiv_rn(zk, resolution);
        const float diff = __fmul_rn((float)(i - r), resolution);
        const float e = __fdiv_rn(__fmul_rn(__fmul_rn(-0.5f, diff), diff), __fmul_rn(sigma, sigma));
        const float occ = __fmul_rn(0.95f, expf(e));
        if (i <= r) return occ > free ? make_float2(occ, 0.0f) : make_float2(0.0f, __fsub_rn(1.0f, free));
        return occ > 0.5f ? make_float2(occ, 0.0f) : make_float2(0.0f, 0.0f);
    }
    return make_float2(0.0f, __fsub_rn(1.0f, free));
}

// combine_masses (measurement_grid.cu:14-30): Dempster's rule for {occ, free}
__device__ __forceinline__ float2 combine(float2 prior, float2 m) {
    const float unk = __fsub_rn(__fsub_rn(1.0f, prior.x), prior.y);
    const float m_unk = __fsub_rn(__fsub_rn(1.0f, m.x), m.y);
    const float K = __fadd_rn(__fmul_rn(prior.y, m.x), __fmul_rn(prior.x, m.y));
    const float den = __fsub_rn(1.0f, K);
    const float occ = __fadd_rn(__fadd_rn(__fmul_rn(prior.x, m_unk), __fmul_rn(unk, m.x)), __fmul_rn(prior.x, m.x));
    const float fre = __fadd_rn(__fadd_rn(__fmul_rn(prior.y, m_unk), __fmul_rn(unk, m.y)), __fmul_rn(prior.y, m.y));
    return make_float2(__fdiv_rn(occ, den), __fdiv_rn(fre, den));
}

// polar[bin * beams + beam]: texture row = range bin, column = beam (surf2Dwrite(x=theta, y=range))
__global__ void k_polar_ism(float2* __restrict__ polar, const float* __restrict__ ranges, int beams, int bins,
                            float resolution, float sigma, int fuse) {
    const int n = beams * bins;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int bin = k / beams, beam = k - bin * beams;
        float2 m = inverse_sensor_model(bin, resolution, ranges[beam], bins, sigma);
        m = make_float2(clamp_mass(m.x), clamp_mass(m.y));
        polar[k] = fuse ? combine(polar[k], m) : m;
    }
}

struct Fan {
    const long long* vx;  // vertex window coordinates x 256 (exact integers); [0] is the apex
    const long long* vy;
    const float* s;       // texture coordinate s of each vertex (t: 0 at the apex, 1 on the arc)
    int nv;               // apex + arc vertices
    int a0;               // angle (degrees) of arc vertex 1
};

// twice the signed area of (a, b, p), exact: coordinates are multiples of 1/256 below 2^13
__device__ __forceinline__ long long edge(long long ax, long long ay, long long bx, long long by, long long px,
                                          long long py) {
    return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}
// the edge a -> b of a counter-clockwise triangle owns the points on it when it is a left edge
// (going down) or a top edge (horizontal, going left): every point of a shared edge belongs to
// exactly one of the two triangles
__device__ __forceinline__ bool owns(long long e, long long ax, long long ay, long long bx, long long by) {
    return e > 0 || (e == 0 && (by < ay || (by == ay && bx < ax)));
}

__global__ void k_polar_warp(dogm_measurement_cell* __restrict__ out, const float2* __restrict__ polar, int beams,
                             int bins, int gs, Fan fan) {
    const int n = gs * gs;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int y = k / gs, x = k - y * gs;  // framebuffer pixel, y up
        const long long px = 256ll * x + 128, py = 256ll * y + 128;  // pixel centre x 256
        const long long cx = fan.vx[0], cy = fan.vy[0];
        float2 val = make_float2(0.0f, 0.0f);  // outside the fan: the clear colour (0, 0)
        if (py > cy || (py == cy && px != cx)) {
            // estimate of the fan triangle from the angle around the apex, then exact tests of
            // it and its neighbours
            const float ang = atan2f((float)(py - cy), (float)(px - cx)) * 57.29577951308232f;
            const int k0 = (int)floorf(ang) - fan.a0 + 1;
            for (int tri = max(1, k0 - 1); tri <= min(fan.nv - 2, k0 + 1); ++tri) {
                const long long ax = fan.vx[tri], ay = fan.vy[tri], bx = fan.vx[tri + 1], by = fan.vy[tri + 1];
                const long long e_ab = edge(ax, ay, bx, by, px, py);   // opposite the apex
                const long long e_bc = edge(bx, by, cx, cy, px, py);   // opposite vertex a
                const long long e_ca = edge(cx, cy, ax, ay, px, py);   // opposite vertex b
                if (!owns(e_ab, ax, ay, bx, by) || !owns(e_bc, bx, by, cx, cy) || !owns(e_ca, cx, cy, ax, ay))
                    continue;
                const float area = __ll2float_rn(edge(cx, cy, ax, ay, bx, by));
                const float la = __fdiv_rn(__ll2float_rn(e_bc), area);
                const float lb = __fdiv_rn(__ll2float_rn(e_ca), area);
                const float t = __fadd_rn(la, lb);
                const float s = __fadd_rn(__fmul_rn(la, fan.s[tri]), __fmul_rn(lb, fan.s[tri + 1]));
                const float u = __fsub_rn(1.0f, __fdiv_rn(s, __fadd_rn(t, 1e-10f)));  // shader.cpp:31
                const float v = t;
                // GL_LINEAR on level 0, GL_CLAMP_TO_BORDER with border (0, 0)
                const float xs = __fsub_rn(__fmul_rn(u, (float)beams), 0.5f);
                const float ys = __fsub_rn(__fmul_rn(v, (float)bins), 0.5f);
                const float fx = floorf(xs), fy = floorf(ys);
                const float a = __fsub_rn(xs, fx), b = __fsub_rn(ys, fy);
                const int i0 = (int)fx, j0 = (int)fy;
                float2 tx[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int i = i0 + (q & 1), j = j0 + (q >> 1);
                    tx[q] = (i >= 0 && i < beams && j >= 0 && j < bins) ? polar[(size_t)j * beams + i]
                                                                       : make_float2(0.0f, 0.0f);
                }
                const float w00 = __fmul_rn(__fsub_rn(1.0f, a), __fsub_rn(1.0f, b));
                const float w10 = __fmul_rn(a, __fsub_rn(1.0f, b));
                const float w01 = __fmul_rn(__fsub_rn(1.0f, a), b);
                const float w11 = __fmul_rn(a, b);
                val.x = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w00, tx[0].x), __fmul_rn(w10, tx[1].x)),
                                            __fmul_rn(w01, tx[2].x)), __fmul_rn(w11, tx[3].x));
                val.y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w00, tx[0].y), __fmul_rn(w10, tx[1].y)),
                                            __fmul_rn(w01, tx[2].y)), __fmul_rn(w11, tx[3].y));
                break;
            }
        }
        dogm_measurement_cell c;
        c.occ_mass = val.x;    // red
        c.free_mass = val.y;   // green
        c.likelihood = 1.0f;   // measurement_grid.cu:129-130
        c.p_A = 1.0f;
        out[(size_t)(gs - 1 - y) * gs + x] = c;  // rows flipped (measurement_grid.cu:119)
    }
}

}  // namespace
}  // namespace dogm_gb300

using namespace dogm_gb300;

struct dogm_meas_grid {
    dogm_laser_params p{};
    int device = 0, num_sms = 0;
    int gs = 0, beams = 0, bins = 0;
    float2* polar = nullptr;
    float* ranges = nullptr;
    long long* vx = nullptr;
    long long* vy = nullptr;
    float* s = nullptr;
    int nv = 0, a0 = 0;
    std::vector<long long> hvx, hvy;
    std::vector<float> hs;
    bool have_polar = false;
};

namespace {

thread_local std::string g_err;
dogm_status mfail(dogm_status s, const std::string& m) {
    g_err = m;
    set_last_error(g_err.c_str());
    return s;
}

#define MCUDA(call)                                                                             \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) return mfail(DOGM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// The fan of generateCircleSegmentVertices (opengl/renderer.cpp:11-31) in window coordinates:
// apex at NDC (0, -1) -- the bottom centre of the viewport -- and one arc vertex per whole degree
// from int(90 - fov/2) while <= 90 + fov/2, radius 2 * max_range / grid_length in NDC; NDC x maps
// to window (x + 1) * gs / 2 (glViewport(0, 0, gs, gs)); coordinates snapped to 1/256 pixel.
void build_fan(dogm_meas_grid* m, float grid_length) {
    const float fov = m->p.fov;
    const float half = fov / 2;
    const float start = 90 - half, end = 90 + half;
    const float radius = 2.0f * (m->p.max_range / grid_length);
    const float cx = 0.0f, cy = -1.0f;
    const float half_gs = (float)m->gs / 2.0f;
    auto snap = [&](float ndc) { return (long long)std::llround((double)((ndc + 1.0f) * half_gs) * 256.0); };
    m->hvx.assign(1, snap(cx));
    m->hvy.assign(1, snap(cy));
    m->hs.assign(1, 0.0f);
    m->a0 = (int)start;
    for (int angle = (int)start; angle <= end; angle++) {
        const float rad = (float)(angle * 3.14159265358979323846 / 180.0f);  // angle * M_PI / 180.0f
        const float xv = std::cos(rad), yv = std::sin(rad);
        m->hvx.push_back(snap(cx + radius * xv));
        m->hvy.push_back(snap(cy + radius * yv));
        m->hs.push_back((angle - start) / fov);
    }
    m->nv = (int)m->hvx.size();
}

}  // namespace

extern "C" {

dogm_status dogm_meas_grid_create(const dogm_laser_params* p, float grid_length, float grid_resolution, int beams,
                                  dogm_meas_grid** out) {
    if (!p || !out) return mfail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (!(p->max_range > 0.f) || !(p->resolution > 0.f) || !(p->fov > 0.f) || p->fov > 360.f ||
        !(p->stddev_range > 0.f) || !(grid_length > 0.f) || !(grid_resolution > 0.f) || beams < 1)
        return mfail(DOGM_ERR_INVALID_ARGUMENT, "laser parameters, grid length and resolution must be > 0");
    const int gs = (int)(grid_length / grid_resolution);  // laser_to_meas_grid.cu:11
    const int bins = (int)(p->max_range / p->resolution);  // laser_to_meas_grid.cu:41
    if (gs < 1 || gs > 8192 || bins < 1) return mfail(DOGM_ERR_UNSUPPORTED, "grid or polar size out of range");
    dogm_meas_grid* m = new dogm_meas_grid();
    m->p = *p;
    m->gs = gs;
    m->beams = beams;
    m->bins = bins;
    build_fan(m, grid_length);
    auto cleanup = [&](dogm_status st) { dogm_meas_grid_destroy(m); return st; };
    if (cudaGetDevice(&m->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, m->device) != cudaSuccess)
        return cleanup(mfail(DOGM_ERR_CUDA, "no CUDA device"));
    if (cudaMalloc(&m->polar, sizeof(float2) * (size_t)beams * bins) != cudaSuccess ||
        cudaMalloc(&m->ranges, sizeof(float) * (size_t)beams) != cudaSuccess ||
        cudaMalloc(&m->vx, sizeof(long long) * m->nv) != cudaSuccess ||
        cudaMalloc(&m->vy, sizeof(long long) * m->nv) != cudaSuccess ||
        cudaMalloc(&m->s, sizeof(float) * m->nv) != cudaSuccess)
        return cleanup(mfail(DOGM_ERR_OUT_OF_MEMORY, "measurement-grid buffers"));
    if (cudaMemcpy(m->vx, m->hvx.data(), sizeof(long long) * m->nv, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(m->vy, m->hvy.data(), sizeof(long long) * m->nv, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(m->s, m->hs.data(), sizeof(float) * m->nv, cudaMemcpyHostToDevice) != cudaSuccess)
        return cleanup(mfail(DOGM_ERR_CUDA, "fan upload"));
    *out = m;
    return DOGM_OK;
}

dogm_status dogm_meas_grid_destroy(dogm_meas_grid* m) {
    if (!m) return DOGM_OK;
    for (void* q : {(void*)m->polar, (void*)m->ranges, (void*)m->vx, (void*)m->vy, (void*)m->s})
        if (q) cudaFree(q);
    delete m;
    return DOGM_OK;
}

dogm_status dogm_meas_grid_generate(dogm_meas_grid* m, const float* ranges, int device, int fuse,
                                    dogm_measurement_cell* out_device, void* stream) {
    if (!m || !ranges || !out_device) return mfail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (fuse && !m->have_polar) return mfail(DOGM_ERR_NOT_READY, "fuse needs a previous scan");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const float* r = ranges;
    if (!device) {
        MCUDA(cudaMemcpyAsync(m->ranges, ranges, sizeof(float) * m->beams, cudaMemcpyHostToDevice, s));
        r = m->ranges;
    }
    const int blocks = m->num_sms * 8;
    k_polar_ism<<<blocks, 256, 0, s>>>(m->polar, r, m->beams, m->bins, m->p.resolution, m->p.stddev_range, fuse);
    MCUDA(cudaGetLastError());
    Fan fan{m->vx, m->vy, m->s, m->nv, m->a0};
    k_polar_warp<<<blocks, 256, 0, s>>>(out_device, m->polar, m->beams, m->bins, m->gs, fan);
    MCUDA(cudaGetLastError());
    MCUDA(cudaStreamSynchronize(s));  // the host range buffer is reused by the next call
    m->have_polar = true;
    return DOGM_OK;
}

int dogm_meas_grid_size(const dogm_meas_grid* m) { return m ? m->gs : 0; }

dogm_status dogm_meas_grid_polar(dogm_meas_grid* m, float* host_out, size_t n, int* beams, int* bins) {
    if (!m) return mfail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (beams) *beams = m->beams;
    if (bins) *bins = m->bins;
    if (host_out) {
        if (n < (size_t)2 * m->beams * m->bins) return mfail(DOGM_ERR_INVALID_ARGUMENT, "n < 2 x beams x bins");
        MCUDA(cudaMemcpy(host_out, m->polar, sizeof(float2) * (size_t)m->beams * m->bins, cudaMemcpyDeviceToHost));
    }
    return DOGM_OK;
}

dogm_status dogm_meas_grid_fan(dogm_meas_grid* m, long long* x256, long long* y256, float* s, int n, int* nv,
                               int* first_angle) {
    if (!m) return mfail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (nv) *nv = m->nv;
    if (first_angle) *first_angle = m->a0;
    if (n < m->nv) return (x256 || y256 || s) ? mfail(DOGM_ERR_INVALID_ARGUMENT, "n < vertices") : DOGM_OK;
    for (int i = 0; i < m->nv; ++i) {
        if (x256) x256[i] = m->hvx[i];
        if (y256) y256[i] = m->hvy[i];
        if (s) s[i] = m->hs[i];
    }
    return DOGM_OK;
}

}  // extern "C"
