// Dynamic-cell extraction on the GPU: the cells a consumer of the grid reads after an update.
//
// The reference does this on the host after copying the whole grid back
// (computeCellsWithVelocity, dogm/demo/utils/image_creation.cpp:19-66): a cell is kept when its
// pignistic occupancy occ + (1 - occ - free) / 2 reaches a threshold and the Mahalanobis length of
// its mean velocity under the velocity covariance, v^T Sigma^-1 v, reaches another.  Here one
// pass flags the cells and counts them per 1024-cell tile, a second writes the kept cells in
// row-major order (the reference's loop order) to a compact device array, and only that array
// crosses to the host.  The 2 x 2 inverse is the closed form in a fixed FP32 order; a singular
// covariance gives 0 (OpenCV's LU inverse returns a zero matrix for it).
#include <algorithm>
#include <string>
#include <vector>

#include "dogm_internal.h"

namespace dogm_gb300 {
namespace {

constexpr int kExtractTile = 1024;
constexpr int kExtractThreads = 256;
constexpr int kExtractIpt = kExtractTile / kExtractThreads;

struct Flagged {
    float occ, maha;
    bool keep;
};

__device__ __forceinline__ Flagged flag_cell(const dogm_grid_cell& c, float min_occ, float min_vel) {
    Flagged f;
    // pignistic_transformation (image_creation.cpp:19-22)
    f.occ = __fadd_rn(c.occ_mass, __fmul_rn(0.5f, __fsub_rn(__fsub_rn(1.0f, c.occ_mass), c.free_mass)));
    const float det = __fsub_rn(__fmul_rn(c.var_x_vel, c.var_y_vel), __fmul_rn(c.covar_xy_vel, c.covar_xy_vel));
    float m = 0.0f;
    if (det != 0.0f) {
        // v^T Sigma^-1 v = (vy mx^2 - 2 c mx my + vx my^2) / det
        const float mx = c.mean_x_vel, my = c.mean_y_vel;
        const float q = __fadd_rn(__fsub_rn(__fmul_rn(c.var_y_vel, __fmul_rn(mx, mx)),
                                            __fmul_rn(2.0f, __fmul_rn(c.covar_xy_vel, __fmul_rn(mx, my)))),
                                  __fmul_rn(c.var_x_vel, __fmul_rn(my, my)));
        m = __fdiv_rn(q, det);
    }
    f.maha = m;
    f.keep = f.occ >= min_occ && m >= min_vel;
    return f;
}

__global__ void __launch_bounds__(kExtractThreads) k_extract_count(const dogm_grid_cell* __restrict__ cells, int C,
                                                                   float min_occ, float min_vel,
                                                                   unsigned int* __restrict__ tile_count) {
    __shared__ unsigned int red[kExtractThreads / 32];
    const int tiles = (C + kExtractTile - 1) / kExtractTile;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
        unsigned int n = 0;
#pragma unroll
        for (int r = 0; r < kExtractIpt; ++r) {
            const int k = t * kExtractTile + r * kExtractThreads + threadIdx.x;
            if (k < C) n += flag_cell(cells[k], min_occ, min_vel).keep ? 1u : 0u;
        }
        for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = n;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned int s = 0;
            for (int w = 0; w < kExtractThreads / 32; ++w) s += red[w];
            tile_count[t] = s;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kExtractThreads) k_extract_write(const dogm_grid_cell* __restrict__ cells, int C,
                                                                   int gs, float min_occ, float min_vel,
                                                                   const unsigned int* __restrict__ tile_count,
                                                                   dogm_dynamic_cell* __restrict__ out, int max_out) {
    __shared__ unsigned int wsum[kExtractThreads / 32];
    __shared__ unsigned int base_s;
    const int tiles = (C + kExtractTile - 1) / kExtractTile;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
        if (tile_count[t] == 0u) continue;  // block-uniform
        // first output slot of the tile: the counts of the tiles before it
        unsigned int part = 0;
        for (int i = threadIdx.x; i < t; i += kExtractThreads) part += tile_count[i];
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        if (lane == 0) wsum[warp] = part;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned int s = 0;
            for (int w = 0; w < kExtractThreads / 32; ++w) s += wsum[w];
            base_s = s;
        }
        __syncthreads();
        unsigned int base = base_s;
        // cells in row-major order: thread-chunks of the tile in order, lanes in order
        for (int r = 0; r < kExtractIpt; ++r) {
            const int k = t * kExtractTile + r * kExtractThreads + threadIdx.x;
            Flagged f{0.0f, 0.0f, false};
            dogm_grid_cell c;
            if (k < C) {
                c = cells[k];
                f = flag_cell(c, min_occ, min_vel);
            }
            const unsigned int ballot = __ballot_sync(0xffffffffu, f.keep);
            if (lane == 0) wsum[warp] = __popc(ballot);
            __syncthreads();
            unsigned int before = 0, total = 0;
            for (int w = 0; w < kExtractThreads / 32; ++w) {
                const unsigned int s = wsum[w];
                if (w < warp) before += s;
                total += s;
            }
            if (f.keep) {
                const unsigned int slot = base + before + __popc(ballot & ((1u << lane) - 1u));
                if ((int)slot < max_out) {
                    dogm_dynamic_cell d;
                    d.index = k;
                    const int y = k / gs;
                    d.x = (float)(k - y * gs);  // grid indices, as image_creation.cpp:53-54
                    d.y = (float)y;
                    d.occupancy = f.occ;
                    d.mahalanobis = f.maha;
                    d.cell = c;
                    out[slot] = d;
                }
            }
            base += total;
            __syncthreads();
        }
    }
}

}  // namespace
}  // namespace dogm_gb300

using namespace dogm_gb300;

extern "C" dogm_status dogm_extract_dynamic_cells_device(const dogm_grid_cell* cells, int grid_size,
                                                         float min_occupancy, float min_velocity,
                                                         dogm_dynamic_cell* out, int max_out, unsigned int* scratch,
                                                         int* n_out, void* stream) {
    if (!cells || !out || !scratch || !n_out || grid_size < 1 || grid_size > 8192 || max_out < 0) {
        set_last_error("dogm_extract_dynamic_cells_device: bad argument");
        return DOGM_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int C = grid_size * grid_size;
    const int tiles = (C + kExtractTile - 1) / kExtractTile;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = std::min(tiles, sms * 8);
    k_extract_count<<<blocks, kExtractThreads, 0, s>>>(cells, C, min_occupancy, min_velocity, scratch);
    k_extract_write<<<blocks, kExtractThreads, 0, s>>>(cells, C, grid_size, min_occupancy, min_velocity, scratch, out,
                                                       max_out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        return DOGM_ERR_CUDA;
    }
    // total = sum of the tile counts, read back for the caller
    std::vector<unsigned int> cnt(tiles);
    e = cudaMemcpyAsync(cnt.data(), scratch, sizeof(unsigned int) * tiles, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        return DOGM_ERR_CUDA;
    }
    long long total = 0;
    for (unsigned int c : cnt) total += c;
    *n_out = (int)total;
    return DOGM_OK;
}
