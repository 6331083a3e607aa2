// Particle-side kernels: frame begin, prediction (with the fused ego shift), first-frame
// particle initialisation, the stand-alone shift stage and Philox draw export.
#include "dogm_device.cuh"

namespace dogm_gb300 {

// ---------------------------------------------------------------------------------------
// Frame begin: zero the per-frame scratch of every grid in the batch.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_frame_begin(Batch* __restrict__ bt) {
    const int stride = gridDim.x * blockDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    for (int gi = 0; gi < bt->n_grids; ++gi) {
        const GridDesc& g = bt->g[gi];
        for (int i = tid; i < g.ctiles; i += stride) g.ctile_cnt[i] = 0u;
        for (int i = tid; i < g.ctiles + g.tiles[kStBirth]; i += stride) g.cell_sum[i] = 0ull;
        for (int i = tid; i < g.tiles[kStResample]; i += stride) g.res_sum[i] = 0ull;
        // (the per-tile bucket counts are written whole each frame)
        if (tid == 0) {
            g.fs->status = 0u;
            g.fs->qb_total = 0ull;
            g.fs->joint_total = 0ull;
            g.fs->qo_total = 0ull;
            g.fs->n_birth = 0;
        }
    }
}

// ---------------------------------------------------------------------------------------
// Prediction (dogm/src/kernel/predict.cu:12-48), fused with the particle half of the ego
// shift (dogm/src/kernel/ego_motion_compensation.cu:16-23).
//   s' = F s + noise, F = [[1,0,dt,0],[0,1,0,dt],[0,0,1,0],[0,0,0,1]]
// evaluated as x' = (x + dt*vx) + n_x (the grouping of the reference's mat4 x vec4);
// the weight is not stored per particle: every persistent particle carries the common
// weight w_res, so the predicted weight is p_S * w_res, or 0 out of the grid (bit 30).
// Each 4096-particle tile also counts its particles per bucket of the sort (2^bucket_bits
// cells): the row of the tile is written whole, the grid's totals are added to ctile_cnt.
// mode 0: full frame (shift + bucket counts); mode 1: particlePrediction stage call (no
// counts); mode 2: particleAssignment stage call (bucket counts of the resident keys only).
// ---------------------------------------------------------------------------------------
// 512 threads per 4096-particle tile (8 particles each): the kernel is issue-bound, and twice
// the warps of a 256-thread block keep about 50 warps per SM in flight over the frame's tiles.
constexpr int kPredictThreads = 512;
static_assert(kPredictTile % kPredictThreads == 0, "whole particles per thread");

template <bool FINE, class View>
__device__ __forceinline__ void predict_body(const View& v, int mode, uint32_t* h2) {
    const int total = v.total(kStPredict);
    const bool counts = mode != 1;
    if (counts) {
        // this frame's exact sums start at zero: the cell and newborn passes add into them
        // after this kernel, and the last reader (the previous frame's resampling) is done
        const int stride = gridDim.x * blockDim.x;
        const int tid = blockIdx.x * blockDim.x + threadIdx.x;
        for (int gi = 0; gi < v.n(); ++gi) {
            const GridDesc& g = v.g(gi);
            for (int i = tid; i < g.tiles[kStResample]; i += stride) g.res_sum[i] = 0ull;
                if (tid == 0) {
                g.fs->status = 0u;
                g.fs->qb_total = 0ull;
                g.fs->joint_total = 0ull;
            }
        }
    }
    const int lane = threadIdx.x & 31;
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int gi = v.grid(kStPredict, t);
        const GridDesc& g = v.g(gi);
        const int lt = t - v.first(gi, kStPredict);
        if (counts) {
            for (int i = threadIdx.x; i < g.ctiles; i += kPredictThreads) h2[i] = 0u;
            __syncthreads();
        }
        const float gsm1 = (float)(g.gs - 1);
        const float dt = g.dt;
        const bool shift = (mode == 0) && g.shifted;
        const float fsx = (float)g.shift_x, fsy = (float)g.shift_y;
        const int base = lt * kPredictTile;
#pragma unroll
        for (int k = 0; k < kPredictTile / kPredictThreads; ++k) {
            const int i = base + k * kPredictThreads + threadIdx.x;
            bool valid = i < g.N;
            uint32_t key = 0xffffffffu;
            if (valid && mode == 2) {
                key = g.P_key[i] & kCellMask;
                valid = key < (uint32_t)g.C;  // injected keys outside the grid are not counted
            } else if (valid) {
                float4 s = g.P_state[i];
                const uint32_t kw = g.P_key[i];
                if (shift) {
                    s.x = __fsub_rn(s.x, fsx);
                    s.y = __fsub_rn(s.y, fsy);
                }
                float4 z;
                if (g.rp_predict) {
                    z = g.rp_predict[i];
                } else {
                    const U4 r = draw_block(g, (uint32_t)i, g.frame, kDrawPredict);
                    const float2 a = box_muller(r.x, r.y);
                    const float2 b = box_muller(r.z, r.w);
                    z = make_float4(a.x, a.y, b.x, b.y);
                }
                const float nx = __fmaf_rn(z.x, g.sigma_pos, 0.0f);
                const float ny = __fmaf_rn(z.y, g.sigma_pos, 0.0f);
                const float nvx = __fmaf_rn(z.z, g.sigma_vel, 0.0f);
                const float nvy = __fmaf_rn(z.w, g.sigma_vel, 0.0f);
                float4 o;
                o.x = __fadd_rn(__fadd_rn(s.x, __fmul_rn(dt, s.z)), nx);
                o.y = __fadd_rn(__fadd_rn(s.y, __fmul_rn(dt, s.w)), ny);
                o.z = __fadd_rn(s.z, nvx);
                o.w = __fadd_rn(s.w, nvy);
                const bool out = (o.x > gsm1) || (o.x < 0.0f) || (o.y > gsm1) || (o.y < 0.0f);
                const int px = min(max(__float2int_rz(o.x), 0), g.gs - 1);
                const int py = min(max(__float2int_rz(o.y), 0), g.gs - 1);
                key = (uint32_t)(px + g.gs * py);
                g.P_state[i] = o;
                g.P_key[i] = key | (out ? kOutBit : 0u) | (kw & kAssocBit);
            }
            if (counts) {
                const uint32_t bucket = valid ? key >> (FINE ? g.bucket_bits : kCellTileBits) : 0xffffffffu;
                const uint32_t peers = __match_any_sync(0xffffffffu, bucket);
                if (valid && lane == __ffs(peers) - 1) atomicAdd(&h2[bucket], (uint32_t)__popc(peers));
            }
        }
        if (counts) {
            __syncthreads();
            // this tile's bucket counts (predict and scatter tiles coincide), row written whole
            uint32_t* row = g.hsort + (size_t)lt * g.bucket_stride;
            for (int i = threadIdx.x; i < g.ctiles; i += kPredictThreads) {
                const uint32_t c = h2[i];
                row[i] = c;
                if (c) atomicAdd(&g.ctile_cnt[i], c);
            }
            __syncthreads();
        }
    }
}


// The frame's descriptors as the device batch holds them, or as one grid's kernel parameter.
struct BatchView {
    const Batch* b;
    __device__ int n() const { return b->n_grids; }
    __device__ int total(int s) const { return batch_total(b, s); }
    __device__ int grid(int s, int t) const { return grid_of_tile(b, s, t); }
    __device__ int first(int gi, int s) const { return b->prefix[gi][s]; }
    __device__ const GridDesc& g(int gi) const { return b->g[gi]; }
};
struct ParamView {
    const FrameParam* p;
    __device__ int n() const { return 1; }
    __device__ int total(int s) const { return p->tiles[s]; }
    __device__ int grid(int, int) const { return 0; }
    __device__ int first(int, int) const { return 0; }
    __device__ const GridDesc& g(int) const { return p->g; }
};

// Writes a one-grid frame from predict's parameter into the device batch, for the kernels after
// predict (they wait for predict to finish before reading it).  Block 0, after the wait for the
// previous kernel, so no earlier kernel still reads the batch.
__device__ void publish_frame(Batch* bt, const FrameParam& fp) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&fp.g);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&bt->g[0]);
    static_assert(sizeof(GridDesc) % 4 == 0, "descriptor copied in words");
    for (int i = threadIdx.x; i < (int)(sizeof(GridDesc) / 4); i += blockDim.x) dst[i] = src[i];
    if (threadIdx.x < kNumStages) {
        bt->counters[threadIdx.x] = 0u;
        bt->prefix[0][threadIdx.x] = 0;
        bt->prefix[1][threadIdx.x] = fp.tiles[threadIdx.x];
    }
    if (threadIdx.x == 0) {
        bt->n_grids = 1;
        bt->status = 0u;
        bt->status_host = fp.status_host;
    }
}

// FINE: some grid of the launch sorts by buckets finer than a cell tile.
template <bool FINE>
__global__ void __launch_bounds__(kPredictThreads, 3) k_predict(Batch* __restrict__ bt, int mode,
                                                             const __grid_constant__ FrameParam fp) {
    grid_dependency_begin();
    __shared__ uint32_t h2[kMaxCellTiles];  // particles per cell tile (bucket of the sort)
    if (fp.valid) {
        if (blockIdx.x == 0) publish_frame(bt, fp);
        predict_body<FINE>(ParamView{&fp}, mode, h2);
    } else {
        predict_body<FINE>(BatchView{bt}, mode, h2);
    }
}

// ---------------------------------------------------------------------------------------
// First frame: particles spread over the cells in proportion to the measured occupied
// mass (dogm/src/dogm.cu:217-241, init_new_particles.cu:76-124).  The proportional
// allocation is an exact fixed-point scan instead of a float scan scaled by N / total.
// An all-zero measurement spreads the particles uniformly (the reference divides by 0).
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_init_scan(Batch* __restrict__ bt) {
    __shared__ unsigned long long red[kThreads / 32];
    const int total = batch_total(bt, kStInitScan);
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int gi = grid_of_tile(bt, kStInitScan, t);
        const GridDesc& g = bt->g[gi];
        const int lt = t - bt->prefix[gi][kStInitScan];
        const int base = lt * kCellTile;
        unsigned long long v = 0ull;
        for (int j = 0; j < kCellIpt; ++j) {
            const int k = base + threadIdx.x * kCellIpt + j;
            if (k < g.C) v += quantize(g.meas_src[k].occ_mass, g.q_shift);
        }
        unsigned long long tile_sum;
        block_excl_scan_u64(v, red, &tile_sum);
        if (threadIdx.x == 0) {
            g.cell_sum[g.tiles[kStCell] + lt] = tile_sum;  // second half: first-frame masses
            atomicAdd(&g.fs->qo_total, tile_sum);
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_init_expand(Batch* __restrict__ bt) {
    __shared__ unsigned long long red[kThreads / 32];
    __shared__ int bnd[kCellTile + 1];  // bnd[0] = first slot of the tile, bnd[1+c] = end of cell c
    const int total = batch_total(bt, kStInitExpand);
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int gi = grid_of_tile(bt, kStInitExpand, t);
        const GridDesc& g = bt->g[gi];
        const int lt = t - bt->prefix[gi][kStInitExpand];
        const unsigned long long T = g.fs->qo_total;
        const bool uniform = (T == 0ull);
        const int base = lt * kCellTile;
        unsigned long long q[kCellIpt];
        unsigned long long v = 0ull;
        for (int j = 0; j < kCellIpt; ++j) {
            const int k = base + threadIdx.x * kCellIpt + j;
            q[j] = (k < g.C) ? (uniform ? 1ull : quantize(g.meas_src[k].occ_mass, g.q_shift)) : 0ull;
            v += q[j];
        }
        unsigned long long tile_sum;
        unsigned long long pre = block_excl_scan_u64(v, red, &tile_sum);
        unsigned long long tile_excl = (unsigned long long)base;
        if (!uniform) tile_excl = block_sum_before(g.cell_sum + g.tiles[kStCell], lt, red);
        const unsigned long long TT = uniform ? (unsigned long long)g.C : T;
        if (threadIdx.x == 0) bnd[0] = alloc_boundary(tile_excl, TT, g.N);
        unsigned long long acc = tile_excl + pre;
        for (int j = 0; j < kCellIpt; ++j) {
            acc += q[j];
            bnd[1 + threadIdx.x * kCellIpt + j] = alloc_boundary(acc, TT, g.N);
        }
        __syncthreads();
        const int ncell = min(kCellTile, g.C - base);
        const int lo = bnd[0], hi = bnd[ncell];
        const float vmax = g.init_max_vel;
        const float span = __fsub_rn(vmax, -vmax);
        for (int s = lo + threadIdx.x; s < hi; s += kThreads) {
            int a = 0, b = ncell - 1;  // first cell c with bnd[1+c] > s
            while (a < b) {
                const int m = (a + b) >> 1;
                if (bnd[1 + m] > s) b = m; else a = m + 1;
            }
            const int k = base + a;
            float2 u;
            if (g.rp_init) {
                u = g.rp_init[s];
            } else {
                const U4 r = draw_block(g, (uint32_t)s, 0u, kDrawInit);
                u = make_float2(u01_open0(r.x), u01_open0(r.y));
            }
            float4 st;
            st.x = __fadd_rn((float)(k % g.gs), 0.5f);
            st.y = __fadd_rn((float)(k / g.gs), 0.5f);
            st.z = __fmaf_rn(span, __fsub_rn(1.0f, u.x), -vmax);
            st.w = __fmaf_rn(span, __fsub_rn(1.0f, u.y), -vmax);
            g.P_state[s] = st;
            g.P_key[s] = (uint32_t)k;
        }
        if (lt == 0 && threadIdx.x == 0) g.fs->w_res = __fdiv_rn(1.0f, (float)g.N);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------
// Stand-alone ego shift (the stage call; the update fuses it into predict and cells):
// particles x -= x_move (ego_motion_compensation.cu:16-23) and the cell records moved by
// (x_move, y_move) with the strict 0 < x,y bounds of ego_motion_compensation.cu:38.
// ---------------------------------------------------------------------------------------
__global__ void k_shift_particles(float4* st, int n, float fx, float fy) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 s = st[i];
        s.x = __fsub_rn(s.x, fx);
        s.y = __fsub_rn(s.y, fy);
        st[i] = s;
    }
}

__global__ void k_shift_cells(dogm_grid_cell* cells, const dogm_grid_cell* old_cells, float* free_new,
                              const float* free_old, int gs, int xm, int ym) {
    const int C = gs * gs;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < C; k += gridDim.x * blockDim.x) {
        const int x = k % gs, y = k / gs;
        const int nx = x + xm, ny = y + ym;
        const bool ok = nx > 0 && nx < gs && ny > 0 && ny < gs;
        dogm_grid_cell c;
        float f = 0.0f;
        if (ok) {
            c = old_cells[nx + gs * ny];
            f = free_old[nx + gs * ny];
        } else {
            memset(&c, 0, sizeof(c));
        }
        cells[k] = c;
        free_new[k] = f;
    }
}

// ---------------------------------------------------------------------------------------
// Philox draw export: exactly the numbers the kernels above draw at `iteration`.
// ---------------------------------------------------------------------------------------
__global__ void k_draws(GridDesc g, uint32_t frame, float2* init_u, float4* predict_z, float2* birth_z,
                        unsigned long long* resample_r) {
    const int stride = gridDim.x * blockDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    for (int i = tid; i < g.N; i += stride) {
        if (init_u) {
            const U4 r = draw_block(g, (uint32_t)i, 0u, kDrawInit);
            init_u[i] = make_float2(u01_open0(r.x), u01_open0(r.y));
        }
        if (predict_z) {
            const U4 r = draw_block(g, (uint32_t)i, frame, kDrawPredict);
            const float2 a = box_muller(r.x, r.y);
            const float2 b = box_muller(r.z, r.w);
            predict_z[i] = make_float4(a.x, a.y, b.x, b.y);
        }
    }
    if (birth_z)
        for (int i = tid; i < g.B; i += stride) {
            const U4 r = draw_block(g, (uint32_t)i, frame, kDrawBirth);
            birth_z[i] = box_muller(r.x, r.y);
        }
    if (resample_r && tid == 0) {
        const U4 r = draw_block(g, 0u, frame, kDrawResample);
        *resample_r = ((unsigned long long)r.x << 32) | r.y;
    }
}

// ---------------------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------------------
cudaError_t launch_frame_begin(const Batch* d_batch, int n_grids, const LaunchCfg& cfg) {
    (void)n_grids;
    k_frame_begin<<<cfg.num_sms * 2, kThreads, 0, cfg.stream>>>(const_cast<Batch*>(d_batch));
    return cudaGetLastError();
}

cudaError_t launch_predict(const Batch* d_batch, int stage_mode, const LaunchCfg& cfg, const FrameParam* fp,
                           bool fine) {
    FrameParam none{};
    if (fine)
        return launch_kernel(cfg, k_predict<true>, launch_blocks(cfg, 3), kPredictThreads, 0,
                             const_cast<Batch*>(d_batch), stage_mode, fp ? *fp : none);
    return launch_kernel(cfg, k_predict<false>, launch_blocks(cfg, 3), kPredictThreads, 0, const_cast<Batch*>(d_batch),
                         stage_mode, fp ? *fp : none);
}

cudaError_t launch_init_particles(const Batch* d_batch, const LaunchCfg& cfg) {
    k_init_scan<<<cfg.num_sms * 4, kThreads, 0, cfg.stream>>>(const_cast<Batch*>(d_batch));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_init_expand<<<cfg.num_sms * 4, kThreads, 0, cfg.stream>>>(const_cast<Batch*>(d_batch));
    return cudaGetLastError();
}

cudaError_t launch_shift_stage(const GridDesc& g, int x_move, int y_move, const LaunchCfg& cfg) {
    k_shift_particles<<<cfg.num_sms * 4, kThreads, 0, cfg.stream>>>(g.P_state, g.N, (float)x_move, (float)y_move);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    dogm_grid_cell* old_cells = nullptr;
    e = cudaMallocAsync((void**)&old_cells, sizeof(dogm_grid_cell) * (size_t)g.C, cfg.stream);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(old_cells, g.cells, sizeof(dogm_grid_cell) * (size_t)g.C, cudaMemcpyDeviceToDevice,
                        cfg.stream);
    if (e != cudaSuccess) return e;
    k_shift_cells<<<cfg.num_sms * 4, kThreads, 0, cfg.stream>>>(g.cells, old_cells, g.free_new, g.free_old, g.gs,
                                                                 x_move, y_move);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaFreeAsync(old_cells, cfg.stream);
}

// ---------------------------------------------------------------------------------------
// Allocation-free shift stage.
//
// Some callers may not allocate device memory once they are running: a real-time loop whose
// device memory is fixed at start-up, or a process whose free device memory is held by
// another allocator (a framework's caching allocator, a fixed arena), where the temporary
// cudaMallocAsync of launch_shift_stage can stall or fail in mid-run.  This variant copies
// the previous cell records into a fixed device array compiled into the library instead.
//
// The array is one per device (per CUDA context) and every call shares it; it keeps the
// contents of the last call.  Nothing in it has to start at zero: the copy overwrites the
// first C records before k_shift_cells reads them, and nothing past them is read.  Calls
// whose work overlaps on the GPU (two host threads shifting two grids at once) race on the
// array, so such callers must serialise them.
// ---------------------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_shift_scratch[kShiftScratchBytes];

// Device address of g_shift_scratch in the current device's context.  In host code the
// array's name is only a host-side stand-in, so the address is asked for with that device
// current.  It is looked up on every call rather than cached: the lookup allocates nothing,
// and a context created anew (after cudaDeviceReset) loads the module again at another
// address, which a cache keyed by the device ordinal would miss.
cudaError_t shift_scratch_address(void** out) {
    *out = nullptr;
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_shift_scratch);
    if (e != cudaSuccess) return e;
    *out = p;
    return cudaSuccess;
}

cudaError_t shift_scratch_setup() {
    void* p;
    return shift_scratch_address(&p);
}

cudaError_t launch_shift_stage_noalloc(const GridDesc& g, int x_move, int y_move, const LaunchCfg& cfg) {
    const size_t bytes = sizeof(dogm_grid_cell) * (size_t)g.C;
    if (bytes > kShiftScratchBytes) return cudaErrorInvalidValue;  // the caller checks first
    void* scratch = nullptr;
    cudaError_t e = shift_scratch_address(&scratch);
    if (e != cudaSuccess) return e;
    dogm_grid_cell* old_cells = static_cast<dogm_grid_cell*>(scratch);
    k_shift_particles<<<cfg.num_sms * 4, kThreads, 0, cfg.stream>>>(g.P_state, g.N, (float)x_move, (float)y_move);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    e = cudaMemcpyAsync(old_cells, g.cells, bytes, cudaMemcpyDeviceToDevice, cfg.stream);
    if (e != cudaSuccess) return e;
    k_shift_cells<<<cfg.num_sms * 4, kThreads, 0, cfg.stream>>>(g.cells, old_cells, g.free_new, g.free_old, g.gs,
                                                                 x_move, y_move);
    return cudaGetLastError();
}

cudaError_t launch_draws(const GridDesc& g, int iteration, float2* init_u, float4* predict_z, float2* birth_z,
                         unsigned long long* resample_r, const LaunchCfg& cfg) {
    k_draws<<<cfg.num_sms * 4, kThreads, 0, cfg.stream>>>(g, (uint32_t)iteration, init_u, predict_z, birth_z,
                                                           resample_r);
    return cudaGetLastError();
}

}  // namespace dogm_gb300
