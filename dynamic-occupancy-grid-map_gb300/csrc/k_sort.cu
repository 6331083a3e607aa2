// Stable particle-to-cell sort, first half: a stable bucket scatter of the predicted particles
// by cell tile (the 1024-cell tiles of the cell pass; by runs of 64-512 cells for a small dense
// grid, GridDesc::bucket_bits).  The second half, a stable counting sort of each job's buckets
// by cell, runs inside the cell pass (k_cells.cu), which then holds them in shared memory
// anyway.  Together they give exactly the permutation of a stable sort by cell index and
// replace thrust::sort_by_key with its zip payload (dogm/src/dogm.cu:262-281).
//   predict      per 4096-particle tile, the particles per bucket (row written whole) and the
//                particles per bucket over the whole grid (ctile_cnt)
//   k_sort_scan  column scan of the [tile][bucket] counts -> the output offset of every
//                (tile, bucket) pair; one block also scans ctile_cnt into the first sorted
//                position of every bucket and orders the buckets for the cell pass
//   k_sort_scatter  stable warp ranking inside the tile, scatter of {state, key} to
//                offset + rank: the payload moves once, read in order and written in runs
//                (consecutive particles of the resampled set lie in few buckets)
#include "dogm_device.cuh"

namespace dogm_gb300 {

// ---------------------------------------------------------------------------------------
// Column scan: for each bucket b, O[t][b] = base(b) + sum_{t' < t} H[t'][b], in place.
// Work item = (grid, group of 32 buckets); 32 warps split the tiles into contiguous chunks.
// ---------------------------------------------------------------------------------------
constexpr int kScanWarps = 32;  // one warp per lane of the transposed chunk scan
static_assert(kScanWarps == 32, "the chunk scan transposes a 32 x 32 matrix");
constexpr int kScanBatch = 8;
constexpr int kScanKeep = 16;  // tiles per warp kept in registers (N up to 2M particles)
constexpr int kCtilePer = kMaxCellTiles / (kScanWarps * 32);
static_assert(kCtilePer * kScanWarps * 32 == kMaxCellTiles, "one block scans every cell-tile count");

// Exclusive scan of the per-bucket particle counts that predict took, written as the cell
// pass's job list.  A job is a run of whole buckets of one cell tile: the tile itself when the
// grid sorts by cell tile, else consecutive buckets of the tile merged while their particles stay
// within kJobTarget (a bucket above it is a job of its own), so that a tile holding many
// particles is shared by several blocks of the cell pass.  ctile_job[j] = {tile, first sorted
// position, end, first cell | end cell << 16 (within the tile)} of the j-th job to claim, jobs
// by decreasing bit length of their particle count (the fullest, slowest start first), in any
// order within a class; entries after the last job are {0xffffffff, 0, 0, 0}.  Run by one block
// as the last work item of the bucket scan (after predict, before the scatter and the cell
// pass).  scratch: >= 64 words.
__device__ __forceinline__ int job_class(uint32_t n) { return 15 - min(15, 32 - __clz((int)n)); }

__device__ void ctile_scan(const GridDesc& g, uint32_t* red, uint32_t* scratch) {
    __shared__ uint32_t s_cnt[kFineMaxBuckets], s_pre[kFineMaxBuckets];  // buckets of a finely sorted grid
    const int n = g.ctiles;
    const int bb = g.bucket_bits;
    const bool fine = bb < kCellTileBits;  // then n <= kFineMaxBuckets
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int i0 = threadIdx.x * kCtilePer;
    uint32_t* cls_count = scratch;       // 16 classes
    uint32_t* cls_next = scratch + 32;
    if (threadIdx.x < 16) cls_count[threadIdx.x] = 0u;
    uint32_t v[kCtilePer], s = 0u;
#pragma unroll
    for (int j = 0; j < kCtilePer; ++j) {
        v[j] = (i0 + j < n) ? g.ctile_cnt[i0 + j] : 0u;
        s += v[j];
    }
    uint32_t x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) red[warp] = x;
    __syncthreads();
    uint32_t e = x - s;
    for (int w = 0; w < warp; ++w) e += red[w];
    const int bpt = 1 << (kCellTileBits - bb);  // buckets per cell tile
    const int ntiles = (n + bpt - 1) / bpt;
    // one job per tile; or, for a finely sorted grid, runs of buckets (counted, then placed)
    auto walk = [&](int t, bool place) {
        int b = t * bpt;
        const int bend = min(n, b + bpt);
        while (b < bend) {
            const int j0 = b;
            uint32_t sum = s_cnt[b++];
            while (b < bend && sum + s_cnt[b] <= (uint32_t)kJobTarget) sum += s_cnt[b++];
            if (!place) {
                atomicAdd(&cls_count[job_class(sum)], 1u);
            } else {
                const uint32_t pos = atomicAdd(&cls_next[job_class(sum)], 1u);
                const uint32_t c_lo = (uint32_t)(j0 - t * bpt) << bb, c_hi = (uint32_t)(b - t * bpt) << bb;
                g.ctile_job[pos] = make_uint4((uint32_t)t, s_pre[j0], s_pre[j0] + sum, c_lo | (c_hi << 16));
            }
        }
    };
    if (fine) {
#pragma unroll
        for (int j = 0; j < kCtilePer; ++j) {
            if (i0 + j < n) {
                s_cnt[i0 + j] = v[j];
                s_pre[i0 + j] = e;
            }
            e += v[j];
        }
        __syncthreads();
        for (int t = threadIdx.x; t < ntiles; t += blockDim.x) walk(t, false);
    } else {
#pragma unroll
        for (int j = 0; j < kCtilePer; ++j)
            if (i0 + j < n) atomicAdd(&cls_count[job_class(v[j])], 1u);
    }
    __syncthreads();
    if (warp == 0) {
        const uint32_t c = lane < 16 ? cls_count[lane] : 0u;
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane < 16) cls_next[lane] = inc - c;
        if (lane == 15) scratch[48] = inc;  // jobs in all
    }
    __syncthreads();
    if (fine) {
        for (int t = threadIdx.x; t < ntiles; t += blockDim.x) walk(t, true);
        for (int i = (int)scratch[48] + threadIdx.x; i < n; i += blockDim.x)
            g.ctile_job[i] = make_uint4(0xffffffffu, 0u, 0u, 0u);
    } else {
#pragma unroll
        for (int j = 0; j < kCtilePer; ++j) {
            if (i0 + j < n) {
                const uint32_t pos = atomicAdd(&cls_next[job_class(v[j])], 1u);
                g.ctile_job[pos] = make_uint4((uint32_t)(i0 + j), e, e + v[j], (uint32_t)kCellTile << 16);
            }
            e += v[j];
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kScanWarps * 32) k_sort_scan(Batch* __restrict__ bt) {
    grid_dependency_begin();
    __shared__ uint32_t chunk[kScanWarps][33];
    __shared__ uint32_t red[kScanWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int total = batch_total(bt, kStScan);
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int gi = grid_of_tile(bt, kStScan, t);
        const GridDesc& g = bt->g[gi];
        const int group = t - bt->prefix[gi][kStScan];
        if (group == g.tiles[kStScan] - 1) {  // block-uniform
            ctile_scan(g, red, &chunk[0][0]);
            continue;
        }
        const int nb = g.ctiles;
        const int b = group * 32 + lane;
        const size_t stride = (size_t)g.bucket_stride;
        // each warp owns a contiguous chunk of tiles; up to kScanKeep counts per lane stay in
        // registers between the sum and the rewrite (one load round), more are reloaded
        uint32_t* H = g.hsort;
        const int T = g.sort_tiles;
        const int per = (T + kScanWarps - 1) / kScanWarps;
        const int t0 = warp * per, t1 = min(T, t0 + per);
        const bool keep = per <= kScanKeep;  // block-uniform
        uint32_t v[kScanKeep];
        uint32_t s = 0;
        if (keep) {
#pragma unroll
            for (int i = 0; i < kScanKeep; ++i) v[i] = (b < nb && t0 + i < t1) ? H[(t0 + i) * stride + b] : 0u;
#pragma unroll
            for (int i = 0; i < kScanKeep; ++i) s += v[i];
        } else if (b < nb) {
            for (int tb = t0; tb < t1; tb += kScanBatch) {
                uint32_t w[kScanBatch];
#pragma unroll
                for (int i = 0; i < kScanBatch; ++i) w[i] = (tb + i < t1) ? H[(tb + i) * stride + b] : 0u;
#pragma unroll
                for (int i = 0; i < kScanBatch; ++i) s += w[i];
            }
        }
        // bucket base: particles in buckets < b over the whole grid (loads issued alongside)
        uint32_t part = 0;
        for (int i = threadIdx.x; i < group * 32; i += blockDim.x) part += g.ctile_cnt[i];
        const uint32_t own = (b < nb) ? g.ctile_cnt[b] : 0u;
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        uint32_t lanepre = own;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, lanepre, o);
            if (lane >= o) lanepre += y;
        }
        if (lane == 0) red[warp] = part;
        chunk[warp][lane] = s;
        __syncthreads();
        // the block's sum of the parts: one load per lane and a warp reduction
        uint32_t base_all = red[lane];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) base_all += __shfl_xor_sync(0xffffffffu, base_all, o);
        // the counts of this lane's bucket in the chunks of the warps before this one: warp w
        // scans bucket w across the 32 chunks (one per lane; the padded rows keep the
        // transposed reads free of bank conflicts) and writes the exclusive prefixes back
        const uint32_t c = chunk[lane][warp];
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        __syncthreads();
        chunk[lane][warp] = inc - c;
        __syncthreads();
        uint32_t pre = lanepre - own + base_all + chunk[warp][lane];
        if (b < nb) {
            if (keep) {
#pragma unroll
                for (int i = 0; i < kScanKeep; ++i) {
                    if (t0 + i < t1) H[(t0 + i) * stride + b] = pre;
                    pre += v[i];
                }
            } else {
                for (int tb = t0; tb < t1; tb += kScanBatch) {
                    uint32_t w[kScanBatch];
#pragma unroll
                    for (int i = 0; i < kScanBatch; ++i) w[i] = (tb + i < t1) ? H[(tb + i) * stride + b] : 0u;
#pragma unroll
                    for (int i = 0; i < kScanBatch; ++i) {
                        if (tb + i < t1) H[(tb + i) * stride + b] = pre;
                        pre += w[i];
                    }
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------
// Bucket scatter: one tile of 4096 particles per block iteration, 512 threads (8 particles
// each), warp-striped: item k of lane l of warp w is tile position w * 256 + k * 32 + l.
// Shared memory (dynamic, W = the batch's largest bucket count rounded up to 8):
//   whist  u16 [16][W]  per-warp bucket counts, then each warp's offset within the tile
//   gbase  u32 [W]      output offset of each bucket for this tile (from the column scan)
// ---------------------------------------------------------------------------------------
constexpr int kScatterThreads = 512;
constexpr int kScatterWarps = kScatterThreads / 32;
constexpr int kScatterIpt = kSortTile / kScatterThreads;
static_assert(kScatterIpt * kScatterThreads == kSortTile, "whole particles per thread");

__host__ __device__ __forceinline__ int scatter_width(int max_ctiles) { return (max_ctiles + 7) & ~7; }
__host__ __device__ __forceinline__ size_t scatter_smem(int W) {
    return (size_t)kScatterWarps * W * sizeof(uint16_t) + (size_t)W * sizeof(uint32_t);
}

// FINE: some grid of the launch sorts by buckets finer than a cell tile (bucket = cell >>
// bucket_bits); without it the bucket is the cell tile.
template <bool FINE>
__global__ void __launch_bounds__(kScatterThreads, 2) k_sort_scatter(Batch* __restrict__ bt, int W) {
    grid_dependency_begin();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint16_t* whist = reinterpret_cast<uint16_t*>(smem_raw);
    uint32_t* gbase = reinterpret_cast<uint32_t*>(smem_raw + (size_t)kScatterWarps * W * sizeof(uint16_t));
    const int total = batch_total(bt, kStSort);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;
    uint16_t* my_hist = whist + warp * W;

    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int gi = grid_of_tile(bt, kStSort, t);
        const GridDesc& g = bt->g[gi];
        const int lt = t - bt->prefix[gi][kStSort];
        const int nb = g.ctiles;
        const uint32_t* O = g.hsort + (size_t)lt * g.bucket_stride;
        for (int i = threadIdx.x; i < nb; i += kScatterThreads) gbase[i] = O[i];
        uint4* wz = reinterpret_cast<uint4*>(whist);  // all warp counts, 16 bytes a store
        for (int i = threadIdx.x; i < kScatterWarps * W / 8; i += kScatterThreads) wz[i] = make_uint4(0u, 0u, 0u, 0u);
        __syncthreads();

        const int base = lt * kSortTile + warp * (32 * kScatterIpt);
        uint32_t key[kScatterIpt];
        uint16_t rank[kScatterIpt];
        // the predicted particles are read here for the last time in the frame: evict-first
        // loads (__ldcs) leave L2 to the bucketed copy the cell pass reads next
#pragma unroll
        for (int k = 0; k < kScatterIpt; ++k) {
            const int pos = base + k * 32 + lane;
            key[k] = pos < g.N ? __ldcs(g.P_key + pos) : 0xffffffffu;
        }
        // stable rank within the warp: rounds in input order, peers by match_any (a key whose
        // bucket lies outside the grid -- only injected state can hold one -- is not placed)
#pragma unroll
        for (int k = 0; k < kScatterIpt; ++k) {
            const uint32_t b = (key[k] & kCellMask) >> (FINE ? g.bucket_bits : kCellTileBits);
            const bool valid = base + k * 32 + lane < g.N && b < (uint32_t)nb;
            const uint32_t d = valid ? b : 0xffffffffu;
            const uint32_t peers = __match_any_sync(0xffffffffu, d);
            uint16_t before = 0;
            if (valid) before = my_hist[d];
            rank[k] = (uint16_t)(before + __popc(peers & lt_mask));
            __syncwarp();
            if (valid && lane == __ffs(peers) - 1) my_hist[d] = (uint16_t)(before + __popc(peers));
            __syncwarp();
        }
        __syncthreads();
        // per bucket: exclusive offsets across the warps of the tile
        for (int b = threadIdx.x; b < nb; b += kScatterThreads) {
            uint32_t acc = 0;
#pragma unroll
            for (int w = 0; w < kScatterWarps; ++w) {
                const uint32_t c = whist[w * W + b];
                whist[w * W + b] = (uint16_t)acc;
                acc += c;
            }
        }
        __syncthreads();

        // scatter {state, key} (and, for debugging, the particle's index) to its bucket slot;
        // per half of the items, every state load is issued before the first store (a load
        // behind its own store's guard would wait for the one before it)
        const float4* __restrict__ p_state = g.P_state;
        float4* __restrict__ t_state = g.T_state;
        uint32_t* __restrict__ t_key = g.T_key;
        constexpr int kHalf = kScatterIpt / 2;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            float4 st[kHalf];
            uint32_t out[kHalf];
#pragma unroll
            for (int j = 0; j < kHalf; ++j) {
                const int k = h * kHalf + j;
                const int pos = base + k * 32 + lane;
                const uint32_t d = (key[k] & kCellMask) >> (FINE ? g.bucket_bits : kCellTileBits);
                out[j] = 0xffffffffu;
                if (pos < g.N && d < (uint32_t)nb) out[j] = gbase[d] + my_hist[d] + rank[k];
                st[j] = __ldcs(p_state + (pos < g.N ? pos : g.N - 1));
            }
#pragma unroll
            for (int j = 0; j < kHalf; ++j) {
                const int k = h * kHalf + j;
                const int pos = base + k * 32 + lane;
                if (pos >= g.N) continue;
                if (out[j] < (uint32_t)g.N) {
                    t_key[out[j]] = key[k];
                    t_state[out[j]] = st[j];
                    if (g.T_idx) g.T_idx[out[j]] = pos;
                } else {  // a bucket outside the grid, or an inconsistent histogram
                    flag_status(g, kStatusBounds);
                }
            }
        }
        __syncthreads();
    }
}

cudaError_t launch_sort_scan(const Batch* d_batch, const LaunchCfg& cfg) {
    return launch_kernel(cfg, k_sort_scan, launch_blocks(cfg, 2), kScanWarps * 32, 0, const_cast<Batch*>(d_batch));
}

cudaError_t prepare_sort() {
    const int smem = (int)scatter_smem(scatter_width(kMaxCellTiles));
    cudaError_t e = cudaFuncSetAttribute(k_sort_scatter<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_sort_scatter<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

cudaError_t launch_sort_scatter(const Batch* d_batch, int max_ctiles, const LaunchCfg& cfg, bool fine) {
    const int W = scatter_width(max_ctiles);
    Batch* b = const_cast<Batch*>(d_batch);
    if (fine) return launch_kernel(cfg, k_sort_scatter<true>, launch_blocks(cfg, 2), kScatterThreads, scatter_smem(W), b, W);
    return launch_kernel(cfg, k_sort_scatter<false>, launch_blocks(cfg, 2), kScatterThreads, scatter_smem(W), b, W);
}

}  // namespace dogm_gb300
