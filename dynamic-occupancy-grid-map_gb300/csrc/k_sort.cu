// Stable particle-to-cell sort: two LSD radix passes over the cell index (<= 11-bit digits),
// reduce-then-scan.  Replaces thrust::sort_by_key with a zip payload (dogm/src/dogm.cu:262-281).
//   upsweep    pass 0: per-tile digit histograms written by predict (same 4096-particle tiles);
//              pass 1: k_sort_hist counts each tile of the pass-0 output in shared memory and
//              writes its row whole (no global atomics, no zeroing between frames)
//   k_sort_scan  column scan of the [tile][digit] histogram -> the global output offset of
//              every (tile, digit) pair (digit base from predict's global histogram)
//   k_sort_pass  stable warp ranking inside the tile, scatter to offset + rank; pass 0 moves
//              {key, index} pairs (one 8-byte store per particle), pass 1 also gathers the
//              predicted particle state, so the payload moves once.
// Stability makes the permutation identical to the reference's stable sort.
#include "dogm_device.cuh"

namespace dogm_gb300 {

// ---------------------------------------------------------------------------------------
// Column scan: for each digit b, O[t][b] = base(b) + sum_{t' < t} H[t'][b], in place.
// Work item = (grid, group of 32 digits); 32 warps split the tiles into contiguous chunks.
// ---------------------------------------------------------------------------------------
constexpr int kScanWarps = 32;  // one warp per lane of the transposed chunk scan
static_assert(kScanWarps == 32, "the chunk scan transposes a 32 x 32 matrix");
constexpr int kScanBatch = 8;
constexpr int kScanKeep = 16;  // tiles per warp kept in registers (N up to 2M particles)
constexpr int kCtilePer = kMaxCellTiles / (kScanWarps * 32);
static_assert(kCtilePer * kScanWarps * 32 == kMaxCellTiles, "one block scans every cell-tile count");

// Exclusive scan of the per-cell-tile particle counts that predict took: ctile_start[i] is
// the first sorted position of cell tile i, ctile_start[n] = N.  Also the claim order of the
// cell pass: tiles by decreasing bit length of their particle count (the fullest, slowest
// tiles start first; the last tiles claimed are the quickest), in any order within a class.
// Run by one block as the last work item of the pass-1 digit scan (after predict, before
// the cell pass).  scratch: >= 64 words.
__device__ void ctile_scan(const GridDesc& g, uint32_t* red, uint32_t* scratch) {
    const int n = g.tiles[kStCell];
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
#pragma unroll
    for (int j = 0; j < kCtilePer; ++j) {
        if (i0 + j < n) {
            g.ctile_start[i0 + j] = e;
            atomicAdd(&cls_count[15 - min(15, 32 - __clz((int)v[j]))], 1u);
        }
        e += v[j];
    }
    if (i0 < n && n <= i0 + kCtilePer) g.ctile_start[n] = e;
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
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kCtilePer; ++j)
        if (i0 + j < n) g.ctile_order[atomicAdd(&cls_next[15 - min(15, 32 - __clz((int)v[j]))], 1u)] = (uint32_t)(i0 + j);
    __syncthreads();
}

__global__ void __launch_bounds__(kScanWarps * 32) k_sort_scan(Batch* __restrict__ bt, int pass) {
    grid_dependency_begin();
    __shared__ uint32_t chunk[kScanWarps][33];
    __shared__ uint32_t red[kScanWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int stage = pass ? kStScan1 : kStScan0;
    const int total = batch_total(bt, stage);
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int gi = grid_of_tile(bt, stage, t);
        const GridDesc& g = bt->g[gi];
        const int group = t - bt->prefix[gi][stage];
        if (pass == 1 && group == g.tiles[kStScan1] - 1) {  // block-uniform
            ctile_scan(g, red, &chunk[0][0]);
            continue;
        }
        const int nb = 1 << (pass ? g.d1_bits : g.d0_bits);
        const int b = group * 32 + lane;
        const uint32_t* hist = g.hist + pass * kSortMaxBins;
        // each warp owns a contiguous chunk of tiles; up to kScanKeep counts per lane stay in
        // registers between the sum and the rewrite (one load round), more are reloaded
        uint32_t* H = g.hsort + (size_t)pass * g.sort_tiles * kSortMaxBins;
        const int T = g.sort_tiles;
        const int per = (T + kScanWarps - 1) / kScanWarps;
        const int t0 = warp * per, t1 = min(T, t0 + per);
        const bool keep = per <= kScanKeep;  // block-uniform
        uint32_t v[kScanKeep];
        uint32_t s = 0;
        if (keep) {
#pragma unroll
            for (int i = 0; i < kScanKeep; ++i)
                v[i] = (b < nb && t0 + i < t1) ? H[(size_t)(t0 + i) * kSortMaxBins + b] : 0u;
#pragma unroll
            for (int i = 0; i < kScanKeep; ++i) s += v[i];
        } else if (b < nb) {
            for (int tb = t0; tb < t1; tb += kScanBatch) {
                uint32_t w[kScanBatch];
#pragma unroll
                for (int i = 0; i < kScanBatch; ++i)
                    w[i] = (tb + i < t1) ? H[(size_t)(tb + i) * kSortMaxBins + b] : 0u;
#pragma unroll
                for (int i = 0; i < kScanBatch; ++i) s += w[i];
            }
        }
        // digit base: sum of the global histogram over digits < b (loads issued alongside)
        uint32_t part = 0;
        for (int i = threadIdx.x; i < group * 32; i += blockDim.x) part += hist[i];
        const uint32_t own = (b < nb) ? hist[b] : 0u;
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
        // the counts of this lane's digit in the chunks of the warps before this one: warp w
        // scans digit w across the 32 chunks (one per lane; the padded rows keep the transposed
        // reads free of bank conflicts) and writes the exclusive prefixes back in place
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
                    if (t0 + i < t1) H[(size_t)(t0 + i) * kSortMaxBins + b] = pre;
                    pre += v[i];
                }
            } else {
                for (int tb = t0; tb < t1; tb += kScanBatch) {
                    uint32_t w[kScanBatch];
#pragma unroll
                    for (int i = 0; i < kScanBatch; ++i)
                        w[i] = (tb + i < t1) ? H[(size_t)(tb + i) * kSortMaxBins + b] : 0u;
#pragma unroll
                    for (int i = 0; i < kScanBatch; ++i) {
                        if (tb + i < t1) H[(size_t)(tb + i) * kSortMaxBins + b] = pre;
                        pre += w[i];
                    }
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------
// Downsweep: one tile of 4096 keys per block iteration.
// ---------------------------------------------------------------------------------------
struct SortSmem {
    uint16_t whist[kThreads / 32][kSortMaxBins];  // per-warp digit counts, then warp offsets
    uint32_t gbase[kSortMaxBins];                  // global offset of each digit for this tile
    uint16_t rank[kSortTile];                      // rank of each key among its warp's equal digits
};

// Four blocks per SM: a 2M-particle frame's 489 tiles run in one wave.
template <bool FINAL>
__global__ void __launch_bounds__(kThreads, 4) k_sort_pass(Batch* __restrict__ bt) {
    grid_dependency_begin();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SortSmem& sm = *reinterpret_cast<SortSmem*>(smem_raw);
    const int stage = FINAL ? kStSort1 : kStSort0;
    const int pass = FINAL ? 1 : 0;
    const int total = batch_total(bt, stage);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;

    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int gi = grid_of_tile(bt, stage, t);
        const GridDesc& g = bt->g[gi];
        const int lt = t - bt->prefix[gi][stage];
        const int bits = pass ? g.d1_bits : g.d0_bits;
        const int shift = pass ? g.d0_bits : 0;
        const int nb = 1 << bits;
        const uint32_t* O = g.hsort + (size_t)pass * g.sort_tiles * kSortMaxBins + (size_t)lt * kSortMaxBins;
        for (int i = threadIdx.x; i < nb; i += kThreads) sm.gbase[i] = O[i];
        uint4* wz = reinterpret_cast<uint4*>(&sm.whist[0][0]);  // all warp counts, 16 bytes a store
        for (int i = threadIdx.x; i < (int)(sizeof(sm.whist) / sizeof(uint4)); i += kThreads)
            wz[i] = make_uint4(0u, 0u, 0u, 0u);
        __syncthreads();

        // load the tile warp-striped (item k of lane l: warp base + k*32 + l)
        const int base = lt * kSortTile + warp * (32 * kSortIpt);
        uint16_t* rank = sm.rank + warp * (32 * kSortIpt) + lane;  // item k at rank[k * 32]
        // one base pointer per thread, items at constant offsets (k * 32 particles)
        const uint32_t* src_kw = FINAL ? reinterpret_cast<const uint32_t*>(g.T_pair + base + lane) : g.P_key + base + lane;
        constexpr int kw_stride = FINAL ? 64 : 32;  // words between a lane's items
        uint32_t key[kSortIpt];
#pragma unroll
        for (int k = 0; k < kSortIpt; ++k)
            key[k] = base + k * 32 + lane < g.N ? src_kw[k * kw_stride] : 0xffffffffu;
        // stable rank within the warp: rounds in input order, peers by match_any
#pragma unroll
        for (int k = 0; k < kSortIpt; ++k) {
            const bool valid = base + k * 32 + lane < g.N;
            const uint32_t d = valid ? (((key[k] & kCellMask) >> shift) & (uint32_t)(nb - 1)) : 0xffffffffu;
            const uint32_t peers = __match_any_sync(0xffffffffu, d);
            uint16_t before = 0;
            if (valid) before = sm.whist[warp][d];
            rank[k * 32] = (uint16_t)(before + __popc(peers & lt_mask));
            __syncwarp();
            if (valid && lane == __ffs(peers) - 1) sm.whist[warp][d] = (uint16_t)(before + __popc(peers));
            __syncwarp();
        }
        __syncthreads();
        // per digit: exclusive offsets across the warps of the tile
        for (int b = threadIdx.x; b < nb; b += kThreads) {
            uint32_t acc = 0;
#pragma unroll
            for (int w = 0; w < kThreads / 32; ++w) {
                const uint32_t c = sm.whist[w][b];
                sm.whist[w][b] = (uint16_t)acc;
                acc += c;
            }
        }
        __syncthreads();

        // scatter to the global sorted position.  The final pass's arrays do not overlap:
        // restrict lets the compiler issue the index loads and state gathers of several items
        // before their stores.
        const uint32_t* __restrict__ t_idx = src_kw + 1;  // .y words of the pass-0 pairs (final pass)
        const float4* __restrict__ p_state = g.P_state;
        float4* __restrict__ s_state = g.S_state;
        uint32_t* __restrict__ s_key = g.S_key;
        uint2* __restrict__ t_pair = g.T_pair;
        const int pos0 = base + lane;
#pragma unroll
        for (int k = 0; k < kSortIpt; ++k) {
            const int pos = base + k * 32 + lane;
            const bool valid = pos < g.N;
            uint32_t out = 0xffffffffu;
            if (valid) {
                const uint32_t d = ((key[k] & kCellMask) >> shift) & (uint32_t)(nb - 1);
                out = sm.gbase[d] + sm.whist[warp][d] + rank[k * 32];
                if (out >= (uint32_t)g.N) {  // only an inconsistent histogram can get here
                    flag_status(g, kStatusBounds);
                    out = 0xffffffffu;
                }
            }
            if (out != 0xffffffffu) {
                if (FINAL) {
                    const uint32_t src = t_idx[k * kw_stride];  // particle index carried by pass 0
                    s_key[out] = key[k];
                    s_state[out] = __ldg(p_state + src);
                    if (g.dbg_perm) g.dbg_perm[out] = (int)src;
                } else {
                    t_pair[out] = make_uint2(key[k], (uint32_t)(pos0 + k * 32));
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------
// Pass-1 digit counts: one tile of the pass-0 output per block iteration, counted in shared
// memory; the row H1[tile][0 .. 2^d1) is written whole.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_sort_hist(Batch* __restrict__ bt) {
    grid_dependency_begin();
    __shared__ uint32_t cnt[kSortMaxBins];
    const int total = batch_total(bt, kStSort1);
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int gi = grid_of_tile(bt, kStSort1, t);
        const GridDesc& g = bt->g[gi];
        const int lt = t - bt->prefix[gi][kStSort1];
        const int nb1 = 1 << g.d1_bits;
        const int shift1 = g.d0_bits;
        for (int i = threadIdx.x; i < nb1; i += kThreads) cnt[i] = 0u;
        const int base = lt * kSortTile;
        const uint32_t* kw = reinterpret_cast<const uint32_t*>(g.T_pair + base + threadIdx.x);
        uint32_t key[kSortIpt];
#pragma unroll
        for (int k = 0; k < kSortIpt; ++k)
            key[k] = base + k * kThreads + (int)threadIdx.x < g.N ? kw[2 * k * kThreads] : 0xffffffffu;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kSortIpt; ++k)
            if (base + k * kThreads + (int)threadIdx.x < g.N)
                atomicAdd(&cnt[((key[k] & kCellMask) >> shift1) & (uint32_t)(nb1 - 1)], 1u);
        __syncthreads();
        uint32_t* H1 = g.hsort + (size_t)g.sort_tiles * kSortMaxBins + (size_t)lt * kSortMaxBins;
        for (int i = threadIdx.x; i < nb1; i += kThreads) H1[i] = cnt[i];
        __syncthreads();
    }
}

cudaError_t launch_sort_scan(const Batch* d_batch, int pass, const LaunchCfg& cfg) {
    return launch_kernel(cfg, k_sort_scan, launch_blocks(cfg, 2), kScanWarps * 32, 0, const_cast<Batch*>(d_batch), pass);
}

cudaError_t launch_sort_pass(const Batch* d_batch, int pass, const LaunchCfg& cfg) {
    const size_t smem = sizeof(SortSmem);  // 48 KB: no opt-in attribute needed
    Batch* b = const_cast<Batch*>(d_batch);
    if (pass == 0)
        return launch_kernel(cfg, k_sort_pass<false>, launch_blocks(cfg, 4), kThreads, smem, b);
    else
        return launch_kernel(cfg, k_sort_pass<true>, launch_blocks(cfg, 4), kThreads, smem, b);
}

cudaError_t launch_sort_offsets1(const Batch* d_batch, const LaunchCfg& cfg) {
    cudaError_t e = launch_kernel(cfg, k_sort_hist, launch_blocks(cfg, 4), kThreads, 0, const_cast<Batch*>(d_batch));
    if (e != cudaSuccess) return e;
    return launch_sort_scan(d_batch, 1, cfg);
}

cudaError_t launch_sort(const Batch* d_batch, const LaunchCfg& cfg) {
    cudaError_t e;
    if ((e = launch_sort_scan(d_batch, 0, cfg)) != cudaSuccess) return e;
    if ((e = launch_sort_pass(d_batch, 0, cfg)) != cudaSuccess) return e;
    if ((e = launch_sort_offsets1(d_batch, cfg)) != cudaSuccess) return e;
    return launch_sort_pass(d_batch, 1, cfg);
}

}  // namespace dogm_gb300
