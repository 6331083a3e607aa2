// Stable particle-to-cell sort: two LSD radix passes over the cell index (<= 11-bit digits)
// with decoupled look-back across tiles.  Replaces thrust::sort_by_key with a zip payload
// (dogm/src/dogm.cu:262-281).  Pass 0 sorts (key, index) by the low digit; pass 1 sorts by
// the high digit and gathers the predicted particle state into sorted order, so the
// payload moves once.  Stability makes the permutation identical to the reference's.
#include "dogm_device.cuh"

namespace dogm_gb300 {

// Sort look-back word: [31:30] status, [29:24] epoch tag, [23:0] count.
constexpr uint32_t kSortAgg = 1u << 30;
constexpr uint32_t kSortInc = 2u << 30;
constexpr uint32_t kSortCount = (1u << 24) - 1u;

struct SortSmem {
    uint16_t whist[kThreads / 32][kSortMaxBins];  // per-warp digit counts, then warp offsets
    uint32_t gbase[kSortMaxBins];                  // global base of each digit for this tile
    int scan[kThreads / 32];
    int slot;
};

template <bool FINAL>
__global__ void __launch_bounds__(kThreads, 2) k_sort_pass(Batch* bt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SortSmem& sm = *reinterpret_cast<SortSmem*>(smem_raw);
    const int stage = FINAL ? kStSort1 : kStSort0;
    const int pass = FINAL ? 1 : 0;
    const int total = batch_total(bt, stage);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;
    constexpr int kBinsPerThread = kSortMaxBins / kThreads;

    for (;;) {
        const int t = claim_tile(bt, stage, &sm.slot);
        if (t >= total) break;
        const int gi = grid_of_tile(bt, stage, t);
        const GridDesc& g = bt->g[gi];
        const int lt = t - bt->prefix[gi][stage];
        const int bits = pass ? g.d1_bits : g.d0_bits;
        const int shift = pass ? g.d0_bits : 0;
        const int nb = 1 << bits;
        const uint32_t epoch = (g.epoch & 63u) << 24;
        uint32_t* lb_all = g.lb_sort + (size_t)pass * g.sort_tiles * kSortMaxBins;

        // 1. global exclusive digit offsets from the histogram predict accumulated
        {
            int v[kBinsPerThread];
            int s = 0;
#pragma unroll
            for (int r = 0; r < kBinsPerThread; ++r) {
                const int b = threadIdx.x * kBinsPerThread + r;
                v[r] = (b < nb) ? (int)g.hist[pass * kSortMaxBins + b] : 0;
                s += v[r];
            }
            int tot;
            int pre = block_excl_scan_i32(s, sm.scan, &tot);
#pragma unroll
            for (int r = 0; r < kBinsPerThread; ++r) {
                const int b = threadIdx.x * kBinsPerThread + r;
                sm.gbase[b] = (uint32_t)pre;
                pre += v[r];
            }
            for (int i = threadIdx.x; i < (kThreads / 32) * nb; i += kThreads) sm.whist[i / nb][i % nb] = 0;
        }
        __syncthreads();

        // 2. load the tile warp-striped (item k of lane l: warp base + k*32 + l)
        const int base = lt * kSortTile + warp * (32 * kSortIpt);
        uint32_t key[kSortIpt], val[kSortIpt], dig[kSortIpt];
        uint16_t rank[kSortIpt];
#pragma unroll
        for (int k = 0; k < kSortIpt; ++k) {
            const int pos = base + k * 32 + lane;
            if (pos < g.N) {
                key[k] = FINAL ? g.T_key[pos] : g.P_key[pos];
                val[k] = FINAL ? g.T_idx[pos] : (uint32_t)pos;
                dig[k] = ((key[k] & kCellMask) >> shift) & (uint32_t)(nb - 1);
            } else {
                key[k] = 0u;
                val[k] = 0u;
                dig[k] = 0xffffffffu;
            }
        }
        // 3. stable rank within the warp: rounds in input order, peers by match_any
#pragma unroll
        for (int k = 0; k < kSortIpt; ++k) {
            const uint32_t peers = __match_any_sync(0xffffffffu, dig[k]);
            const bool valid = dig[k] != 0xffffffffu;
            uint16_t before = 0;
            if (valid) before = sm.whist[warp][dig[k]];
            rank[k] = (uint16_t)(before + __popc(peers & lt_mask));
            __syncwarp();
            if (valid && lane == __ffs(peers) - 1) sm.whist[warp][dig[k]] = (uint16_t)(before + __popc(peers));
            __syncwarp();
        }
        __syncthreads();

        // 4. per digit: warp offsets, tile total, decoupled look-back across tiles
        uint32_t* lb = lb_all + (size_t)lt * kSortMaxBins;
        uint32_t tot[kBinsPerThread];
#pragma unroll
        for (int r = 0; r < kBinsPerThread; ++r) {
            const int b = threadIdx.x + r * kThreads;
            uint32_t acc = 0;
            if (b < nb) {
#pragma unroll
                for (int w = 0; w < kThreads / 32; ++w) {
                    const uint32_t c = sm.whist[w][b];
                    sm.whist[w][b] = (uint16_t)acc;
                    acc += c;
                }
                st_volatile(lb + b, (lt == 0 ? kSortInc : kSortAgg) | epoch | acc);
            }
            tot[r] = acc;
        }
        if (lt > 0) {
#pragma unroll
            for (int r = 0; r < kBinsPerThread; ++r) {
                const int b = threadIdx.x + r * kThreads;
                if (b >= nb) break;
                uint32_t excl = 0;
                int p = lt - 1;
                int spins = 0;
                while (p >= 0) {
                    const uint32_t v = ld_volatile(lb_all + (size_t)p * kSortMaxBins + b);
                    const bool cur = (v & (63u << 24)) == epoch;
                    if (cur && (v & kSortInc)) { excl += v & kSortCount; break; }
                    if (cur && (v & kSortAgg)) { excl += v & kSortCount; --p; continue; }
                    if (++spins > kSpinLimit) { flag_timeout(g); break; }
                    __nanosleep(32);
                }
                st_volatile(lb + b, kSortInc | epoch | ((excl + tot[r]) & kSortCount));
                sm.gbase[b] += excl;
            }
        }
        __syncthreads();

        // 5. scatter to the global sorted position
#pragma unroll
        for (int k = 0; k < kSortIpt; ++k) {
            if (dig[k] == 0xffffffffu) continue;
            const uint32_t out = sm.gbase[dig[k]] + sm.whist[warp][dig[k]] + rank[k];
            if (out >= (uint32_t)g.N) {  // only a corrupted histogram can get here
                flag_status(g, kStatusBounds);
                continue;
            }
            if (FINAL) {
                g.S_key[out] = key[k];
                g.S_state[out] = g.P_state[val[k]];
                if (g.dbg_perm) g.dbg_perm[out] = (int)val[k];
            } else {
                g.T_key[out] = key[k];
                g.T_idx[out] = val[k];
            }
        }
        __syncthreads();
    }
}

cudaError_t launch_sort_pass(const Batch* d_batch, int pass, const LaunchCfg& cfg) {
    const size_t smem = sizeof(SortSmem);  // < 48 KB: no opt-in attribute needed
    Batch* b = const_cast<Batch*>(d_batch);
    if (pass == 0)
        k_sort_pass<false><<<cfg.num_sms * 2, kThreads, smem, cfg.stream>>>(b);
    else
        k_sort_pass<true><<<cfg.num_sms * 2, kThreads, smem, cfg.stream>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_sort(const Batch* d_batch, const LaunchCfg& cfg) {
    cudaError_t e = launch_sort_pass(d_batch, 0, cfg);
    if (e != cudaSuccess) return e;
    return launch_sort_pass(d_batch, 1, cfg);
}

}  // namespace dogm_gb300
