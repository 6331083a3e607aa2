// Resampling: one pass over the joint particle array [persistent (sorted) | newborn].
// The newborns are created here from the slot key words the newborn kernel wrote (the
// reference initialises them in initNewParticlesKernel2, init_new_particles.cu:157-195).
// Replaces the joint concatenation, float scan, random draws, float sort, lower_bound and
// gather of dogm.cu:386-423 / resampling.cu:17-68.  Joint weights are quantised to
// 2^-q_shift and scanned exactly (integer, order-independent; a tile's prefix is the sum of the
// per-tile sums that the cell and newborn kernels accumulated), and
// systematic resampling assigns output slot i to the joint particle j with
// A[j-1]*N <= i*T + U < A[j]*N, so each particle writes its own copies directly.
// The new common weight is T / N (dogm.cu:417).
#include "dogm_device.cuh"

namespace dogm_gb300 {

// A heavy item (more copies than an item writes itself) expanded by the whole block.
struct HeavyItem {
    float4 st;
    uint32_t kw;
    int first, end, item;
};
constexpr int kOwnCopies = 8;        // an item writes up to this many copies itself
constexpr int kMaxHeavy = 768;       // heavy items per tile expanded cooperatively (more: by their thread)

struct ResSmem {
    HeavyItem heavy[kMaxHeavy];    // items with many copies
    unsigned long long red[2 * (kThreads / 32)];
    int nheavy;
    int claim;
};

__global__ void __launch_bounds__(kThreads, 3) k_resample(Batch* __restrict__ bt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ResSmem& sm = *reinterpret_cast<ResSmem*>(smem_raw);
    const int total = batch_total(bt, kStResample);
    // tiles are taken dynamically from the end: the newborn tiles (last in the joint order,
    // with the heaviest copy counts) start first and the light tiles fill in around them
    for (;;) {
        const int c = claim_tile(bt, kStResample, &sm.claim);
        if (c >= total) break;
        const int t = total - 1 - c;
        const int gi = grid_of_tile(bt, kStResample, t);
        const GridDesc& g = bt->g[gi];
        const int lt = t - bt->prefix[gi][kStResample];
        const int base = lt * kResTile;
        const int N = g.N, C = g.C, gs = g.gs, S = g.q_shift;
        const int M = N + g.fs->n_birth;
        const unsigned long long T = g.fs->joint_total;
        const uint32_t* __restrict__ S_key = g.S_key;
        const float4* __restrict__ S_state = g.S_state;
        const float* __restrict__ w_cell = g.w_cell;
        const dogm_grid_cell* __restrict__ cells = g.cells;
        float4* __restrict__ P_state = g.P_state;
        uint32_t* __restrict__ P_key = g.P_key;
        int* __restrict__ dbg_src = g.dbg_src;
        if (threadIdx.x == 0) sm.nheavy = 0;
        unsigned long long r64;
        if (g.rp_resample) {
            r64 = *g.rp_resample;
        } else {
            const U4 r = draw_block(g, 0u, g.frame, kDrawResample);
            r64 = ((unsigned long long)r.x << 32) | r.y;
        }
        const unsigned long long U = __umul64hi(r64, T);  // floor(u * T), u = r64 / 2^64

        // this thread's kResIpt consecutive joint items, in registers
        float4 st[kResIpt];
        uint32_t kw[kResIpt];
        float wq[kResIpt];
        unsigned long long v = 0ull;
        const int j0 = threadIdx.x * kResIpt;
#pragma unroll
        for (int r = 0; r < kResIpt; ++r) {
            const int p = base + j0 + r;
            float w = 0.0f;
            st[r] = make_float4(0.f, 0.f, 0.f, 0.f);
            kw[r] = 0u;
            if (p < N) {
                kw[r] = S_key[p];
                st[r] = S_state[p];
                w = (kw[r] & kOutBit) ? 0.0f : w_cell[kw[r] & kCellMask];
            } else if (p < M) {
                // newborn slot b (initNewParticlesKernel2, init_new_particles.cu:157-195): cell
                // and associated flag from the key word the newborn kernel wrote
                const int b = p - N;
                const uint32_t bk = g.B_key[b];
                const int k = min((int)(bk & kCellMask), C - 1);
                const bool assoc = (bk & kAssocBit) != 0u;
                float2 z;
                if (g.rp_birth) {
                    z = g.rp_birth[b];
                } else {
                    const U4 rr = draw_block(g, (uint32_t)b, g.frame, kDrawBirth);
                    z = box_muller(rr.x, rr.y);
                }
                st[r].x = __fadd_rn((float)(k % gs), 0.5f);
                st[r].y = __fadd_rn(__fdiv_rn((float)k, (float)gs), 0.5f);  // float division, as the reference
                st[r].z = __fmaf_rn(z.x, g.sigma_birth, 0.0f);
                st[r].w = __fmaf_rn(z.y, g.sigma_birth, 0.0f);
                kw[r] = (uint32_t)k | (assoc ? kAssocBit : 0u);
                w = assoc ? cells[k].w_A : cells[k].w_UA;
                if (g.dbg_perm) {  // debug export of the newborns
                    g.B_state[b] = st[r];
                    g.B_w[b] = w;
                }
            }
            kw[r] &= ~kOutBit;
            wq[r] = (p < M) ? w : 0.0f;
            v += quantize(wq[r], S);
        }
        unsigned long long tile_sum;
        unsigned long long acc = block_scan_after(v, g.res_sum, lt, sm.red, &tile_sum);
        int lo_s = (base + j0 == 0) ? 0 : comb_count(acc, T, U, N);
#pragma unroll
        for (int r = 0; r < kResIpt; ++r) {
            acc += quantize(wq[r], S);
            const int hi_s = comb_count(acc, T, U, N);
            bool own = hi_s - lo_s <= kOwnCopies;
            if (!own) {
                const int h = atomicAdd(&sm.nheavy, 1);
                if (h < kMaxHeavy) {
                    HeavyItem e;
                    e.st = st[r]; e.kw = kw[r]; e.first = lo_s; e.end = hi_s; e.item = base + j0 + r;
                    sm.heavy[h] = e;
                } else {
                    own = true;  // list full: this thread writes the copies itself
                }
            }
            if (own) {
                for (int s = lo_s; s < hi_s; ++s) {
                    P_state[s] = st[r];
                    P_key[s] = kw[r];
                    if (dbg_src) dbg_src[s] = base + j0 + r;
                }
            }
            lo_s = hi_s;
        }
        __syncthreads();
        const int nh = min(sm.nheavy, kMaxHeavy);
        for (int h = 0; h < nh; ++h) {
            const HeavyItem e = sm.heavy[h];
            for (int s = e.first + threadIdx.x; s < e.end; s += kThreads) {
                P_state[s] = e.st;
                P_key[s] = e.kw;
                if (dbg_src) dbg_src[s] = e.item;
            }
        }
        if (lt == 0 && threadIdx.x == 0) {
            const float jf = ldexpf(__ull2float_rn(T), -S);
            g.fs->w_res = __fdiv_rn(jf, (float)N);
        }
        __syncthreads();
    }
}

cudaError_t prepare_kernels() {
    return cudaFuncSetAttribute(k_resample, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(ResSmem));
}

cudaError_t launch_resample(const Batch* d_batch, const LaunchCfg& cfg) {
    const int smem = (int)sizeof(ResSmem);
    k_resample<<<cfg.num_sms * 3, kThreads, smem, cfg.stream>>>(const_cast<Batch*>(d_batch));
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// Multinomial index search of the reference (resampling.cu:34-47): optional clamp of the
// last accumulator to the largest query, then lower_bound of every sorted query.
// ---------------------------------------------------------------------------------------
__global__ void k_lower_bound(const float* __restrict__ acc, int n, const float* __restrict__ qv, int nq,
                              int* __restrict__ out, int clamp_last) {
    const float qmax = qv[nq - 1];
    const float last = acc[n - 1];
    const float last_eff = (clamp_last && last != qmax) ? qmax : last;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += gridDim.x * blockDim.x) {
        const float x = qv[i];
        int a = 0, b = n;  // first index with acc >= x
        while (a < b) {
            const int m = (a + b) >> 1;
            const float am = (m == n - 1) ? last_eff : acc[m];
            if (am < x) a = m + 1; else b = m;
        }
        out[i] = a;
    }
}

cudaError_t launch_lower_bound(const float* accum, int n_accum, const float* q, int n_q, int* out, int clamp_last,
                               cudaStream_t s) {
    if (n_q <= 0) return cudaSuccess;
    k_lower_bound<<<(n_q + 255) / 256 < 4096 ? (n_q + 255) / 256 : 4096, 256, 0, s>>>(accum, n_accum, q, n_q, out,
                                                                                  clamp_last);
    return cudaGetLastError();
}

}  // namespace dogm_gb300
