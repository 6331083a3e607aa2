// Resampling: one pass over the joint particle array [persistent (sorted) | newborn].
// The newborns are created here from the slot key words the newborn kernel wrote (the
// reference initialises them in initNewParticlesKernel2, init_new_particles.cu:157-195).
// Replaces the joint concatenation, float scan, random draws, float sort, lower_bound and
// gather of dogm.cu:386-423 / resampling.cu:17-68.  Joint weights are quantised to
// 2^-q_shift and scanned exactly (integer, order-independent; a tile's prefix is the sum of the
// per-tile sums that the cell and newborn kernels accumulated), and
// systematic resampling assigns output slot i to the joint particle j with
// A[j-1]*N <= i*T + U < A[j]*N.  A tile's items are staged in shared memory; their first
// output slots come from the blocked exact scan, and the copies are written with
// consecutive items on consecutive lanes, so the stores of a warp are contiguous.
// The new common weight is T / N (dogm.cu:417).
#include "dogm_device.cuh"

namespace dogm_gb300 {

// Copy counts per item: comb_count(a) = #{ i in [0,N) : i*T + U < a*N }, starting from a
// float estimate (inv_T = 1/T rounded) that the exact 96-bit checks then correct.
__device__ __forceinline__ int comb_count_est(unsigned long long a, unsigned long long T, unsigned long long U, int N,
                                              float inv_T) {
    if (T == 0ull || a >= T) return N;
    const U96 rhs = mul_u64_u32(a, (unsigned int)N);
    const float f = __fmul_rn(__fsub_rn(__fmul_rn(__ull2float_rn(a), (float)N), __ull2float_rn(U)), inv_T);
    int c = (int)ceilf(f);
    c = c < 0 ? 0 : (c > N ? N : c);
    // P(i): i*T + U < a*N holds for i < result and fails from result on
    while (c > 0 && !lt96(add96(mul_u64_u32(T, (unsigned int)(c - 1)), U), rhs)) --c;
    while (c < N && lt96(add96(mul_u64_u32(T, (unsigned int)c), U), rhs)) ++c;
    return c;
}

// Shared words of a tile indexed with one pad word per 32, so that both the blocked
// (thread t: items IPT t .. IPT t + IPT - 1) and the warp-striped (item r*256 + t) accesses are
// free of bank conflicts.
__device__ __forceinline__ int pad_idx(int j) { return j + (j >> 5); }
template <int IPT>
struct ResShape {
    static constexpr int kTile = kThreads * IPT;
    static constexpr int kPadded = kTile + 1 + ((kTile + 1) >> 5) + 1;
};

struct HeavyRef {
    int item, first, end;  // a joint item with more copies than one thread writes
};
constexpr int kOwnCopies = 8;
constexpr int kWarpCopies = 256;  // output slots a warp writes together (8 stores of 32)
constexpr int kMaxHeavy = 256;

template <int IPT>
struct ResSmem {
    float4 st[ResShape<IPT>::kTile];         // states of the tile's joint items
    uint32_t kw[ResShape<IPT>::kTile];       // their key words
    uint32_t lw[ResShape<IPT>::kPadded];     // weight (float bits), then first output slot of each item (+ end)
    HeavyRef heavy[kMaxHeavy];
    unsigned long long red[2 * (kThreads / 32)];
    unsigned long long r64;  // the frame's comb draw (one Philox block, drawn by thread 0)
    int nheavy;
    int claim;
};

// IPT joint particles per thread: tiles of 512, 1024 or 2048 (GridDesc::res_bits 9, 10, 11)
template <int IPT>
__global__ void __launch_bounds__(kThreads, IPT <= 4 ? 5 : 4) k_resample(Batch* __restrict__ bt) {
    grid_dependency_begin();
    // the frame's status bits are final here (only the sort and cell passes set them): they are
    // ORed into the mapped host word, where they stay until the host's next synchronisation reads
    // and clears it (no device-to-host copy after the frame; a clean frame touches nothing)
    if (blockIdx.x == 0 && threadIdx.x == 0 && bt->status_host) {
        const unsigned int st = bt->status;
        if (st) *(volatile unsigned int*)bt->status_host |= st;
    }
    constexpr int kResIpt = IPT;
    constexpr int kResTile = ResShape<IPT>::kTile;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ResSmem<IPT>& sm = *reinterpret_cast<ResSmem<IPT>*>(smem_raw);
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
        if (threadIdx.x == 0) {
            sm.nheavy = 0;
            if (g.rp_resample) {
                sm.r64 = *g.rp_resample;
            } else {
                const U4 r = draw_block(g, 0u, g.frame, kDrawResample);
                sm.r64 = ((unsigned long long)r.x << 32) | r.y;
            }
        }

        // ---- 1: the tile's joint items, warp-striped into shared memory -------------------
        // persistent items: asynchronous copies, then one batch of cell-weight gathers
#pragma unroll
        for (int r = 0; r < kResIpt; ++r) {
            const int p = base + r * kThreads + (int)threadIdx.x;
            if (p < N) {
                cp_async16(&sm.st[p - base], g.S_state + p);
                cp_async4(&sm.kw[p - base], g.S_key + p);
            }
        }
        cp_async_wait_all();
        {
            // every cell-weight load of the thread is issued before the first shared store
            uint32_t kw[kResIpt];
            float w[kResIpt];
#pragma unroll
            for (int r = 0; r < kResIpt; ++r) {
                const int j = r * kThreads + threadIdx.x;
                kw[r] = base + j < N ? sm.kw[j] : 0u;
            }
#pragma unroll
            for (int r = 0; r < kResIpt; ++r) w[r] = g.w_cell[min((int)(kw[r] & kCellMask), C - 1)];
#pragma unroll
            for (int r = 0; r < kResIpt; ++r) {
                const int j = r * kThreads + threadIdx.x;
                if (base + j < N) {
                    sm.lw[pad_idx(j)] = __float_as_uint((kw[r] & kOutBit) ? 0.0f : w[r]);
                    sm.kw[j] = kw[r] & ~kOutBit;
                }
            }
        }
        // newborn items, created here, and the empty tail of the last tile
        for (int r = 0; r < kResIpt; ++r) {
            const int j = r * kThreads + threadIdx.x;
            const int p = base + j;
            if (p < N) continue;
            float4 st = make_float4(0.f, 0.f, 0.f, 0.f);
            uint32_t kw = 0u;
            float w = 0.0f;
            if (p < M) {
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
                st.x = __fadd_rn((float)(k - cell_row(g, k) * gs), 0.5f);
                st.y = __fadd_rn(__fdiv_rn((float)k, (float)gs), 0.5f);  // float division, as the reference
                st.z = __fmaf_rn(z.x, g.sigma_birth, 0.0f);
                st.w = __fmaf_rn(z.y, g.sigma_birth, 0.0f);
                kw = (uint32_t)k | (assoc ? kAssocBit : 0u);
                w = assoc ? g.cells[k].w_A : g.cells[k].w_UA;
                if (g.dbg_perm) {  // debug export of the newborns
                    g.B_state[b] = st;
                    g.B_w[b] = w;
                }
            }
            sm.st[j] = st;
            sm.kw[j] = kw;
            sm.lw[pad_idx(j)] = __float_as_uint(w);
        }
        __syncthreads();

        // ---- 2: exact scan (blocked) -> first output slot of every item -----------------
        const unsigned long long U = __umul64hi(sm.r64, T);  // floor(u * T), u = r64 / 2^64
        const float inv_T = T ? __frcp_rn(__ull2float_rn(T)) : 0.0f;
        const int j0 = threadIdx.x * kResIpt;
        unsigned long long q[kResIpt];
        unsigned long long v = 0ull;
#pragma unroll
        for (int r = 0; r < kResIpt; ++r) {
            q[r] = quantize(__uint_as_float(sm.lw[pad_idx(j0 + r)]), S);
            v += q[r];
        }
        unsigned long long tile_sum;
        unsigned long long acc = block_scan_after(v, g.res_sum, lt, sm.red, &tile_sum);
        // first slot of the thread's first item; later boundaries walk the comb tooth by tooth
        // (tooth = lo_s*T + U, exact 96-bit), or jump for an item with many copies
        int lo_s = (base + j0 == 0) ? 0 : comb_count_est(acc, T, U, N, inv_T);
        U96 tooth = add96(mul_u64_u32(T, (unsigned int)lo_s), U);
#pragma unroll
        for (int r = 0; r < kResIpt; ++r) {
            sm.lw[pad_idx(j0 + r)] = (uint32_t)lo_s;  // this thread read the slot above
            acc += q[r];
            if (T == 0ull) {
                lo_s = N;  // no weight at all: every slot goes to the first item
            } else if (q[r]) {
                const float copies = __fmul_rn(__fmul_rn(__ull2float_rn(q[r]), (float)N), inv_T);
                if (copies < 32.0f) {
                    const U96 rhs = mul_u64_u32(acc, (unsigned int)N);
                    while (lo_s < N && lt96(tooth, rhs)) {
                        ++lo_s;
                        tooth = add96(tooth, T);
                    }
                } else {
                    lo_s = comb_count_est(acc, T, U, N, inv_T);
                    tooth = add96(mul_u64_u32(T, (unsigned int)lo_s), U);
                }
            }
        }
        if (threadIdx.x == kThreads - 1) sm.lw[pad_idx(kResTile)] = (uint32_t)lo_s;
        __syncthreads();

        // ---- 3: copies.  The 32 consecutive items of a warp own one contiguous range of
        // output slots; a warp whose range is short writes it together, 32 consecutive slots
        // per store, each lane finding the owner of its slot (the last lane whose first slot
        // is <= it; items without copies share their first slot with the next item).  A warp
        // with a long range writes per item, and items with many copies go to the block.
        // the resampled set is read again only by the next frame's predict, after hundreds of MB
        // of other traffic: evict-first stores (__stcs)
        float4* __restrict__ P_state = g.P_state;
        uint32_t* __restrict__ P_key = g.P_key;
        int* __restrict__ dbg_src = g.dbg_src;
        const int lane = threadIdx.x & 31;
#pragma unroll 2
        for (int r = 0; r < kResIpt; ++r) {
            const int j = r * kThreads + threadIdx.x;
            const int first = (int)sm.lw[pad_idx(j)], end = (int)sm.lw[pad_idx(j + 1)];
            const int wf = __shfl_sync(0xffffffffu, first, 0), we = __shfl_sync(0xffffffffu, end, 31);
            if (we - wf <= kWarpCopies) {  // warp-uniform
                const int j0 = j - lane;
                for (int s0 = wf; s0 < we; s0 += 32) {
                    const int slot = s0 + lane;
                    int owner = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        const int f = __shfl_sync(0xffffffffu, first, owner + step);
                        if (f <= slot) owner += step;
                    }
                    if (slot < we) {
                        __stcs(P_state + slot, sm.st[j0 + owner]);
                        __stcs(P_key + slot, sm.kw[j0 + owner]);
                        if (dbg_src) dbg_src[slot] = base + j0 + owner;
                    }
                }
            } else if (end > first) {
                bool own = end - first <= kOwnCopies;
                if (!own) {
                    const int h = atomicAdd(&sm.nheavy, 1);
                    if (h < kMaxHeavy) sm.heavy[h] = HeavyRef{j, first, end};
                    else own = true;  // list full: this thread writes the copies itself
                }
                if (own) {
                    const float4 st = sm.st[j];
                    const uint32_t kw = sm.kw[j];
                    for (int s = first; s < end; ++s) {
                        __stcs(P_state + s, st);
                        __stcs(P_key + s, kw);
                        if (dbg_src) dbg_src[s] = base + j;
                    }
                }
            }
        }
        __syncthreads();
        const int nh = min(sm.nheavy, kMaxHeavy);
        for (int h = 0; h < nh; ++h) {
            const HeavyRef e = sm.heavy[h];
            const float4 st = sm.st[e.item];
            const uint32_t kw = sm.kw[e.item];
            for (int s = e.first + threadIdx.x; s < e.end; s += kThreads) {
                __stcs(P_state + s, st);
                __stcs(P_key + s, kw);
                if (dbg_src) dbg_src[s] = base + e.item;
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
    cudaError_t e = cudaFuncSetAttribute(k_resample<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(ResSmem<2>));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_resample<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(ResSmem<4>));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_resample<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(ResSmem<8>));
    return e;
}

cudaError_t launch_resample(const Batch* d_batch, int res_bits, const LaunchCfg& cfg) {
    Batch* b = const_cast<Batch*>(d_batch);
    switch (res_bits) {
        case 9: return launch_kernel(cfg, k_resample<2>, launch_blocks(cfg, 5), kThreads, sizeof(ResSmem<2>), b);
        case 10: return launch_kernel(cfg, k_resample<4>, launch_blocks(cfg, 5), kThreads, sizeof(ResSmem<4>), b);
        case 11: return launch_kernel(cfg, k_resample<8>, launch_blocks(cfg, 4), kThreads, sizeof(ResSmem<8>), b);
    }
    return cudaErrorInvalidValue;
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
