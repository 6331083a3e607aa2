// Cell-side kernels.
//  k_segments : one pass over the sorted particles; per cell (segment) the in-grid count
//               and the velocity sums sum(v), sum(v^2), sum(vx*vy).  Replaces
//               particleToGridKernel (particle_to_grid.cu:22-40), the weight-array copy and
//               the five statistical-moment prefix scans (dogm.cu:350-384).
//  k_cells    : one pass over all cells; fuses the predicted/free mass, the Dempster-Shafer
//               measurement update and newborn split (mass_update.cu:57-89), the persistent
//               reweighting (update_persistent_particles.cu:49-87), the moments
//               (statistical_moments.cu:78-106), the ego shift of the free mass
//               (ego_motion_compensation.cu:25-43) and the measurement copy (dogm.cu:205-208).
//  k_newborn  : newborn allocation over an exact scan of the newborn masses
//               (init_new_particles.cu:126-155, dogm.cu:323-348): records w_A / w_UA and
//               the key word of every newborn slot; the newborn particles themselves are
//               created where they are consumed, in the resample kernel.
#include "dogm_device.cuh"

namespace dogm_gb300 {

// ---------------------------------------------------------------------------------------
// Segmented reduction over sorted particles.
// ---------------------------------------------------------------------------------------
struct SegRun {
    int head;      // sorted position of the segment head inside this tile, -1 if it began earlier
    int n;
    float vx, vy, vxx, vyy, vxy;
};

__device__ __forceinline__ SegRun seg_combine(const SegRun& a, const SegRun& b) {
    if (b.head >= 0) return b;
    SegRun r;
    r.head = a.head;
    r.n = a.n + b.n;
    r.vx = __fadd_rn(a.vx, b.vx);
    r.vy = __fadd_rn(a.vy, b.vy);
    r.vxx = __fadd_rn(a.vxx, b.vxx);
    r.vyy = __fadd_rn(a.vyy, b.vyy);
    r.vxy = __fadd_rn(a.vxy, b.vxy);
    return r;
}

__device__ __forceinline__ SegRun seg_shfl_up(const SegRun& a, int o) {
    SegRun r;
    r.head = __shfl_up_sync(0xffffffffu, a.head, o);
    r.n = __shfl_up_sync(0xffffffffu, a.n, o);
    r.vx = __shfl_up_sync(0xffffffffu, a.vx, o);
    r.vy = __shfl_up_sync(0xffffffffu, a.vy, o);
    r.vxx = __shfl_up_sync(0xffffffffu, a.vxx, o);
    r.vyy = __shfl_up_sync(0xffffffffu, a.vyy, o);
    r.vxy = __shfl_up_sync(0xffffffffu, a.vxy, o);
    return r;
}

__device__ __forceinline__ SegSums to_sums(const SegRun& r) {
    SegSums s;
    s.n_in = r.n;
    s.vx = r.vx; s.vy = r.vy; s.vxx = r.vxx; s.vyy = r.vyy; s.vxy = r.vxy;
    return s;
}

__device__ __forceinline__ SegRun seg_item(uint32_t kw, float4 st, bool head, int pos) {
    SegRun it;
    it.head = head ? pos : -1;
    if (kw & kOutBit) {
        it.n = 0;
        it.vx = it.vy = it.vxx = it.vyy = it.vxy = 0.0f;
    } else {
        it.n = 1;
        it.vx = st.z;
        it.vy = st.w;
        it.vxx = __fmul_rn(st.z, st.z);
        it.vyy = __fmul_rn(st.w, st.w);
        it.vxy = __fmul_rn(st.z, st.w);
    }
    return it;
}

// One tile = kSegTile consecutive sorted particles, staged in shared memory with coalesced
// loads; thread i reduces items [i*kSegIpt, (i+1)*kSegIpt) in order, then a block-wide
// segmented scan joins the threads.  The combine order depends only on positions, so the
// sums are deterministic.
__global__ void __launch_bounds__(kThreads) k_segments(Batch* __restrict__ bt) {
    __shared__ uint32_t skey[kSegTile + 2];
    __shared__ float2 svel[kSegTile];
    __shared__ SegRun wagg[kThreads / 32];
    const int total = batch_total(bt, kStSeg);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int gi = grid_of_tile(bt, kStSeg, t);
        const GridDesc& g = bt->g[gi];
        const int lt = t - bt->prefix[gi][kStSeg];
        const int base = lt * kSegTile;
        const int n = min(kSegTile, g.N - base);
        for (int i = threadIdx.x; i < n; i += kThreads) {
            skey[1 + i] = g.S_key[base + i];
            const float4 st = g.S_state[base + i];
            svel[i] = make_float2(st.z, st.w);
        }
        if (threadIdx.x == 0) {
            skey[0] = base > 0 ? (g.S_key[base - 1] & kCellMask) : 0xffffffffu;
            skey[n + 1] = (base + n < g.N) ? (g.S_key[base + n] & kCellMask) : 0xffffffffu;
        }
        __syncthreads();

        const int j0 = threadIdx.x * kSegIpt;
        SegRun agg;
        agg.head = -1; agg.n = 0; agg.vx = agg.vy = agg.vxx = agg.vyy = agg.vxy = 0.0f;
        for (int r = 0; r < kSegIpt; ++r) {
            const int j = j0 + r;
            if (j >= n) break;
            const uint32_t kw = skey[1 + j];
            const uint32_t prev = (j == 0) ? skey[0] : (skey[j] & kCellMask);
            const float2 v = svel[j];
            agg = seg_combine(agg, seg_item(kw, make_float4(0.f, 0.f, v.x, v.y), (kw & kCellMask) != prev, base + j));
        }
        // block-wide exclusive segmented scan of the thread aggregates
        SegRun inc = agg;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const SegRun other = seg_shfl_up(inc, o);
            if (lane >= o) inc = seg_combine(other, inc);
        }
        if (lane == 31) wagg[warp] = inc;
        SegRun excl = seg_shfl_up(inc, 1);
        __syncthreads();
        SegRun wpre;
        wpre.head = -1; wpre.n = 0; wpre.vx = wpre.vy = wpre.vxx = wpre.vyy = wpre.vxy = 0.0f;
        for (int w = 0; w < warp; ++w) wpre = seg_combine(wpre, wagg[w]);
        excl = (lane == 0) ? wpre : seg_combine(wpre, excl);

        // re-walk and emit at segment tails
        SegRun run = excl;
        for (int r = 0; r < kSegIpt; ++r) {
            const int j = j0 + r;
            if (j >= n) break;
            const uint32_t kw = skey[1 + j];
            const uint32_t c = kw & kCellMask;
            const uint32_t prev = (j == 0) ? skey[0] : (skey[j] & kCellMask);
            const uint32_t next = (j == n - 1) ? skey[n + 1] : (skey[2 + j] & kCellMask);
            const float2 v = svel[j];
            run = seg_combine(run, seg_item(kw, make_float4(0.f, 0.f, v.x, v.y), c != prev, base + j));
            const int pos = base + j;
            if (c != next) {
                if (run.head >= 0) {
                    g.seg_i[c] = make_int4(run.head, pos, run.n, __float_as_int(run.vxy));
                    g.seg_f[c] = make_float4(run.vx, run.vy, run.vxx, run.vyy);
                    atomicOr(&g.occ_bits[c >> 5], 1u << (c & 31));
                } else {
                    g.seg_head[lt] = to_sums(run);
                    g.seg_i[c].y = pos;
                }
            } else if (j == n - 1) {
                if (run.head >= 0) {
                    g.seg_tail[lt] = to_sums(run);
                    g.seg_i[c].x = run.head;
                    atomicOr(&g.occ_bits[c >> 5], 1u << (c & 31));
                } else {
                    g.seg_head[lt] = to_sums(run);
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------
// Fused per-cell update.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_cells(Batch* __restrict__ bt) {
    __shared__ unsigned long long red[kThreads / 32];
    __shared__ unsigned long long red2[kThreads / 32];
    const int total = batch_total(bt, kStCell);
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int gi = grid_of_tile(bt, kStCell, t);
        const GridDesc& g = bt->g[gi];
        const int lt = t - bt->prefix[gi][kStCell];
        const int base = lt * kCellTile;
        const float c_pred = __fmul_rn(g.p_S, g.fs->w_res);  // predicted weight of an in-grid particle
        unsigned long long qb = 0ull, jq = 0ull;
        for (int r = 0; r < kCellIpt; ++r) {
            const int k = base + r * kThreads + threadIdx.x;
            if (k >= g.C) break;
            const int x = k % g.gs, y = k / g.gs;
            const bool occupied = (g.occ_bits[k >> 5] >> (k & 31)) & 1u;
            int start = -1, end = -1;
            SegSums s;
            s.n_in = 0; s.vx = s.vy = s.vxx = s.vyy = s.vxy = 0.0f;
            if (occupied) {
                const int4 si = g.seg_i[k];
                start = si.x;
                end = si.y;
                const int ts = start / kSegTile, te = end / kSegTile;
                if (ts == te) {
                    const float4 sf = g.seg_f[k];
                    s.n_in = si.z;
                    s.vxy = __int_as_float(si.w);
                    s.vx = sf.x; s.vy = sf.y; s.vxx = sf.z; s.vyy = sf.w;
                } else {
                    s = g.seg_tail[ts];
                    for (int tt = ts + 1; tt <= te; ++tt) {
                        const SegSums h = g.seg_head[tt];
                        s.n_in += h.n_in;
                        s.vx = __fadd_rn(s.vx, h.vx);
                        s.vy = __fadd_rn(s.vy, h.vy);
                        s.vxx = __fadd_rn(s.vxx, h.vxx);
                        s.vyy = __fadd_rn(s.vyy, h.vyy);
                        s.vxy = __fadd_rn(s.vxy, h.vxy);
                    }
                }
            }
            float free_prev;
            if (g.shifted) {
                const int sx = x + g.shift_x, sy = y + g.shift_y;
                const bool ok = sx > 0 && sx < g.gs && sy > 0 && sy < g.gs;  // strict, as the reference
                free_prev = ok ? g.free_old[sx + g.gs * sy] : 0.0f;
            } else {
                free_prev = g.free_old[k];
            }
            const dogm_measurement_cell m = g.meas_src[k];
            if (g.copy_meas) g.meas_own[k] = m;
            const CellOut o = cell_masses(s.n_in, c_pred, free_prev, g.alpha, g.p_B, m.free_mass, m.occ_mass);
            float muA = 0.0f, muUA = 0.0f, wp = 0.0f;
            float mx = 0.0f, my = 0.0f, vx = 0.0f, vy = 0.0f, cxy = 0.0f;
            if (occupied) {
                const float wu = __fmul_rn(m.likelihood, o.w_norm);
                const float swu = __fmul_rn((float)s.n_in, wu);
                muA = swu > 0.0f ? __fdiv_rn(o.rho_p, swu) : 0.0f;
                muUA = o.m_occ_pred > 0.0f ? __fdiv_rn(o.rho_p, o.m_occ_pred) : 0.0f;
                wp = __fadd_rn(__fmul_rn(__fmul_rn(m.p_A, muA), wu),
                               __fmul_rn(__fmul_rn(__fsub_rn(1.0f, m.p_A), muUA), o.w_norm));
                if (o.rho_p > 0.0f) {
                    const float inv = __fdiv_rn(1.0f, o.rho_p);
                    mx = __fmul_rn(inv, __fmul_rn(wp, s.vx));
                    my = __fmul_rn(inv, __fmul_rn(wp, s.vy));
                    vx = __fsub_rn(__fmul_rn(inv, __fmul_rn(wp, s.vxx)), __fmul_rn(mx, mx));
                    vy = __fsub_rn(__fmul_rn(inv, __fmul_rn(wp, s.vyy)), __fmul_rn(my, my));
                    cxy = __fsub_rn(__fmul_rn(inv, __fmul_rn(wp, s.vxy)), __fmul_rn(mx, my));
                }
            }
            float4* rec = reinterpret_cast<float4*>(g.cells + k);
            rec[0] = make_float4(__int_as_float(start), __int_as_float(end), o.rho_b, o.rho_p);
            rec[1] = make_float4(o.free_up, o.occ_up, o.m_occ_pred, muA);
            rec[2] = make_float4(muUA, 0.0f, 0.0f, mx);
            rec[3] = make_float4(my, vx, vy, cxy);
            g.free_new[k] = o.free_up;
            g.rho_b[k] = o.rho_b;
            g.w_cell[k] = wp;
            qb += quantize(o.rho_b, g.q_shift);
            // this cell's persistent particles sit at sorted positions [start, end]; their
            // quantised weights go to the resample tiles that hold them (exact integer adds)
            const unsigned long long qw = quantize(wp, g.q_shift);
            if (s.n_in > 0 && qw > 0ull) {
                jq += (unsigned long long)s.n_in * qw;
                const int ts = start / kResTile, te = end / kResTile;
                if (ts == te) {
                    atomicAdd(&g.res_sum[ts], (unsigned long long)s.n_in * qw);
                } else {
                    atomicAdd(&g.res_sum[ts], (unsigned long long)g.seg_tail[ts].n_in * qw);
                    for (int tt = ts + 1; tt <= te; ++tt)
                        atomicAdd(&g.res_sum[tt], (unsigned long long)g.seg_head[tt].n_in * qw);
                }
            }
        }
        unsigned long long tile_qb, tile_jq;
        block_excl_scan_u64(qb, red, &tile_qb);
        block_excl_scan_u64(jq, red2, &tile_jq);
        if (threadIdx.x == 0) {
            g.cell_sum[lt] = tile_qb;
            atomicAdd(&g.fs->qb_total, tile_qb);
            if (tile_jq) atomicAdd(&g.fs->joint_total, tile_jq);
        }
    }
}

// ---------------------------------------------------------------------------------------
// Newborn allocation.  Cell k owns newborn slots [floor(Q[k-1] B / Q), floor(Q[k] B / Q))
// of the exact prefix Q of quantised newborn masses; nu_A = round(n p_A) of them are
// associated (the reference marks nu_A + 1, racing with the next cell:
// init_new_particles.cu:145-153).  Writes w_A / w_UA into the records, the key word of each
// newborn slot, and the newborns' quantised weights into the resample tiles that will hold
// them.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void add_joint_range(TileAgg& agg, unsigned long long* res_sum, long long a, long long b,
                                                unsigned long long q) {
    if (q == 0ull) return;
    for (long long t = a / kResTile; t * kResTile < b; ++t) {
        const long long lo = max(a, t * (long long)kResTile);
        const long long hi = min(b, (t + 1) * (long long)kResTile);
        if (hi > lo) agg_add(agg, res_sum, t, (unsigned long long)(hi - lo) * q);
    }
}

constexpr int kOwnSlots = 16;  // newborn slots a thread fills for its own cell

__global__ void __launch_bounds__(kThreads) k_newborn(Batch* __restrict__ bt) {
    __shared__ unsigned long long red[2 * (kThreads / 32)];
    __shared__ TileAgg agg;
    __shared__ int s_bnd[kCellTile + 1];  // s_bnd[c]: first slot of cell c of the tile
    __shared__ int s_nuA[kCellTile];
    __shared__ int s_heavy[kCellTile];
    __shared__ int s_nheavy;
    const int total = batch_total(bt, kStBirth);
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int gi = grid_of_tile(bt, kStBirth, t);
        const GridDesc& g = bt->g[gi];
        const int lt = t - bt->prefix[gi][kStBirth];
        const int base = lt * kCellTile;
        const unsigned long long T = g.fs->qb_total;
        unsigned long long q[kCellIpt];
        float rb[kCellIpt];
        unsigned long long v = 0ull;
#pragma unroll
        for (int j = 0; j < kCellIpt; ++j) {
            const int k = base + threadIdx.x * kCellIpt + j;
            rb[j] = (k < g.C) ? g.rho_b[k] : 0.0f;
            q[j] = (k < g.C) ? quantize(rb[j], g.q_shift) : 0ull;
            v += q[j];
        }
        unsigned long long tile_sum;
        unsigned long long acc = block_scan_after(v, g.cell_sum, lt, red, &tile_sum);
        const float sc = T ? __fdiv_rn((float)g.B, __ull2float_rn(T)) : 0.0f;
        int lo_c = alloc_boundary_fast(acc, T, g.B, sc);
        if (threadIdx.x == 0) {
            s_bnd[0] = lo_c;
            s_nheavy = 0;
        }
        __syncthreads();
        agg_reset(agg, ((long long)g.N + s_bnd[0]) / kResTile);
        int bnd[kCellIpt + 1];
        bnd[0] = lo_c;
#pragma unroll
        for (int j = 0; j < kCellIpt; ++j) {
            acc += q[j];
            bnd[j + 1] = q[j] ? alloc_boundary_fast(acc, T, g.B, sc) : bnd[j];
            s_bnd[threadIdx.x * kCellIpt + j + 1] = bnd[j + 1];
        }
        __syncthreads();
        unsigned long long jq = 0ull;
        const long long N = g.N;
#pragma unroll
        for (int j = 0; j < kCellIpt; ++j) {
            const int k = base + threadIdx.x * kCellIpt + j;
            const int nnew = bnd[j + 1] - bnd[j];
            if (nnew > 0 && k < g.C) {
                const float pA = g.meas_own[k].p_A;
                const int nuA = (int)roundf(__fmul_rn((float)nnew, pA));
                const int nuUA = nnew - nuA;
                const float wA = nuA > 0 ? __fdiv_rn(__fmul_rn(pA, rb[j]), (float)nuA) : 0.0f;
                const float wUA = nuUA > 0 ? __fdiv_rn(__fmul_rn(__fsub_rn(1.0f, pA), rb[j]), (float)nuUA) : 0.0f;
                g.cells[k].w_A = wA;
                g.cells[k].w_UA = wUA;
                s_nuA[threadIdx.x * kCellIpt + j] = nuA;
                const int nA = min(max(nuA, 0), nnew);
                const unsigned long long qA = quantize(wA, g.q_shift), qU = quantize(wUA, g.q_shift);
                jq += (unsigned long long)nA * qA + (unsigned long long)(nnew - nA) * qU;
                add_joint_range(agg, g.res_sum, N + bnd[j], N + bnd[j] + nA, qA);
                add_joint_range(agg, g.res_sum, N + bnd[j] + nA, N + bnd[j + 1], qU);
            }
        }
        jq = warp_sum_u64(jq);
        if ((threadIdx.x & 31) == 0 && jq) atomicAdd(&g.fs->joint_total, jq);
        __syncthreads();  // every shared add and s_nuA entry is done
        agg_flush(agg, g.res_sum, g.tiles[kStResample]);
        // key word of every newborn slot of the tile: cell | associated bit.  A cell with few
        // newborns is filled by its own thread; the block fills the heavy cells together.
        uint32_t* __restrict__ B_key = g.B_key;
#pragma unroll
        for (int j = 0; j < kCellIpt; ++j) {
            const int c = threadIdx.x * kCellIpt + j;
            const int lo = bnd[j], hi = bnd[j + 1];
            if (hi - lo > 0 && hi - lo <= kOwnSlots) {
                const uint32_t key = (uint32_t)(base + c);
                const int nA = s_nuA[c];
                for (int sl = lo; sl < hi; ++sl) B_key[sl] = key | ((sl - lo) < nA ? kAssocBit : 0u);
            } else if (hi - lo > kOwnSlots) {
                s_heavy[atomicAdd(&s_nheavy, 1)] = c;
            }
        }
        __syncthreads();
        for (int h = 0; h < s_nheavy; ++h) {
            const int c = s_heavy[h];
            const int lo = s_bnd[c], hi = s_bnd[c + 1];
            const uint32_t key = (uint32_t)(base + c);
            const int nA = s_nuA[c];
            for (int sl = lo + threadIdx.x; sl < hi; sl += kThreads) B_key[sl] = key | ((sl - lo) < nA ? kAssocBit : 0u);
        }
        if (threadIdx.x == 0 && lt == 0) g.fs->n_birth = (T > 0ull) ? g.B : 0;
        __syncthreads();
    }
}

cudaError_t launch_segments(const Batch* d_batch, const LaunchCfg& cfg) {
    k_segments<<<cfg.num_sms * 4, kThreads, 0, cfg.stream>>>(const_cast<Batch*>(d_batch));
    return cudaGetLastError();
}

cudaError_t launch_cells(const Batch* d_batch, const LaunchCfg& cfg) {
    k_cells<<<cfg.num_sms * 4, kThreads, 0, cfg.stream>>>(const_cast<Batch*>(d_batch));
    return cudaGetLastError();
}

cudaError_t launch_newborn(const Batch* d_batch, const LaunchCfg& cfg) {
    k_newborn<<<cfg.num_sms * 4, kThreads, 0, cfg.stream>>>(const_cast<Batch*>(d_batch));
    return cudaGetLastError();
}

}  // namespace dogm_gb300
