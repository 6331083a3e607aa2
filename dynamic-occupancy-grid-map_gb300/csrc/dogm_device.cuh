// Device helpers shared by the DOGM kernels: Philox draws, exact fixed-point arithmetic,
// the per-cell Dempster-Shafer update, tile claiming and bounded waits.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "dogm_internal.h"

namespace dogm_gb300 {

// ---------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers: As Easy as 1, 2, 3",
// SC'11): 10 rounds of two 32x32->64 multiplies per round, Weyl-sequence key schedule.
// ---------------------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
    constexpr uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    constexpr uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
        const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += W0;
        k1 += W1;
    }
    return c;
}

__device__ __forceinline__ U4 draw_block(const GridDesc& g, uint32_t index, uint32_t frame, uint32_t stage) {
    return philox4x32_10(U4{index, frame, stage, g.stream_id}, g.seed_lo, g.seed_hi);
}

// 24-bit uniforms: (0,1] for logarithms and the reference's (0,1] curand_uniform range,
// [0,1) for angles.
__device__ __forceinline__ float u01_open0(uint32_t x) { return (float)((x >> 8) + 1u) * 5.9604644775390625e-8f; }
__device__ __forceinline__ float u01_open1(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-8f; }

// Box-Muller: two standard normals from two uniforms, with the hardware approximations of
// log, sin and cos (absolute error ~1e-6 on these ranges, far below the noise scales).
__device__ __forceinline__ float2 box_muller(uint32_t a, uint32_t b) {
    const float u1 = u01_open0(a);
    const float u2 = u01_open1(b);
    const float r = sqrtf(-2.0f * __logf(u1));
    float s, c;
    __sincosf(6.28318530717958647692f * u2 - 3.14159265358979323846f, &s, &c);
    return make_float2(-r * c, -r * s);  // angle shifted into [-pi, pi): cos(x+pi) = -cos x
}

// ---------------------------------------------------------------------------------------
// Exact fixed point.  Weights and masses are quantised to multiples of 2^-S (S = q_shift,
// chosen per grid so that every sum stays below 2^62); all scans over them are exact
// integer scans, so any summation order gives the same bits.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long quantize(float w, int S) {
    // round-to-nearest-even of w * 2^S for w in [0, 2]; <= 0 or NaN -> 0, > 2 clamps to 2.
    // Scaling by 2^S (0 <= S <= 61) is exact in float: a normal w stays normal, a denormal w
    // only moves its bits up, and w * 2^S <= 2^62 stays finite.  One round-to-nearest-even
    // conversion of the exact product is then the rounded integer.
    if (!(w > 0.0f)) return 0ull;
    if (w > 2.0f) w = 2.0f;
    return __float2ull_rn(__fmul_rn(w, __int_as_float((127 + S) << 23)));
}

// 96-bit products of a 64-bit and a 32-bit factor (every product here is below 2^86:
// weights < 2^62 times counts < 2^24).
struct U96 { unsigned long long lo; unsigned int hi; };
__device__ __forceinline__ U96 mul_u64_u32(unsigned long long a, unsigned int b) {
    const unsigned long long p0 = (unsigned long long)(unsigned int)a * b;
    const unsigned long long p1 = (a >> 32) * b;
    const unsigned long long lo = p0 + (p1 << 32);
    return U96{lo, (unsigned int)(p1 >> 32) + (lo < p0 ? 1u : 0u)};
}
__device__ __forceinline__ U96 add96(U96 a, unsigned long long x) {
    const unsigned long long lo = a.lo + x;
    return U96{lo, a.hi + (lo < a.lo ? 1u : 0u)};
}
__device__ __forceinline__ bool lt96(U96 a, U96 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }

// floor(Q * M / T) for Q <= T, T > 0: how many of M slots a prefix mass Q owns.
// (The reference scales a float prefix sum by M / total and truncates:
//  dogm/src/kernel/init_new_particles.cu:30-43,66-74.)
__device__ __forceinline__ int alloc_boundary(unsigned long long Q, unsigned long long T, int M) {
    if (T == 0ull) return 0;
    if (Q >= T) return M;
    const U96 qm = mul_u64_u32(Q, (unsigned int)M);
    const float f = __fmul_rn(__fdiv_rn(__ull2float_rn(Q), __ull2float_rn(T)), (float)M);
    int b = (int)f;
    b = b < 0 ? 0 : (b > M ? M : b);
    // b = largest value with b*T <= Q*M
    while (b > 0 && lt96(qm, mul_u64_u32(T, (unsigned int)b))) --b;
    while (b < M && !lt96(qm, mul_u64_u32(T, (unsigned int)(b + 1)))) ++b;
    return b;
}

// The same with a precomputed scale sc = fl(M / fl(T)): when the float estimate Q * sc is
// farther from an integer than its error bound (4 roundings, relative 2.4e-7 < 3e-7), its
// floor is exact and the 96-bit check is skipped; otherwise the exact path decides.
__device__ __forceinline__ int alloc_boundary_fast(unsigned long long Q, unsigned long long T, int M, float sc) {
    if (T == 0ull) return 0;
    if (Q >= T) return M;
    const float f = __fmul_rn(__ull2float_rn(Q), sc);
    const float err = __fmaf_rn(f, 3e-7f, 1e-30f);
    const float lo = floorf(__fsub_rn(f, err)), hi = floorf(__fadd_rn(f, err));
    if (lo == hi && lo >= 0.0f && lo <= (float)M) return (int)lo;
    return alloc_boundary(Q, T, M);
}

// Systematic resampling comb: slot i takes the joint particle j with
// A[j-1]*N <= i*T + U < A[j]*N (A = inclusive exact prefix, T = total, U in [0,T)).
// comb_count(a) = #{ i in [0,N) : i*T + U < a*N }.  T == 0 sends every slot to particle 0.
__device__ __forceinline__ int comb_count(unsigned long long a, unsigned long long T, unsigned long long U, int N) {
    if (T == 0ull) return N;
    if (a >= T) return N;
    const U96 rhs = mul_u64_u32(a, (unsigned int)N);
    const float f = __fdiv_rn(__fsub_rn(__fmul_rn(__ull2float_rn(a), (float)N), __ull2float_rn(U)),
                              __ull2float_rn(T));
    int c = (int)ceilf(f);
    c = c < 0 ? 0 : (c > N ? N : c);
    // P(i): i*T + U < a*N holds for i < result and fails from result on
    while (c > 0 && !lt96(add96(mul_u64_u32(T, (unsigned int)(c - 1)), U), rhs)) --c;
    while (c < N && lt96(add96(mul_u64_u32(T, (unsigned int)c), U), rhs)) ++c;
    return c;
}

// ---------------------------------------------------------------------------------------
// Per-cell update (FP32).  Order of operations is fixed with _rn intrinsics so the host
// oracle reproduces every bit.  Formulas follow dogm/src/kernel/mass_update.cu:12-45 and
// dogm/src/kernel/update_persistent_particles.cu:16-47.
// ---------------------------------------------------------------------------------------
struct CellOut {
    float m_occ_pred, w_norm, free_up, occ_up, rho_b, rho_p;
};

__device__ __forceinline__ CellOut cell_masses(int n_in, float c, float free_prev, float alpha, float p_B,
                                               float z_free, float z_occ) {
    CellOut o;
    float m = __fmul_rn((float)n_in, c);  // sum of the predicted weights of the cell
    float wn = c;
    if (m > 1.0f) {                        // mass_update.cu:75-79
        wn = __fdiv_rn(c, m);
        m = 1.0f;
    }
    const float one_m = __fsub_rn(1.0f, m);
    const float mf = fminf(__fmul_rn(alpha, free_prev), one_m);         // predict_free_mass
    const float unk = __fsub_rn(one_m, mf);                              // update_masses
    const float meas_unk = __fsub_rn(__fsub_rn(1.0f, z_free), z_occ);
    const float K = __fadd_rn(__fmul_rn(mf, z_occ), __fmul_rn(m, z_free));
    const float den = __fsub_rn(1.0f, K);
    const float occ = __fdiv_rn(__fadd_rn(__fadd_rn(__fmul_rn(m, meas_unk), __fmul_rn(unk, z_occ)), __fmul_rn(m, z_occ)), den);
    const float fre = __fdiv_rn(__fadd_rn(__fadd_rn(__fmul_rn(mf, meas_unk), __fmul_rn(unk, z_free)), __fmul_rn(mf, z_free)), den);
    // separate_newborn_part: rho_b = occ*p_B*(1-m) / (m + p_B*(1-m))
    const float pb1m = __fmul_rn(p_B, one_m);
    const float rb = __fdiv_rn(__fmul_rn(__fmul_rn(occ, p_B), one_m), __fadd_rn(m, pb1m));
    o.m_occ_pred = m;
    o.w_norm = wn;
    o.free_up = fre;
    o.occ_up = occ;
    o.rho_b = rb;
    o.rho_p = __fsub_rn(occ, rb);
    return o;
}

// ---------------------------------------------------------------------------------------
// Programmatic dependent launch: wait until the previous kernel of the stream has completed
// and its writes are visible (a no-op for a launch without the attribute).  First statement of
// every frame kernel, so no global access of this kernel overlaps the previous one.  No kernel
// triggers its dependents early: the next launch is prepared while this one completes (an
// early trigger, with the next kernel's blocks parked on the SMs, measured 3 % slower).
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void grid_dependency_begin() {
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
}

// ---------------------------------------------------------------------------------------
// Asynchronous global -> shared copies (cp.async): a thread's copies land while it works on
// something else; cp_async_wait_all() makes that thread's own copies visible to it.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// ---------------------------------------------------------------------------------------
// Batches: tile claiming and grid lookup.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ int batch_total(const Batch* bt, int stage) { return bt->prefix[bt->n_grids][stage]; }

__device__ __forceinline__ int grid_of_tile(const Batch* bt, int stage, int t) {
    int lo = 0, hi = bt->n_grids - 1;
    while (lo < hi) {  // largest i with prefix[i][stage] <= t
        const int mid = (lo + hi + 1) >> 1;
        if (bt->prefix[mid][stage] <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Dynamic tile claim: the next index of the stage's work counter (reset with every frame's
// descriptors).  Every thread of the block gets the same tile.
__device__ __forceinline__ int claim_tile(Batch* bt, int stage, int* smem_slot) {
    if (threadIdx.x == 0) *smem_slot = (int)atomicAdd(&bt->counters[stage], 1u);
    __syncthreads();
    const int t = *smem_slot;
    __syncthreads();
    return t;
}

// ---------------------------------------------------------------------------------------
// Status bits (kernels record failed checks and finish; the host turns them into status
// codes).  No kernel of the update waits on another block.
// ---------------------------------------------------------------------------------------

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) { return *(const volatile uint32_t*)p; }
__device__ __forceinline__ unsigned long long ld_volatile(const unsigned long long* p) {
    return *(const volatile unsigned long long*)p;
}
__device__ __forceinline__ void st_volatile(uint32_t* p, uint32_t v) { *(volatile uint32_t*)p = v; }
__device__ __forceinline__ void st_volatile(unsigned long long* p, unsigned long long v) {
    *(volatile unsigned long long*)p = v;
}

__device__ __forceinline__ void flag_status(const GridDesc& g, uint32_t bits) {
    atomicOr(&g.fs->status, bits);
    atomicOr(g.status_out, bits);
}
__device__ __forceinline__ void flag_timeout(const GridDesc& g) { flag_status(g, kStatusTimeout); }

// Adds v to the exact joint-weight sum of resample tile t.
__device__ __forceinline__ void add_res_sum(const GridDesc& g, long long t, unsigned long long v) {
    atomicAdd(&g.res_sum[t], v);
}

// Block-wide exclusive scan of one 64-bit value per thread (NT threads).  Returns the
// exclusive prefix; *total receives the block sum.  scratch: >= 8 entries.
template <int NT = kThreads>
__device__ __forceinline__ unsigned long long block_excl_scan_u64(unsigned long long v, unsigned long long* scratch,
                                                                  unsigned long long* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) scratch[warp] = x;
    __syncthreads();
    unsigned long long wpre = 0ull, tot = 0ull;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) {
        const unsigned long long s = scratch[w];
        if (w < warp) wpre += s;
        tot += s;
    }
    __syncthreads();
    *total = tot;
    return wpre + x - v;
}

// Sum of sums[0 .. t) by the whole block (the exclusive prefix of tile t from per-tile
// sums that a previous kernel completed; exact, so any order gives the same bits).
__device__ __forceinline__ unsigned long long block_sum_before(const unsigned long long* sums, int t,
                                                               unsigned long long* scratch) {
    unsigned long long v = 0ull;
    for (int i = threadIdx.x; i < t; i += blockDim.x) v += sums[i];
    unsigned long long total;
    block_excl_scan_u64(v, scratch, &total);
    return total;
}

// This thread's share of sums[0 .. t) (the per-tile sums a previous kernel completed), four
// independent loads in flight per thread.  Split from the scan below so that a caller can
// issue these loads next to its own before waiting on either.
__device__ __forceinline__ unsigned long long block_prefix_part(const unsigned long long* sums, int t) {
    unsigned long long part = 0ull;
    for (int i0 = 0; i0 < t; i0 += 4 * kThreads) {
        unsigned long long a[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i = i0 + u * kThreads + (int)threadIdx.x;
            a[u] = i < t ? sums[i] : 0ull;
        }
        part += (a[0] + a[1]) + (a[2] + a[3]);
    }
    return part;
}

// Exclusive scan of one 64-bit value per thread, offset by the block total of the threads'
// parts (block_prefix_part): returns sum(parts) + (exclusive prefix of v); *total gets the
// block's sum of v.  One barrier round for both.
__device__ __forceinline__ unsigned long long block_scan_with_part(unsigned long long v, unsigned long long part,
                                                                   unsigned long long* scratch16,
                                                                   unsigned long long* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
        part += __shfl_xor_sync(0xffffffffu, part, o);
    }
    if (lane == 31) scratch16[warp] = x;
    if (lane == 0) scratch16[8 + warp] = part;
    __syncthreads();
    unsigned long long wpre = 0ull, tot = 0ull, before = 0ull;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) {
        const unsigned long long s = scratch16[w];
        if (w < warp) wpre += s;
        tot += s;
        before += scratch16[8 + w];
    }
    __syncthreads();
    *total = tot;
    return before + wpre + x - v;
}

// Exclusive scan of one 64-bit value per thread, offset by sums[0 .. t) (the per-tile sums a
// previous kernel completed): returns sums[0..t) + (exclusive prefix of v); *total gets the
// block's sum of v.
__device__ __forceinline__ unsigned long long block_scan_after(unsigned long long v, const unsigned long long* sums,
                                                               int t, unsigned long long* scratch16,
                                                               unsigned long long* total) {
    return block_scan_with_part(v, block_prefix_part(sums, t), scratch16, total);
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Per-block accumulation of exact integer sums into a window of consecutive global
// counters [first, first + kAggSlots): shared atomics inside the window, global atomics
// outside it.  flush() adds each non-zero shared counter to its global counter once.
constexpr int kAggSlots = 64;
struct TileAgg {
    unsigned long long v[kAggSlots];
    long long first;
};
__device__ __forceinline__ void agg_reset(TileAgg& a, long long first) {
    for (int i = threadIdx.x; i < kAggSlots; i += blockDim.x) a.v[i] = 0ull;
    if (threadIdx.x == 0) a.first = first;
}
__device__ __forceinline__ void agg_add(TileAgg& a, unsigned long long* global, long long idx,
                                        unsigned long long x) {
    const long long o = idx - a.first;
    if (o >= 0 && o < kAggSlots) atomicAdd(&a.v[o], x);
    else atomicAdd(&global[idx], x);
}
__device__ __forceinline__ void agg_flush(TileAgg& a, unsigned long long* global, long long limit) {
    for (int i = threadIdx.x; i < kAggSlots; i += blockDim.x)
        if (a.v[i] && a.first + i < limit) atomicAdd(&global[a.first + i], a.v[i]);
}

// Block-wide exclusive scan of one int per thread.
__device__ __forceinline__ int block_excl_scan_i32(int v, int* scratch, int* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) scratch[warp] = x;
    __syncthreads();
    int wpre = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) {
        const int s = scratch[w];
        if (w < warp) wpre += s;
        tot += s;
    }
    __syncthreads();
    *total = tot;
    return wpre + x - v;
}

}  // namespace dogm_gb300
