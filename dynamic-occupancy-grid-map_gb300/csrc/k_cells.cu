// Cell-side kernels.
//  k_cells    : one pass over all cells and the particles in them; fuses the second half of
//               the particle sort (a stable counting sort of the job's buckets by cell), the
//               particle-to-cell segmented reduction, the mass update, reweighting, moments,
//               ego shift of the free mass and the measurement copy.
//  k_newborn  : newborn allocation over an exact scan of the newborn masses
//               (init_new_particles.cu:126-155, dogm.cu:323-348): records w_A / w_UA and
//               the key word of every newborn slot; the newborn particles themselves are
//               created where they are consumed, in the resample kernel.
#include <cstddef>

#include "dogm_device.cuh"

namespace dogm_gb300 {

// ---------------------------------------------------------------------------------------
// Open runs of the segmented reduction: the sums that flow from one thread's particles into
// the next thread's.  Bit 31 of fn marks a run that starts (has a segment head) inside the
// span it summarises; bits 0..30 count in-grid particles.
// ---------------------------------------------------------------------------------------
struct Run {
    uint32_t fn;
    float vx, vy, vxx, vyy, vxy;
};
constexpr uint32_t kRunHead = 1u << 31;

__device__ __forceinline__ Run run_empty(uint32_t flag) {
    Run r;
    r.fn = flag;
    r.vx = r.vy = r.vxx = r.vyy = r.vxy = 0.0f;
    return r;
}

// a followed by b
__device__ __forceinline__ Run run_combine(const Run& a, const Run& b) {
    if (b.fn & kRunHead) return b;
    Run r;
    r.fn = a.fn + b.fn;
    r.vx = __fadd_rn(a.vx, b.vx);
    r.vy = __fadd_rn(a.vy, b.vy);
    r.vxx = __fadd_rn(a.vxx, b.vxx);
    r.vyy = __fadd_rn(a.vyy, b.vyy);
    r.vxy = __fadd_rn(a.vxy, b.vxy);
    return r;
}

__device__ __forceinline__ void run_add(Run& r, uint32_t kw, float2 v) {
    if (kw & kOutBit) return;
    r.fn += 1u;
    r.vx = __fadd_rn(r.vx, v.x);
    r.vy = __fadd_rn(r.vy, v.y);
    r.vxx = __fadd_rn(r.vxx, __fmul_rn(v.x, v.x));
    r.vyy = __fadd_rn(r.vyy, __fmul_rn(v.y, v.y));
    r.vxy = __fadd_rn(r.vxy, __fmul_rn(v.x, v.y));
}

__device__ __forceinline__ Run run_shfl_up(const Run& a, int o) {
    Run r;
    r.fn = __shfl_up_sync(0xffffffffu, a.fn, o);
    r.vx = __shfl_up_sync(0xffffffffu, a.vx, o);
    r.vy = __shfl_up_sync(0xffffffffu, a.vy, o);
    r.vxx = __shfl_up_sync(0xffffffffu, a.vxx, o);
    r.vyy = __shfl_up_sync(0xffffffffu, a.vyy, o);
    r.vxy = __shfl_up_sync(0xffffffffu, a.vxy, o);
    return r;
}

// ---------------------------------------------------------------------------------------
// Fused per-cell update over one tile of kCellTile cells and the particles that lie in it,
// positions [start, end) of the bucketed (T) and sorted (S) arrays (the tile's ctile_job).
//   S  stable counting sort of the bucket by cell, T -> S: per-cell counts, their exclusive
//      scan, then, chunk by chunk in bucket order, each particle's rank among the earlier
//      particles of its cell (warp ranks by match_any, per-warp counts, offsets across warps).
//      The writes land in the tile's own window of S, which stays in L2 for phase A.
//   A  segmented reduction of those particles into per-cell shared sums (sorted range,
//      in-grid count, sum(v), sum(v^2), sum(vx*vy)).  Each thread walks its own share of
//      consecutive particles: a cell whose particles start and end inside the thread is
//      written directly; the run still open at the thread's end flows through a block scan
//      to the thread holding the cell's last particle, which writes it.  Plain stores only (every
//      slot has one writer), and the add order depends only on positions, so the sums are
//      deterministic.  Replaces particleToGridKernel (particle_to_grid.cu:22-40), the
//      weight-array copy and the five statistical-moment prefix scans (dogm.cu:350-384).
//   B  per cell: predicted and free mass, Dempster-Shafer update and newborn split
//      (mass_update.cu:57-89), persistent reweighting (update_persistent_particles.cu:49-87),
//      moments (statistical_moments.cu:78-106), ego shift of the free mass
//      (ego_motion_compensation.cu:25-43) and the measurement copy (dogm.cu:205-208).
//      The quantised weight of each cell's persistent particles goes to the resample
//      tiles that hold them.
// ---------------------------------------------------------------------------------------
constexpr int kCellThreads = 512;  // two cells per thread: a tile finishes in half the time
static_assert(kCellTile % kCellThreads == 0, "whole cells per thread");

constexpr int kCellWarps = kCellThreads / 32;
constexpr int kBucketIpt = 8;  // bucket particles per thread in a chunk of the counting sort
constexpr int kBucketChunk = kCellThreads * kBucketIpt;
static_assert(kCellTile == 2 * kCellThreads && kBucketChunk < 65536, "one pair of 16-bit cell counts per thread");

// Records a warp stages at a time in B (half of its 32 cells): the staging area then fits in the
// space the sort's counts use, and two blocks of the pass leave the SM the larger L1 split.
constexpr int kStageRecs = 16;

struct CellSmem {
    dogm_measurement_cell meas[kCellTile];  // prefetched (cp.async) while S and A run
    float free_prev[kCellTile];             // previous free mass, ego shift applied
    union {
        // S: per-warp particle counts per cell in the current chunk, then offsets across warps
        uint16_t whist[kCellWarps][kCellTile];
        struct {            // A and B: each occupied cell's range, in-grid count and sums
            int start[kCellTile];   // sorted position of the first particle
            int end[kCellTile];     // sorted position of the last particle
            int n_in[kCellTile];    // in-grid particles
            float vx[kCellTile], vy[kCellTile], vxx[kCellTile], vyy[kCellTile], vxy[kCellTile];
        } cell;
    } u1;
    union {
        struct {            // S: particles per cell, then running offsets (two chunks in turn)
            uint32_t cnt[kCellTile];
            uint32_t off[2][kCellTile];
        } srt;
        // B, per warp: kStageRecs of its cell records, staged so that the warp stores them as
        // 512 contiguous bytes per instruction instead of four 16-byte pieces at 64-byte stride
        float4 stage[kCellWarps][kStageRecs * 4];
    } u2;
    uint8_t occ[kCellTile];  // cell holds particles (from the sort's counts; read by its B thread)
    int scan[kCellWarps];
    Run wagg[kCellThreads / 32];  // each warp's run, then (wpre) the runs before each warp
    Run wpre[kCellThreads / 32];
    unsigned long long red[kCellThreads / 32], red2[kCellThreads / 32];
    uint4 job[2];  // the block's current tile and the one claimed for the next iteration:
    int jt[2];     // work index (>= total: none left), grid, and ctile_job entry
    int jgrid[2];
};
static_assert(offsetof(CellSmem, meas) % 16 == 0, "16-byte cp.async destination");
static_assert(offsetof(CellSmem, u2) % 16 == 0, "16-byte staged records");
static_assert(sizeof(CellSmem) <= 80 * 1024, "two blocks per SM within the 164 KB shared-memory split");
static_assert(offsetof(CellSmem, job) % 16 == 0, "16-byte cp.async destination");
static_assert(sizeof(dogm_grid_cell) == 64, "a record is four float4");

// Record chunk j of record l is staged at float4 slot 4 l + (j ^ ((l >> 1) & 3)): for each j the
// eight records of a 128-byte shared-memory wavefront hit eight distinct 16-byte bank groups, and
// reading record r's chunk c back from slot 4 r + (c ^ ((r >> 1) & 3)) gives lanes 4 q .. 4 q + 3
// one whole record, again without conflicts.
__device__ __forceinline__ int stage_slot(int rec, int chunk) { return rec * 4 + (chunk ^ ((rec >> 1) & 3)); }

// The quantised weights of a cell's in-grid persistent particles (sorted positions
// [start, end]) added to the resample tiles that hold them.  Out-of-grid particles (weight
// 0) lie only in border cells; only for those is a split across tiles counted from the keys.
__device__ __forceinline__ void add_persistent(const GridDesc& g, int start, int end, int n_in,
                                               unsigned long long qw) {
    const int rb = g.res_bits;
    const int ts = start >> rb, te = end >> rb;
    if (ts == te) {
        add_res_sum(g, ts, (unsigned long long)n_in * qw);
        return;
    }
    const bool all_in = n_in == end - start + 1;
    for (int rt = ts; rt <= te; ++rt) {
        const int lo = max(start, rt << rb), hi = min(end + 1, (rt + 1) << rb);
        int cnt = hi - lo;
        if (!all_in) {
            cnt = 0;
            for (int i = lo; i < hi; ++i) cnt += (g.S_key[i] & kOutBit) ? 0 : 1;
        }
        if (cnt) add_res_sum(g, rt, (unsigned long long)cnt * qw);
    }
}

__device__ __forceinline__ void put_cell(CellSmem& sm, const GridDesc& g, uint32_t cl, int last, const Run& r) {
    if (cl >= (uint32_t)kCellTile) {  // only inconsistent tile counts get here
        flag_status(g, kStatusBounds);
        return;
    }
    sm.u1.cell.end[cl] = last;
    sm.u1.cell.n_in[cl] = (int)(r.fn & ~kRunHead);
    sm.u1.cell.vx[cl] = r.vx;
    sm.u1.cell.vy[cl] = r.vy;
    sm.u1.cell.vxx[cl] = r.vxx;
    sm.u1.cell.vyy[cl] = r.vyy;
    sm.u1.cell.vxy[cl] = r.vxy;
}

// S: the stable counting sort of one bucket (bucketed positions [p0, p1) of T, whose cells lie
// in [base, base + kCellTile)) into the same positions of S.  The bucket is ranked in chunks of
// at most kBucketChunk particles; within a chunk warp w takes the contiguous segment
// [w * 32 R, (w + 1) * 32 R) in R rounds of 32 (R = the chunk's particles / 512, rounded up), so
// that bucket order is (warp, round, lane) and per-warp counts give stable ranks.  A bucket of
// one chunk is ranked in a single pass: its per-warp counts also give the per-cell totals.
// Ends with a barrier.
__device__ __forceinline__ int chunk_rounds(int n) { return min(kBucketIpt, (n + kCellThreads - 1) / kCellThreads); }

__device__ __forceinline__ void sort_bucket(CellSmem& sm, const GridDesc& g, int base, int p0, int p1) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const int np = p1 - p0;
    const bool single = np <= kBucketChunk;  // block-uniform
    uint32_t key[kBucketIpt];
    uint16_t rank[kBucketIpt];

    // the cell (within the tile) of key word kw, or ~0 for no particle; a key outside the
    // tile can only come from inconsistent counts and is not placed
    auto cell_of = [&](uint32_t kw) -> uint32_t {
        const uint32_t c = kw == 0xffffffffu ? 0xffffffffu : (kw & kCellMask) - (uint32_t)base;
        return c < (uint32_t)kCellTile ? c : 0xffffffffu;
    };
    // the bucketed particles are last read in this pass: evict-first loads (__ldcs) keep L2
    // for the sorted copy, which resampling reads again
    auto load_chunk = [&](int c0, int R) {
        const int wbase = c0 + warp * 32 * R;
#pragma unroll
        for (int k = 0; k < kBucketIpt; ++k) {
            const int i = wbase + k * 32 + lane;
            key[k] = (k < R && i < p1) ? __ldcs(g.T_key + i) : 0xffffffffu;
        }
    };
    auto zero_whist = [&]() {
        uint4* wz = reinterpret_cast<uint4*>(&sm.u1.whist[0][0]);
        for (int i = threadIdx.x; i < (int)(sizeof(sm.u1.whist) / sizeof(uint4)); i += kCellThreads)
            wz[i] = make_uint4(0u, 0u, 0u, 0u);
    };
    // warp ranks of the loaded chunk: rank[k] = earlier same-cell particles of the warp
    auto rank_chunk = [&](int R) {
#pragma unroll
        for (int k = 0; k < kBucketIpt; ++k) {
            if (k >= R) break;  // block-uniform
            const uint32_t d = cell_of(key[k]);
            const uint32_t peers = __match_any_sync(0xffffffffu, d);
            uint16_t before = 0;
            if (d != 0xffffffffu) before = sm.u1.whist[warp][d];
            rank[k] = (uint16_t)(before + __popc(peers & lt_mask));
            __syncwarp();
            if (d != 0xffffffffu && lane == __ffs(peers) - 1) sm.u1.whist[warp][d] = (uint16_t)(before + __popc(peers));
            __syncwarp();
        }
    };
    // exclusive scan of cnt[] into off[0][] (the first position of each cell in the bucket)
    auto scan_counts = [&]() {
        constexpr int kPer = kCellTile / kCellThreads;
        const int c0 = threadIdx.x * kPer;
        uint32_t v[kPer], s = 0u;
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            v[j] = sm.u2.srt.cnt[c0 + j];
            s += v[j];
        }
        uint32_t x = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) sm.scan[warp] = (int)x;
        __syncthreads();
        uint32_t e = x - s;
        for (int w = 0; w < warp; ++w) e += (uint32_t)sm.scan[w];
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            sm.u2.srt.off[0][c0 + j] = e;
            e += v[j];
        }
    };
    // the loaded chunk to its sorted positions; per half of the rounds every state load is
    // issued before the first store
    auto scatter_chunk = [&](int c0, int R, int cur) {
        const int wbase = c0 + warp * 32 * R;
        constexpr int kHalf = kBucketIpt / 2;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (h * kHalf >= R) break;  // block-uniform
            float4 st[kHalf];
            int out[kHalf];
#pragma unroll
            for (int j = 0; j < kHalf; ++j) {
                const int k = h * kHalf + j;
                const int i = wbase + k * 32 + lane;
                const uint32_t c = cell_of(key[k]);
                out[j] = -1;
                if (k < R && c != 0xffffffffu)
                    out[j] = p0 + (int)(sm.u2.srt.off[cur][c] + sm.u1.whist[warp][c] + rank[k]);
                st[j] = __ldcs(g.T_state + ((k < R && i < p1) ? i : p1 - 1));
            }
#pragma unroll
            for (int j = 0; j < kHalf; ++j) {
                const int k = h * kHalf + j;
                const int i = wbase + k * 32 + lane;
                if (k >= R || i >= p1) continue;
                if (out[j] < p0 || out[j] >= p1) {  // only inconsistent counts get here
                    flag_status(g, kStatusBounds);
                    continue;
                }
                g.S_key[out[j]] = key[k];
                g.S_state[out[j]] = st[j];
                if (g.dbg_perm) g.dbg_perm[out[j]] = g.T_idx[i];
            }
        }
    };

    if (single) {
        // one pass: warp ranks and counts; the column prefix over the warps gives each warp's
        // offset within its cell and the cell's total
        const int R = chunk_rounds(np);
        load_chunk(p0, R);
        zero_whist();
        __syncthreads();
        rank_chunk(R);
        __syncthreads();
        {
            // two cells per 32-bit word: the halves never carry (a chunk holds <= 4096)
            uint32_t* wh = reinterpret_cast<uint32_t*>(&sm.u1.whist[0][0]);
            const int cp = threadIdx.x;  // cells 2 cp, 2 cp + 1
            uint32_t acc = 0u;
#pragma unroll
            for (int w = 0; w < kCellWarps; ++w) {
                const uint32_t n = wh[w * (kCellTile / 2) + cp];
                wh[w * (kCellTile / 2) + cp] = acc;
                acc += n;
            }
            sm.u2.srt.cnt[2 * cp] = acc & 0xffffu;
            sm.u2.srt.cnt[2 * cp + 1] = acc >> 16;
        }
        __syncthreads();
        scan_counts();
        __syncthreads();
        scatter_chunk(p0, R, 0);
        __syncthreads();
        return;
    }

    // several chunks: particles per cell over the whole bucket first
    for (int c = threadIdx.x; c < kCellTile; c += kCellThreads) sm.u2.srt.cnt[c] = 0u;
    __syncthreads();
    for (int c0 = p0; c0 < p1; c0 += kBucketChunk) {
        const int R = chunk_rounds(min(kBucketChunk, p1 - c0));
        load_chunk(c0, R);
#pragma unroll
        for (int k = 0; k < kBucketIpt; ++k) {
            if (k >= R) break;  // block-uniform
            const uint32_t d = cell_of(key[k]);
            const uint32_t peers = __match_any_sync(0xffffffffu, d);
            if (d != 0xffffffffu && lane == __ffs(peers) - 1) atomicAdd(&sm.u2.srt.cnt[d], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    scan_counts();
    // then chunk by chunk in bucket order, the cells' offsets carried from chunk to chunk
    int cur = 0;
    for (int c0 = p0; c0 < p1; c0 += kBucketChunk, cur ^= 1) {
        const int R = chunk_rounds(min(kBucketChunk, p1 - c0));
        load_chunk(c0, R);
        zero_whist();
        __syncthreads();
        rank_chunk(R);
        __syncthreads();
        {
            // two cells per 32-bit word, as above
            uint32_t* wh = reinterpret_cast<uint32_t*>(&sm.u1.whist[0][0]);
            const int cp = threadIdx.x;
            uint32_t acc = 0u;
#pragma unroll
            for (int w = 0; w < kCellWarps; ++w) {
                const uint32_t n = wh[w * (kCellTile / 2) + cp];
                wh[w * (kCellTile / 2) + cp] = acc;
                acc += n;
            }
            sm.u2.srt.off[cur ^ 1][2 * cp] = sm.u2.srt.off[cur][2 * cp] + (acc & 0xffffu);
            sm.u2.srt.off[cur ^ 1][2 * cp + 1] = sm.u2.srt.off[cur][2 * cp + 1] + (acc >> 16);
        }
        __syncthreads();
        scatter_chunk(c0, R, cur);
        __syncthreads();
    }
}

// STAGED: a stage call (GridDesc::stage_mask selects the parts); the update's instantiation runs
// every part with no mask tests.  FINE: some grid of the launch sorts by buckets finer than a
// cell tile, so a job may be a run of buckets or an unused slot; without it every job is a whole
// tile.
template <bool STAGED, bool FINE>
__global__ void __launch_bounds__(kCellThreads, 2) k_cells(Batch* __restrict__ bt) {
    grid_dependency_begin();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CellSmem& sm = *reinterpret_cast<CellSmem*>(smem_raw);
    const int total = batch_total(bt, kStCell);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    {
        // the next frame's bucket totals start at zero: predict adds them; their readers (the
        // bucket scan) finished before this kernel
        const int stride = gridDim.x * blockDim.x;
        const int tid = blockIdx.x * blockDim.x + threadIdx.x;
        for (int gi = 0; gi < bt->n_grids; ++gi) {
            const GridDesc& g = bt->g[gi];
            for (int i = tid; i < g.ctiles; i += stride) g.ctile_cnt[i] = 0u;
        }
    }
    // jobs are claimed one ahead: thread 0 takes the next work index at the start of a job
    // and, once the in-bucket sort is done, copies its ctile_job entry to shared memory
    // (cp.async); the body's barriers publish both, so a job starts without a load chain.  A job
    // is a cell tile, or for a finely sorted grid a run of its buckets: cells [c_lo, c_hi) of the
    // tile and the sorted positions [p0, p1) of their particles.
    if (threadIdx.x == 0) {
        const int t0 = (int)atomicAdd(&bt->counters[kStCell], 1u);
        sm.jt[0] = t0;
        if (t0 < total) {
            const int gi = grid_of_tile(bt, kStCell, t0);
            sm.jgrid[0] = gi;
            sm.job[0] = bt->g[gi].ctile_job[t0 - bt->prefix[gi][kStCell]];
        }
    }
    __syncthreads();
    for (int it = 0;; it ^= 1) {
        if (sm.jt[it] >= total) break;
        int next = 0;
        if (threadIdx.x == 0) next = (int)atomicAdd(&bt->counters[kStCell], 1u);
        const GridDesc& g = bt->g[sm.jgrid[it]];
        const uint4 job = sm.job[it];
        if (FINE && job.x == 0xffffffffu) {  // an unused slot after a grid's last job (block-uniform)
            if (threadIdx.x == 0) {
                sm.jt[it ^ 1] = next;
                if (next < total) {
                    const int gn = grid_of_tile(bt, kStCell, next);
                    sm.jgrid[it ^ 1] = gn;
                    sm.job[it ^ 1] = bt->g[gn].ctile_job[next - bt->prefix[gn][kStCell]];
                }
            }
            __syncthreads();
            continue;
        }
        const int lt = (int)job.x;  // full jobs first
        const int base = lt * kCellTile;
        const int p0 = (int)job.y, p1 = (int)job.z;
        // prefetch the measurement and the (shifted) previous free mass of this thread's cells
        const bool meas16 = (reinterpret_cast<uintptr_t>(g.meas_src) & 15u) == 0u;
        for (int r = 0; r < kCellTile / kCellThreads; ++r) {
            const int cl = r * kCellThreads + threadIdx.x;
            const int k = base + cl;
            if (k >= g.C) break;
            if (FINE && (cl < (int)(job.w & 0xffffu) || cl >= (int)(job.w >> 16))) continue;  // another job's cell
            if (meas16) {
                cp_async16(&sm.meas[cl], g.meas_src + k);
            } else {
                for (int w = 0; w < 4; ++w)
                    cp_async4(reinterpret_cast<float*>(&sm.meas[cl]) + w, reinterpret_cast<const float*>(g.meas_src + k) + w);
            }
            int src = k;
            if (g.shifted) {
                const int row = cell_row(g, k);
                const int sx = k - row * g.gs + g.shift_x, sy = row + g.shift_y;
                const bool ok = sx > 0 && sx < g.gs && sy > 0 && sy < g.gs;  // strict, as the reference
                src = ok ? sx + g.gs * sy : -1;
            }
            if (src >= 0) cp_async4(&sm.free_prev[cl], g.free_old + src);
            else sm.free_prev[cl] = 0.0f;
        }

        // ---- S: stable counting sort of the job's particles into S -----------------------
        const int np = p1 - p0;
        if (np > 0) sort_bucket(sm, g, base, p0, p1);  // block-uniform; ends with a barrier
        else __syncthreads();
        // which of this thread's B cells hold particles (the counts are overwritten in B; A's
        // barriers order these reads before any staging)
        for (int r = 0; r < kCellTile / kCellThreads; ++r) {
            const int cl = r * kCellThreads + threadIdx.x;
            sm.occ[cl] = (np > 0 && sm.u2.srt.cnt[cl] != 0u) ? 1 : 0;
        }
        if (threadIdx.x == 0) {  // the next tile's job (slot it ^ 1 was last read before the barrier)
            sm.jt[it ^ 1] = next;
            if (next < total) {
                const int gn = grid_of_tile(bt, kStCell, next);
                sm.jgrid[it ^ 1] = gn;
                cp_async16(&sm.job[it ^ 1], bt->g[gn].ctile_job + (next - bt->prefix[gn][kStCell]));
            }
        }

        // ---- A: segmented reduction of the tile's particles ------------------------------
        // thread t walks its own consecutive share [i_beg, i_end) of the tile's particles, so
        // a full tile costs one block scan however many particles it holds
        if (np > 0) {  // block-uniform
            const int per = (np + kCellThreads - 1) / kCellThreads;
            const int i_beg = min(p1, p0 + (int)threadIdx.x * per), i_end = min(p1, i_beg + per);
            const uint32_t kSent = 0xffffffffu;  // cell "outside the tile"
            uint32_t prev = (i_beg > p0 && i_beg < p1) ? (g.S_key[i_beg - 1] & kCellMask) : kSent;
            Run cur = run_empty(0u);    // run open at the current particle
            Run first = run_empty(0u);  // the thread's first run, when it continues an earlier one
            uint32_t first_cell = kSent;
            int first_last = -1;
            bool last_tail = false;
            for (int ib = i_beg; ib < i_end; ib += kSegIpt) {
                uint32_t kw[kSegIpt];
                float2 v[kSegIpt];
#pragma unroll
                for (int r = 0; r < kSegIpt; ++r) {
                    const int i = ib + r;
                    kw[r] = kSent;
                    v[r] = make_float2(0.0f, 0.0f);
                    if (i < p1) kw[r] = g.S_key[i];
                    if (i < i_end) {
                        const float4 st = g.S_state[i];
                        v[r] = make_float2(st.z, st.w);
                    }
                }
                const uint32_t after = (ib + kSegIpt < p1) ? (g.S_key[ib + kSegIpt] & kCellMask) : kSent;
#pragma unroll
                for (int r = 0; r < kSegIpt; ++r) {
                    const int i = ib + r;
                    if (i < i_end) {
                        const uint32_t c = kw[r] & kCellMask;
                        const uint32_t next = (r + 1 < kSegIpt) ? (kw[r + 1] == kSent ? kSent : (kw[r + 1] & kCellMask))
                                                                : after;
                        if (c != prev) {  // segment head
                            cur = run_empty(kRunHead);
                            const uint32_t cl = c - (uint32_t)base;
                            if (cl < (uint32_t)kCellTile) sm.u1.cell.start[cl] = i;
                        }
                        run_add(cur, kw[r], v[r]);
                        last_tail = c != next;
                        if (last_tail) {  // segment tail
                            if (cur.fn & kRunHead) {
                                put_cell(sm, g, c - (uint32_t)base, i, cur);
                            } else {
                                first = cur;
                                first_cell = c;
                                first_last = i;
                            }
                            cur = run_empty(kRunHead);
                        }
                        prev = c;
                    }
                }
            }
            // the run this thread passes on: empty after a tail, else the open run
            const Run out = last_tail ? run_empty(kRunHead) : cur;
            Run inc = out;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const Run other = run_shfl_up(inc, o);
                if (lane >= o) inc = run_combine(other, inc);
            }
            if (lane == 31) sm.wagg[warp] = inc;
            Run excl = run_shfl_up(inc, 1);
            __syncthreads();
            if (warp == 0) {  // exclusive scan of the warps' runs by one warp
                constexpr int kWarps = kCellThreads / 32;
                Run a = lane < kWarps ? sm.wagg[lane] : run_empty(0u);
#pragma unroll
                for (int o = 1; o < kWarps; o <<= 1) {
                    const Run other = run_shfl_up(a, o);
                    if (lane >= o) a = run_combine(other, a);
                }
                Run ex = run_shfl_up(a, 1);
                if (lane == 0) ex = run_empty(0u);
                if (lane < kWarps) sm.wpre[lane] = ex;
            }
            __syncthreads();
            Run pre = sm.wpre[warp];
            if (lane > 0) pre = run_combine(pre, excl);
            if (first_last >= 0) put_cell(sm, g, first_cell - (uint32_t)base, first_last, run_combine(pre, first));
            __syncthreads();
        }

        // ---- B: per-cell update ----------------------------------------------------------
        // (a stage call runs one part of the pass: it starts from the records as they are and
        // replaces only its own fields)
        const uint32_t mask = STAGED ? g.stage_mask : kPartAll;
        const bool all = !STAGED;
        const float c_pred = g.weights_predicted ? g.fs->w_res                    // predicted weight of
                                                 : __fmul_rn(g.p_S, g.fs->w_res);  // an in-grid particle
        unsigned long long qb = 0ull, jq = 0ull;
        // the job's cells (read again here, not held through S and A): whole warps of B
        const int c_lo = FINE ? (int)(sm.job[it].w & 0xffffu) : 0, c_hi = FINE ? (int)(sm.job[it].w >> 16) : kCellTile;
        cp_async_wait_all();  // this thread's own prefetches (B reads only its own cells' slots)
        for (int r = 0; r < kCellTile / kCellThreads; ++r) {
            const int cl = r * kCellThreads + threadIdx.x;
            const int k = base + cl;
            const int warp_first = base + r * kCellThreads + warp * 32;  // the warp's 32 cells
            if (warp_first >= g.C) break;                                // warp-uniform
            if (FINE && (warp_first - base < c_lo || warp_first - base >= c_hi)) continue;  // another job's
            float4* stage = sm.u2.stage[warp];
            const int n_rec = min(32, g.C - warp_first);
            float4* dst = reinterpret_cast<float4*>(g.cells + warp_first);
            // the lane's new record, every field (a stage call keeps only its parts' fields)
            float4 n0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), n1 = n0, n2 = n0, n3 = n0;
            if (k < g.C) {
                const bool occupied = sm.occ[cl] != 0;  // range, count and sums are set only then
                const int start = occupied ? sm.u1.cell.start[cl] : -1, end = occupied ? sm.u1.cell.end[cl] : -1;
                const int n_in = occupied ? sm.u1.cell.n_in[cl] : 0;
                const float free_prev = sm.free_prev[cl];
                const dogm_measurement_cell m = sm.meas[cl];
                const CellOut o = cell_masses(n_in, c_pred, free_prev, g.alpha, g.p_B, m.free_mass, m.occ_mass);
                float muA = 0.0f, muUA = 0.0f, wp = 0.0f;
                float mx = 0.0f, my = 0.0f, vx = 0.0f, vy = 0.0f, cxy = 0.0f;
                if (occupied) {
                    const float wu = __fmul_rn(m.likelihood, o.w_norm);
                    const float swu = __fmul_rn((float)n_in, wu);
                    muA = swu > 0.0f ? __fdiv_rn(o.rho_p, swu) : 0.0f;
                    muUA = o.m_occ_pred > 0.0f ? __fdiv_rn(o.rho_p, o.m_occ_pred) : 0.0f;
                    wp = __fadd_rn(__fmul_rn(__fmul_rn(m.p_A, muA), wu),
                                   __fmul_rn(__fmul_rn(__fsub_rn(1.0f, m.p_A), muUA), o.w_norm));
                    if (o.rho_p > 0.0f && (mask & kPartMoments)) {
                        const float inv = __fdiv_rn(1.0f, o.rho_p);
                        mx = __fmul_rn(inv, __fmul_rn(wp, sm.u1.cell.vx[cl]));
                        my = __fmul_rn(inv, __fmul_rn(wp, sm.u1.cell.vy[cl]));
                        vx = __fsub_rn(__fmul_rn(inv, __fmul_rn(wp, sm.u1.cell.vxx[cl])), __fmul_rn(mx, mx));
                        vy = __fsub_rn(__fmul_rn(inv, __fmul_rn(wp, sm.u1.cell.vyy[cl])), __fmul_rn(my, my));
                        cxy = __fsub_rn(__fmul_rn(inv, __fmul_rn(wp, sm.u1.cell.vxy[cl])), __fmul_rn(mx, my));
                    }
                }
                n0 = make_float4(__int_as_float(start), __int_as_float(end), o.rho_b, o.rho_p);
                n1 = make_float4(o.free_up, o.occ_up, o.m_occ_pred, muA);
                n2 = make_float4(muUA, 0.0f, 0.0f, mx);  // w_A / w_UA: the newborn pass sets them
                n3 = make_float4(my, vx, vy, cxy);
                if (mask & kPartMasses) {
                    // read by nothing later in the frame: stored with the evict-first hint, so they
                    // do not push the sorted particles and cell weights (read by resampling) out of L2
                    if (g.copy_meas)
                        __stcs(reinterpret_cast<float4*>(g.meas_own + k), make_float4(m.free_mass, m.occ_mass, m.likelihood, m.p_A));
                    __stcs(g.free_new + k, o.free_up);
                    g.rho_b[k] = make_float2(o.rho_b, m.p_A);
                    qb += quantize(o.rho_b, g.q_shift);
                }
                if (mask & kPartReweight) {
                    if (n_in > 0) g.w_cell[k] = wp;  // read only through the keys of in-grid particles
                    const unsigned long long qw = n_in > 0 ? quantize(wp, g.q_shift) : 0ull;
                    if (qw) {
                        jq += (unsigned long long)n_in * qw;
                        add_persistent(g, start, end, n_in, qw);
                    }
                }
            }
            // the warp's records, kStageRecs at a time: 512 contiguous bytes per store instruction
            // (evict-first: only the newborn pass and the readback touch them again)
#pragma unroll
            for (int h = 0; h < 32 / kStageRecs; ++h) {
                const int rec0 = h * kStageRecs;
                if (rec0 >= n_rec) break;  // warp-uniform
                const int nr = min(kStageRecs, n_rec - rec0);
                if (!all) {  // block-uniform: the records as they are
#pragma unroll
                    for (int q = 0; q < kStageRecs / 8; ++q) {
                        const int rec = q * 8 + (lane >> 2), chunk = lane & 3;
                        if (rec < nr) stage[stage_slot(rec, chunk)] = dst[(rec0 + rec) * 4 + chunk];
                    }
                    __syncwarp();
                }
                const int rl = lane - rec0;  // this lane's record in the half
                if (rl >= 0 && rl < nr) {
                    if (all) {
                        stage[stage_slot(rl, 0)] = n0;
                        stage[stage_slot(rl, 1)] = n1;
                        stage[stage_slot(rl, 2)] = n2;
                        stage[stage_slot(rl, 3)] = n3;
                    } else {
                        float4 s0 = stage[stage_slot(rl, 0)], s1 = stage[stage_slot(rl, 1)];
                        float4 s2 = stage[stage_slot(rl, 2)], s3 = stage[stage_slot(rl, 3)];
                        if (mask & kPartRanges) {
                            s0.x = n0.x;
                            s0.y = n0.y;
                        }
                        if (mask & kPartMasses) {
                            s0.z = n0.z; s0.w = n0.w;
                            s1.x = n1.x; s1.y = n1.y; s1.z = n1.z;
                            s2.y = n2.y; s2.z = n2.z;
                        }
                        if (mask & kPartReweight) {
                            s1.w = n1.w;
                            s2.x = n2.x;
                        }
                        if (mask & kPartMoments) {
                            s2.w = n2.w;
                            s3 = n3;
                        }
                        stage[stage_slot(rl, 0)] = s0;
                        stage[stage_slot(rl, 1)] = s1;
                        stage[stage_slot(rl, 2)] = s2;
                        stage[stage_slot(rl, 3)] = s3;
                    }
                }
                __syncwarp();
#pragma unroll
                for (int q = 0; q < kStageRecs / 8; ++q) {
                    const int rec = q * 8 + (lane >> 2), chunk = lane & 3;
                    if (rec < nr) __stcs(dst + (rec0 + rec) * 4 + chunk, stage[stage_slot(rec, chunk)]);
                }
                __syncwarp();  // the stage is refilled by the next half
            }
        }
        // the tile's exact sums: warp sums, then thread 0 adds the warps' (sm.red is next
        // written at the end of the next tile, after that tile's barriers)
        qb = warp_sum_u64(qb);
        jq = warp_sum_u64(jq);
        if (lane == 0) {
            sm.red[warp] = qb;
            sm.red2[warp] = jq;
        }
        if (threadIdx.x == 0) cp_async_wait_all();  // the next tile's job has landed
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long tile_qb = 0ull, tile_jq = 0ull;
            for (int w = 0; w < kCellWarps; ++w) {
                tile_qb += sm.red[w];
                tile_jq += sm.red2[w];
            }
            if (mask & kPartMasses) {
                // the job's sum at its first bucket, zeros at its others (the newborn pass sums
                // the buckets before a tile)
                if (FINE) {
                    const int b0 = (lt << (kCellTileBits - g.bucket_bits)) + (c_lo >> g.bucket_bits);
                    const int b1 = min(g.ctiles, (lt << (kCellTileBits - g.bucket_bits)) + (c_hi >> g.bucket_bits));
                    g.cell_sum[b0] = tile_qb;
                    for (int b = b0 + 1; b < b1; ++b) g.cell_sum[b] = 0ull;
                } else {
                    g.cell_sum[lt] = tile_qb;
                }
                atomicAdd(&g.fs->qb_total, tile_qb);
            }
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
constexpr int kRunTiles = 4;  // resample tiles a thread accumulates in registers

// q per slot over joint positions [a, b), added per resample tile: the first kRunTiles tiles
// from rt0 in registers, any further ones straight to the global sums.
__device__ __forceinline__ void add_joint_range(unsigned long long (&racc)[kRunTiles], long long rt0,
                                                const GridDesc& g, long long a, long long b,
                                                unsigned long long q) {
    if (q == 0ull) return;
    const int rb = g.res_bits;
    for (long long rt = a >> rb; (rt << rb) < b; ++rt) {
        const long long lo = max(a, rt << rb);
        const long long hi = min(b, (rt + 1) << rb);
        if (hi <= lo) continue;
        const unsigned long long v = (unsigned long long)(hi - lo) * q;
        const long long o = rt - rt0;
        if (o >= 0 && o < kRunTiles) {
#pragma unroll
            for (int i = 0; i < kRunTiles; ++i) racc[i] += (o == i) ? v : 0ull;
        } else {
            add_res_sum(g, rt, v);
        }
    }
}

// FINE: some grid of the launch sorts by buckets finer than a cell tile (its tile sums are per
// bucket); without it they are per tile.
template <bool FINE>
__global__ void __launch_bounds__(kThreads, 6) k_newborn(Batch* __restrict__ bt) {
    grid_dependency_begin();
    __shared__ unsigned long long red[2 * (kThreads / 32)];
    __shared__ int s_bnd[kCellTile + 1];  // s_bnd[c]: first slot of cell c of the tile; [kCellTile]: end
    __shared__ int s_nuA[kCellTile];
    // the tile's cells that receive newborns, compacted so that all threads share their work
    __shared__ uint16_t s_list[kCellTile];
    __shared__ float2 s_bp[kCellTile];
    __shared__ int s_wcnt[kThreads / 32];
    const int total = batch_total(bt, kStBirth);
    const int lane = threadIdx.x & 31;
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int gi = grid_of_tile(bt, kStBirth, t);
        const GridDesc& g = bt->g[gi];
        const int lt = t - bt->prefix[gi][kStBirth];
        const int base = lt * kCellTile;
        const unsigned long long T = g.fs->qb_total;
        unsigned long long q[kCellIpt];
        float rb[kCellIpt];
        float2 bp[kCellIpt];
#pragma unroll
        for (int j = 0; j < kCellIpt; ++j) {
            const int k = base + threadIdx.x * kCellIpt + j;
            bp[j] = (k < g.C) ? __ldcs(g.rho_b + k) : make_float2(0.0f, 0.0f);  // {rho_b, p_A}
        }
        // the earlier tiles' sums load while the cells' values are in flight
        const unsigned long long part =
            block_prefix_part(g.cell_sum, FINE ? lt << (kCellTileBits - g.bucket_bits) : lt);
        unsigned long long v = 0ull;
#pragma unroll
        for (int j = 0; j < kCellIpt; ++j) {
            rb[j] = bp[j].x;
            q[j] = quantize(rb[j], g.q_shift);
            v += q[j];
        }
        unsigned long long tile_sum;
        unsigned long long acc = block_scan_with_part(v, part, red, &tile_sum);
        const float sc = T ? __fdiv_rn((float)g.B, __ull2float_rn(T)) : 0.0f;
        int bnd[kCellIpt + 1];
        bnd[0] = alloc_boundary_fast(acc, T, g.B, sc);
        // boundaries are monotone in the prefix: when the thread's first and last agree, so do
        // the ones between (most threads' cells get no newborn at all)
        const int b_last = alloc_boundary_fast(acc + v, T, g.B, sc);  // v: the thread's q sum
#pragma unroll
        for (int j = 0; j < kCellIpt; ++j) {
            acc += q[j];
            if (j + 1 == kCellIpt) bnd[j + 1] = b_last;
            else bnd[j + 1] = (b_last == bnd[0] || !q[j]) ? bnd[j] : alloc_boundary_fast(acc, T, g.B, sc);
            s_bnd[threadIdx.x * kCellIpt + j] = bnd[j];
        }
        if (threadIdx.x == kThreads - 1) s_bnd[kCellTile] = bnd[kCellIpt];
        // cells with newborns: count per thread, exclusive scan over the block
        uint32_t mask = 0u;
#pragma unroll
        for (int j = 0; j < kCellIpt; ++j)
            if (bnd[j + 1] > bnd[j] && base + (int)threadIdx.x * kCellIpt + j < g.C) mask |= 1u << j;
        const int cnt = __popc(mask);
        int wpos = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, wpos, o);
            if (lane >= o) wpos += y;
        }
        if (lane == 31) s_wcnt[threadIdx.x >> 5] = wpos;
        __syncthreads();
        int pos = wpos - cnt, n_list = 0;
#pragma unroll
        for (int w = 0; w < kThreads / 32; ++w) {
            const int c = s_wcnt[w];
            if (w < (int)(threadIdx.x >> 5)) pos += c;
            n_list += c;
        }
#pragma unroll
        for (int j = 0; j < kCellIpt; ++j)
            if (mask & (1u << j)) {
                s_list[pos] = (uint16_t)(threadIdx.x * kCellIpt + j);
                s_bp[pos] = bp[j];
                ++pos;
            }
        __syncthreads();
        const int lo_tile = s_bnd[0], hi_tile = s_bnd[kCellTile];
        const long long N = g.N;
        const long long rt0 = (N + lo_tile) >> g.res_bits;
        unsigned long long racc[kRunTiles] = {0ull, 0ull, 0ull, 0ull};
        unsigned long long jq = 0ull;
        // w_A / w_UA of each listed cell (init_new_particles.cu:145-153) and its joint weights
        for (int i = threadIdx.x; i < n_list; i += kThreads) {
            const int lc = s_list[i];
            const int k = base + lc;
            const int b0 = s_bnd[lc], b1 = s_bnd[lc + 1];
            const int nnew = b1 - b0;
            const float rbj = s_bp[i].x, pAj = s_bp[i].y;
            const int nuA = (int)roundf(__fmul_rn((float)nnew, pAj));
            const int nuUA = nnew - nuA;
            const float wA = nuA > 0 ? __fdiv_rn(__fmul_rn(pAj, rbj), (float)nuA) : 0.0f;
            const float wUA = nuUA > 0 ? __fdiv_rn(__fmul_rn(__fsub_rn(1.0f, pAj), rbj), (float)nuUA) : 0.0f;
            g.cells[k].w_A = wA;
            g.cells[k].w_UA = wUA;
            s_nuA[lc] = nuA;
            const int nA = min(max(nuA, 0), nnew);
            const unsigned long long qA = quantize(wA, g.q_shift), qU = quantize(wUA, g.q_shift);
            jq += (unsigned long long)nA * qA + (unsigned long long)(nnew - nA) * qU;
            add_joint_range(racc, rt0, g, N + b0, N + b0 + nA, qA);
            add_joint_range(racc, rt0, g, N + b0 + nA, N + b1, qU);
        }
#pragma unroll
        for (int i = 0; i < kRunTiles; ++i) {
            if (!__any_sync(0xffffffffu, racc[i] != 0ull)) continue;  // warp-uniform
            const unsigned long long s = warp_sum_u64(racc[i]);
            if (lane == 0 && s) add_res_sum(g, rt0 + i, s);
        }
        if (__any_sync(0xffffffffu, jq != 0ull)) {
            jq = warp_sum_u64(jq);
            if (lane == 0 && jq) atomicAdd(&g.fs->joint_total, jq);
        }
        __syncthreads();  // every s_nuA entry is written
        // key word of every newborn slot of the tile (cell | associated bit), slot by slot on
        // consecutive threads; the owner cell is the last c with s_bnd[c] <= slot
        for (int sl = lo_tile + threadIdx.x; sl < hi_tile; sl += kThreads) {
            int lo = 0, hi = kCellTile - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_bnd[mid] <= sl) lo = mid; else hi = mid - 1;
            }
            g.B_key[sl] = (uint32_t)(base + lo) | ((sl - s_bnd[lo]) < s_nuA[lo] ? kAssocBit : 0u);
        }
        if (threadIdx.x == 0 && lt == 0) g.fs->n_birth = (T > 0ull) ? g.B : 0;
        __syncthreads();
    }
}

cudaError_t prepare_cells() {
    cudaError_t e = cudaFuncSetAttribute(k_cells<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(CellSmem));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_cells<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(CellSmem));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_cells<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(CellSmem));
}

cudaError_t launch_cells(const Batch* d_batch, const LaunchCfg& cfg, bool staged, bool fine) {
    Batch* b = const_cast<Batch*>(d_batch);
    // (a stage call takes the instantiation that handles every job form)
    if (staged) return launch_kernel(cfg, k_cells<true, true>, launch_blocks(cfg, 2), kCellThreads, sizeof(CellSmem), b);
    if (fine) return launch_kernel(cfg, k_cells<false, true>, launch_blocks(cfg, 2), kCellThreads, sizeof(CellSmem), b);
    return launch_kernel(cfg, k_cells<false, false>, launch_blocks(cfg, 2), kCellThreads, sizeof(CellSmem), b);
}

cudaError_t launch_newborn(const Batch* d_batch, const LaunchCfg& cfg, bool fine) {
    Batch* b = const_cast<Batch*>(d_batch);
    if (fine) return launch_kernel(cfg, k_newborn<true>, launch_blocks(cfg, 6), kThreads, 0, b);
    return launch_kernel(cfg, k_newborn<false>, launch_blocks(cfg, 6), kThreads, 0, b);
}

}  // namespace dogm_gb300
