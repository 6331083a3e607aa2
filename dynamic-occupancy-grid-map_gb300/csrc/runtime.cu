// Host runtime behind the C ABI (include/dogm_gb300.h): handle lifetime, pose bookkeeping,
// batch upload, the per-frame launch sequence and its CUDA graph, readback and test hooks.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <unistd.h>

#include "dogm_internal.h"

using namespace dogm_gb300;

namespace {

thread_local std::string g_last_error;

dogm_status fail(dogm_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

#define DOGM_CUDA(call)                                                                               \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return fail(e_ == cudaErrorMemoryAllocation ? DOGM_ERR_OUT_OF_MEMORY : DOGM_ERR_CUDA,     \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                          \
    } while (0)

int bitlen(unsigned long long v) {
    int b = 0;
    while (v) { ++b; v >>= 1; }
    return b;
}

int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }

constexpr int kStages = 6;
const char* const kStageNames[kStages] = {"predict", "sort_scan", "sort_scatter", "cells", "newborn", "resample"};

// One launch context: a device copy of a Batch, two pinned host mirrors (the host fills one
// while the device may still read the other, so frame k+1 is queued while frame k runs) and
// the CUDA graphs of the steady-state frame, keyed by (batch size, mirror).
struct Ctx {
    int device = -1;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    Batch* d_batch = nullptr;                    // the device batch of mirror `cur`
    Batch* d_batch_m[2] = {nullptr, nullptr};    // one device batch per mirror
    // graph frames upload their descriptors on this stream, ahead of the frame before them
    cudaStream_t up_stream = nullptr;
    cudaEvent_t up_done[2] = {nullptr, nullptr};
    Batch* h_batch[2] = {nullptr, nullptr};      // pinned
    unsigned int* h_status = nullptr;            // pinned and mapped: one word per mirror, one for copies
    unsigned int* d_h_status = nullptr;          // its device address
    cudaEvent_t done[2] = {nullptr, nullptr};    // the frame that read mirror i has finished
    bool pending[2] = {false, false};
    int cur = 0;                                 // mirror of the frame being built
    std::map<int, cudaGraphExec_t> graphs;
    bool profile = false;
    cudaEvent_t ev[kStages + 1] = {};
    int mult[kStages] = {};  // tuned blocks per SM per stage (0: the kernel's default)
    // programmatic dependent launch between the frame's kernels (environment DOGM_PDL=0 turns
    // it off, for comparison)
    bool pdl = true;
    // how steady-state frames are launched (dogm_set_launch_mode): chained (one grid of a
    // handle's own context; otherwise a graph), a CUDA graph, or plain launches
    int launch_mode = DOGM_LAUNCH_CHAINED;
    // bucket-count class of the batch being built: the bucket scatter's shared memory is sized
    // for 2048 buckets, or 4096 when a grid of the batch has more than 2048 cell tiles
    int scatter_ctiles = 2048;
    // resampling tile of this context's launches: 2^res_bits joint particles
    int res_bits = kResBitsDefault;
    // a handle's own context: a steady-state frame of its one grid runs chained (no graph, no
    // upload, no event between frames; predict takes the descriptor as a parameter and follows
    // the previous frame's resampling programmatically).  Launch slots and the batch context
    // keep graphs, since their callers wait on the frames' events.
    bool chain = false;
    // some grid of the current batch sorts by buckets finer than a cell tile (the cell pass then
    // takes jobs of bucket runs)
    bool fine = false;
    bool last_chained = false;  // the last frame queued ran chained

    // Captured graphs hold the launch widths: drop them when the widths change.
    void drop_graphs() {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
    }

    ~Ctx() {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        for (int i = 0; i < 2; ++i) {
            if (d_batch_m[i]) cudaFree(d_batch_m[i]);
            if (h_batch[i]) cudaFreeHost(h_batch[i]);
            if (done[i]) cudaEventDestroy(done[i]);
            if (up_done[i]) cudaEventDestroy(up_done[i]);
        }
        if (up_stream) cudaStreamDestroy(up_stream);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        if (h_status) cudaFreeHost(h_status);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};

dogm_status ctx_init(Ctx& c, int device) {
    c.device = device;
    if (const char* v = std::getenv("DOGM_PDL")) c.pdl = std::strcmp(v, "0") != 0;
    DOGM_CUDA(cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, device));
    DOGM_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    c.own_stream = true;
    DOGM_CUDA(cudaStreamCreateWithFlags(&c.up_stream, cudaStreamNonBlocking));
    for (int i = 0; i < 2; ++i) {
        DOGM_CUDA(cudaMalloc(&c.d_batch_m[i], sizeof(Batch)));
        DOGM_CUDA(cudaMemset(c.d_batch_m[i], 0, sizeof(Batch)));
        DOGM_CUDA(cudaMallocHost(&c.h_batch[i], sizeof(Batch)));
        std::memset(c.h_batch[i], 0, sizeof(Batch));
        DOGM_CUDA(cudaEventCreateWithFlags(&c.done[i], cudaEventDisableTiming));
        DOGM_CUDA(cudaEventCreateWithFlags(&c.up_done[i], cudaEventDisableTiming));
    }
    c.d_batch = c.d_batch_m[0];
    DOGM_CUDA(cudaHostAlloc((void**)&c.h_status, 3 * sizeof(unsigned int), cudaHostAllocMapped | cudaHostAllocPortable));
    c.h_status[0] = c.h_status[1] = c.h_status[2] = 0;
    DOGM_CUDA(cudaHostGetDevicePointer((void**)&c.d_h_status, c.h_status, 0));
    for (auto& e : c.ev) DOGM_CUDA(cudaEventCreate(&e));
    return DOGM_OK;
}

// Makes mirror m the current one (its pinned host batch and its device batch).
void set_mirror(Ctx& c, int m) {
    c.cur = m;
    c.d_batch = c.d_batch_m[m];
}

// The mirror for the next frame: waits until the frame that last read it has finished.
dogm_status acquire_mirror(Ctx& c) {
    const int i = c.cur;
    if (c.pending[i]) {
        DOGM_CUDA(cudaEventSynchronize(c.done[i]));
        c.pending[i] = false;
    }
    return DOGM_OK;
}

}  // namespace

struct dogm_handle {
    int device = 0;
    dogm_params params{};
    dogm_options opt{};
    int gs = 0, N = 0, B = 0, C = 0;
    bool first_pose_received = false, first_measurement_received = false;
    float position_x = 0.f, position_y = 0.f, yaw = 0.f;
    int iteration = 0;
    bool need_clear = true;
    int last_launches = 0;
    GridDesc desc{};                     // persistent pointers + sizes; per-frame fields set per call
    std::vector<void*> allocations;
    Ctx ctx;
    // replay and debug buffers
    float2* rp_init = nullptr;
    float4* rp_predict = nullptr;
    float2* rp_birth = nullptr;
    unsigned long long* rp_resample = nullptr;
    bool debug = false;
    // dynamic-cell extraction staging (allocated on first use)
    dogm_dynamic_cell* dyn_out = nullptr;
    int dyn_cap = 0;
    unsigned int* dyn_scratch = nullptr;
    // asynchronous grid readback (dogm_get_grid_cells_async), created on first use: a second
    // cell-record buffer that the updates alternate with, a copy stream, and per buffer the
    // event after its last queued copy (0: the primary buffer, 1: cells_alt)
    dogm_grid_cell* cells_primary = nullptr;
    dogm_grid_cell* cells_alt = nullptr;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t frame_ready = nullptr;
    cudaEvent_t copy_done[2] = {nullptr, nullptr};
    float stage_dt = 0.1f;  // dt of the last gridCellOccupancyUpdate stage call
};

namespace {

template <class T>
dogm_status dalloc(dogm_handle* h, T** p, size_t count) {
    void* q = nullptr;
    const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) return fail(DOGM_ERR_OUT_OF_MEMORY, "cudaMalloc of " + std::to_string(bytes) + " B failed");
    e = cudaMemset(q, 0, bytes);
    if (e != cudaSuccess) return fail(DOGM_ERR_CUDA, cudaGetErrorString(e));
    h->allocations.push_back(q);
    *p = static_cast<T*>(q);
    return DOGM_OK;
}

// A handle's frame buffers are carved from one allocation: a first pass over the buffer list
// sums their sizes, a second assigns the pointers.  One mapping per grid keeps its buffers
// together whatever earlier handles of the process allocated and freed.
constexpr size_t kCarveAlign = 256;
struct Carver {
    unsigned char* base = nullptr;  // null: sizing pass
    size_t off = 0;
    template <class T>
    void take(T** p, size_t count) {
        off = (off + kCarveAlign - 1) & ~(kCarveAlign - 1);
        if (base) *p = reinterpret_cast<T*>(base + off);
        off += std::max<size_t>(count, 1) * sizeof(T);
    }
};

struct Sizes {
    int gs, N, B, C, key_bits, sort_tiles, cell_tiles, res_tiles, pred_tiles, scan;
    int bucket_bits, buckets;  // buckets of the particle sort (= cell tiles unless the grid is small)
};

dogm_status derive_sizes(const dogm_params& p, Sizes& s) {
    if (!(p.size > 0.f) || !(p.resolution > 0.f)) return fail(DOGM_ERR_INVALID_ARGUMENT, "size/resolution must be > 0");
    s.gs = static_cast<int>(p.size / p.resolution);  // dogm.cu:34
    if (s.gs < 1) return fail(DOGM_ERR_INVALID_ARGUMENT, "grid_size < 1");
    s.C = s.gs * s.gs;
    s.key_bits = std::max(1, bitlen((unsigned long long)(s.C - 1)));
    if (s.key_bits > kMaxKeyBits)
        return fail(DOGM_ERR_UNSUPPORTED, "grid_size " + std::to_string(s.gs) + " > 2048 is not supported");
    s.N = p.particle_count;
    s.B = p.new_born_particle_count;
    if (s.N < 1 || s.N > kMaxParticles) return fail(DOGM_ERR_UNSUPPORTED, "particle_count must be in [1, 2^24)");
    if (s.B < 0 || s.B > kMaxParticles) return fail(DOGM_ERR_UNSUPPORTED, "new_born_particle_count must be in [0, 2^24)");
    s.pred_tiles = div_up(s.N, kPredictTile);
    s.sort_tiles = div_up(s.N, kSortTile);
    s.cell_tiles = div_up(s.C, kCellTile);
    s.bucket_bits = kCellTileBits;
    if (s.cell_tiles <= kFineMaxTiles && (long long)s.N > (long long)kFineMinPerTile * s.cell_tiles)
        while (s.bucket_bits > kMinBucketBits && div_up(s.C, 1 << (s.bucket_bits - 1)) <= kFineMaxBuckets)
            --s.bucket_bits;
    s.buckets = div_up(s.C, 1 << s.bucket_bits);
    s.res_tiles = div_up((long long)s.N + s.B, 1 << kResBitsMin);  // the finest resampling tiling
    s.scan = div_up(s.buckets, 32) + 1;  // bucket groups of the column scan + the job list
    return DOGM_OK;
}

void set_tiles(GridDesc& g, const Sizes& s) {
    for (int i = 0; i < kNumStages; ++i) g.tiles[i] = 0;
    g.tiles[kStPredict] = s.pred_tiles;
    g.tiles[kStScan] = s.scan;
    g.tiles[kStSort] = s.sort_tiles;
    g.tiles[kStCell] = s.buckets;  // job slots of the cell pass (at most one job per bucket)
    g.tiles[kStBirth] = s.cell_tiles;
    g.tiles[kStResample] = div_up((long long)s.N + s.B, 1 << kResBitsDefault);
    g.res_bits = kResBitsDefault;
    g.tiles[kStInitScan] = s.cell_tiles;
    g.tiles[kStInitExpand] = s.cell_tiles;
    g.sort_tiles = s.sort_tiles;
}

// Fills the per-frame fields of h->desc.  Pose bookkeeping follows DOGM::updatePose
// (dogm/src/dogm.cu:161-203): the first pose is stored; later poses shift the grid only
// when |dx| or |dy| exceeds one cell, by -int(d / resolution) cells, dropping the
// remainder and ignoring yaw.
void pose_update(dogm_handle* h, float new_x, float new_y, float new_yaw, int* shifted, int* xm, int* ym) {
    *shifted = 0;
    *xm = *ym = 0;
    if (!h->first_pose_received) {
        h->position_x = new_x;
        h->position_y = new_y;
        h->yaw = new_yaw;
        h->first_pose_received = true;
        return;
    }
    const float x_diff = new_x - h->position_x;
    const float y_diff = new_y - h->position_y;
    const float res = h->params.resolution;
    if (std::fabs(x_diff) > res || std::fabs(y_diff) > res) {
        *xm = -static_cast<int>(x_diff / res);
        *ym = -static_cast<int>(y_diff / res);
        *shifted = 1;
        h->position_x = new_x;
        h->position_y = new_y;
        h->yaw = new_yaw;
    }
}

void fill_frame(dogm_handle* h, float dt, int shifted, int xm, int ym, const dogm_measurement_cell* meas_src,
                int copy_meas) {
    GridDesc& g = h->desc;
    g.dt = dt;
    g.alpha = std::pow(h->params.freespace_discount, dt);  // float pow, as dogm.cu:291
    g.shifted = shifted;
    g.shift_x = xm;
    g.shift_y = ym;
    g.meas_src = meas_src;
    g.copy_meas = copy_meas;
    g.frame = (uint32_t)h->iteration;
    g.stage_mask = kPartAll;      // the update runs every part of the cell pass
    g.weights_predicted = 0;
    g.rp_init = h->rp_init;
    g.rp_predict = h->rp_predict;
    g.rp_birth = h->rp_birth;
    g.rp_resample = h->rp_resample;
}

// Writes n grid descriptors and the per-stage tile prefix into the current pinned mirror
// (call acquire_mirror first).  init_mask[i] != 0 schedules grid i's first-frame init.
void build_batch(Ctx& c, dogm_handle* const* hs, int n, const std::vector<int>& init_mask) {
    Batch& b = *c.h_batch[c.cur];
    b.n_grids = n;
    b.status = 0u;
    b.status_host = c.d_h_status + c.cur;
    c.scatter_ctiles = 2048;
    c.fine = false;
    for (int i = 0; i < n; ++i) {
        if (hs[i]->desc.ctiles > c.scatter_ctiles) c.scatter_ctiles = kMaxCellTiles;
        if (hs[i]->desc.bucket_bits < kCellTileBits) c.fine = true;
    }
    for (int s = 0; s < kNumStages; ++s) b.counters[s] = 0u;
    for (int s = 0; s < kNumStages; ++s) b.prefix[0][s] = 0;
    for (int i = 0; i < n; ++i) {
        b.g[i] = hs[i]->desc;
        b.g[i].status_out = &c.d_batch->status;
        // the context's resampling tile (the per-tile sums are scratch of one frame)
        b.g[i].res_bits = c.res_bits;
        b.g[i].tiles[kStResample] = div_up((long long)b.g[i].N + b.g[i].B, 1 << c.res_bits);
        for (int s = 0; s < kNumStages; ++s) {
            int tiles = b.g[i].tiles[s];
            if ((s == kStInitScan || s == kStInitExpand) && !init_mask[i]) tiles = 0;
            b.prefix[i + 1][s] = b.prefix[i][s] + tiles;
        }
    }
}

// The header (with the unused prefix rows past n, about 2 KB) and n descriptors in one copy:
// a second copy cost about 2 us of every graph-launched frame.
size_t batch_upload_bytes(int n) { return offsetof(Batch, g) + sizeof(GridDesc) * (size_t)n; }

cudaError_t upload_batch(Ctx& c, int n) {
    return cudaMemcpyAsync(c.d_batch, c.h_batch[c.cur], batch_upload_bytes(n), cudaMemcpyHostToDevice, c.stream);
}

// Status of a frame launched without a graph, copied into the third word (stage calls end with
// other kernels than the resampling, which ORs the bits into its mirror's word itself).
cudaError_t download_status(Ctx& c) {
    return cudaMemcpyAsync(c.h_status + 2, &c.d_batch->status, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                           c.stream);
}

// The steady-state frame: 6 kernels; with profiling, a CUDA event before each stage and at the
// end.
// fp: a chained frame's descriptor (predict then follows the previous frame's resampling
// programmatically too).
cudaError_t frame_kernels(Ctx& c, bool with_init, bool with_begin, const FrameParam* fp = nullptr) {
    LaunchCfg cfg{c.num_sms, c.stream};
    const bool prof = c.profile && !with_init;
    cudaError_t e;
#define STAGE(i, call)                                                              \
    do {                                                                            \
        if (prof && (e = cudaEventRecord(c.ev[i], c.stream)) != cudaSuccess) return e; \
        cfg.mult = c.mult[i];                                                       \
        cfg.pdl = c.pdl && !prof && (i > 0 || fp); /* else predict follows the upload */ \
        if ((e = (call)) != cudaSuccess) return e;                                  \
    } while (0)
    // the per-frame counters are reset by predict and the cell pass of the previous frame; a
    // full reset runs only on a grid's first frame or after a failed frame
    if ((with_begin || with_init) && (e = launch_frame_begin(c.d_batch, 0, cfg)) != cudaSuccess) return e;
    if (with_init && (e = launch_init_particles(c.d_batch, cfg)) != cudaSuccess) return e;
    STAGE(0, launch_predict(c.d_batch, 0, cfg, fp, c.fine));
    STAGE(1, launch_sort_scan(c.d_batch, cfg));
    STAGE(2, launch_sort_scatter(c.d_batch, c.scatter_ctiles, cfg, c.fine));
    STAGE(3, launch_cells(c.d_batch, cfg, false, c.fine));
    STAGE(4, launch_newborn(c.d_batch, cfg, c.fine));
    STAGE(5, launch_resample(c.d_batch, c.res_bits, cfg));
#undef STAGE
    if (prof && (e = cudaEventRecord(c.ev[kStages], c.stream)) != cudaSuccess) return e;
    return cudaSuccess;
}

// Steady-state graphs are keyed by a power-of-two bucket of the batch size: the kernels read
// only descriptors [0, n_grids), so a graph that uploads bucket(n) >= n descriptors serves
// every batch size in the bucket and a serving loop with changing batch sizes instantiates at
// most 9 graphs per mirror.
int graph_bucket(int n) {
    int b = 1;
    while (b < n) b <<= 1;
    return std::min(b, kMaxBatch);
}

// A graph is keyed by its batch-size bucket, mirror, bucket-scatter class, resampling tile and
// the cell pass's job form (whole tiles, or runs of finer buckets).
int graph_key(int nb, int mirror, int scatter_ctiles, int res_bits, bool fine) {
    return (res_bits << 21) + (scatter_ctiles > 2048 ? 1 << 20 : 0) + (fine ? 1 << 19 : 0) + nb * 2 + mirror;
}

// A device-to-host copy queued after a frame's kernels and before its completion event.
struct HostCopy {
    void* dst;
    const void* src;
    size_t bytes;
};

// Queues one frame from the current mirror and advances to the other mirror.
dogm_status run_frame(Ctx& c, int n, bool any_init, bool any_clear, int* launches,
                      const std::vector<HostCopy>* after = nullptr) {
    cudaError_t e;
    const bool plain = any_init || any_clear || c.profile || c.launch_mode == DOGM_LAUNCH_PLAIN;
    const bool chained = !plain && n == 1 && c.chain && c.pdl && c.launch_mode == DOGM_LAUNCH_CHAINED;
    if (!chained && c.last_chained) {
        // chained frames record no completion event: let them finish before a frame that
        // relies on the mirrors' events and uploads into the device batches
        DOGM_CUDA(cudaStreamSynchronize(c.stream));
        c.last_chained = false;
    }
    if (chained) {
        const Batch& hb = *c.h_batch[c.cur];
        FrameParam fp{};
        fp.g = hb.g[0];
        for (int s = 0; s < kNumStages; ++s) fp.tiles[s] = hb.prefix[1][s];
        fp.status_host = hb.status_host;
        fp.valid = 1;
        DOGM_CUDA(frame_kernels(c, false, false, &fp));
        *launches = kLaunchesPerFrame;
        c.last_chained = true;
    } else if (plain) {
        // first frame of some grid (init runs between begin and predict), a frame after a
        // failed one (full counter reset first) or per-stage timing
        DOGM_CUDA(upload_batch(c, n));
        DOGM_CUDA(frame_kernels(c, any_init, any_clear));
        DOGM_CUDA(download_status(c));
        *launches = kLaunchesPerFrame + (any_init || any_clear ? 1 : 0) + (any_init ? kLaunchesInit : 0);
    } else {
        const int nb = graph_bucket(n);
        // the descriptors go up on the upload stream into this mirror's device batch (the frame
        // that last read it has finished: acquire_mirror), so the copy runs while the frame
        // before this one is still on the device instead of between the two
        DOGM_CUDA(cudaMemcpyAsync(c.d_batch, c.h_batch[c.cur], batch_upload_bytes(nb), cudaMemcpyHostToDevice,
                                  c.up_stream));
        DOGM_CUDA(cudaEventRecord(c.up_done[c.cur], c.up_stream));
        DOGM_CUDA(cudaStreamWaitEvent(c.stream, c.up_done[c.cur], 0));
        const int key = graph_key(nb, c.cur, c.scatter_ctiles, c.res_bits, c.fine);
        auto it = c.graphs.find(key);
        if (it == c.graphs.end()) {
            cudaGraph_t graph;
            // the six kernels; the resampling kernel ORs the frame's status bits into mapped
            // host memory, so no copy follows them
            DOGM_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
            e = frame_kernels(c, false, false);
            cudaError_t e2 = cudaStreamEndCapture(c.stream, &graph);
            if (e != cudaSuccess) return fail(DOGM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
            if (e2 != cudaSuccess) return fail(DOGM_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e2));
            cudaGraphExec_t exec;
            e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess)
                return fail(DOGM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
            it = c.graphs.emplace(key, exec).first;
        }
        DOGM_CUDA(cudaGraphLaunch(it->second, c.stream));
        *launches = kLaunchesPerFrame;
    }
    if (after)
        for (const HostCopy& hc : *after)
            DOGM_CUDA(cudaMemcpyAsync(hc.dst, hc.src, hc.bytes, cudaMemcpyDeviceToHost, c.stream));
    if (!chained) {  // a chained frame's parameters were copied at launch: its mirror is free
        DOGM_CUDA(cudaEventRecord(c.done[c.cur], c.stream));
        c.pending[c.cur] = true;
    }
    set_mirror(c, c.cur ^ 1);
    return DOGM_OK;
}

// Waits for the context's stream and turns device status bits into a status code.
dogm_status finish_frame(Ctx& c, dogm_handle* const* hs, int n) {
    DOGM_CUDA(cudaStreamSynchronize(c.stream));
    c.pending[0] = c.pending[1] = false;
    // the resampling kernel ORs a frame's bits into its mirror's word, so the bits of every frame
    // since the last synchronisation are here, not only the last two frames'
    const unsigned int st = c.h_status[0] | c.h_status[1] | c.h_status[2];
    c.h_status[0] = c.h_status[1] = c.h_status[2] = 0;
    if (st & kStatusTimeout) {
        for (int i = 0; i < n; ++i) hs[i]->need_clear = true;
        return fail(DOGM_ERR_DEVICE_TIMEOUT, "a bounded device-side wait gave up");
    }
    if (st & kStatusBounds) {
        for (int i = 0; i < n; ++i) hs[i]->need_clear = true;
        return fail(DOGM_ERR_CUDA, "a device index check refused an out-of-range write (inconsistent histogram)");
    }
    return DOGM_OK;
}

// Per-frame host bookkeeping after the launches were queued.
void advance(dogm_handle* h) {
    std::swap(h->desc.free_old, h->desc.free_new);
    h->iteration += 1;
    h->need_clear = false;
    h->first_measurement_received = true;
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

// Shared batch contexts, one per device.
std::mutex g_ctx_mu;
std::map<int, Ctx*> g_batch_ctx;

template <class T>
dogm_status upload_replay(T** dst, const void* src, size_t bytes) {
    if (!src) {
        if (*dst) cudaFree(*dst);
        *dst = nullptr;
        return DOGM_OK;
    }
    if (!*dst) DOGM_CUDA(cudaMalloc((void**)dst, bytes));
    DOGM_CUDA(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
    return DOGM_OK;
}

}  // namespace

extern "C" {

int dogm_abi_version(void) { return DOGM_ABI_VERSION; }
const char* dogm_last_error(void) { return g_last_error.c_str(); }

const char* dogm_status_string(dogm_status s) {
    switch (s) {
        case DOGM_OK: return "ok";
        case DOGM_ERR_INVALID_ARGUMENT: return "invalid argument";
        case DOGM_ERR_OUT_OF_MEMORY: return "out of memory";
        case DOGM_ERR_CUDA: return "CUDA error";
        case DOGM_ERR_DEVICE_TIMEOUT: return "device wait timed out";
        case DOGM_ERR_NOT_READY: return "not ready";
        case DOGM_ERR_UNSUPPORTED: return "unsupported";
        case DOGM_ERR_BUDGET: return "over budget";
    }
    return "unknown";
}

dogm_status dogm_default_options(dogm_options* opt) {
    if (!opt) return fail(DOGM_ERR_INVALID_ARGUMENT, "opt is NULL");
    opt->seed = 123456ull;
    opt->stream_id = 0u;
    opt->resample_mode = DOGM_RESAMPLE_SYSTEMATIC;
    opt->sync_each_update = 1;
    return DOGM_OK;
}

size_t dogm_state_bytes(const dogm_params* p) {
    if (!p) return 0;
    Sizes s;
    if (derive_sizes(*p, s) != DOGM_OK) return 0;
    const size_t N = (size_t)s.N, B = (size_t)s.B, C = (size_t)s.C;
    size_t b = 0;
    b += 3 * N * (16 + 4);                            // P, T (bucketed), S (sorted) particles
    b += B * (16 + 4 + 4);                            // newborns
    // per cell: record 64, measurement copy 16, free mass 2 x 4, {newborn mass, p_A} 8, cell weight 4
    b += C * (sizeof(dogm_grid_cell) + sizeof(dogm_measurement_cell) + 2 * 4 + 8 + 4);
    b += (size_t)s.sort_tiles * (size_t)((s.buckets + 3) & ~3) * 4;  // per-tile bucket counts
    b += (size_t)s.buckets * (4 + 16 + 8) + (size_t)s.cell_tiles * 8 + (size_t)s.res_tiles * 8;
    b += 2 * sizeof(Batch);  // the launch context's device batch of each mirror
    return b;
}

dogm_status dogm_create(const dogm_params* params, const dogm_options* opt, dogm_handle** out) {
    if (!params || !out) return fail(DOGM_ERR_INVALID_ARGUMENT, "params/out is NULL");
    *out = nullptr;
    Sizes s;
    dogm_status st = derive_sizes(*params, s);
    if (st != DOGM_OK) return st;
    dogm_handle* h = new dogm_handle();
    h->params = *params;
    if (opt) h->opt = *opt; else dogm_default_options(&h->opt);
    cudaError_t e = cudaGetDevice(&h->device);
    if (e != cudaSuccess) { delete h; return fail(DOGM_ERR_CUDA, cudaGetErrorString(e)); }
    h->gs = s.gs; h->N = s.N; h->B = s.B; h->C = s.C;
    auto cleanup = [&](dogm_status s2) { dogm_destroy(h); return s2; };
    if ((st = ctx_init(h->ctx, h->device)) != DOGM_OK) return cleanup(st);
    h->ctx.chain = true;
    if (prepare_kernels() != cudaSuccess || prepare_cells() != cudaSuccess || prepare_sort() != cudaSuccess)
        return cleanup(fail(DOGM_ERR_CUDA, "kernel attribute setup failed"));

    GridDesc& g = h->desc;
    g.N = s.N; g.B = s.B; g.C = s.C; g.gs = s.gs;
    g.ctiles = s.buckets;
    g.bucket_stride = (s.buckets + 3) & ~3;
    g.bucket_bits = s.bucket_bits;
    g.q_shift = 61 - bitlen((unsigned long long)s.C);
    g.gs_div = (1ull << 42) / (unsigned long long)s.gs + 1ull;
    g.p_S = params->persistence_prob;
    g.sigma_pos = params->stddev_process_noise_position;
    g.sigma_vel = params->stddev_process_noise_velocity;
    g.p_B = params->birth_prob;
    g.sigma_birth = params->stddev_velocity;
    g.init_max_vel = params->init_max_velocity;
    g.stream_id = h->opt.stream_id;
    g.seed_lo = (uint32_t)(h->opt.seed & 0xffffffffull);
    g.seed_hi = (uint32_t)(h->opt.seed >> 32);
    set_tiles(g, s);

    dogm_measurement_cell* meas_own = nullptr;
    float* fa = nullptr; float* fb = nullptr;
    auto carve = [&](Carver& cv) {
        cv.take(&g.P_state, s.N); cv.take(&g.P_key, s.N);
        cv.take(&g.T_state, s.N); cv.take(&g.T_key, s.N);
        cv.take(&g.S_state, s.N); cv.take(&g.S_key, s.N);
        cv.take(&g.B_state, s.B); cv.take(&g.B_key, s.B); cv.take(&g.B_w, s.B);
        cv.take(&g.cells, s.C);
        cv.take(&meas_own, s.C);
        cv.take(&fa, s.C); cv.take(&fb, s.C);
        cv.take(&g.rho_b, s.C); cv.take(&g.w_cell, s.C);
        cv.take(&g.hsort, (size_t)s.sort_tiles * g.bucket_stride);
        cv.take(&g.ctile_cnt, s.buckets); cv.take(&g.ctile_job, s.buckets);
        cv.take(&g.cell_sum, (size_t)s.buckets + s.cell_tiles);
        cv.take(&g.res_sum, s.res_tiles);
        cv.take(&g.fs, 1);
    };
    {
        Carver sizing;
        carve(sizing);
        unsigned char* arena = nullptr;  // zeroed, freed with the handle's allocations
        if ((st = dalloc(h, &arena, sizing.off)) != DOGM_OK) return cleanup(st);
        Carver cv;
        cv.base = arena;
        carve(cv);
    }
    g.meas_own = meas_own;
    g.meas_src = meas_own;
    g.free_old = fa; g.free_new = fb;
    // measurement cells start as in initGridCellsKernel (init.cu:65-80): no evidence,
    // likelihood 1, p_A 1; cells start with zero masses and empty ranges.
    {
        std::vector<dogm_measurement_cell> m((size_t)s.C, dogm_measurement_cell{0.f, 0.f, 1.f, 1.f});
        e = cudaMemcpy(meas_own, m.data(), sizeof(dogm_measurement_cell) * m.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cleanup(fail(DOGM_ERR_CUDA, cudaGetErrorString(e)));
        std::vector<dogm_grid_cell> c((size_t)s.C);
        for (auto& x : c) { std::memset(&x, 0, sizeof(x)); x.start_idx = -1; x.end_idx = -1; }
        e = cudaMemcpy(g.cells, c.data(), sizeof(dogm_grid_cell) * c.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cleanup(fail(DOGM_ERR_CUDA, cudaGetErrorString(e)));
        FrameState fs{};
        fs.w_res = 0.0f;
        e = cudaMemcpy(g.fs, &fs, sizeof(fs), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cleanup(fail(DOGM_ERR_CUDA, cudaGetErrorString(e)));
    }
    *out = h;
    return DOGM_OK;
}

dogm_status dogm_destroy(dogm_handle* h) {
    if (!h) return DOGM_OK;
    DeviceGuard dg(h->device);
    cudaDeviceSynchronize();
    for (void* p : h->allocations) cudaFree(p);
    for (void* p : {(void*)h->rp_init, (void*)h->rp_predict, (void*)h->rp_birth, (void*)h->rp_resample,
                    (void*)h->dyn_out, (void*)h->dyn_scratch})
        if (p) cudaFree(p);
    if (h->cells_alt) cudaFree(h->desc.cells == h->cells_primary ? h->cells_alt : h->desc.cells);
    for (cudaEvent_t e : {h->frame_ready, h->copy_done[0], h->copy_done[1]})
        if (e) cudaEventDestroy(e);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    delete h;
    return DOGM_OK;
}

// With asynchronous readback in use, each update writes the cell-record buffer the previous
// update did not, after the copy last queued from it has finished (on `stream`).  Records are
// rewritten whole every frame, so the results do not depend on the buffer.
static dogm_status alternate_cells(dogm_handle* h, cudaStream_t stream) {
    if (!h->cells_alt) return DOGM_OK;
    std::swap(h->desc.cells, h->cells_alt);
    const int b = h->desc.cells == h->cells_primary ? 0 : 1;
    DOGM_CUDA(cudaStreamWaitEvent(stream, h->copy_done[b], 0));
    return DOGM_OK;
}

// Makes `stream` wait for every queued asynchronous copy of the handle's cell records.
static dogm_status wait_readback(dogm_handle* h, cudaStream_t stream) {
    for (cudaEvent_t e : h->copy_done)
        if (e) DOGM_CUDA(cudaStreamWaitEvent(stream, e, 0));
    return DOGM_OK;
}

// Host pages that a copy engine reads: on the Grace host of a GB300, host-to-device copies from
// pinned pages that the CPU has not accessed for some seconds slow down the longer the pages stay
// untouched (from 160 to 16 GB/s over 40 s, pages copied every 3 s), while pages that the CPU read
// or wrote just before copy at full speed.  The calling thread therefore reads one byte of every
// page of a host measurement grid before its copy is queued: a few microseconds per grid.
static void touch_host_pages(const void* p, size_t bytes) {
    static const size_t page = [] {
        const long s = sysconf(_SC_PAGESIZE);
        return s >= 4096 ? (size_t)s : (size_t)4096;
    }();
    const volatile unsigned char* b = static_cast<const volatile unsigned char*>(p);
    unsigned int acc = 0;
    for (size_t o = 0; o < bytes; o += page) acc += b[o];
    if (bytes) acc += b[bytes - 1];
    (void)acc;
}

static dogm_status prepare_measurement(dogm_handle* h, const dogm_measurement_cell* meas, int device,
                                       cudaStream_t stream, const dogm_measurement_cell** src, int* copy) {
    *src = h->desc.meas_own;
    *copy = 0;
    if (!meas) return DOGM_OK;  // keep the resident grid
    if (device) {
        *src = meas;
        *copy = 1;
        return DOGM_OK;
    }
    touch_host_pages(meas, sizeof(dogm_measurement_cell) * (size_t)h->C);
    DOGM_CUDA(cudaMemcpyAsync(h->desc.meas_own, meas, sizeof(dogm_measurement_cell) * (size_t)h->C,
                              cudaMemcpyHostToDevice, stream));
    return DOGM_OK;
}

dogm_status dogm_update(dogm_handle* h, const dogm_measurement_cell* meas, float new_x, float new_y, float new_yaw,
                        float dt, int device) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    DeviceGuard dg(h->device);
    Ctx& c = h->ctx;
    dogm_status st = acquire_mirror(c);  // frame k+1 is built while frame k may still run
    if (st != DOGM_OK) return st;
    const dogm_measurement_cell* src;
    int copy;
    st = prepare_measurement(h, meas, device, c.stream, &src, &copy);
    if (st != DOGM_OK) return st;
    st = alternate_cells(h, c.stream);
    if (st != DOGM_OK) return st;
    const bool init = !h->first_measurement_received;
    int shifted, xm, ym;
    pose_update(h, new_x, new_y, new_yaw, &shifted, &xm, &ym);
    fill_frame(h, dt, shifted, xm, ym, src, copy);
    dogm_handle* hs[1] = {h};
    std::vector<int> init_mask(1, init ? 1 : 0);
    build_batch(c, hs, 1, init_mask);
    st = run_frame(c, 1, init, h->need_clear, &h->last_launches);
    if (st != DOGM_OK) { h->need_clear = true; return st; }
    advance(h);
    if (h->opt.sync_each_update) return finish_frame(c, hs, 1);
    return DOGM_OK;
}

dogm_status dogm_update_batch(dogm_handle* const* hs, int n, const dogm_measurement_cell* const* meas,
                              const float* new_x, const float* new_y, const float* new_yaw, const float* dt,
                              int device) {
    if (!hs || n <= 0 || n > kMaxBatch || !new_x || !new_y || !new_yaw || !dt)
        return fail(DOGM_ERR_INVALID_ARGUMENT, "bad batch arguments");
    const int dev = hs[0]->device;
    for (int i = 0; i < n; ++i) {
        if (!hs[i] || hs[i]->device != dev) return fail(DOGM_ERR_INVALID_ARGUMENT, "all handles must share a device");
        for (int j = 0; j < i; ++j)
            if (hs[j] == hs[i]) return fail(DOGM_ERR_INVALID_ARGUMENT, "a handle appears twice in a batch");
    }
    DeviceGuard dg(dev);
    Ctx* c;
    {
        std::lock_guard<std::mutex> lk(g_ctx_mu);
        auto it = g_batch_ctx.find(dev);
        if (it == g_batch_ctx.end()) {
            c = new Ctx();
            dogm_status st = ctx_init(*c, dev);
            if (st != DOGM_OK) { delete c; return st; }
            g_batch_ctx[dev] = c;
        } else {
            c = it->second;
        }
    }
    DOGM_CUDA(cudaStreamSynchronize(c->stream));
    dogm_status st0 = acquire_mirror(*c);
    if (st0 != DOGM_OK) return st0;
    std::vector<int> init_mask(n, 0);
    bool any_init = false;
    for (int i = 0; i < n; ++i) {
        dogm_handle* h = hs[i];
        DOGM_CUDA(cudaStreamSynchronize(h->ctx.stream));
        const dogm_measurement_cell* src;
        int copy;
        dogm_status st = prepare_measurement(h, meas ? meas[i] : nullptr, device, c->stream, &src, &copy);
        if (st != DOGM_OK) return st;
        st = alternate_cells(h, c->stream);
        if (st != DOGM_OK) return st;
        init_mask[i] = h->first_measurement_received ? 0 : 1;
        any_init |= init_mask[i] != 0;
        int shifted, xm, ym;
        pose_update(h, new_x[i], new_y[i], new_yaw[i], &shifted, &xm, &ym);
        fill_frame(h, dt[i], shifted, xm, ym, src, copy);
    }
    build_batch(*c, hs, n, init_mask);
    bool any_clear = false;
    for (int i = 0; i < n; ++i) any_clear |= hs[i]->need_clear;
    int launches = 0;
    dogm_status st = run_frame(*c, n, any_init, any_clear, &launches);
    if (st != DOGM_OK) {
        for (int i = 0; i < n; ++i) hs[i]->need_clear = true;
        return st;
    }
    for (int i = 0; i < n; ++i) {
        advance(hs[i]);
        hs[i]->last_launches = launches;
    }
    return finish_frame(*c, hs, n);
}

dogm_status dogm_synchronize(dogm_handle* h) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    DeviceGuard dg(h->device);
    dogm_status st = wait_readback(h, h->ctx.stream);  // queued asynchronous copies finish too
    if (st != DOGM_OK) return st;
    dogm_handle* hs[1] = {h};
    return finish_frame(h->ctx, hs, 1);
}

dogm_status dogm_get_grid_cells(dogm_handle* h, dogm_grid_cell* host_out, size_t n) {
    if (!h || !host_out) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n != (size_t)h->C) return fail(DOGM_ERR_INVALID_ARGUMENT, "n must equal grid_size^2");
    DeviceGuard dg(h->device);
    DOGM_CUDA(cudaMemcpyAsync(host_out, h->desc.cells, sizeof(dogm_grid_cell) * n, cudaMemcpyDeviceToHost,
                              h->ctx.stream));
    DOGM_CUDA(cudaStreamSynchronize(h->ctx.stream));
    return DOGM_OK;
}

dogm_status dogm_get_grid_cells_async(dogm_handle* h, dogm_grid_cell* host_out, size_t n) {
    if (!h || !host_out) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n != (size_t)h->C) return fail(DOGM_ERR_INVALID_ARGUMENT, "n must equal grid_size^2");
    DeviceGuard dg(h->device);
    if (!h->cells_alt) {
        dogm_grid_cell* alt = nullptr;
        dogm_status st = dalloc(h, &alt, (size_t)h->C);
        if (st != DOGM_OK) return st;
        h->allocations.pop_back();  // owned through cells_alt / desc.cells, freed in dogm_destroy
        if (cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->frame_ready, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->copy_done[0], cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->copy_done[1], cudaEventDisableTiming) != cudaSuccess) {
            for (cudaEvent_t* e : {&h->frame_ready, &h->copy_done[0], &h->copy_done[1]})
                if (*e) { cudaEventDestroy(*e); *e = nullptr; }
            if (h->copy_stream) { cudaStreamDestroy(h->copy_stream); h->copy_stream = nullptr; }
            cudaFree(alt);
            return fail(DOGM_ERR_CUDA, "readback stream or event creation failed");
        }
        h->cells_primary = h->desc.cells;
        h->cells_alt = alt;
    }
    const int b = h->desc.cells == h->cells_primary ? 0 : 1;
    DOGM_CUDA(cudaEventRecord(h->frame_ready, h->ctx.stream));
    DOGM_CUDA(cudaStreamWaitEvent(h->copy_stream, h->frame_ready, 0));
    DOGM_CUDA(cudaMemcpyAsync(host_out, h->desc.cells, sizeof(dogm_grid_cell) * n, cudaMemcpyDeviceToHost,
                              h->copy_stream));
    DOGM_CUDA(cudaEventRecord(h->copy_done[b], h->copy_stream));
    return DOGM_OK;
}

dogm_status dogm_get_grid_cells_device(dogm_handle* h, dogm_grid_cell* dev_out, size_t n) {
    if (!h || !dev_out) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n != (size_t)h->C) return fail(DOGM_ERR_INVALID_ARGUMENT, "n must equal grid_size^2");
    DeviceGuard dg(h->device);
    DOGM_CUDA(cudaMemcpyAsync(dev_out, h->desc.cells, sizeof(dogm_grid_cell) * n, cudaMemcpyDeviceToDevice,
                              h->ctx.stream));
    DOGM_CUDA(cudaStreamSynchronize(h->ctx.stream));
    return DOGM_OK;
}

dogm_status dogm_get_measurement_cells(dogm_handle* h, dogm_measurement_cell* host_out, size_t n) {
    if (!h || !host_out) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n != (size_t)h->C) return fail(DOGM_ERR_INVALID_ARGUMENT, "n must equal grid_size^2");
    DeviceGuard dg(h->device);
    DOGM_CUDA(cudaMemcpyAsync(host_out, h->desc.meas_own, sizeof(dogm_measurement_cell) * n, cudaMemcpyDeviceToHost,
                              h->ctx.stream));
    DOGM_CUDA(cudaStreamSynchronize(h->ctx.stream));
    return DOGM_OK;
}

dogm_status dogm_get_particles(dogm_handle* h, float* state, int* idx, float* weight, unsigned char* assoc, size_t n) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    if (n != (size_t)h->N) return fail(DOGM_ERR_INVALID_ARGUMENT, "n must equal particle_count");
    DeviceGuard dg(h->device);
    cudaStream_t s = h->ctx.stream;
    std::vector<uint32_t> keys(n);
    FrameState fs;
    if (state) DOGM_CUDA(cudaMemcpyAsync(state, h->desc.P_state, 16 * n, cudaMemcpyDeviceToHost, s));
    DOGM_CUDA(cudaMemcpyAsync(keys.data(), h->desc.P_key, 4 * n, cudaMemcpyDeviceToHost, s));
    DOGM_CUDA(cudaMemcpyAsync(&fs, h->desc.fs, sizeof(fs), cudaMemcpyDeviceToHost, s));
    DOGM_CUDA(cudaStreamSynchronize(s));
    for (size_t i = 0; i < n; ++i) {
        if (idx) idx[i] = (int)(keys[i] & kCellMask);
        if (assoc) assoc[i] = (keys[i] & kAssocBit) ? 1 : 0;
        if (weight) weight[i] = (keys[i] & kOutBit) ? 0.0f : fs.w_res;
    }
    return DOGM_OK;
}

int dogm_get_grid_size(const dogm_handle* h) { return h ? h->gs : 0; }
float dogm_get_resolution(const dogm_handle* h) { return h ? h->params.resolution : 0.f; }
float dogm_get_position_x(const dogm_handle* h) { return h ? h->position_x : 0.f; }
float dogm_get_position_y(const dogm_handle* h) { return h ? h->position_y : 0.f; }
float dogm_get_yaw(const dogm_handle* h) { return h ? h->yaw : 0.f; }
int dogm_get_iteration(const dogm_handle* h) { return h ? h->iteration : 0; }
int dogm_get_particle_count(const dogm_handle* h) { return h ? h->N : 0; }
int dogm_get_new_born_particle_count(const dogm_handle* h) { return h ? h->B : 0; }
int dogm_last_launch_count(const dogm_handle* h) { return h ? h->last_launches : 0; }

dogm_status dogm_set_launch_mode(dogm_handle* h, int mode) {
    if (!h || (mode != DOGM_LAUNCH_CHAINED && mode != DOGM_LAUNCH_GRAPH && mode != DOGM_LAUNCH_PLAIN))
        return fail(DOGM_ERR_INVALID_ARGUMENT, "bad handle or launch mode");
    h->ctx.launch_mode = mode;
    return DOGM_OK;
}

// ---- stage calls -----------------------------------------------------------------------

dogm_status dogm_particle_prediction(dogm_handle* h, float dt) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    DeviceGuard dg(h->device);
    Ctx& c = h->ctx;
    DOGM_CUDA(cudaStreamSynchronize(c.stream));
    fill_frame(h, dt, 0, 0, 0, h->desc.meas_own, 0);
    dogm_handle* hs[1] = {h};
    c.pending[0] = c.pending[1] = false;  // the stream was synchronised above
    build_batch(c, hs, 1, std::vector<int>(1, 0));
    DOGM_CUDA(upload_batch(c, 1));
    LaunchCfg cfg{c.num_sms, c.stream};
    DOGM_CUDA(launch_predict(c.d_batch, 1, cfg));
    DOGM_CUDA(cudaStreamSynchronize(c.stream));
    // the common weight becomes p_S * w (predict.cu:30); out-of-grid particles read as 0
    FrameState fs;
    DOGM_CUDA(cudaMemcpy(&fs, h->desc.fs, sizeof(fs), cudaMemcpyDeviceToHost));
    fs.w_res = fs.w_res * h->params.persistence_prob;
    DOGM_CUDA(cudaMemcpy(&h->desc.fs->w_res, &fs.w_res, sizeof(float), cudaMemcpyHostToDevice));
    h->last_launches = 1;
    return DOGM_OK;
}

}  // extern "C"

// Runs stage launches on the handle's resident state (the reference's public stage methods):
// the handle alone in a batch, kernels launched one by one and waited for; the cell pass runs
// only the parts in `mask`, and the weights are taken as already predicted (particlePrediction
// multiplies them by p_S, predict.cu:30).  Returns the launches' device status.
template <class Launch>
static dogm_status run_stage(dogm_handle* h, float dt, uint32_t mask, int n_launches, Launch launch) {
    DeviceGuard dg(h->device);
    Ctx& c = h->ctx;
    DOGM_CUDA(cudaStreamSynchronize(c.stream));
    c.pending[0] = c.pending[1] = false;  // the stream was synchronised above
    dogm_status st = wait_readback(h, c.stream);  // the cell records may be rewritten
    if (st != DOGM_OK) return st;
    fill_frame(h, dt, 0, 0, 0, h->desc.meas_own, 0);
    h->desc.stage_mask = mask;
    h->desc.weights_predicted = 1;
    dogm_handle* hs[1] = {h};
    build_batch(c, hs, 1, std::vector<int>(1, 0));
    h->desc.stage_mask = kPartAll;
    h->desc.weights_predicted = 0;
    DOGM_CUDA(upload_batch(c, 1));
    LaunchCfg cfg{c.num_sms, c.stream};
    DOGM_CUDA(launch(cfg));
    DOGM_CUDA(download_status(c));
    h->last_launches = n_launches;
    return finish_frame(c, hs, 1);
}

extern "C" {

dogm_status dogm_particle_assignment(dogm_handle* h) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    const bool clear = h->need_clear;  // first frame, or after a failed one: all counters reset
    Ctx& c = h->ctx;
    return run_stage(h, h->stage_dt, kPartRanges, 4 + (clear ? 1 : 0), [&](const LaunchCfg& cfg) {
        cudaError_t e;
        if (clear && (e = launch_frame_begin(c.d_batch, 1, cfg)) != cudaSuccess) return e;
        if ((e = launch_predict(c.d_batch, 2, cfg)) != cudaSuccess) return e;
        if ((e = launch_sort_scan(c.d_batch, cfg)) != cudaSuccess) return e;
        if ((e = launch_sort_scatter(c.d_batch, c.scatter_ctiles, cfg)) != cudaSuccess) return e;
        return launch_cells(c.d_batch, cfg, true);
    });
}

dogm_status dogm_grid_cell_occupancy_update(dogm_handle* h, float dt) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    h->stage_dt = dt;  // freespace_discount^dt (dogm.cu:291) is also what the later parts use
    Ctx& c = h->ctx;
    return run_stage(h, dt, kPartMasses, 1, [&](const LaunchCfg& cfg) { return launch_cells(c.d_batch, cfg, true); });
}

dogm_status dogm_update_persistent_particles(dogm_handle* h) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    Ctx& c = h->ctx;
    return run_stage(h, h->stage_dt, kPartReweight, 1, [&](const LaunchCfg& cfg) { return launch_cells(c.d_batch, cfg, true); });
}

dogm_status dogm_initialize_new_particles(dogm_handle* h) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    Ctx& c = h->ctx;
    return run_stage(h, h->stage_dt, 0u, 1, [&](const LaunchCfg& cfg) { return launch_newborn(c.d_batch, cfg); });
}

dogm_status dogm_statistical_moments(dogm_handle* h) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    Ctx& c = h->ctx;
    return run_stage(h, h->stage_dt, kPartMoments, 1, [&](const LaunchCfg& cfg) { return launch_cells(c.d_batch, cfg, true); });
}

dogm_status dogm_resampling(dogm_handle* h) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    Ctx& c = h->ctx;
    dogm_status st = run_stage(h, h->stage_dt, 0u, 1,
                               [&](const LaunchCfg& cfg) { return launch_resample(c.d_batch, c.res_bits, cfg); });
    if (st != DOGM_OK) return st;
    // the resampled particles are the current ones (the reference's particle_array =
    // particle_array_next, dogm.cu:128), and the frame ends as an update's does
    advance(h);
    return DOGM_OK;
}

dogm_status dogm_update_pose(dogm_handle* h, float new_x, float new_y, float new_yaw) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    DeviceGuard dg(h->device);
    int shifted, xm, ym;
    pose_update(h, new_x, new_y, new_yaw, &shifted, &xm, &ym);
    if (!shifted) return DOGM_OK;
    // the shift rewrites the cell records in place: copies queued from them by
    // dogm_get_grid_cells_async finish first
    dogm_status st = wait_readback(h, h->ctx.stream);
    if (st != DOGM_OK) return st;
    LaunchCfg cfg{h->ctx.num_sms, h->ctx.stream};
    DOGM_CUDA(launch_shift_stage(h->desc, xm, ym, cfg));
    DOGM_CUDA(cudaStreamSynchronize(h->ctx.stream));
    std::swap(h->desc.free_old, h->desc.free_new);
    return DOGM_OK;
}

// dogm_update_pose without device allocation: the shift's copy of the previous cell records
// goes to the library's fixed shift array (launch_shift_stage_noalloc) instead of a temporary
// buffer.  A grid too large for the array is refused before the pose changes.
dogm_status dogm_update_pose_noalloc(dogm_handle* h, float new_x, float new_y, float new_yaw) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    const size_t need = sizeof(dogm_grid_cell) * (size_t)h->C;
    if (need > kShiftScratchBytes)
        return fail(DOGM_ERR_INVALID_ARGUMENT,
                    "dogm_update_pose_noalloc: a grid of " + std::to_string(h->C) + " cells needs " +
                        std::to_string(need) + " B of shift scratch, more than the fixed " +
                        std::to_string(kShiftScratchBytes) + " B (" +
                        std::to_string(kShiftScratchBytes / sizeof(dogm_grid_cell)) +
                        " cells); use dogm_update_pose for this grid");
    DeviceGuard dg(h->device);
    DOGM_CUDA(shift_scratch_setup());
    int shifted, xm, ym;
    pose_update(h, new_x, new_y, new_yaw, &shifted, &xm, &ym);
    if (!shifted) return DOGM_OK;
    dogm_status st = wait_readback(h, h->ctx.stream);  // as dogm_update_pose
    if (st != DOGM_OK) return st;
    LaunchCfg cfg{h->ctx.num_sms, h->ctx.stream};
    DOGM_CUDA(launch_shift_stage_noalloc(h->desc, xm, ym, cfg));
    DOGM_CUDA(cudaStreamSynchronize(h->ctx.stream));
    std::swap(h->desc.free_old, h->desc.free_new);
    return DOGM_OK;
}

dogm_status dogm_initialize_particles(dogm_handle* h) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    DeviceGuard dg(h->device);
    Ctx& c = h->ctx;
    DOGM_CUDA(cudaStreamSynchronize(c.stream));
    fill_frame(h, 0.f, 0, 0, 0, h->desc.meas_own, 0);
    dogm_handle* hs[1] = {h};
    c.pending[0] = c.pending[1] = false;  // the stream was synchronised above
    build_batch(c, hs, 1, std::vector<int>(1, 1));
    DOGM_CUDA(upload_batch(c, 1));
    LaunchCfg cfg{c.num_sms, c.stream};
    DOGM_CUDA(launch_frame_begin(c.d_batch, 1, cfg));
    DOGM_CUDA(launch_init_particles(c.d_batch, cfg));
    DOGM_CUDA(cudaStreamSynchronize(c.stream));
    h->first_measurement_received = true;
    h->need_clear = true;
    return DOGM_OK;
}

// ---- state injection, replay, debug ------------------------------------------------------

dogm_status dogm_set_measurement_cells(dogm_handle* h, const dogm_measurement_cell* host_in, size_t n) {
    if (!h || !host_in) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n != (size_t)h->C) return fail(DOGM_ERR_INVALID_ARGUMENT, "n must equal grid_size^2");
    DeviceGuard dg(h->device);
    DOGM_CUDA(cudaMemcpy(h->desc.meas_own, host_in, sizeof(dogm_measurement_cell) * n, cudaMemcpyHostToDevice));
    return DOGM_OK;
}

dogm_status dogm_set_particles(dogm_handle* h, const float* state, const int* idx, const unsigned char* assoc,
                               float weight, size_t n) {
    if (!h || !state) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n != (size_t)h->N) return fail(DOGM_ERR_INVALID_ARGUMENT, "n must equal particle_count");
    DeviceGuard dg(h->device);
    std::vector<uint32_t> keys(n);
    for (size_t i = 0; i < n; ++i)
        keys[i] = (idx ? ((uint32_t)idx[i] & kCellMask) : 0u) | ((assoc && assoc[i]) ? kAssocBit : 0u);
    DOGM_CUDA(cudaMemcpy(h->desc.P_state, state, 16 * n, cudaMemcpyHostToDevice));
    DOGM_CUDA(cudaMemcpy(h->desc.P_key, keys.data(), 4 * n, cudaMemcpyHostToDevice));
    DOGM_CUDA(cudaMemcpy(&h->desc.fs->w_res, &weight, sizeof(float), cudaMemcpyHostToDevice));
    h->first_measurement_received = true;
    return DOGM_OK;
}

dogm_status dogm_set_replay(dogm_handle* h, const float* init_u, const float* predict_z, const float* birth_z,
                            const uint64_t* resample_r) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    DeviceGuard dg(h->device);
    DOGM_CUDA(cudaStreamSynchronize(h->ctx.stream));
    dogm_status st;
    if ((st = upload_replay(&h->rp_init, init_u, 8 * (size_t)h->N)) != DOGM_OK) return st;
    if ((st = upload_replay(&h->rp_predict, predict_z, 16 * (size_t)h->N)) != DOGM_OK) return st;
    if ((st = upload_replay(&h->rp_birth, birth_z, 8 * (size_t)std::max(h->B, 1))) != DOGM_OK) return st;
    if ((st = upload_replay(&h->rp_resample, resample_r, 8)) != DOGM_OK) return st;
    return DOGM_OK;
}

dogm_status dogm_clear_replay(dogm_handle* h) { return dogm_set_replay(h, nullptr, nullptr, nullptr, nullptr); }

dogm_status dogm_generate_draws(dogm_handle* h, int iteration, float* init_u, float* predict_z, float* birth_z,
                                uint64_t* resample_r) {
    if (!h || iteration < 0) return fail(DOGM_ERR_INVALID_ARGUMENT, "bad argument");
    DeviceGuard dg(h->device);
    cudaStream_t s = h->ctx.stream;
    float2* di = nullptr; float4* dp = nullptr; float2* db = nullptr; unsigned long long* dr = nullptr;
    if (init_u) DOGM_CUDA(cudaMalloc(&di, 8 * (size_t)h->N));
    if (predict_z) DOGM_CUDA(cudaMalloc(&dp, 16 * (size_t)h->N));
    if (birth_z && h->B > 0) DOGM_CUDA(cudaMalloc(&db, 8 * (size_t)h->B));
    if (resample_r) DOGM_CUDA(cudaMalloc(&dr, 8));
    LaunchCfg cfg{h->ctx.num_sms, s};
    DOGM_CUDA(launch_draws(h->desc, iteration, di, dp, db, dr, cfg));
    DOGM_CUDA(cudaStreamSynchronize(s));
    if (di) DOGM_CUDA(cudaMemcpy(init_u, di, 8 * (size_t)h->N, cudaMemcpyDeviceToHost));
    if (dp) DOGM_CUDA(cudaMemcpy(predict_z, dp, 16 * (size_t)h->N, cudaMemcpyDeviceToHost));
    if (db) DOGM_CUDA(cudaMemcpy(birth_z, db, 8 * (size_t)h->B, cudaMemcpyDeviceToHost));
    if (dr) DOGM_CUDA(cudaMemcpy(resample_r, dr, 8, cudaMemcpyDeviceToHost));
    for (void* p : {(void*)di, (void*)dp, (void*)db, (void*)dr}) if (p) cudaFree(p);
    return DOGM_OK;
}

dogm_status dogm_debug_enable(dogm_handle* h, int enable) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    DeviceGuard dg(h->device);
    if (enable && !h->debug) {
        dogm_status st;
        if ((st = dalloc(h, &h->desc.dbg_perm, h->N)) != DOGM_OK) return st;
        if ((st = dalloc(h, &h->desc.T_idx, h->N)) != DOGM_OK) return st;
        if ((st = dalloc(h, &h->desc.dbg_src, h->N)) != DOGM_OK) return st;
        h->debug = true;
    } else if (!enable) {
        h->desc.dbg_perm = nullptr;
        h->desc.T_idx = nullptr;
        h->desc.dbg_src = nullptr;
        h->debug = false;
    }
    return DOGM_OK;
}

dogm_status dogm_debug_export(dogm_handle* h, int* sorted_cell, float* sorted_state, int* sort_perm,
                              float* birth_state, int* birth_cell, unsigned char* birth_assoc, float* birth_weight,
                              int* resample_src, uint64_t* joint_total, int* q_shift, int* n_birth) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    DeviceGuard dg(h->device);
    DOGM_CUDA(cudaStreamSynchronize(h->ctx.stream));
    const size_t N = (size_t)h->N, B = (size_t)h->B;
    if (sorted_cell) {
        std::vector<uint32_t> k(N);
        DOGM_CUDA(cudaMemcpy(k.data(), h->desc.S_key, 4 * N, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < N; ++i) sorted_cell[i] = (int)(k[i] & kCellMask);
    }
    if (sorted_state) DOGM_CUDA(cudaMemcpy(sorted_state, h->desc.S_state, 16 * N, cudaMemcpyDeviceToHost));
    if (sort_perm) {
        if (!h->debug) return fail(DOGM_ERR_NOT_READY, "enable debug before the update to export the permutation");
        DOGM_CUDA(cudaMemcpy(sort_perm, h->desc.dbg_perm, 4 * N, cudaMemcpyDeviceToHost));
    }
    if (B > 0) {
        if (birth_state) DOGM_CUDA(cudaMemcpy(birth_state, h->desc.B_state, 16 * B, cudaMemcpyDeviceToHost));
        if (birth_weight) DOGM_CUDA(cudaMemcpy(birth_weight, h->desc.B_w, 4 * B, cudaMemcpyDeviceToHost));
        if (birth_cell || birth_assoc) {
            std::vector<uint32_t> k(B);
            DOGM_CUDA(cudaMemcpy(k.data(), h->desc.B_key, 4 * B, cudaMemcpyDeviceToHost));
            for (size_t i = 0; i < B; ++i) {
                if (birth_cell) birth_cell[i] = (int)(k[i] & kCellMask);
                if (birth_assoc) birth_assoc[i] = (k[i] & kAssocBit) ? 1 : 0;
            }
        }
    }
    if (resample_src) {
        if (!h->debug) return fail(DOGM_ERR_NOT_READY, "enable debug before the update to export resample sources");
        DOGM_CUDA(cudaMemcpy(resample_src, h->desc.dbg_src, 4 * N, cudaMemcpyDeviceToHost));
    }
    FrameState fs;
    DOGM_CUDA(cudaMemcpy(&fs, h->desc.fs, sizeof(fs), cudaMemcpyDeviceToHost));
    if (joint_total) *joint_total = fs.joint_total;
    if (q_shift) *q_shift = h->desc.q_shift;
    if (n_birth) *n_birth = fs.n_birth;
    return DOGM_OK;
}

dogm_status dogm_debug_joint_weights(dogm_handle* h, float* weights, size_t n, int* n_joint) {
    if (!h || !weights) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!h->debug) return fail(DOGM_ERR_NOT_READY, "enable debug before the update to export the joint weights");
    if (n < (size_t)h->N + (size_t)h->B) return fail(DOGM_ERR_INVALID_ARGUMENT, "n < particle_count + newborns");
    DeviceGuard dg(h->device);
    DOGM_CUDA(cudaStreamSynchronize(h->ctx.stream));
    const size_t N = (size_t)h->N, C = (size_t)h->C;
    FrameState fs;
    DOGM_CUDA(cudaMemcpy(&fs, h->desc.fs, sizeof(fs), cudaMemcpyDeviceToHost));
    std::vector<uint32_t> k(N);
    std::vector<float> wc(C);
    DOGM_CUDA(cudaMemcpy(k.data(), h->desc.S_key, 4 * N, cudaMemcpyDeviceToHost));
    DOGM_CUDA(cudaMemcpy(wc.data(), h->desc.w_cell, 4 * C, cudaMemcpyDeviceToHost));
    // persistent items in sorted order: the reweighted weight of their cell, 0 out of the grid
    for (size_t i = 0; i < N; ++i) weights[i] = (k[i] & kOutBit) ? 0.0f : wc[k[i] & kCellMask];
    const size_t nb = (size_t)std::max(fs.n_birth, 0);
    if (nb) DOGM_CUDA(cudaMemcpy(weights + N, h->desc.B_w, 4 * nb, cudaMemcpyDeviceToHost));
    if (n_joint) *n_joint = (int)(N + nb);
    return DOGM_OK;
}

// ---- measurement -------------------------------------------------------------------------

void* dogm_get_stream(dogm_handle* h) { return h ? (void*)h->ctx.stream : nullptr; }

dogm_status dogm_profile_enable(dogm_handle* h, int enable) {
    if (!h) return fail(DOGM_ERR_INVALID_ARGUMENT, "handle is NULL");
    h->ctx.profile = enable != 0;
    return DOGM_OK;
}

int dogm_stage_times(dogm_handle* h, float* ms, int n) {
    if (!h || !h->ctx.profile) return 0;
    DeviceGuard dg(h->device);
    if (cudaEventSynchronize(h->ctx.ev[kStages]) != cudaSuccess) return 0;
    for (int i = 0; i < kStages && i < n; ++i) {
        float t = 0.f;
        cudaEventElapsedTime(&t, h->ctx.ev[i], h->ctx.ev[i + 1]);
        if (ms) ms[i] = t;
    }
    return kStages;
}

const char* dogm_stage_name(int i) { return (i >= 0 && i < kStages) ? kStageNames[i] : ""; }

// ---- snapshot and restore --------------------------------------------------------------------

namespace {
struct SnapshotHeader {
    char magic[8];  // "DOGMSNP1"
    uint32_t header_bytes;
    int32_t gs, N, B;
    dogm_params params;
    uint64_t seed;
    uint32_t stream_id;
    int32_t iteration;
    int32_t first_pose, first_measurement, need_clear;
    float position_x, position_y, yaw;
    FrameState fs;
};
constexpr char kSnapMagic[8] = {'D', 'O', 'G', 'M', 'S', 'N', 'P', '1'};

size_t snapshot_payload(const dogm_handle* h) {
    const size_t N = (size_t)h->N, C = (size_t)h->C;
    return N * (16 + 4) + C * (4 + sizeof(dogm_measurement_cell) + sizeof(dogm_grid_cell));
}
}  // namespace

size_t dogm_snapshot_bytes(const dogm_handle* h) { return h ? sizeof(SnapshotHeader) + snapshot_payload(h) : 0; }

dogm_status dogm_snapshot(dogm_handle* h, void* host_buf, size_t n) {
    if (!h || !host_buf) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n < dogm_snapshot_bytes(h)) return fail(DOGM_ERR_INVALID_ARGUMENT, "buffer smaller than dogm_snapshot_bytes");
    DeviceGuard dg(h->device);
    dogm_status st = dogm_synchronize(h);
    if (st != DOGM_OK) return st;
    SnapshotHeader hd;
    std::memset(&hd, 0, sizeof(hd));
    std::memcpy(hd.magic, kSnapMagic, 8);
    hd.header_bytes = sizeof(SnapshotHeader);
    hd.gs = h->gs;
    hd.N = h->N;
    hd.B = h->B;
    hd.params = h->params;
    hd.seed = h->opt.seed;
    hd.stream_id = h->opt.stream_id;
    hd.iteration = h->iteration;
    hd.first_pose = h->first_pose_received;
    hd.first_measurement = h->first_measurement_received;
    hd.need_clear = h->need_clear;
    hd.position_x = h->position_x;
    hd.position_y = h->position_y;
    hd.yaw = h->yaw;
    DOGM_CUDA(cudaMemcpy(&hd.fs, h->desc.fs, sizeof(FrameState), cudaMemcpyDeviceToHost));
    unsigned char* p = static_cast<unsigned char*>(host_buf);
    std::memcpy(p, &hd, sizeof(hd));
    p += sizeof(hd);
    const size_t N = (size_t)h->N, C = (size_t)h->C;
    DOGM_CUDA(cudaMemcpy(p, h->desc.P_state, 16 * N, cudaMemcpyDeviceToHost));
    p += 16 * N;
    DOGM_CUDA(cudaMemcpy(p, h->desc.P_key, 4 * N, cudaMemcpyDeviceToHost));
    p += 4 * N;
    DOGM_CUDA(cudaMemcpy(p, h->desc.free_old, 4 * C, cudaMemcpyDeviceToHost));  // carried into the next update
    p += 4 * C;
    DOGM_CUDA(cudaMemcpy(p, h->desc.meas_own, sizeof(dogm_measurement_cell) * C, cudaMemcpyDeviceToHost));
    p += sizeof(dogm_measurement_cell) * C;
    DOGM_CUDA(cudaMemcpy(p, h->desc.cells, sizeof(dogm_grid_cell) * C, cudaMemcpyDeviceToHost));
    return DOGM_OK;
}

dogm_status dogm_restore(dogm_handle* h, const void* host_buf, size_t n) {
    if (!h || !host_buf) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n < sizeof(SnapshotHeader)) return fail(DOGM_ERR_INVALID_ARGUMENT, "buffer shorter than a snapshot header");
    SnapshotHeader hd;
    std::memcpy(&hd, host_buf, sizeof(hd));
    if (std::memcmp(hd.magic, kSnapMagic, 8) != 0 || hd.header_bytes != sizeof(SnapshotHeader))
        return fail(DOGM_ERR_INVALID_ARGUMENT, "not a snapshot of this library version");
    if (hd.gs != h->gs || hd.N != h->N || hd.B != h->B || std::memcmp(&hd.params, &h->params, sizeof(dogm_params)) != 0)
        return fail(DOGM_ERR_INVALID_ARGUMENT, "snapshot of a handle with other parameters");
    if (n < dogm_snapshot_bytes(h)) return fail(DOGM_ERR_INVALID_ARGUMENT, "truncated snapshot");
    DeviceGuard dg(h->device);
    dogm_status st = dogm_synchronize(h);
    if (st != DOGM_OK) return st;
    const unsigned char* p = static_cast<const unsigned char*>(host_buf) + sizeof(hd);
    const size_t N = (size_t)h->N, C = (size_t)h->C;
    DOGM_CUDA(cudaMemcpy(h->desc.P_state, p, 16 * N, cudaMemcpyHostToDevice));
    p += 16 * N;
    DOGM_CUDA(cudaMemcpy(h->desc.P_key, p, 4 * N, cudaMemcpyHostToDevice));
    p += 4 * N;
    DOGM_CUDA(cudaMemcpy(h->desc.free_old, p, 4 * C, cudaMemcpyHostToDevice));
    p += 4 * C;
    DOGM_CUDA(cudaMemcpy(h->desc.meas_own, p, sizeof(dogm_measurement_cell) * C, cudaMemcpyHostToDevice));
    p += sizeof(dogm_measurement_cell) * C;
    DOGM_CUDA(cudaMemcpy(h->desc.cells, p, sizeof(dogm_grid_cell) * C, cudaMemcpyHostToDevice));
    FrameState fs = hd.fs;
    fs.status = 0u;
    DOGM_CUDA(cudaMemcpy(h->desc.fs, &fs, sizeof(FrameState), cudaMemcpyHostToDevice));
    h->opt.seed = hd.seed;
    h->opt.stream_id = hd.stream_id;
    h->desc.seed_lo = (uint32_t)(hd.seed & 0xffffffffull);
    h->desc.seed_hi = (uint32_t)(hd.seed >> 32);
    h->desc.stream_id = hd.stream_id;
    h->iteration = hd.iteration;
    h->first_pose_received = hd.first_pose != 0;
    h->first_measurement_received = hd.first_measurement != 0;
    h->position_x = hd.position_x;
    h->position_y = hd.position_y;
    h->yaw = hd.yaw;
    h->need_clear = true;  // the restored frame starts with a full reset of the per-frame counters
    return DOGM_OK;
}

dogm_status dogm_extract_dynamic_cells(dogm_handle* h, float min_occupancy, float min_velocity,
                                       dogm_dynamic_cell* host_out, int max_out, int* n_found) {
    if (!h || !n_found || max_out < 0 || (max_out > 0 && !host_out))
        return fail(DOGM_ERR_INVALID_ARGUMENT, "bad dynamic-cell extraction arguments");
    DeviceGuard dg(h->device);
    Ctx& c = h->ctx;
    if (!h->dyn_scratch) DOGM_CUDA(cudaMalloc(&h->dyn_scratch, sizeof(unsigned int) * (size_t)div_up(h->C, 1024)));
    if (max_out > h->dyn_cap) {
        if (h->dyn_out) cudaFree(h->dyn_out);
        h->dyn_out = nullptr;
        h->dyn_cap = 0;
        DOGM_CUDA(cudaMalloc(&h->dyn_out, sizeof(dogm_dynamic_cell) * (size_t)max_out));
        h->dyn_cap = max_out;
    }
    dogm_dynamic_cell* out = h->dyn_out ? h->dyn_out : reinterpret_cast<dogm_dynamic_cell*>(h->dyn_scratch);
    dogm_status st = dogm_extract_dynamic_cells_device(h->desc.cells, h->gs, min_occupancy, min_velocity, out, max_out,
                                                       h->dyn_scratch, n_found, (void*)c.stream);
    if (st != DOGM_OK) return st;
    const int n = std::min(*n_found, max_out);
    if (n > 0) {
        DOGM_CUDA(cudaMemcpyAsync(host_out, h->dyn_out, sizeof(dogm_dynamic_cell) * (size_t)n, cudaMemcpyDeviceToHost,
                                  c.stream));
        DOGM_CUDA(cudaStreamSynchronize(c.stream));
    }
    return DOGM_OK;
}

// ---- autotuning ----------------------------------------------------------------------------

// ms per update over `reps` graph-launched updates on the resident measurement grid.
static dogm_status time_updates(dogm_handle* h, int reps, float* ms) {
    Ctx& c = h->ctx;
    dogm_status st;
    for (int i = 0; i < 2; ++i)  // graph capture of both mirrors
        if ((st = dogm_update(h, nullptr, 0.f, 0.f, 0.f, 0.1f, 0)) != DOGM_OK) return st;
    DOGM_CUDA(cudaStreamSynchronize(c.stream));
    DOGM_CUDA(cudaEventRecord(c.ev[0], c.stream));
    for (int i = 0; i < reps; ++i)
        if ((st = dogm_update(h, nullptr, 0.f, 0.f, 0.f, 0.1f, 0)) != DOGM_OK) return st;
    DOGM_CUDA(cudaEventRecord(c.ev[kStages], c.stream));
    DOGM_CUDA(cudaEventSynchronize(c.ev[kStages]));
    float t = 0.f;
    DOGM_CUDA(cudaEventElapsedTime(&t, c.ev[0], c.ev[kStages]));
    *ms = t / (float)reps;
    return dogm_synchronize(h);
}

static std::string tune_key(const dogm_handle* h) {
    cudaDeviceProp prop;
    std::string name = cudaGetDeviceProperties(&prop, h->device) == cudaSuccess ? prop.name : "unknown";
    for (char& ch : name)
        if (ch == '|' || ch == '\n') ch = '_';
    return "dogm-tune v3|" + name + "|gs=" + std::to_string(h->gs) + "|N=" + std::to_string(h->N) +
           "|B=" + std::to_string(h->B);
}

dogm_status dogm_get_tune(dogm_handle* h, dogm_tune* out) {
    if (!h || !out) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    for (int i = 0; i < kStages; ++i) out->blocks_per_sm[i] = h->ctx.mult[i];
    out->resample_tile_bits = h->ctx.res_bits == kResBitsDefault ? 0 : h->ctx.res_bits;
    return DOGM_OK;
}

dogm_status dogm_set_tune(dogm_handle* h, const dogm_tune* t) {
    if (!h || !t) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    for (int i = 0; i < 8; ++i)
        if (t->blocks_per_sm[i] < 0 || t->blocks_per_sm[i] > 32 || (i >= kStages && t->blocks_per_sm[i] != 0))
            return fail(DOGM_ERR_INVALID_ARGUMENT, "blocks_per_sm must be in [0, 32] for the 6 stages and 0 after them");
    if (t->resample_tile_bits != 0 && (t->resample_tile_bits < kResBitsMin || t->resample_tile_bits > kResBitsMax))
        return fail(DOGM_ERR_INVALID_ARGUMENT, "resample_tile_bits must be 0 or in [9, 11] (tiles of 512 .. 2048)");
    DeviceGuard dg(h->device);
    dogm_status st = dogm_synchronize(h);  // no frame of the old shape in flight
    if (st != DOGM_OK) return st;
    for (int i = 0; i < kStages; ++i) h->ctx.mult[i] = t->blocks_per_sm[i];
    h->ctx.res_bits = t->resample_tile_bits ? t->resample_tile_bits : kResBitsDefault;
    h->ctx.drop_graphs();
    return DOGM_OK;
}

dogm_status dogm_autotune(dogm_handle* h, const dogm_measurement_cell* meas, int device, int reps,
                          const char* cache_path, dogm_tune* out) {
    if (!h || !meas || !out) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (reps <= 0) reps = 10;
    reps = std::min(reps, 1000);
    DeviceGuard dg(h->device);
    const std::string key = tune_key(h);
    if (cache_path) {
        if (FILE* f = std::fopen(cache_path, "r")) {
            char line[1024];
            dogm_tune t{};
            bool found = false;
            while (std::fgets(line, sizeof(line), f)) {
                const std::string ln(line);
                const size_t sep = ln.find(" : ");
                if (sep == std::string::npos || ln.compare(0, sep, key) != 0) continue;
                int* m = t.blocks_per_sm;
                found = std::sscanf(ln.c_str() + sep + 3, "%d %d %d %d %d %d %d %d %d %f %f", &m[0], &m[1], &m[2],
                                    &m[3], &m[4], &m[5], &m[6], &m[7], &t.resample_tile_bits, &t.ms_tuned,
                                    &t.ms_default) == 11;
            }
            std::fclose(f);
            if (found) {
                dogm_status st = dogm_set_tune(h, &t);
                if (st == DOGM_OK) *out = t;
                return st;
            }
        }
    }
    // a scratch handle with the same parameters, the measurement grid resident in it
    dogm_options opt = h->opt;
    opt.sync_each_update = 0;
    dogm_handle* s = nullptr;
    dogm_status st = dogm_create(&h->params, &opt, &s);
    if (st != DOGM_OK) return st;
    struct Drop {
        dogm_handle* s;
        ~Drop() { dogm_destroy(s); }
    } drop{s};
    const size_t mbytes = sizeof(dogm_measurement_cell) * (size_t)s->C;
    DOGM_CUDA(cudaMemcpy(s->desc.meas_own, meas, mbytes, device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
    for (int i = 0; i < 3; ++i)
        if ((st = dogm_update(s, nullptr, 0.f, 0.f, 0.f, 0.1f, 0)) != DOGM_OK) return st;
    // The scratch state keeps evolving while it is timed, so candidates are timed in
    // interleaved rounds (each round times every candidate once) and compared on their sums;
    // a choice other than the built-in one must win by 2 %.
    constexpr int kRounds = 3;
    auto time_bits = [&](int bits, float* ms) {
        s->ctx.res_bits = bits;
        s->ctx.drop_graphs();
        return time_updates(s, reps, ms);
    };

    // 1: the resampling tile (512, 1024 or 2048 joint particles; a template instance each),
    // whole-update time
    float bits_ms[kResBitsMax + 1] = {};
    for (int round = 0; round < kRounds; ++round)
        for (int bits = kResBitsMin; bits <= kResBitsMax; ++bits) {
            float ms = 0.f;
            if ((st = time_bits(bits, &ms)) != DOGM_OK) return st;
            bits_ms[bits] += ms;
        }
    int best_bits = kResBitsDefault;
    for (int bits = kResBitsMin; bits <= kResBitsMax; ++bits)
        if (bits_ms[bits] < 0.98f * bits_ms[best_bits]) best_bits = bits;
    s->ctx.res_bits = best_bits;
    s->ctx.drop_graphs();

    // 2: each stage's width, timed by the per-stage events (plain launches), in interleaved
    // rounds over the candidates
    static const int kCand[] = {0, 1, 2, 3, 4, 6, 8};  // 0: the kernel's built-in width
    constexpr int kNumCand = (int)(sizeof(kCand) / sizeof(kCand[0]));
    int best_mult[kStages] = {};
    s->ctx.profile = true;
    for (int stage = 0; stage < kStages; ++stage) {
        float acc[kNumCand] = {};
        for (int round = 0; round < kRounds; ++round)
            for (int ci = 0; ci < kNumCand; ++ci) {
                s->ctx.mult[stage] = kCand[ci];
                for (int r = 0; r < reps; ++r) {
                    if ((st = dogm_update(s, nullptr, 0.f, 0.f, 0.f, 0.1f, 0)) != DOGM_OK) return st;
                    if ((st = dogm_synchronize(s)) != DOGM_OK) return st;
                    float ms[kStages];
                    dogm_stage_times(s, ms, kStages);
                    acc[ci] += ms[stage];
                }
            }
        int bc = 0;
        for (int ci = 1; ci < kNumCand; ++ci)
            if (acc[ci] < 0.98f * acc[bc]) bc = ci;
        s->ctx.mult[stage] = kCand[bc];
        best_mult[stage] = kCand[bc];
    }
    s->ctx.profile = false;

    // 3: the tuned shape against the built-in one, again interleaved
    float sum_def = 0.f, sum_tuned = 0.f;
    int saved_mult[kStages];
    for (int i = 0; i < kStages; ++i) saved_mult[i] = s->ctx.mult[i];
    for (int round = 0; round < kRounds; ++round) {
        float ms = 0.f;
        for (int i = 0; i < kStages; ++i) s->ctx.mult[i] = 0;
        if ((st = time_bits(kResBitsDefault, &ms)) != DOGM_OK) return st;
        sum_def += ms;
        for (int i = 0; i < kStages; ++i) s->ctx.mult[i] = saved_mult[i];
        if ((st = time_bits(best_bits, &ms)) != DOGM_OK) return st;
        sum_tuned += ms;
    }
    const float ms_tuned = sum_tuned / (float)kRounds, ms_def = sum_def / (float)kRounds;

    dogm_tune t{};
    if (sum_tuned < 0.98f * sum_def) {
        for (int i = 0; i < kStages; ++i) t.blocks_per_sm[i] = best_mult[i];
        t.resample_tile_bits = best_bits == kResBitsDefault ? 0 : best_bits;
        t.ms_tuned = ms_tuned;
    } else {
        t.ms_tuned = ms_def;  // nothing beat the defaults
    }
    t.ms_default = ms_def;
    if ((st = dogm_set_tune(h, &t)) != DOGM_OK) return st;
    if (cache_path) {
        if (FILE* f = std::fopen(cache_path, "a")) {
            const int* m = t.blocks_per_sm;
            std::fprintf(f, "%s : %d %d %d %d %d %d %d %d %d %.5f %.5f\n", key.c_str(), m[0], m[1], m[2], m[3], m[4],
                         m[5], m[6], m[7], t.resample_tile_bits, t.ms_tuned, t.ms_default);
            std::fclose(f);
        }
    }
    *out = t;
    return DOGM_OK;
}

// ---- utilities ---------------------------------------------------------------------------

dogm_status dogm_lower_bound_f32(const float* accum, int n_accum, const float* q, int n_q, int* out, int clamp_last,
                                 void* stream) {
    if (!accum || !q || !out || n_accum <= 0 || n_q < 0) return fail(DOGM_ERR_INVALID_ARGUMENT, "bad argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DOGM_CUDA(launch_lower_bound(accum, n_accum, q, n_q, out, clamp_last, s));
    DOGM_CUDA(cudaStreamSynchronize(s));
    return DOGM_OK;
}

dogm_status dogm_host_alloc(void** ptr, size_t bytes) {
    if (!ptr) return fail(DOGM_ERR_INVALID_ARGUMENT, "ptr is NULL");
    DOGM_CUDA(cudaMallocHost(ptr, bytes));
    return DOGM_OK;
}
dogm_status dogm_host_free(void* ptr) {
    DOGM_CUDA(cudaFreeHost(ptr));
    return DOGM_OK;
}
dogm_status dogm_device_alloc(void** ptr, size_t bytes) {
    if (!ptr) return fail(DOGM_ERR_INVALID_ARGUMENT, "ptr is NULL");
    DOGM_CUDA(cudaMalloc(ptr, bytes));
    return DOGM_OK;
}
dogm_status dogm_device_free(void* ptr) {
    DOGM_CUDA(cudaFree(ptr));
    return DOGM_OK;
}
dogm_status dogm_memcpy(void* dst, const void* src, size_t bytes, int kind) {
    DOGM_CUDA(cudaMemcpy(dst, src, bytes, static_cast<cudaMemcpyKind>(kind)));
    return DOGM_OK;
}

}  // extern "C"

// ---- batch slots of the serving loop ---------------------------------------------------------

namespace dogm_gb300 {

struct BatchSlot {
    Ctx ctx;
    std::vector<dogm_handle*> hs;  // handles of the unfinished launch
    int mirror = -1;               // mirror whose done event marks that launch
};

dogm_status slot_create(int device, BatchSlot** out) {
    *out = nullptr;
    DeviceGuard dg(device);
    BatchSlot* s = new BatchSlot();
    dogm_status st = ctx_init(s->ctx, device);
    if (st != DOGM_OK) { delete s; return st; }
    if (prepare_kernels() != cudaSuccess || prepare_cells() != cudaSuccess || prepare_sort() != cudaSuccess) {
        delete s;
        return fail(DOGM_ERR_CUDA, "kernel attribute setup failed");
    }
    *out = s;
    return DOGM_OK;
}

void slot_destroy(BatchSlot* s) {
    if (!s) return;
    DeviceGuard dg(s->ctx.device);
    cudaStreamSynchronize(s->ctx.stream);
    delete s;
}

// The same per-handle steps as dogm_update_batch (measurement copy, pose bookkeeping, frame
// descriptors, one launch per stage for all handles), without the waits: the caller
// guarantees that no handle has unfinished work elsewhere.
dogm_status slot_launch(BatchSlot* s, const SlotFrame* fr, int n) {
    if (!s || !fr || n <= 0 || n > kMaxBatch) return fail(DOGM_ERR_INVALID_ARGUMENT, "bad slot launch");
    if (s->mirror >= 0) return fail(DOGM_ERR_NOT_READY, "slot launch before the previous one was finished");
    Ctx& c = s->ctx;
    DeviceGuard dg(c.device);
    dogm_status st = acquire_mirror(c);
    if (st != DOGM_OK) return st;
    s->hs.assign(n, nullptr);
    std::vector<int> init_mask(n, 0);
    std::vector<HostCopy> copies;
    bool any_init = false, any_clear = false;
    for (int i = 0; i < n; ++i) {
        dogm_handle* h = fr[i].h;
        s->hs[i] = h;
        const dogm_measurement_cell* src;
        int copy;
        st = prepare_measurement(h, fr[i].meas, fr[i].device, c.stream, &src, &copy);
        if (st != DOGM_OK) return st;
        st = alternate_cells(h, c.stream);
        if (st != DOGM_OK) return st;
        init_mask[i] = h->first_measurement_received ? 0 : 1;
        any_init |= init_mask[i] != 0;
        any_clear |= h->need_clear;
        int shifted, xm, ym;
        pose_update(h, fr[i].x, fr[i].y, fr[i].yaw, &shifted, &xm, &ym);
        fill_frame(h, fr[i].dt, shifted, xm, ym, src, copy);
        if (fr[i].cells_out)
            copies.push_back({fr[i].cells_out, h->desc.cells, sizeof(dogm_grid_cell) * (size_t)h->C});
    }
    build_batch(c, s->hs.data(), n, init_mask);
    const int mirror = c.cur;
    int launches = 0;
    st = run_frame(c, n, any_init, any_clear, &launches, &copies);
    if (st != DOGM_OK) {
        for (int i = 0; i < n; ++i) s->hs[i]->need_clear = true;
        s->hs.clear();
        return st;
    }
    for (int i = 0; i < n; ++i) {
        advance(s->hs[i]);
        s->hs[i]->last_launches = launches;
    }
    s->mirror = mirror;
    return DOGM_OK;
}

// Captures and instantiates the steady-state graph of every batch-size bucket up to max_n for
// both mirrors, without launching it: a graph records the kernel launches on the mirror's
// device batch, which depend on none of the handles of a frame.
dogm_status slot_prewarm(BatchSlot* s, int max_n) {
    if (!s) return fail(DOGM_ERR_INVALID_ARGUMENT, "slot is NULL");
    Ctx& c = s->ctx;
    DeviceGuard dg(c.device);
    const int cur = c.cur;
    for (int m = 0; m < 4; ++m) {  // two mirrors, each with both job forms of the cell pass
        for (int nb = 1; nb <= graph_bucket(std::max(1, max_n)); nb <<= 1) {
            c.scatter_ctiles = 2048;  // streams of the serving loop have at most 2048 cell tiles
            c.fine = (m & 2) != 0;
            const int key = graph_key(nb, m & 1, c.scatter_ctiles, c.res_bits, c.fine);
            if (c.graphs.count(key)) continue;
            set_mirror(c, m & 1);
            cudaGraph_t graph;
            DOGM_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = frame_kernels(c, false, false);
            cudaError_t e2 = cudaStreamEndCapture(c.stream, &graph);
            set_mirror(c, cur);
            if (e != cudaSuccess || e2 != cudaSuccess)
                return fail(DOGM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
            cudaGraphExec_t exec;
            e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return fail(DOGM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
            c.graphs.emplace(key, exec);
        }
    }
    set_mirror(c, cur);
    return DOGM_OK;
}

bool slot_done(BatchSlot* s) {
    if (!s || s->mirror < 0) return true;
    DeviceGuard dg(s->ctx.device);
    return cudaEventQuery(s->ctx.done[s->mirror]) != cudaErrorNotReady;
}

dogm_status slot_finish(BatchSlot* s) {
    if (!s || s->mirror < 0) return DOGM_OK;
    DeviceGuard dg(s->ctx.device);
    s->mirror = -1;
    dogm_status st = finish_frame(s->ctx, s->hs.data(), (int)s->hs.size());
    s->hs.clear();
    return st;
}

cudaStream_t handle_stream(dogm_handle* h) { return h->ctx.stream; }
const dogm_grid_cell* handle_cells(dogm_handle* h) { return h->desc.cells; }
int handle_cell_count(const dogm_handle* h) { return h->C; }
void set_last_error(const char* msg) { g_last_error = msg; }

}  // namespace dogm_gb300
