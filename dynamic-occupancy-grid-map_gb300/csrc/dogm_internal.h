// Internal device-side layout shared by the kernels and the host runtime.
//
// One grid (one dogm_handle) is described by a GridDesc.  A launch processes a Batch of
// GridDescs: every stage kernel is a persistent kernel whose blocks pull tiles from the
// concatenated tile space of all grids in the batch, so the same launch sequence (and the
// same CUDA graph) serves one grid or many uneven grids.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "dogm_gb300.h"

namespace dogm_gb300 {

// ---- tile shapes (elements per tile; 256-thread blocks everywhere) ---------------------
constexpr int kThreads = 256;
constexpr int kPredictTile = 4096;   // particles per predict tile (16 per thread)
constexpr int kSortIpt = 16;         // keys per thread in the bucket scatter
constexpr int kSortTile = kThreads * kSortIpt;
constexpr int kSegIpt = 4;           // sorted particles per thread in a chunk of the cell pass
constexpr int kSegTile = kThreads * kSegIpt;
constexpr int kCellIpt = 4;          // cells per thread in the cell passes
constexpr int kCellTile = kThreads * kCellIpt;
// resampling tile: 2^res_bits joint particles (256 threads, 2, 4 or 8 each); a launch-shape
// choice of the autotuner, the same for every grid of a launch
constexpr int kResBitsMin = 9, kResBitsDefault = 10, kResBitsMax = 11;

static_assert(kPredictTile == kSortTile, "predict writes the bucket counts of the scatter tiles");

constexpr int kMaxKeyBits = 22;      // grid_size <= 2048 -> cells < 2^22
constexpr int kCellTileBits = 10;
constexpr int kMaxCellTiles = (1 << kMaxKeyBits) >> kCellTileBits;  // buckets of the particle sort
static_assert(kCellTile == (1 << kCellTileBits), "cell tiles are indexed by cell >> kCellTileBits");
// Buckets of the particle sort: 2^bucket_bits cells.  A grid of at most kFineMaxTiles cell tiles
// with more than kFineMinPerTile particles per tile on average sorts by finer buckets (down to
// 2^kMinBucketBits cells, at most kFineMaxBuckets of them), so that the cell pass can split a
// cell tile whose particles are many into jobs of whole buckets of about kJobTarget particles;
// other grids sort by cell tile (on a sparser or larger grid the finer rows cost more than the
// split gains).  The choice depends on the grid's parameters alone, so a grid gives the same bits
// alone and in any batch.
constexpr int kMinBucketBits = 6;
constexpr int kFineMaxTiles = 128;
constexpr int kFineMinPerTile = 2048;
constexpr int kFineMaxBuckets = 1024;
constexpr int kJobTarget = 4096;     // particles of a cell-pass job (one chunk of its counting sort)
static_assert(kMinBucketBits >= 6, "a job's cell range covers whole warps of the per-cell part");
static_assert((1 << kResBitsMin) % 32 == 0, "32 aligned sorted positions lie in one resample tile");
constexpr int kMaxParticles = (1 << 24) - 1;  // keys, counts and slot indices stay below 2^24

// Particle key word: bits 0..29 cell index, bit 30 "out of grid" (weight 0), bit 31 associated.
constexpr uint32_t kCellMask = 0x3fffffffu;
constexpr uint32_t kOutBit = 1u << 30;
constexpr uint32_t kAssocBit = 1u << 31;

// Philox counter word 2: which draw family.
enum DrawStage : uint32_t { kDrawInit = 1, kDrawPredict = 2, kDrawBirth = 3, kDrawResample = 4 };

// Stages of the update; each has a tile count per grid and a work counter for dynamic claims.
// The particle sort is one stable bucket scatter by cell tile (kStScan: bucket offsets, kStSort:
// the scatter) followed by a stable counting sort of each bucket inside the cell pass.
enum Stage : int {
    kStPredict = 0, kStScan, kStSort, kStCell, kStBirth, kStResample, kStInitScan, kStInitExpand, kNumStages
};


// Per-grid state that lives on the device across frames.
struct FrameState {
    // written by one update, read by the next
    float w_res;          // common particle weight after the last resampling (or 1/N)
    uint32_t status;      // sticky error bits (kStatus*)
    // per-frame accumulators (zeroed by predict; all of them by the frame-begin kernel)
    unsigned long long qb_total;   // sum of quantised newborn masses (exact)
    unsigned long long joint_total;// sum of quantised joint weights (exact)
    unsigned long long qo_total;   // first frame: sum of quantised measured occupancy
    int n_birth;                   // newborns created this frame (B or 0)
    int pad;
};
// Parts of the cell pass (GridDesc::stage_mask).  The update runs them all in one pass; the
// stage calls of the reference's public stage methods run one each and merge their fields into
// the cell records (dogm/src/dogm.cu:262-384: particleAssignment, gridCellOccupancyUpdate,
// updatePersistentParticles, statisticalMoments).
constexpr uint32_t kPartRanges = 1u;    // start_idx / end_idx
constexpr uint32_t kPartMasses = 2u;    // masses, free mass, newborn mass, measurement copy
constexpr uint32_t kPartReweight = 4u;  // mu_A / mu_UA, reweighted weights, joint weight sums
constexpr uint32_t kPartMoments = 8u;   // velocity mean / variance / covariance
constexpr uint32_t kPartAll = 15u;

constexpr uint32_t kStatusTimeout = 1u;  // a bounded wait gave up
constexpr uint32_t kStatusBounds = 2u;   // an index check refused a write

struct GridDesc {
    // sizes
    int N, B, C, gs;
    int q_shift;            // fixed point: weight w -> round(w * 2^q_shift)
    int ctiles;             // buckets of the particle sort (2^bucket_bits cells each)
    int bucket_stride;      // words per row of the per-tile bucket counts (ctiles rounded up to 4)
    int bucket_bits;        // log2 of the cells per bucket (kCellTileBits, or finer for small grids)
    int res_bits;           // resampling tile = 2^res_bits joint particles (set per launch)
    unsigned long long gs_div;  // floor(2^42 / gs) + 1: k / gs == (k * gs_div) >> 42 for k < 2^22
    // filter parameters
    float p_S, sigma_pos, sigma_vel, p_B, sigma_birth, init_max_vel;
    // per-frame parameters
    float dt, alpha;        // alpha = freespace_discount^dt (host powf, as dogm.cu:291)
    int shift_x, shift_y;   // cells to shift (x_move, y_move of dogm.cu:177-178)
    int shifted;            // 1 when the pose moved by more than one cell this frame
    int copy_meas;          // 1: meas_src is a caller buffer to copy into meas_own
    uint32_t stage_mask;    // parts of the cell pass to run (kPart*)
    int weights_predicted;  // 1: w_res already holds p_S * w (stage calls: particlePrediction ran)
    uint32_t frame;         // iteration number (Philox counter word 1)
    uint32_t stream_id;     // Philox counter word 3
    uint32_t seed_lo, seed_hi;
    // particles (persistent: P, bucketed by cell tile: T, sorted: S, newborn: Bp)
    float4* P_state; uint32_t* P_key;
    float4* T_state; uint32_t* T_key;  // stable bucket scatter of P by cell tile
    int* T_idx;             // debug: index in P of each bucketed particle (NULL: off)
    float4* S_state; uint32_t* S_key;
    float4* B_state; uint32_t* B_key; float* B_w;  // newborns: key words always, state/weight for debug export
    // cells
    dogm_grid_cell* cells;
    const dogm_measurement_cell* meas_src;
    dogm_measurement_cell* meas_own;
    float* free_old; float* free_new;   // free mass of the previous / this frame (ping-pong)
    float2* rho_b;          // per cell {newborn mass, p_A} of this frame (the newborn kernel's input)
    float* w_cell;          // per cell weight of an in-grid persistent particle after reweighting
    // scratch
    uint32_t* hsort;        // sort_tiles x bucket_stride: per-tile bucket counts, then offsets
    uint32_t* ctile_cnt;    // per bucket: particles whose cell lies in it (counted by predict)
    uint4* ctile_job;       // jobs of the cell pass in claim order (many particles first): {cell
                            // tile, first sorted position, end, first cell | end cell << 16 within
                            // the tile}; unused entries at the end: {0xffffffff, 0, 0, 0}
    unsigned long long* cell_sum;  // per bucket: quantised newborn mass of the job that starts at
                                   // it (0 inside a job); then per cell tile (offset
                                   // tiles[kStCell]): first-frame occupied mass
    unsigned long long* res_sum;   // per resample tile: quantised joint weight (exact atomics)
    FrameState* fs;
    unsigned int* status_out;  // the batch-level status word
    // replay inputs (NULL: Philox) and debug outputs (NULL: off)
    const float2* rp_init; const float4* rp_predict; const float2* rp_birth; const unsigned long long* rp_resample;
    int* dbg_perm; int* dbg_src;
    // tiles per stage (sort_tiles sizes the per-tile digit counts)
    int tiles[kNumStages];
    int sort_tiles;
    int pad1;
};

// Row of cell k: exact for k < 2^22 and gs <= 2048 (the error k * e / 2^42 < 2^-20 stays below
// the 1 / gs margin of floor(k / gs)).
__host__ __device__ __forceinline__ int cell_row(const GridDesc& g, int k) {
    return (int)(((unsigned long long)k * g.gs_div) >> 42);
}

constexpr int kMaxBatch = 256;

// Device copy of one batch.  The host uploads the header, prefix rows 0..n and g[0..n)
// before every frame; the upload also zeroes the tile counters.
struct Batch {
    int n_grids;
    unsigned int status;                     // OR of every grid's error bits this frame
    unsigned int counters[kNumStages];       // dynamic tile counters
    unsigned int* status_host;               // this frame's status word in mapped host memory
    int prefix[kMaxBatch + 1][kNumStages];   // prefix[i][s]: tiles of stage s in grids < i
    GridDesc g[kMaxBatch];
};

// One grid's frame passed to predict as a kernel parameter instead of through an upload of the
// device batch: predict reads it from its parameters and writes the device batch for the later
// kernels (valid = 0: the kernel reads the device batch as uploaded).
struct FrameParam {
    GridDesc g;
    int tiles[kNumStages];
    unsigned int* status_host;
    int valid;
};

// ---- kernel launchers (defined in the .cu files) ---------------------------------------
struct LaunchCfg {
    int num_sms;
    cudaStream_t stream;
    int mult = 0;      // blocks per SM of this launch (0: the kernel's built-in default)
    bool pdl = false;  // programmatic dependent launch after the previous kernel on the stream
};

// Launches a frame kernel.  With cfg.pdl the launch is programmatically serialised after the
// previous kernel on the stream (its launch is processed while that kernel completes); every
// frame kernel begins with grid_dependency_begin(), which waits for the previous kernel to
// complete and flush before any of its own memory accesses.
template <typename... KArgs, typename... Args>
cudaError_t launch_kernel(const LaunchCfg& cfg, void (*kernel)(KArgs...), int grid, int block, size_t smem,
                          Args... args) {
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)grid);
    lc.blockDim = dim3((unsigned)block);
    lc.dynamicSmemBytes = smem;
    lc.stream = cfg.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = attr;
    lc.numAttrs = cfg.pdl ? 1 : 0;
    return cudaLaunchKernelEx(&lc, kernel, args...);
}
// Blocks of a persistent launch: num_sms x the tuned multiplier, or x the default.
inline int launch_blocks(const LaunchCfg& cfg, int default_mult) {
    return cfg.num_sms * (cfg.mult > 0 ? cfg.mult : default_mult);
}

cudaError_t prepare_kernels();  // per device, before the first launch
cudaError_t prepare_cells();
cudaError_t prepare_sort();
cudaError_t launch_frame_begin(const Batch* d_batch, int n_grids, const LaunchCfg& cfg);
cudaError_t launch_init_particles(const Batch* d_batch, const LaunchCfg& cfg);
// stage_mode 0: the update's predict (ego shift, motion, bucket counts, per-frame sums zeroed);
// 1: the particlePrediction stage call (motion only); 2: the particleAssignment stage call
// (bucket counts of the resident keys and per-frame sums zeroed, no motion)
cudaError_t launch_predict(const Batch* d_batch, int stage_mode, const LaunchCfg& cfg, const FrameParam* fp = nullptr,
                           bool fine = true);
// bucket offsets (column scan of the per-tile bucket counts) and the stable bucket scatter;
// max_ctiles: the largest bucket count of the batch's grids (sizes the scatter's shared memory)
cudaError_t launch_sort_scan(const Batch* d_batch, const LaunchCfg& cfg);
cudaError_t launch_sort_scatter(const Batch* d_batch, int max_ctiles, const LaunchCfg& cfg, bool fine = true);
// staged: a stage call, running the parts of GridDesc::stage_mask
cudaError_t launch_cells(const Batch* d_batch, const LaunchCfg& cfg, bool staged = false, bool fine = true);
cudaError_t launch_newborn(const Batch* d_batch, const LaunchCfg& cfg, bool fine = true);
cudaError_t launch_resample(const Batch* d_batch, int res_bits, const LaunchCfg& cfg);
cudaError_t launch_shift_stage(const GridDesc& g, int x_move, int y_move, const LaunchCfg& cfg);
// Allocation-free shift stage: the copy of the previous cell records goes to a fixed device
// array of kShiftScratchBytes (16 MiB = 262,144 cells, e.g. a 512 x 512 grid).
constexpr size_t kShiftScratchBytes = size_t(16) << 20;
cudaError_t shift_scratch_setup();  // once per device, with that device current
cudaError_t launch_shift_stage_noalloc(const GridDesc& g, int x_move, int y_move, const LaunchCfg& cfg);
cudaError_t launch_draws(const GridDesc& g, int iteration, float2* init_u, float4* predict_z, float2* birth_z,
                         unsigned long long* resample_r, const LaunchCfg& cfg);
cudaError_t launch_lower_bound(const float* accum, int n_accum, const float* q, int n_q, int* out, int clamp_last,
                               cudaStream_t s);

// Kernel launches per steady-state update (for the launch-count claim): predict, bucket scan,
// bucket scatter, cells, newborn, resample.  A grid's first frame, and a frame after a failed
// one, adds the frame-begin reset.
constexpr int kLaunchesPerFrame = 6;
constexpr int kLaunchesInit = 2;

// ---- batch slots (runtime.cu): the launch contexts of the serving loop (serving.cu) ------
// A slot owns a stream, a device batch and its pinned mirrors.  slot_launch queues one
// batched frame of n distinct handles and returns without waiting; slot_done tells whether
// that frame finished; slot_finish waits for it and returns its status.  A handle must not
// be in two unfinished launches at once (the serving loop keeps one frame per stream in
// flight); a slot takes its next launch only after slot_finish.
struct BatchSlot;
struct SlotFrame {
    dogm_handle* h;
    const dogm_measurement_cell* meas;  // NULL keeps the resident grid
    int device;                         // meas is a device pointer
    float x, y, yaw, dt;
    dogm_grid_cell* cells_out;          // host buffer for the grid after the update, or NULL
};
dogm_status slot_create(int device, BatchSlot** out);
void slot_destroy(BatchSlot* s);
dogm_status slot_launch(BatchSlot* s, const SlotFrame* frames, int n);
dogm_status slot_prewarm(BatchSlot* s, int max_n);  // build the graphs of batches up to max_n
bool slot_done(BatchSlot* s);
dogm_status slot_finish(BatchSlot* s);
// Per-handle helpers of the per-stream serving mode.
cudaStream_t handle_stream(dogm_handle* h);
const dogm_grid_cell* handle_cells(dogm_handle* h);
int handle_cell_count(const dogm_handle* h);
void set_last_error(const char* msg);

}  // namespace dogm_gb300
