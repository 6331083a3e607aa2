/*
 * dogm_gb300.h — C ABI of the GB300-native dynamic occupancy grid map (DOGM) update.
 *
 * The reference exposes no C ABI: its boundary is the C++ class dogm::DOGM
 * (dogm/include/dogm/dogm.h:20-199), linked statically.  Every entry point below
 * replaces one member of that class (cited per function) with a plain-pointer C call
 * that a cgo / JNI / ctypes / C++ caller can bind.  The header-only C++ class in
 * include/dogm/dogm.h restores the reference's exact C++ signatures on top of it.
 *
 * Conventions
 *  - Every call returns a dogm_status; DOGM_OK == 0.  The reference only prints CUDA
 *    errors and continues (dogm/include/dogm/cuda_utils.h:13-24); here the caller decides.
 *  - A handle owns all device state of one grid (particles, cells, measurement copy) on
 *    the device that was current when it was created (dogm/src/dogm.cu:39-43).
 *  - Host buffers passed in are only read/written during the call.  Device buffers
 *    passed in (device != 0) must be device pointers of the handle's device.
 *  - Handles are not thread-safe; distinct handles may be used from distinct threads.
 */
#ifndef DOGM_GB300_H
#define DOGM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DOGM_ABI_VERSION 1

typedef enum dogm_status {
    DOGM_OK = 0,
    DOGM_ERR_INVALID_ARGUMENT = 1, /* bad pointer, size or parameter                        */
    DOGM_ERR_OUT_OF_MEMORY = 2,    /* device or pinned-host allocation failed               */
    DOGM_ERR_CUDA = 3,             /* a CUDA runtime call failed (see dogm_last_error)     */
    DOGM_ERR_DEVICE_TIMEOUT = 4,   /* a bounded device-side wait gave up; state is suspect */
    DOGM_ERR_NOT_READY = 5,        /* call needs a state the handle has not reached yet    */
    DOGM_ERR_UNSUPPORTED = 6,      /* size or mode outside what this build supports        */
    DOGM_ERR_BUDGET = 7            /* serving: admission refused by the HBM budget         */
} dogm_status;

/* Filter parameters.  Field order and meaning are those of dogm::DOGM::Params
 * (dogm/include/dogm/dogm.h:26-60); the struct is layout-compatible with it. */
typedef struct dogm_params {
    float size;                          /* grid side [m]                                  */
    float resolution;                    /* cell side [m/cell]                             */
    int particle_count;                  /* persistent particles N                         */
    int new_born_particle_count;         /* newborn particles B                            */
    float persistence_prob;              /* p_S                                            */
    float stddev_process_noise_position; /* sigma of the position process noise [m]        */
    float stddev_process_noise_velocity; /* sigma of the velocity process noise [m/s]      */
    float birth_prob;                    /* p_B                                            */
    float stddev_velocity;               /* sigma of newborn velocities [m/s]              */
    float init_max_velocity;             /* first-frame velocities ~ U(-v, v) [m/s]        */
    float freespace_discount;            /* free mass decays by freespace_discount^dt      */
} dogm_params;

/* One grid cell: 16 x 4 B, layout of dogm::GridCell (dogm/include/dogm/dogm_types.h:13-33). */
typedef struct dogm_grid_cell {
    int start_idx, end_idx;
    float new_born_occ_mass, pers_occ_mass, free_mass, occ_mass, pred_occ_mass;
    float mu_A, mu_UA, w_A, w_UA;
    float mean_x_vel, mean_y_vel, var_x_vel, var_y_vel, covar_xy_vel;
} dogm_grid_cell;

/* One measurement cell: layout of dogm::MeasurementCell (dogm/include/dogm/dogm_types.h:35-41). */
typedef struct dogm_measurement_cell {
    float free_mass, occ_mass, likelihood, p_A;
} dogm_measurement_cell;

/* Resampling scheme (the reference draws N sorted uniforms: dogm/src/dogm.cu:386-423). */
typedef enum dogm_resample_mode {
    DOGM_RESAMPLE_SYSTEMATIC = 0 /* one uniform offset, comb of N teeth over the exact scan */
} dogm_resample_mode;

/* Options that have no counterpart in dogm::DOGM::Params (kept apart so Params stays ABI). */
typedef struct dogm_options {
    uint64_t seed;      /* Philox key; the reference seeds curand with 123456 (dogm/src/dogm.cu:101) */
    uint32_t stream_id; /* Philox counter word: distinct sensor streams draw independent noise       */
    int resample_mode;  /* dogm_resample_mode                                                       */
    int sync_each_update; /* 1 (default): dogm_update returns after the device is done, like
                             the reference's cudaDeviceSynchronize (dogm/src/dogm.cu:130)          */
} dogm_options;

typedef struct dogm_handle dogm_handle;

/* ---- lifetime ------------------------------------------------------------------------ */

/* Fills *opt with the defaults (seed 123456, stream 0, systematic, synchronous). */
dogm_status dogm_default_options(dogm_options* opt);

/* Replaces DOGM::DOGM(const Params&) (dogm/src/dogm.cu:33-71): allocates all device state
 * on the current device.  Particles are initialised on the first update, as in the
 * reference (dogm/src/dogm.cu:210-214).  opt may be NULL (defaults). */
dogm_status dogm_create(const dogm_params* params, const dogm_options* opt, dogm_handle** out);

/* Replaces DOGM::~DOGM (dogm/src/dogm.cu:73-93). NULL is a no-op. */
dogm_status dogm_destroy(dogm_handle* h);

/* ---- the update (hot path) ----------------------------------------------------------- */

/* Replaces DOGM::updateGrid (dogm/src/dogm.cu:115-131): copy in the measurement grid
 * (grid_size^2 cells, row-major), ego-shift, predict, sort, mass update, persistent
 * reweighting, newborn initialisation, moments and resampling.  device != 0 means meas
 * is a device pointer, else a host pointer (pinned host memory copies fastest).
 * meas == NULL keeps the resident measurement grid (the reference's failed copy at
 * dogm/src/dogm.cu:208 leaves it unchanged as well). */
dogm_status dogm_update(dogm_handle* h, const dogm_measurement_cell* meas, float new_x, float new_y,
                        float new_yaw, float dt, int device);

/* Batched form: n independent handles (uneven sizes allowed, all on one device) updated
 * by one launch per stage, captured in a CUDA graph.  Arrays have n entries.  The result
 * of each handle is bit-identical to updating it alone with dogm_update. */
dogm_status dogm_update_batch(dogm_handle* const* hs, int n, const dogm_measurement_cell* const* meas,
                              const float* new_x, const float* new_y, const float* new_yaw, const float* dt,
                              int device);

/* Waits for all work queued on the handle's stream (only needed with sync_each_update=0) and
 * for the copies queued by dogm_get_grid_cells_async. */
dogm_status dogm_synchronize(dogm_handle* h);

/* ---- readback (dogm/src/dogm.cu:133-159) ---------------------------------------------- */

/* Replaces DOGM::getGridCells: copies n == grid_size^2 cells to host memory. */
dogm_status dogm_get_grid_cells(dogm_handle* h, dogm_grid_cell* host_out, size_t n);
/* Same into a device buffer of the handle's device (no host round trip). */
dogm_status dogm_get_grid_cells_device(dogm_handle* h, dogm_grid_cell* dev_out, size_t n);
/* Queues the copy of the current grid (n == grid_size^2 cells) to host_out on a copy stream of
 * the handle and returns: the copy overlaps the next update's measurement copy and kernels.
 * From the first call on the handle keeps a second cell-record buffer (C x 64 bytes) and its
 * updates alternate between the two, each waiting for the copy last queued from the buffer it
 * writes; results are bit-identical to the synchronous path.  host_out holds the grid once
 * dogm_synchronize(h) returns; it must stay valid until then and should be pinned
 * (dogm_host_alloc) for the copy to run asynchronously. */
dogm_status dogm_get_grid_cells_async(dogm_handle* h, dogm_grid_cell* host_out, size_t n);

/* Replaces DOGM::getMeasurementCells. */
dogm_status dogm_get_measurement_cells(dogm_handle* h, dogm_measurement_cell* host_out, size_t n);

/* Replaces DOGM::getParticles (dogm/src/dogm.cu:153-159, layout dogm_types.h:51-144):
 * state is n x {x, y, vx, vy}; any output pointer may be NULL to skip that field. */
dogm_status dogm_get_particles(dogm_handle* h, float* state_xyvv, int* grid_cell_idx, float* weight,
                               unsigned char* associated, size_t n);

/* Getters of dogm.h:106-139, plus the iteration count (completed updates). */
int dogm_get_grid_size(const dogm_handle* h);
float dogm_get_resolution(const dogm_handle* h);
float dogm_get_position_x(const dogm_handle* h);
float dogm_get_position_y(const dogm_handle* h);
float dogm_get_yaw(const dogm_handle* h);
int dogm_get_iteration(const dogm_handle* h);
int dogm_get_particle_count(const dogm_handle* h);
int dogm_get_new_born_particle_count(const dogm_handle* h);

/* ---- stage-level calls (the reference's public stage methods, dogm.h:147-156) -------- */

/* Replaces DOGM::particlePrediction(dt) (dogm/src/dogm.cu:243-260) on the resident
 * particles, without the rest of the update. */
dogm_status dogm_particle_prediction(dogm_handle* h, float dt);

/* Replaces the private DOGM::updatePose (dogm/src/dogm.cu:161-203): pose bookkeeping and,
 * when the pose moved by more than one cell, the particle and grid shift. */
dogm_status dogm_update_pose(dogm_handle* h, float new_x, float new_y, float new_yaw);

/* dogm_update_pose that allocates no device memory; it has no counterpart in the reference.
 * Same arguments, results and errors as dogm_update_pose.  It is for callers that may not
 * allocate device memory while they run -- a real-time loop whose device memory is fixed at
 * start-up, or a process whose free device memory belongs to another allocator -- because
 * dogm_update_pose takes a temporary buffer for the copy of the previous cell records.  Here
 * that copy goes to a fixed 16 MiB device array built into the library, one per device, so
 * grids of at most 262,144 cells (for example 512 x 512) are accepted; a larger grid returns
 * DOGM_ERR_INVALID_ARGUMENT and leaves the handle unchanged.  Every call looks up the array's
 * address in the current context (a lookup, not an allocation), so a context created anew after
 * cudaDeviceReset is handled; the first call on a device may load the library's device code into
 * that context: make that first call before any stream capture.  Like dogm_update_pose, it
 * waits for grid copies queued by dogm_get_grid_cells_async before it moves the cells.  All calls on a
 * device share the one array, so calls whose work overlaps on the GPU (several host threads at
 * once) race on it and must be serialised by the caller. */
dogm_status dogm_update_pose_noalloc(dogm_handle* h, float new_x, float new_y, float new_yaw);

/* Replaces DOGM::initializeParticles (dogm/src/dogm.cu:217-241) from the resident
 * measurement grid (set by a previous update, or by dogm_set_measurement_cells). */
dogm_status dogm_initialize_particles(dogm_handle* h);

/* The remaining stage methods, in the order DOGM::updateGrid runs them (dogm/src/dogm.cu:119-127).
 * Each runs one part of the update on the handle's resident state and waits for it.  Called in
 * this order once per frame -- after dogm_set_measurement_cells (and dogm_initialize_particles on
 * the first frame), dogm_update_pose and dogm_particle_prediction -- they compute the same bits
 * as dogm_update with the same inputs.  The particle weights are taken as they are, i.e. as
 * dogm_particle_prediction left them (p_S times the previous weight). */

/* Replaces DOGM::particleAssignment (dogm/src/dogm.cu:262-281): the stable particle-to-cell
 * sort and the cells' start_idx / end_idx. */
dogm_status dogm_particle_assignment(dogm_handle* h);

/* Replaces DOGM::gridCellOccupancyUpdate (dogm/src/dogm.cu:283-298): predicted, free, occupied,
 * persistent and newborn masses (freespace_discount^dt), written into the cell records. */
dogm_status dogm_grid_cell_occupancy_update(dogm_handle* h, float dt);

/* Replaces DOGM::updatePersistentParticles (dogm/src/dogm.cu:300-321): mu_A, mu_UA and the
 * reweighted persistent weights. */
dogm_status dogm_update_persistent_particles(dogm_handle* h);

/* Replaces DOGM::initializeNewParticles (dogm/src/dogm.cu:323-348): newborn allocation over the
 * cells' newborn masses, w_A / w_UA of the records. */
dogm_status dogm_initialize_new_particles(dogm_handle* h);

/* Replaces DOGM::statisticalMoments (dogm/src/dogm.cu:350-384): velocity mean, variance and
 * covariance of the cell records. */
dogm_status dogm_statistical_moments(dogm_handle* h);

/* Replaces DOGM::resampling (dogm/src/dogm.cu:386-423) and the particle_array =
 * particle_array_next copy of updateGrid (dogm/src/dogm.cu:128): systematic resampling over the
 * exact joint-weight scan; the resampled set becomes the current particles and the frame ends
 * (dogm_get_iteration counts it). */
dogm_status dogm_resampling(dogm_handle* h);

/* ---- state injection and draw replay (parity tests; not on the hot path) -------------- */

/* Overwrites the resident measurement grid from host memory. */
dogm_status dogm_set_measurement_cells(dogm_handle* h, const dogm_measurement_cell* host_in, size_t n);

/* Overwrites the resident particles from host arrays (state n x 4 floats, cell indices,
 * associated flags) and sets the common particle weight. */
dogm_status dogm_set_particles(dogm_handle* h, const float* state_xyvv, const int* grid_cell_idx,
                               const unsigned char* associated, float weight, size_t n);

/* Draw replay: when set, the next updates take their random numbers from these host
 * arrays instead of Philox.  init: N x 2 uniforms in (0,1]; predict: N x 4 normals;
 * birth: B x 2 normals; resample: one 64-bit fraction (u = r / 2^64).  Each pointer may
 * be NULL (that stage keeps Philox).  The arrays are copied to the device at this call
 * and used by every following update until dogm_clear_replay. */
dogm_status dogm_set_replay(dogm_handle* h, const float* init_u, const float* predict_z, const float* birth_z,
                            const uint64_t* resample_r);
dogm_status dogm_clear_replay(dogm_handle* h);

/* Generates the Philox draws the handle would use at update number `iteration`
 * (0-based) into host arrays of the replay shapes above (NULL skips a stage). */
dogm_status dogm_generate_draws(dogm_handle* h, int iteration, float* init_u, float* predict_z, float* birth_z,
                                uint64_t* resample_r);

/* Debug exports of the last update (host arrays, n entries each; NULL skips):
 * sorted_cell[N] / sorted_state[N x 4] / sort_perm[N] are the particles after the stable
 * sort by cell; birth_* are the newborns [B]; resample_src[N] is the joint index
 * (persistent < N <= birth) each new particle was copied from; joint_total is the exact
 * fixed-point joint weight and q_shift its scale (weight = q / 2^q_shift). */
dogm_status dogm_debug_enable(dogm_handle* h, int enable);
dogm_status dogm_debug_export(dogm_handle* h, int* sorted_cell, float* sorted_state, int* sort_perm,
                              float* birth_state, int* birth_cell, unsigned char* birth_assoc, float* birth_weight,
                              int* resample_src, uint64_t* joint_total, int* q_shift, int* n_birth);

/* Debug export of the last update's resampling input (debug enabled before the update): the
 * joint weights in joint order -- the N persistent particles in sorted order with their
 * reweighted weights (the reference's weight_array, dogm.cu:393), then the newborns' weights
 * (birth_particle_array.weight, dogm.cu:394) -- as float; n >= particle_count + newborns;
 * *n_joint receives the count. */
dogm_status dogm_debug_joint_weights(dogm_handle* h, float* weights, size_t n, int* n_joint);

/* ---- utilities ------------------------------------------------------------------------ */

/* Multinomial index search of the reference (thrust::lower_bound at
 * dogm/src/kernel/resampling.cu:34-47, including the last-accumulator clamp): for each of
 * the q sorted queries, the first i with accum[i] >= query.  All pointers are device
 * pointers; runs on `stream` (a cudaStream_t, 0 = legacy default). */
dogm_status dogm_lower_bound_f32(const float* accum, int n_accum, const float* sorted_queries, int n_queries,
                                 int* out_idx, int clamp_last, void* stream);

/* Pinned host buffers for fast host<->device copies (cudaMallocHost). */
dogm_status dogm_host_alloc(void** ptr, size_t bytes);
dogm_status dogm_host_free(void* ptr);
/* Plain device buffers on the current device (tests and benches without a framework). */
dogm_status dogm_device_alloc(void** ptr, size_t bytes);
dogm_status dogm_device_free(void* ptr);
dogm_status dogm_memcpy(void* dst, const void* src, size_t bytes, int kind /* cudaMemcpyKind */);

/* Device bytes a handle with these parameters holds (admission control); a handle that uses
 * dogm_get_grid_cells_async holds 64 * grid_size^2 bytes more. */
size_t dogm_state_bytes(const dogm_params* params);

/* ---- serving loop ----------------------------------------------------------------------
 *
 * No counterpart in the reference (one dogm::DOGM per sensor, updated synchronously by its
 * caller, dogm/demo/main.cpp:81-92).  A server keeps many sensor streams resident on one
 * device -- each stream is a dogm_handle with its particles and grid -- admits streams under an
 * HBM budget, and updates the frames that callers submit by continuous batching: a worker
 * thread takes the oldest pending frame of every stream that has no frame on the device, up to
 * max_batch of them, and queues them as one batched update (dogm_update_batch's launch
 * sequence and CUDA graph) on one of max_inflight launch slots, so that frames arriving while
 * others run join the next launch and launches overlap on the device.  Each frame's result is
 * bit-identical to updating its stream alone with dogm_update (same handle, same frames).
 * DOGM_SERVE_PER_STREAM instead updates every frame on its own with dogm_update on the
 * stream's own CUDA stream, and DOGM_SERVE_PER_STREAM_PLAIN also waits for each frame before
 * the next (the two per-stream comparisons).  All calls are thread-safe. */

typedef enum dogm_serve_mode {
    DOGM_SERVE_BATCHED = 0,    /* continuous batching over launch slots                      */
    DOGM_SERVE_PER_STREAM = 1, /* one dogm_update per frame on the stream's own CUDA stream,
                                  chained launches, frames of several streams in flight      */
    DOGM_SERVE_PER_STREAM_PLAIN = 2 /* one dogm_update per frame with plain kernel launches,
                                  each waited for before the next frame starts (the
                                  reference's synchronous updateGrid, dogm/src/dogm.cu:115-131) */
} dogm_serve_mode;

typedef struct dogm_server_config {
    size_t hbm_budget_bytes; /* resident stream state (dogm_state_bytes) stays within this      */
    int mode;                /* dogm_serve_mode                                                */
    int max_batch;           /* frames per batched launch, 1..256                              */
    int max_inflight;        /* batched launches queued on the device at once, 1..4            */
    int queue_admission;     /* 1: a stream that does not fit waits for memory to free up;
                                0: dogm_server_open_stream refuses it with DOGM_ERR_BUDGET      */
} dogm_server_config;

/* One finished frame.  Times are nanoseconds of the monotonic clock of dogm_server_now_ns. */
typedef struct dogm_server_result {
    int stream;          /* id from dogm_server_open_stream                                    */
    int status;          /* dogm_status of the frame                                           */
    uint64_t tag;        /* the caller's tag from dogm_server_submit                           */
    int iteration;       /* completed updates of the stream, this one included                 */
    int batch_size;      /* frames in the launch that carried this one (1 per stream)          */
    int64_t t_submit_ns; /* dogm_server_submit accepted the frame                              */
    int64_t t_launch_ns; /* the frame's launch was queued on the device                        */
    int64_t t_done_ns;   /* the worker saw the launch finished (update and readback done)      */
} dogm_server_result;

typedef struct dogm_server_stats {
    uint64_t frames_submitted, frames_done, launches;
    int streams_active;      /* admitted, with device state                                    */
    int streams_waiting;     /* opened, waiting for the budget                                 */
    size_t resident_bytes;   /* dogm_state_bytes of the admitted streams                       */
    size_t budget_bytes;
    double mean_batch;       /* frames per launch so far                                       */
} dogm_server_stats;

typedef struct dogm_server dogm_server;

/* Stream states reported by dogm_server_stream_state. */
#define DOGM_STREAM_WAITING 0 /* opened, not admitted yet (over budget)                          */
#define DOGM_STREAM_ACTIVE 1  /* admitted: device state allocated                                 */
#define DOGM_STREAM_CLOSED 2  /* closed, or admission failed                                      */

/* Defaults: 150 GB budget, batched, max_batch 64, max_inflight 2, queued admission. */
dogm_status dogm_server_default_config(dogm_server_config* cfg);

/* Creates a server on the current device and starts its worker thread. */
dogm_status dogm_server_create(const dogm_server_config* cfg, dogm_server** out);

/* Finishes every submitted frame of the admitted streams, frees all streams, stops the worker. */
dogm_status dogm_server_destroy(dogm_server* s);

/* Opens a stream with the filter parameters of one dogm_handle (opt may be NULL).  If its
 * dogm_state_bytes fit the budget next to the admitted streams (and no earlier stream waits),
 * its device state is allocated now; otherwise, with queue_admission, it waits (state
 * DOGM_STREAM_WAITING; frames may already be submitted) until closed streams free the budget,
 * and without queue_admission the call returns DOGM_ERR_BUDGET.  A stream larger than the
 * whole budget is always refused with DOGM_ERR_BUDGET. */
dogm_status dogm_server_open_stream(dogm_server* s, const dogm_params* params, const dogm_options* opt,
                                    int* stream_id);

/* Finishes the stream's submitted frames, frees its device state and admits waiting streams
 * that now fit.  Returns when the stream is closed. */
dogm_status dogm_server_close_stream(dogm_server* s, int stream_id);

/* Queues one frame of a stream (the arguments of dogm_update).  meas (host, or device with
 * device != 0; pinned host memory copies fastest) must stay valid and unchanged until the
 * frame's result is returned.  cells_out, if not NULL, is a host buffer of grid_size^2 cells
 * that receives the stream's grid after this update.  A stream's frames run in submission
 * order, one at a time. */
dogm_status dogm_server_submit(dogm_server* s, int stream_id, const dogm_measurement_cell* meas, int device,
                               float new_x, float new_y, float new_yaw, float dt, dogm_grid_cell* cells_out,
                               uint64_t tag);

/* paused != 0 holds back new launches (launches in flight finish; submitted frames queue);
 * paused == 0 resumes, and the next launches take every frame that queued meanwhile. */
dogm_status dogm_server_pause(dogm_server* s, int paused);

/* Moves up to max finished frames into out, waiting up to timeout_us for the first one;
 * *n_out receives the count (0 on timeout). */
dogm_status dogm_server_poll(dogm_server* s, dogm_server_result* out, int max, int timeout_us, int* n_out);

/* Waits until every submitted frame has finished (DOGM_ERR_NOT_READY after timeout_ms, for
 * example while frames of a waiting stream cannot run). */
dogm_status dogm_server_drain(dogm_server* s, int timeout_ms);

dogm_status dogm_server_get_stats(dogm_server* s, dogm_server_stats* out);

/* DOGM_STREAM_* state of a stream, or -1 for an unknown id. */
int dogm_server_stream_state(dogm_server* s, int stream_id);

/* The dogm_handle of an admitted stream, for the readback calls (dogm_get_grid_cells ...).
 * Use it only while none of the stream's frames is pending (after dogm_server_drain). */
dogm_status dogm_server_stream_handle(dogm_server* s, int stream_id, dogm_handle** out);

/* The clock of dogm_server_result (monotonic, nanoseconds). */
int64_t dogm_server_now_ns(void);

/* ---- snapshot and restore -----------------------------------------------------------------
 *
 * No counterpart in the reference.  A snapshot is the state one update carries into the next:
 * particles (state and key words), the free mass, the common particle weight, the resident
 * measurement grid, the last cell records, the pose bookkeeping, the update count and the
 * random-number identity (seed, stream id).  Restoring it into a handle created with the same
 * dogm_params makes that handle continue bit-identically to the original (used to move a
 * serving stream, or to resume after a restart).  The buffer is host memory in native byte
 * order, starting with a versioned header. */
size_t dogm_snapshot_bytes(const dogm_handle* h);
dogm_status dogm_snapshot(dogm_handle* h, void* host_buf, size_t n);
/* DOGM_ERR_INVALID_ARGUMENT (handle unchanged) if the buffer is not a snapshot of a handle with
 * the same parameters. */
dogm_status dogm_restore(dogm_handle* h, const void* host_buf, size_t n);

/* ---- dynamic-cell extraction -------------------------------------------------------------
 *
 * Replaces the demo's host-side computeCellsWithVelocity (dogm/demo/utils/image_creation.cpp:
 * 19-66), which copies the whole grid back and filters it on the CPU: here the filter runs on
 * the GPU and only the kept cells cross to the host.  A cell is kept when its pignistic
 * occupancy occ + (1 - occ - free) / 2 >= min_occupancy and the Mahalanobis length of its mean
 * velocity, v^T Sigma^-1 v with Sigma = [[var_x, cov], [cov, var_y]], >= min_velocity (0 for a
 * singular Sigma).  Cells come in row-major order, as the reference's loops visit them. */
typedef struct dogm_dynamic_cell {
    int index;          /* y * grid_size + x                                              */
    float x, y;         /* column and row of the cell (image_creation.cpp:53-54)          */
    float occupancy;    /* pignistic occupancy                                            */
    float mahalanobis;  /* v^T Sigma^-1 v                                                 */
    dogm_grid_cell cell;
} dogm_dynamic_cell;

/* Extracts from the handle's current grid into host_out (up to max_out cells, the first in
 * row-major order); *n_found receives how many cells pass, which may exceed max_out.  The
 * handle keeps a device staging buffer of max_out cells (allocated on first use or growth). */
dogm_status dogm_extract_dynamic_cells(dogm_handle* h, float min_occupancy, float min_velocity,
                                       dogm_dynamic_cell* host_out, int max_out, int* n_found);

/* The same over any grid in device memory: cells (grid_size^2), out (device, max_out entries),
 * scratch (device, ceil(grid_size^2 / 1024) words); runs on `stream` and returns when done. */
dogm_status dogm_extract_dynamic_cells_device(const dogm_grid_cell* cells, int grid_size, float min_occupancy,
                                              float min_velocity, dogm_dynamic_cell* out, int max_out,
                                              unsigned int* scratch, int* n_found, void* stream);

/* ---- accuracy evaluation against ground truth (host code) --------------------------------
 *
 * Replaces the demo's PrecisionEvaluator with its DBSCAN and MAE/RMSE metrics
 * (dogm/demo/utils/precision_evaluator.cpp:16-139, dbscan.cpp:24-114, metrics.cpp:8-56):
 * the dynamic cells of a frame are clustered (eps 3 cells, at least 5 cells within eps counting
 * the cell itself), each cluster's mean (x, y, vx, vy) is converted to metres with y up
 * (x * r, grid_length - y * r, vx * r, -vy * r, precision_evaluator.cpp:98-121) and matched to the
 * nearest object closer than 5 m; errors accumulate into MAE and RMSE, unmatched clusters into
 * the unassigned count.  The functions touch no GPU. */
typedef enum dogm_dbscan_mode {
    DOGM_DBSCAN_REFERENCE = 0, /* dbscan.cpp:55-98 exactly, including its labelling of the first
                                  |seeds| input points (dbscan.cpp:64-67) instead of the seeds   */
    DOGM_DBSCAN_STANDARD = 1   /* the published DBSCAN, same visiting order                      */
} dogm_dbscan_mode;

/* Vehicle of the simulator (dogm/demo/simulator/include/simulator.h:11-31): position of the
 * facing side's centre and velocity, metres and m/s, x right, y up. */
typedef struct dogm_object_truth {
    float x, y, vx, vy;
} dogm_object_truth;

typedef struct dogm_cluster {
    float x, y, vx, vy;                  /* cluster mean in metres / m/s, y up (NaN if empty) */
    int cells;                           /* cells in the cluster                              */
    int truth;                           /* matched object, -1 if none within 5 m             */
    float err_x, err_y, err_vx, err_vy;  /* mean - object (0 if unmatched)                    */
} dogm_cluster;

/* DBSCAN over the cells' (x, y); label[i] receives the cluster of cell i or -1.  Cells must have
 * distinct coordinates. */
dogm_status dogm_cluster_cells(const dogm_dynamic_cell* cells, int n, float eps, int min_cells, int mode,
                               int* label, int* n_clusters);

typedef struct dogm_evaluator dogm_evaluator;

/* resolution: metres per cell; grid_length: the grid's side in metres (GridParams::size). */
dogm_status dogm_evaluator_create(float resolution, float grid_length, int dbscan_mode, dogm_evaluator** out);
dogm_status dogm_evaluator_destroy(dogm_evaluator* e);

/* PrecisionEvaluator::evaluateAndStoreStep: clusters the frame's cells and accumulates the errors
 * of the matched clusters.  With no cells or no objects the frame adds nothing.  Up to
 * max_clusters clusters are written to `clusters` (may be NULL); *n_clusters receives how many
 * the frame had. */
dogm_status dogm_evaluator_add_step(dogm_evaluator* e, const dogm_dynamic_cell* cells, int n,
                                    const dogm_object_truth* truth, int n_truth, dogm_cluster* clusters,
                                    int max_clusters, int* n_clusters);

/* MAE and RMSE of (x, y, vx, vy) over all matched clusters so far (NaN before the first match),
 * the number of matched clusters and of unassigned ones.  Any output may be NULL. */
dogm_status dogm_evaluator_summary(const dogm_evaluator* e, float* mae4, float* rmse4, int* detections,
                                   int* unassigned);

/* ---- measurement-grid generation from a lidar scan --------------------------------------
 *
 * Replaces the demo's LaserMeasurementGrid (dogm/demo/simulator/include/mapping/
 * laser_to_meas_grid.h:13-35), which needs OpenGL for its polar -> cartesian step: here the
 * inverse sensor model (kernel/measurement_grid.cu:33-89) and the warp over the sensor's
 * field of view (opengl/renderer.cpp:11-31, shader.cpp:22-35) are CUDA kernels.  The sensor
 * sits at the centre of the grid's last row and looks towards row 0; beam 0 points
 * 90 + fov/2 degrees from the x axis and the last beam 90 - fov/2 (the texture's u runs
 * against the fan's angle).  Differences from the OpenGL path: the polar grid is sampled with
 * level-0 bilinear filtering (no mipmaps, no anisotropy: those depend on the graphics driver)
 * and coverage uses exact edge functions on vertices snapped to 1/256 pixel. */

/* LaserMeasurementGrid::Params (laser_to_meas_grid.h:16-22). */
typedef struct dogm_laser_params {
    float max_range;    /* [m]; polar range bins = int(max_range / resolution)            */
    float resolution;   /* range-bin length [m]                                           */
    float fov;          /* field of view [degrees]                                        */
    float stddev_range; /* range noise of the inverse sensor model [m]                    */
} dogm_laser_params;

typedef struct dogm_meas_grid dogm_meas_grid;

/* LaserMeasurementGrid(params, grid_length, resolution) (laser_to_meas_grid.cu:10-18) for
 * scans of `beams` ranges; grid_size = int(grid_length / grid_resolution). */
dogm_status dogm_meas_grid_create(const dogm_laser_params* p, float grid_length, float grid_resolution, int beams,
                                  dogm_meas_grid** out);
dogm_status dogm_meas_grid_destroy(dogm_meas_grid* m);

/* LaserMeasurementGrid::generateGrid (laser_to_meas_grid.cu:25-70): ranges[beams] in metres
 * (host, or device with device != 0; non-finite = no return) -> grid_size^2 measurement cells
 * written to out_device, a device buffer (then dogm_update(h, out_device, ..., 1)).  fuse != 0
 * combines this scan into the previous polar grid by Dempster's rule instead of replacing it
 * (fusePolarGridTextureKernel, measurement_grid.cu:91-113).  Runs on `stream`
 * (a cudaStream_t, 0 = legacy default) and returns when the grid is written. */
dogm_status dogm_meas_grid_generate(dogm_meas_grid* m, const float* ranges, int device, int fuse,
                                    dogm_measurement_cell* out_device, void* stream);
int dogm_meas_grid_size(const dogm_meas_grid* m);

/* Debug exports: the polar grid (bins x beams float pairs {occ, free}, row = range bin) and the
 * fan (apex, then one vertex per degree: window coordinates x 256 and texture s; the first arc
 * vertex's angle in degrees). */
dogm_status dogm_meas_grid_polar(dogm_meas_grid* m, float* host_out, size_t n, int* beams, int* bins);
dogm_status dogm_meas_grid_fan(dogm_meas_grid* m, long long* x256, long long* y256, float* s, int n, int* nv,
                               int* first_angle);

/* ---- measurement ---------------------------------------------------------------------- */

/* The cudaStream_t (as void*) the handle launches on: record CUDA events on it to time updates. */
void* dogm_get_stream(dogm_handle* h);

/* Per-stage timing (the reference has only a wall-clock timer around updateGrid,
 * dogm/demo/main.cpp:81,91-92).  When enabled, updates run as plain launches with a CUDA
 * event between stages instead of the CUDA graph; dogm_stage_times fills up to n values in
 * milliseconds for the last update, in the order of dogm_stage_name(0..n-1), and returns
 * the number of stages. */
dogm_status dogm_profile_enable(dogm_handle* h, int enable);
int dogm_stage_times(dogm_handle* h, float* ms, int n);
const char* dogm_stage_name(int i);

/* ---- autotuning -------------------------------------------------------------------------
 * No counterpart in the reference (its launch shape is fixed: SMs x maxThreadsPerSM / 256
 * blocks of 256 threads for every kernel, dogm/src/dogm.cu:45-47).  The tunable shape of an
 * update is the width of each stage's persistent launch (blocks per SM) and the resampling tile
 * (one of three compiled tile shapes). */
typedef struct dogm_tune {
    int blocks_per_sm[8];   /* per stage, in dogm_stage_name order (6 stages, the last two entries
                               0); 0 = the built-in default                                       */
    int resample_tile_bits; /* joint particles per resampling tile = 2^bits: 9, 10 or 11 (three
                               compiled tile shapes); 0 = the default 10                        */
    float ms_tuned;         /* dogm_autotune: ms per update with these settings               */
    float ms_default;       /* dogm_autotune: ms per update with the defaults                 */
} dogm_tune;

/* The handle's current settings (zeros: defaults). */
dogm_status dogm_get_tune(dogm_handle* h, dogm_tune* out);

/* Applies settings to the handle's own updates (dogm_update); a batch uses its own launch
 * context's defaults.  Results do not change: every setting computes the same bits.
 * blocks_per_sm in [0, 32]; resample_tile_bits 0 or in [9, 11]. */
dogm_status dogm_set_tune(dogm_handle* h, const dogm_tune* t);

/* Times candidate settings on a scratch handle with the same parameters, fed `meas`
 * (grid_size^2 cells, a device pointer if device != 0): each resampling tile shape (whole
 * updates), then each stage's width in {1, 2, 3, 4, 6, 8} blocks per SM with per-stage CUDA
 * events, `reps` updates per candidate and timing.  Candidates are timed in three interleaved
 * rounds (the scratch state evolves while it is timed) and compared on their sums; a setting
 * other than the built-in one, and the tuned shape as a whole, must win by 2 %.  The result is
 * applied to h and returned in *out.  With cache_path (may be NULL), a line keyed by device
 * name, grid size and particle counts is read instead of tuning, or appended after tuning. */
dogm_status dogm_autotune(dogm_handle* h, const dogm_measurement_cell* meas, int device, int reps,
                          const char* cache_path, dogm_tune* out);

/* Number of kernel launches the last update issued, and the text of the last error. */
int dogm_last_launch_count(const dogm_handle* h);

/* How a handle's steady-state updates are launched (no counterpart in the reference, whose
 * updateGrid issues every kernel itself).  DOGM_LAUNCH_CHAINED (the default): the six kernels
 * are launched one after another, each programmatically dependent on the one before it (the
 * first on the previous update's last), with the update's descriptor passed to the first
 * kernel as a parameter, so nothing else runs on the stream between two updates.
 * DOGM_LAUNCH_GRAPH: one captured CUDA graph per update, its descriptor uploaded on a second
 * stream (the form a batch's update and the serving loop's launch slots always take).
 * DOGM_LAUNCH_PLAIN: the kernels one by one, the descriptor copied up before them and the
 * status back after, as the reference does.  The results are the same bits in every mode. */
typedef enum dogm_launch_mode {
    DOGM_LAUNCH_CHAINED = 0,
    DOGM_LAUNCH_PLAIN = 1,
    DOGM_LAUNCH_GRAPH = 2
} dogm_launch_mode;
dogm_status dogm_set_launch_mode(dogm_handle* h, int mode);
const char* dogm_last_error(void);
const char* dogm_status_string(dogm_status s);
int dogm_abi_version(void);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* DOGM_GB300_H */
