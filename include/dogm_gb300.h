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

/* Waits for all work queued on the handle's stream (only needed with sync_each_update=0). */
dogm_status dogm_synchronize(dogm_handle* h);

/* ---- readback (dogm/src/dogm.cu:133-159) ---------------------------------------------- */

/* Replaces DOGM::getGridCells: copies n == grid_size^2 cells to host memory. */
dogm_status dogm_get_grid_cells(dogm_handle* h, dogm_grid_cell* host_out, size_t n);
/* Same into a device buffer of the handle's device (no host round trip). */
dogm_status dogm_get_grid_cells_device(dogm_handle* h, dogm_grid_cell* dev_out, size_t n);

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
 * DOGM_ERR_INVALID_ARGUMENT and leaves the handle unchanged.  The first call on a device looks
 * up the array's address: make that first call before any stream capture.  All calls on a
 * device share the one array, so calls whose work overlaps on the GPU (several host threads at
 * once) race on it and must be serialised by the caller. */
dogm_status dogm_update_pose_noalloc(dogm_handle* h, float new_x, float new_y, float new_yaw);

/* Replaces DOGM::initializeParticles (dogm/src/dogm.cu:217-241) from the resident
 * measurement grid (set by a previous update, or by dogm_set_measurement_cells). */
dogm_status dogm_initialize_particles(dogm_handle* h);

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

/* Device bytes a handle with these parameters holds (admission control). */
size_t dogm_state_bytes(const dogm_params* params);

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

/* Number of kernel launches the last update issued, and the text of the last error. */
int dogm_last_launch_count(const dogm_handle* h);
const char* dogm_last_error(void);
const char* dogm_status_string(dogm_status s);
int dogm_abi_version(void);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* DOGM_GB300_H */
