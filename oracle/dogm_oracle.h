/*
 * dogm_oracle.h — CPU restatement of the dynamic occupancy grid map update.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker the GPU path is compared with,
 * and the timed CPU baseline of bench.py; the product (libdogm_gb300.so) never calls it.
 *
 * Two restatements live here:
 *   dogm_oracle_update_f32 / _f64
 *       the update exactly as the GPU path computes it (same stage semantics, same fixed
 *       operation order, exact integer scans), instantiated in float and in double.  The
 *       float instance reproduces every bit of the GPU path given the same random draws,
 *       except the per-cell velocity sums whose summation order differs; the double
 *       instance is the high-precision reference for tolerances.
 *   dogm_oracle_reference_f32
 *       the reference's own stage sequence (dogm/src/dogm.cu:115-131): global float prefix
 *       sums with segment differences, float-scan newborn allocation, multinomial
 *       resampling over sorted uniforms with lower_bound.  OpenMP-parallel; it is the CPU
 *       baseline ("the reference's pipeline transcribed to host code").
 *
 * Parity pins: the Philox generator is checked against the published Random123 answers;
 * the prediction and the ego shift are checked against the known answers of the
 * reference's own tests (dogm/test/dogm_spec.cpp:10-103).  No reference test pins the
 * mass update, reweighting, newborn, moment or resampling results (parity for those
 * stages rests on this restatement and on the cited reference lines).
 */
#ifndef DOGM_ORACLE_H
#define DOGM_ORACLE_H

#include <stdint.h>

typedef struct dogm_oracle_params {
    int gs, N, B, q_shift;
    float p_S, sigma_pos, sigma_vel, p_B, sigma_birth, init_max_vel, freespace_discount;
} dogm_oracle_params;

typedef struct dogm_oracle_frame {
    float dt;
    int shifted, shift_x, shift_y;
    int first_frame;
    const float* meas;      /* C x {free, occ, likelihood, p_A}        */
    const float* init_u;    /* N x 2 uniforms in (0,1] (first frame)    */
    const float* predict_z; /* N x 4 standard normals                   */
    const float* birth_z;   /* B x 2 standard normals                   */
    uint64_t resample_r;    /* systematic offset u = r / 2^64           */
} dogm_oracle_frame;

/* Outputs of one frame; any pointer may be NULL.  REAL = float for _f32, double for _f64. */
typedef struct dogm_oracle_out {
    void* cells;       /* C x 16 REAL: the GridCell fields in order (indices as REAL)    */
    void* S_state;     /* N x 4 REAL: particles after the stable sort                    */
    uint32_t* S_key;   /* N: sorted key words (cell | out-of-grid bit 30 | assoc bit 31) */
    int* perm;         /* N: input index of each sorted particle                         */
    void* B_state;     /* B x 4 REAL newborn states                                      */
    uint32_t* B_key;   /* B newborn key words                                            */
    void* B_w;         /* B REAL newborn weights                                         */
    int* res_src;      /* N: joint index each resampled particle was copied from         */
    uint64_t joint_total, qb_total;
    int n_birth;
} dogm_oracle_out;

/* State in/out: P_state (N x 4 REAL), P_key (N), free_mass (C REAL), w_res (1 REAL). */
int dogm_oracle_update_f32(const dogm_oracle_params* p, const dogm_oracle_frame* f, float* P_state,
                           uint32_t* P_key, float* free_mass, float* w_res, dogm_oracle_out* out);
int dogm_oracle_update_f64(const dogm_oracle_params* p, const dogm_oracle_frame* f, double* P_state,
                           uint32_t* P_key, double* free_mass, double* w_res, dogm_oracle_out* out);

/* Stage helpers for the reference's known-answer tests. */
void dogm_oracle_predict_f32(const dogm_oracle_params* p, float dt, const float* predict_z, float* P_state,
                             uint32_t* P_key, float* weights, int n);
void dogm_oracle_shift_particles_f32(float* P_state, int n, int x_move, int y_move);
/* Host pose bookkeeping of DOGM::updatePose: returns 1 and the moves when the grid shifts. */
int dogm_oracle_pose(float resolution, int* first, float* px, float* py, float* yaw, float nx, float ny,
                     float nyaw, int* x_move, int* y_move);

/* Philox4x32-10 block and the exact helpers shared with the GPU path. */
void dogm_oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
uint64_t dogm_oracle_quantize(double w, int S);
int dogm_oracle_alloc_boundary(uint64_t Q, uint64_t T, int M);
int dogm_oracle_comb_count(uint64_t a, uint64_t T, uint64_t U, int N);
/* Philox draws of one update in the GPU path's replay layouts (NULL skips a stage). */
void dogm_oracle_draws(uint64_t seed, uint32_t stream_id, int N, int B, int iteration, float* init_u,
                       float* predict_z, float* birth_z, uint64_t* resample_r);

/* The reference's pipeline in float (see above).  State: P_state (N x 4), P_idx (N),
 * P_w (N), P_assoc (N), cells (C x 16 floats, the GridCell records), meas (C x 4, in).
 * Draws come from Philox seeded with (seed, frame); threads = 0 uses all cores.
 * Returns the number of OpenMP threads used. */
int dogm_oracle_reference_f32(const dogm_oracle_params* p, const float* meas, float dt, int first_frame,
                              int shifted, int x_move, int y_move, uint64_t seed, uint32_t frame, float* P_state,
                              int* P_idx, float* P_w, unsigned char* P_assoc, float* cells, int threads);

/* Resampling-scan precision study: systematic comb of n slots over joint weights w[0..m) with
 * offset u in [0,1) and the prefix in float32 (mode 0), compensated float32 (1) or float64 (2);
 * out[i] = joint item of slot i. */
void dogm_oracle_comb_indices(const float* w, int m, int n, double u, int mode, int* out);

#endif /* DOGM_ORACLE_H */
