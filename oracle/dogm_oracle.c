/*
 * dogm_oracle.c — CPU restatements of the dynamic occupancy grid map update.
 * TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline as the checker; the product library never links or calls it.  See dogm_oracle.h.
 *
 * Build: gcc -O2 -std=gnu11 -fPIC -shared -fopenmp -ffp-contract=off (no fast-math, no
 * contraction, so float expressions round after every operation, like the GPU path's
 * _rn intrinsics).
 */
#include "dogm_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define CELL_MASK 0x3fffffffu
#define OUT_BIT (1u << 30)
#define ASSOC_BIT (1u << 31)

/* ---------------------------------------------------------------------------------------
 * Philox4x32-10 (Salmon et al., SC'11): two 32x32->64 multiplies per round, Weyl key
 * schedule; counter {index, frame, stage, stream}, key = seed.
 * ------------------------------------------------------------------------------------- */
void dogm_oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n1 = (uint32_t)p1;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        const uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

enum { DRAW_INIT = 1, DRAW_PREDICT = 2, DRAW_BIRTH = 3, DRAW_RESAMPLE = 4 };

static void draw_block(uint64_t seed, uint32_t stream, uint32_t index, uint32_t frame, uint32_t stage, uint32_t o[4]) {
    const uint32_t c[4] = {index, frame, stage, stream};
    const uint32_t k[2] = {(uint32_t)(seed & 0xffffffffu), (uint32_t)(seed >> 32)};
    dogm_oracle_philox(c, k, o);
}

static float u01_open0(uint32_t x) { return (float)((x >> 8) + 1u) * 5.9604644775390625e-8f; }
static float u01_open1(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-8f; }

static void box_muller_f(uint32_t a, uint32_t b, float* z0, float* z1) {
    const float u1 = u01_open0(a), u2 = u01_open1(b);
    const float r = sqrtf(-2.0f * logf(u1));
    const float th = 6.28318530717958647692f * u2;
    *z0 = r * cosf(th);
    *z1 = r * sinf(th);
}

void dogm_oracle_draws(uint64_t seed, uint32_t stream, int N, int B, int iteration, float* init_u, float* predict_z,
                       float* birth_z, uint64_t* resample_r) {
    uint32_t o[4];
#pragma omp parallel for private(o) schedule(static)
    for (int i = 0; i < N; ++i) {
        if (init_u) {
            draw_block(seed, stream, (uint32_t)i, 0u, DRAW_INIT, o);
            init_u[2 * (size_t)i] = u01_open0(o[0]);
            init_u[2 * (size_t)i + 1] = u01_open0(o[1]);
        }
        if (predict_z) {
            draw_block(seed, stream, (uint32_t)i, (uint32_t)iteration, DRAW_PREDICT, o);
            box_muller_f(o[0], o[1], &predict_z[4 * (size_t)i], &predict_z[4 * (size_t)i + 1]);
            box_muller_f(o[2], o[3], &predict_z[4 * (size_t)i + 2], &predict_z[4 * (size_t)i + 3]);
        }
    }
    if (birth_z) {
#pragma omp parallel for private(o) schedule(static)
        for (int i = 0; i < B; ++i) {
            draw_block(seed, stream, (uint32_t)i, (uint32_t)iteration, DRAW_BIRTH, o);
            box_muller_f(o[0], o[1], &birth_z[2 * (size_t)i], &birth_z[2 * (size_t)i + 1]);
        }
    }
    if (resample_r) {
        draw_block(seed, stream, 0u, (uint32_t)iteration, DRAW_RESAMPLE, o);
        *resample_r = ((uint64_t)o[0] << 32) | o[1];
    }
}

/* ---------------------------------------------------------------------------------------
 * Exact fixed point (shared semantics with the GPU path).
 * ------------------------------------------------------------------------------------- */
uint64_t dogm_oracle_quantize(double w, int S) {
    if (!(w > 0.0)) return 0;
    if (w > 2.0) w = 2.0;
    return (uint64_t)llrint(ldexp(w, S));
}

/* floor(Q * M / T) */
int dogm_oracle_alloc_boundary(uint64_t Q, uint64_t T, int M) {
    if (T == 0) return 0;
    if (Q >= T) return M;
    return (int)(((unsigned __int128)Q * (uint64_t)M) / T);
}

/* #{ i in [0,N) : i*T + U < a*N } */
int dogm_oracle_comb_count(uint64_t a, uint64_t T, uint64_t U, int N) {
    if (T == 0) return N;
    if (a >= T) return N;
    const unsigned __int128 rhs = (unsigned __int128)a * (uint64_t)N;
    if (rhs <= U) return 0;
    const unsigned __int128 num = rhs - U;
    unsigned __int128 c = (num + T - 1) / T;
    if (c > (unsigned __int128)N) c = N;
    return (int)c;
}

/* DOGM::updatePose (dogm/src/dogm.cu:161-203) */
int dogm_oracle_pose(float resolution, int* first, float* px, float* py, float* yaw, float nx, float ny, float nyaw,
                     int* x_move, int* y_move) {
    *x_move = *y_move = 0;
    if (!*first) {
        *px = nx; *py = ny; *yaw = nyaw;
        *first = 1;
        return 0;
    }
    const float x_diff = nx - *px;
    const float y_diff = ny - *py;
    if (fabsf(x_diff) > resolution || fabsf(y_diff) > resolution) {
        *x_move = -(int)(x_diff / resolution);
        *y_move = -(int)(y_diff / resolution);
        *px = nx; *py = ny; *yaw = nyaw;
        return 1;
    }
    return 0;
}

/* moveParticlesKernel (ego_motion_compensation.cu:16-23) */
void dogm_oracle_shift_particles_f32(float* st, int n, int x_move, int y_move) {
    for (int i = 0; i < n; ++i) {
        st[4 * (size_t)i] = st[4 * (size_t)i] - (float)x_move;
        st[4 * (size_t)i + 1] = st[4 * (size_t)i + 1] - (float)y_move;
    }
}

/* ---- the two instantiations of the update restatement --------------------------------- */
#define REAL float
#define SFX f32
#define RFMA fmaf
#define RROUND roundf
#define LDEXP ldexpf
#include "dogm_oracle_impl.h"
#undef REAL
#undef SFX
#undef RFMA
#undef RROUND
#undef LDEXP

#define REAL double
#define SFX f64
#define RFMA fma
#define RROUND round
#define LDEXP ldexp
#include "dogm_oracle_impl.h"
#undef REAL
#undef SFX
#undef RFMA
#undef RROUND
#undef LDEXP

/* =======================================================================================
 * The reference's pipeline in float, stage by stage (dogm/src/dogm.cu:115-131), OpenMP.
 * ===================================================================================== */

typedef struct ref_cell {
    int start_idx, end_idx;
    float new_born_occ_mass, pers_occ_mass, free_mass, occ_mass, pred_occ_mass, mu_A, mu_UA, w_A, w_UA;
    float mean_x_vel, mean_y_vel, var_x_vel, var_y_vel, covar_xy_vel;
} ref_cell;

/* inclusive float scan, two passes over per-thread blocks (thrust::inclusive_scan, common.h:11-22) */
static void scan_f32(const float* in, float* out, size_t n) {
    const int T = omp_get_max_threads();
    float* part = (float*)calloc((size_t)T + 1, sizeof(float));
#pragma omp parallel num_threads(T)
    {
        const int t = omp_get_thread_num(), nt = omp_get_num_threads();
        const size_t lo = n * (size_t)t / (size_t)nt, hi = n * (size_t)(t + 1) / (size_t)nt;
        float s = 0.0f;
        for (size_t i = lo; i < hi; ++i) { s += in[i]; out[i] = s; }
        part[t + 1] = s;
#pragma omp barrier
#pragma omp single
        for (int k = 1; k <= nt; ++k) part[k] += part[k - 1];
        const float off = part[t];
        if (t > 0)
            for (size_t i = lo; i < hi; ++i) out[i] += off;
    }
    free(part);
}

/* stable LSD radix sort of an index permutation by 32-bit keys (8-bit digits) */
static void radix_perm_u32(const uint32_t* key, int* perm, size_t n, int bits) {
    const int T = omp_get_max_threads();
    int* tmp = (int*)malloc(sizeof(int) * n);
    size_t* hist = (size_t*)malloc(sizeof(size_t) * 256 * (size_t)T);
    for (size_t i = 0; i < n; ++i) perm[i] = (int)i;
    int* src = perm;
    int* dst = tmp;
    const int passes = (bits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        const int sh = 8 * p;
        memset(hist, 0, sizeof(size_t) * 256 * (size_t)T);
#pragma omp parallel num_threads(T)
        {
            const int t = omp_get_thread_num(), nt = omp_get_num_threads();
            const size_t lo = n * (size_t)t / (size_t)nt, hi = n * (size_t)(t + 1) / (size_t)nt;
            size_t* h = hist + 256 * (size_t)t;
            for (size_t i = lo; i < hi; ++i) h[(key[src[i]] >> sh) & 255u]++;
#pragma omp barrier
#pragma omp single
            {
                size_t acc = 0;
                for (int d = 0; d < 256; ++d)
                    for (int u = 0; u < nt; ++u) {
                        const size_t c = hist[256 * (size_t)u + d];
                        hist[256 * (size_t)u + d] = acc;
                        acc += c;
                    }
            }
            for (size_t i = lo; i < hi; ++i) dst[h[(key[src[i]] >> sh) & 255u]++] = src[i];
        }
        int* s2 = src; src = dst; dst = s2;
    }
    if (src != perm) memcpy(perm, src, sizeof(int) * n);
    free(tmp);
    free(hist);
}

static float ref_subtract(const float* acc, int s, int e) { return s == 0 ? acc[e] : acc[e] - acc[s - 1]; }

int dogm_oracle_reference_f32(const dogm_oracle_params* p, const float* meas, float dt, int first_frame, int shifted,
                              int x_move, int y_move, uint64_t seed, uint32_t frame, float* P_state, int* P_idx,
                              float* P_w, unsigned char* P_assoc, float* cells_raw, int threads) {
    if (threads > 0) omp_set_num_threads(threads);
    const int nthreads = omp_get_max_threads();
    const int gs = p->gs, N = p->N, B = p->B, C = gs * gs;
    ref_cell* cells = (ref_cell*)cells_raw;
    float* weight_array = (float*)malloc(sizeof(float) * (size_t)N);
    float* accN = (float*)malloc(sizeof(float) * (size_t)(N + B));
    float* born = (float*)malloc(sizeof(float) * (size_t)C);
    float* accC = (float*)malloc(sizeof(float) * (size_t)C);
    float* Bs = (float*)calloc((size_t)(B > 0 ? B : 1) * 4, sizeof(float));
    int* Bi = (int*)calloc((size_t)(B > 0 ? B : 1), sizeof(int));
    float* Bw = (float*)calloc((size_t)(B > 0 ? B : 1), sizeof(float));
    unsigned char* Ba = (unsigned char*)calloc((size_t)(B > 0 ? B : 1), 1);
    int* perm = (int*)malloc(sizeof(int) * (size_t)(N > B ? N : B) * 1);
    float* tmp4 = (float*)malloc(sizeof(float) * 4 * (size_t)N);
    float* tmp1 = (float*)malloc(sizeof(float) * (size_t)N);
    int* tmpi = (int*)malloc(sizeof(int) * (size_t)N);
    unsigned char* tmpa = (unsigned char*)malloc((size_t)N);
    float* vel[5];
    for (int k = 0; k < 5; ++k) vel[k] = (float*)malloc(sizeof(float) * (size_t)N);
    float* vacc[5];
    for (int k = 0; k < 5; ++k) vacc[k] = (float*)malloc(sizeof(float) * (size_t)N);

    /* 1. first measurement: initializeParticles (dogm.cu:217-241) */
    if (first_frame) {
#pragma omp parallel for
        for (int j = 0; j < C; ++j) born[j] = meas[4 * (size_t)j + 1];
        scan_f32(born, accC, (size_t)C);
        const float mx = accC[C - 1];
        const float sc = (float)N / mx;
#pragma omp parallel for
        for (int j = 0; j < C; ++j) accC[j] = accC[j] * sc;
        memset(P_idx, 0, sizeof(int) * (size_t)N);
#pragma omp parallel for schedule(dynamic, 1024)
        for (int j = 0; j < C; ++j) {
            const int s = j == 0 ? 0 : (int)accC[j - 1];
            const int e = (int)accC[j] - 1;
            for (int i = s; i <= e && i < N; ++i)
                if (i >= 0) P_idx[i] = j;
        }
        const float w0 = 1.0f / (float)N, v = p->init_max_vel;
#pragma omp parallel for
        for (int i = 0; i < N; ++i) {
            uint32_t o[4];
            draw_block(seed, 0u, (uint32_t)i, 0u, DRAW_INIT, o);
            const int c = P_idx[i];
            P_state[4 * (size_t)i + 0] = (float)(c % gs) + 0.5f;
            P_state[4 * (size_t)i + 1] = (float)(c / gs) + 0.5f;
            P_state[4 * (size_t)i + 2] = -v + (v - (-v)) * (1.0f - u01_open0(o[0]));
            P_state[4 * (size_t)i + 3] = -v + (v - (-v)) * (1.0f - u01_open0(o[1]));
            P_w[i] = w0;
            P_assoc[i] = 0;
        }
    }

    /* 2. updatePose: particle and cell shift (dogm.cu:180-196) */
    if (shifted) {
#pragma omp parallel for
        for (int i = 0; i < N; ++i) {
            P_state[4 * (size_t)i] -= (float)x_move;
            P_state[4 * (size_t)i + 1] -= (float)y_move;
        }
        ref_cell* old = (ref_cell*)malloc(sizeof(ref_cell) * (size_t)C);
        memcpy(old, cells, sizeof(ref_cell) * (size_t)C);
        memset(cells, 0, sizeof(ref_cell) * (size_t)C);
#pragma omp parallel for
        for (int k = 0; k < C; ++k) {
            const int x = k % gs, y = k / gs, nx = x + x_move, ny = y + y_move;
            if (nx > 0 && nx < gs && ny > 0 && ny < gs) cells[k] = old[nx + gs * ny];
        }
        free(old);
    }

    /* 3. particlePrediction (predict.cu:12-48) */
    {
        const float gsm1 = (float)(gs - 1);
        uint32_t* key = (uint32_t*)tmpi;
#pragma omp parallel for
        for (int i = 0; i < N; ++i) {
            uint32_t o[4];
            float z[4];
            draw_block(seed, 0u, (uint32_t)i, frame, DRAW_PREDICT, o);
            box_muller_f(o[0], o[1], &z[0], &z[1]);
            box_muller_f(o[2], o[3], &z[2], &z[3]);
            float* s = P_state + 4 * (size_t)i;
            const float x = (s[0] + dt * s[2]) + z[0] * p->sigma_pos;
            const float y = (s[1] + dt * s[3]) + z[1] * p->sigma_pos;
            s[2] = s[2] + z[2] * p->sigma_vel;
            s[3] = s[3] + z[3] * p->sigma_vel;
            s[0] = x;
            s[1] = y;
            P_w[i] = p->p_S * P_w[i];
            if (x > gsm1 || x < 0.0f || y > gsm1 || y < 0.0f) P_w[i] = 0.0f;
            int px = (int)x, py = (int)y;
            px = px < 0 ? 0 : (px > gs - 1 ? gs - 1 : px);
            py = py < 0 ? 0 : (py > gs - 1 ? gs - 1 : py);
            P_idx[i] = px + gs * py;
            key[i] = (uint32_t)P_idx[i];
        }
    }

    /* 4. particleAssignment: stable sort by cell, ranges, weight array (dogm.cu:262-281) */
    {
#pragma omp parallel for
        for (int k = 0; k < C; ++k) { cells[k].start_idx = -1; cells[k].end_idx = -1; }
        int bits = 1;
        while ((1u << bits) < (unsigned)C) ++bits;
        uint32_t* key = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)N);
        for (int i = 0; i < N; ++i) key[i] = (uint32_t)P_idx[i];
        radix_perm_u32(key, perm, (size_t)N, bits);
        free(key);
#pragma omp parallel for
        for (int d = 0; d < N; ++d) {
            const int i = perm[d];
            memcpy(tmp4 + 4 * (size_t)d, P_state + 4 * (size_t)i, 16);
            tmp1[d] = P_w[i];
            tmpi[d] = P_idx[i];
            tmpa[d] = P_assoc[i];
        }
        memcpy(P_state, tmp4, 16 * (size_t)N);
        memcpy(P_w, tmp1, 4 * (size_t)N);
        memcpy(P_idx, tmpi, 4 * (size_t)N);
        memcpy(P_assoc, tmpa, (size_t)N);
#pragma omp parallel for
        for (int i = 0; i < N; ++i) {
            const int c = P_idx[i];
            if (i == 0 || P_idx[i - 1] != c) cells[c].start_idx = i;
            if (i == N - 1 || P_idx[i + 1] != c) cells[c].end_idx = i;
            weight_array[i] = P_w[i];
        }
    }

    /* 5. gridCellOccupancyUpdate (mass_update.cu:57-89) */
    {
        scan_f32(weight_array, accN, (size_t)N);
        const float alpha = powf(p->freespace_discount, dt);
#pragma omp parallel for schedule(dynamic, 4096)
        for (int k = 0; k < C; ++k) {
            ref_cell* g = &cells[k];
            float m = 0.0f;
            if (g->start_idx != -1) m = ref_subtract(accN, g->start_idx, g->end_idx);
            if (m > 1.0f) {
                for (int i = g->start_idx; i <= g->end_idx; ++i) {
                    weight_array[i] = weight_array[i] / m;
                    P_w[i] = weight_array[i];
                }
                m = 1.0f;
            }
            const float* z = meas + 4 * (size_t)k;
            const float mf = fminf(alpha * g->free_mass, 1.0f - m);
            const float unk = 1.0f - m - mf;
            const float mu = 1.0f - z[0] - z[1];
            const float K = mf * z[1] + m * z[0];
            const float occ = (m * mu + unk * z[1] + m * z[1]) / (1.0f - K);
            const float fre = (mf * mu + unk * z[0] + mf * z[0]) / (1.0f - K);
            const float rb = (occ * p->p_B * (1.0f - m)) / (m + p->p_B * (1.0f - m));
            born[k] = rb;
            g->pers_occ_mass = occ - rb;
            g->new_born_occ_mass = rb;
            g->free_mass = fre;
            g->occ_mass = occ;
            g->pred_occ_mass = m;
        }
    }

    /* 6. updatePersistentParticles (update_persistent_particles.cu:49-87) */
    {
#pragma omp parallel for
        for (int i = 0; i < N; ++i) weight_array[i] = meas[4 * (size_t)P_idx[i] + 2] * P_w[i];
        scan_f32(weight_array, accN, (size_t)N);
#pragma omp parallel for
        for (int k = 0; k < C; ++k) {
            ref_cell* g = &cells[k];
            if (g->start_idx != -1) {
                const float acc = ref_subtract(accN, g->start_idx, g->end_idx);
                g->mu_A = acc > 0.0f ? g->pers_occ_mass / acc : 0.0f;
                g->mu_UA = g->pred_occ_mass > 0.0f ? g->pers_occ_mass / g->pred_occ_mass : 0.0f;
            }
        }
#pragma omp parallel for
        for (int i = 0; i < N; ++i) {
            const ref_cell* g = &cells[P_idx[i]];
            const float pA = meas[4 * (size_t)P_idx[i] + 3];
            weight_array[i] = pA * g->mu_A * weight_array[i] + (1.0f - pA) * g->mu_UA * P_w[i];
        }
    }

    /* 7. initializeNewParticles (init_new_particles.cu:126-195) */
    if (B > 0) {
        scan_f32(born, accC, (size_t)C);
        const float mx = accC[C - 1];
        const float sc = (float)B / mx;
#pragma omp parallel for
        for (int j = 0; j < C; ++j) accC[j] = accC[j] * sc;
#pragma omp parallel for schedule(dynamic, 1024)
        for (int j = 0; j < C; ++j) {
            const int s = j == 0 ? 0 : (int)accC[j - 1];
            const int e = (int)accC[j] - 1;
            const int n = s <= e ? e - s + 1 : 0;
            const float pA = meas[4 * (size_t)j + 3];
            const int nuA = (int)roundf((float)n * pA), nuUA = n - nuA;
            cells[j].w_A = nuA > 0 ? (pA * born[j]) / (float)nuA : 0.0f;
            cells[j].w_UA = nuUA > 0 ? ((1.0f - pA) * born[j]) / (float)nuUA : 0.0f;
            for (int i = s; i <= e && i < B; ++i) {
                if (i < 0) continue;
                Bi[i] = j;
                Ba[i] = (i < s + nuA) ? 1 : 0;
                Bw[i] = -1.0f; /* assigned */
            }
        }
#pragma omp parallel for
        for (int i = 0; i < B; ++i) {
            uint32_t o[4];
            float z0, z1;
            draw_block(seed, 0u, (uint32_t)i, frame, DRAW_BIRTH, o);
            box_muller_f(o[0], o[1], &z0, &z1);
            const int c = Bi[i];
            Bs[4 * (size_t)i + 0] = (float)(c % gs) + 0.5f;
            Bs[4 * (size_t)i + 1] = (float)c / (float)gs + 0.5f;
            Bs[4 * (size_t)i + 2] = z0 * p->sigma_birth;
            Bs[4 * (size_t)i + 3] = z1 * p->sigma_birth;
            Bw[i] = (Bw[i] < 0.0f) ? (Ba[i] ? cells[c].w_A : cells[c].w_UA) : 0.0f;
        }
    }

    /* 8. statisticalMoments (statistical_moments.cu:58-106) */
    {
#pragma omp parallel for
        for (int i = 0; i < N; ++i) {
            const float w = weight_array[i], vx = P_state[4 * (size_t)i + 2], vy = P_state[4 * (size_t)i + 3];
            vel[0][i] = w * vx;
            vel[1][i] = w * vy;
            vel[2][i] = w * vx * vx;
            vel[3][i] = w * vy * vy;
            vel[4][i] = w * vx * vy;
        }
        for (int k = 0; k < 5; ++k) scan_f32(vel[k], vacc[k], (size_t)N);
#pragma omp parallel for
        for (int k = 0; k < C; ++k) {
            ref_cell* g = &cells[k];
            const float rp = g->pers_occ_mass;
            if (g->start_idx != -1 && rp > 0.0f) {
                const int s = g->start_idx, e = g->end_idx;
                const float mxv = (1.0f / rp) * ref_subtract(vacc[0], s, e);
                const float myv = (1.0f / rp) * ref_subtract(vacc[1], s, e);
                g->mean_x_vel = mxv;
                g->mean_y_vel = myv;
                g->var_x_vel = (1.0f / rp) * ref_subtract(vacc[2], s, e) - mxv * mxv;
                g->var_y_vel = (1.0f / rp) * ref_subtract(vacc[3], s, e) - myv * myv;
                g->covar_xy_vel = (1.0f / rp) * ref_subtract(vacc[4], s, e) - mxv * myv;
            } else {
                g->mean_x_vel = g->mean_y_vel = g->var_x_vel = g->var_y_vel = g->covar_xy_vel = 0.0f;
            }
        }
    }

    /* 9. resampling: multinomial over sorted uniforms (dogm.cu:386-423, resampling.cu) */
    {
        const size_t M = (size_t)N + (size_t)B;
        float* joint = (float*)malloc(sizeof(float) * M);
        memcpy(joint, weight_array, sizeof(float) * (size_t)N);
        if (B > 0) memcpy(joint + N, Bw, sizeof(float) * (size_t)B);
        scan_f32(joint, accN, M);
        const float J = accN[M - 1];
        float* rnd = (float*)malloc(sizeof(float) * (size_t)N);
        uint32_t* rbits = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)N);
#pragma omp parallel for
        for (int i = 0; i < N; ++i) {
            uint32_t o[4];
            draw_block(seed, 0u, (uint32_t)i, frame, DRAW_RESAMPLE, o);
            rnd[i] = 0.0f + (J - 0.0f) * (1.0f - u01_open0(o[0]));
            memcpy(&rbits[i], &rnd[i], 4);
        }
        radix_perm_u32(rbits, perm, (size_t)N, 32);
#pragma omp parallel for
        for (int i = 0; i < N; ++i) tmp1[i] = rnd[perm[i]];
        const float rmax = tmp1[N - 1];
        if (J != rmax) accN[M - 1] = rmax;
#pragma omp parallel for
        for (int i = 0; i < N; ++i) {
            const float x = tmp1[i];
            size_t a = 0, b = M;
            while (a < b) {
                const size_t m = (a + b) >> 1;
                if (accN[m] < x) a = m + 1; else b = m;
            }
            tmpi[i] = (int)a;
        }
        const float nw = J / (float)N;
        float* ns = (float*)malloc(16 * (size_t)N);
        int* ni = (int*)malloc(4 * (size_t)N);
        unsigned char* na = (unsigned char*)malloc((size_t)N);
#pragma omp parallel for
        for (int i = 0; i < N; ++i) {
            const int idx = tmpi[i];
            if (idx < N) {
                memcpy(ns + 4 * (size_t)i, P_state + 4 * (size_t)idx, 16);
                ni[i] = P_idx[idx];
                na[i] = P_assoc[idx];
            } else {
                const int b = idx - N < B ? idx - N : B - 1;
                memcpy(ns + 4 * (size_t)i, Bs + 4 * (size_t)b, 16);
                ni[i] = Bi[b];
                na[i] = Ba[b];
            }
        }
        /* 10. particle_array = particle_array_next (dogm.cu:128) */
        memcpy(P_state, ns, 16 * (size_t)N);
        memcpy(P_idx, ni, 4 * (size_t)N);
        memcpy(P_assoc, na, (size_t)N);
#pragma omp parallel for
        for (int i = 0; i < N; ++i) P_w[i] = nw;
        free(ns); free(ni); free(na); free(joint); free(rnd); free(rbits);
    }

    free(weight_array); free(accN); free(born); free(accC); free(Bs); free(Bi); free(Bw); free(Ba);
    free(perm); free(tmp4); free(tmp1); free(tmpi); free(tmpa);
    for (int k = 0; k < 5; ++k) { free(vel[k]); free(vacc[k]); }
    return nthreads;
}

/* ---- resampling-scan precision study (test infrastructure) ---------------------------------
 * Systematic resampling of n slots over the joint weights w[0..m): slot i takes the first item
 * j whose inclusive prefix A[j] exceeds the tooth (i + u) * A[m-1] / n, u in [0, 1) -- the comb
 * of the GB300 path, here with the prefix kept in
 *   mode 0: float32, summed sequentially (what a plain float scan gives at best),
 *   mode 1: compensated float32 -- a float pair (hi, lo) per prefix built with TwoSum, teeth
 *           and comparisons on the pair (about 48 significant bits),
 *   mode 2: float64.
 * out[i] = the item of slot i.  Merge walk, O(m + n). */
static void two_sum_f(float a, float b, float* s, float* e) {
    const float x = a + b;
    const float bv = x - a;
    *e = (a - (x - bv)) + (b - bv);
    *s = x;
}

void dogm_oracle_comb_indices(const float* w, int m, int n, double u, int mode, int* out) {
    if (m <= 0 || n <= 0) return;
    int j = 0;
    if (mode == 0) {
        float* acc = (float*)malloc(sizeof(float) * (size_t)m);
        float s = 0.0f;
        for (int k = 0; k < m; ++k) { s = s + w[k]; acc[k] = s; }
        const float step = acc[m - 1] / (float)n;
        for (int i = 0; i < n; ++i) {
            const float t = ((float)i + (float)u) * step;
            while (j < m - 1 && !(acc[j] > t)) ++j;
            out[i] = j;
        }
        free(acc);
    } else if (mode == 1) {
        float* hi = (float*)malloc(sizeof(float) * (size_t)m);
        float* lo = (float*)malloc(sizeof(float) * (size_t)m);
        float sh = 0.0f, sl = 0.0f;
        for (int k = 0; k < m; ++k) {
            float e;
            two_sum_f(sh, w[k], &sh, &e);
            sl = sl + e;
            float h2, l2;
            two_sum_f(sh, sl, &h2, &l2);  /* renormalise the pair */
            sh = h2;
            sl = l2;
            hi[k] = sh;
            lo[k] = sl;
        }
        /* tooth (i + u) * J / n with J = (hi, lo): double-float product, compared as a pair */
        const double J = (double)hi[m - 1] + (double)lo[m - 1];
        for (int i = 0; i < n; ++i) {
            const double t = ((double)i + u) * (J / (double)n);
            const float th = (float)t, tl = (float)(t - (double)th);
            while (j < m - 1 && !(hi[j] > th || (hi[j] == th && lo[j] > tl))) ++j;
            out[i] = j;
        }
        free(hi);
        free(lo);
    } else {
        double* acc = (double*)malloc(sizeof(double) * (size_t)m);
        double s = 0.0;
        for (int k = 0; k < m; ++k) { s += (double)w[k]; acc[k] = s; }
        const double step = acc[m - 1] / (double)n;
        for (int i = 0; i < n; ++i) {
            const double t = ((double)i + u) * step;
            while (j < m - 1 && !(acc[j] > t)) ++j;
            out[i] = j;
        }
        free(acc);
    }
}
