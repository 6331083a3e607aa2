/*
 * One instantiation of the update restatement, included by dogm_oracle.c with
 *   REAL  float | double      arithmetic and state type
 *   SFX   f32 | f64           function-name suffix
 *   RFMA  fmaf | fma
 *   RROUND roundf | round
 * TEST INFRASTRUCTURE ONLY (see dogm_oracle.h).
 *
 * Stage order and formulas, with the reference lines each restates:
 *   first frame    dogm.cu:217-241, init_new_particles.cu:76-124 (exact allocation)
 *   ego shift      dogm.cu:161-203, ego_motion_compensation.cu:16-43 (strict bounds)
 *   prediction     dogm.cu:243-260, predict.cu:12-48
 *   sort + ranges  dogm.cu:262-281, particle_to_grid.cu:12-40 (stable by cell)
 *   masses         mass_update.cu:12-89
 *   reweighting    update_persistent_particles.cu:16-87
 *   newborns       dogm.cu:323-348, init_new_particles.cu:18-195 (nu_A, not nu_A + 1)
 *   moments        statistical_moments.cu:16-106
 *   resampling     dogm.cu:386-423, systematic over an exact fixed-point scan
 */

#define CAT2(a, b) a##_##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SFX)

typedef struct FN(cell_out) {
    REAL m_occ_pred, w_norm, free_up, occ_up, rho_b, rho_p;
} FN(cell_out);

/* mass_update.cu:12-45 with the prediction of dogm.cu:283-298 */
static FN(cell_out) FN(cell_masses)(int n_in, REAL c, REAL free_prev, REAL alpha, REAL p_B, REAL z_free, REAL z_occ) {
    FN(cell_out) o;
    REAL m = (REAL)n_in * c;
    REAL wn = c;
    if (m > (REAL)1) {
        wn = c / m;
        m = (REAL)1;
    }
    const REAL one_m = (REAL)1 - m;
    const REAL a = alpha * free_prev;
    const REAL mf = a < one_m ? a : one_m;
    const REAL unk = one_m - mf;
    const REAL meas_unk = ((REAL)1 - z_free) - z_occ;
    const REAL K = mf * z_occ + m * z_free;
    const REAL den = (REAL)1 - K;
    const REAL occ = ((m * meas_unk + unk * z_occ) + m * z_occ) / den;
    const REAL fre = ((mf * meas_unk + unk * z_free) + mf * z_free) / den;
    const REAL pb1m = p_B * one_m;
    const REAL rb = ((occ * p_B) * one_m) / (m + pb1m);
    o.m_occ_pred = m;
    o.w_norm = wn;
    o.free_up = fre;
    o.occ_up = occ;
    o.rho_b = rb;
    o.rho_p = occ - rb;
    return o;
}

static int FN(sat_int)(REAL x) {
    if (!(x == x)) return 0;
    if (x >= (REAL)2147483647.0) return 2147483647;
    if (x <= (REAL)-2147483648.0) return (-2147483647 - 1);
    return (int)x;
}

void FN(dogm_oracle_predict)(const dogm_oracle_params* p, float dtf, const float* z, REAL* st, uint32_t* key,
                             REAL* weights, int n) {
    const REAL dt = (REAL)dtf;
    const REAL gsm1 = (REAL)(p->gs - 1);
    for (int i = 0; i < n; ++i) {
        REAL* s = st + 4 * (size_t)i;
        const REAL nx = RFMA((REAL)z[4 * (size_t)i + 0], (REAL)p->sigma_pos, (REAL)0);
        const REAL ny = RFMA((REAL)z[4 * (size_t)i + 1], (REAL)p->sigma_pos, (REAL)0);
        const REAL nvx = RFMA((REAL)z[4 * (size_t)i + 2], (REAL)p->sigma_vel, (REAL)0);
        const REAL nvy = RFMA((REAL)z[4 * (size_t)i + 3], (REAL)p->sigma_vel, (REAL)0);
        const REAL x = (s[0] + dt * s[2]) + nx;
        const REAL y = (s[1] + dt * s[3]) + ny;
        const REAL vx = s[2] + nvx;
        const REAL vy = s[3] + nvy;
        const int out = (x > gsm1) || (x < (REAL)0) || (y > gsm1) || (y < (REAL)0);
        int px = FN(sat_int)(x), py = FN(sat_int)(y);
        px = px < 0 ? 0 : (px > p->gs - 1 ? p->gs - 1 : px);
        py = py < 0 ? 0 : (py > p->gs - 1 ? p->gs - 1 : py);
        s[0] = x; s[1] = y; s[2] = vx; s[3] = vy;
        key[i] = (uint32_t)(px + p->gs * py) | (out ? OUT_BIT : 0u) | (key[i] & ASSOC_BIT);
        if (weights) weights[i] = out ? (REAL)0 : (REAL)p->p_S * weights[i];
    }
}

int FN(dogm_oracle_update)(const dogm_oracle_params* p, const dogm_oracle_frame* f, REAL* P_state, uint32_t* P_key,
                           REAL* free_mass, REAL* w_res, dogm_oracle_out* out) {
    const int gs = p->gs, N = p->N, B = p->B, C = gs * gs, S = p->q_shift;
    int rc = 0;

    /* ---- first frame: particles in proportion to the measured occupied mass ---------- */
    if (f->first_frame) {
        uint64_t T0 = 0;
        for (int k = 0; k < C; ++k) T0 += dogm_oracle_quantize((double)(REAL)f->meas[4 * (size_t)k + 1], S);
        const REAL vmax = (REAL)p->init_max_vel;
        const REAL span = vmax - (-vmax);
        uint64_t Q = 0;
        int lo = 0;
        for (int k = 0; k < C; ++k) {
            int hi;
            if (T0 == 0) {
                hi = dogm_oracle_alloc_boundary((uint64_t)(k + 1), (uint64_t)C, N);
            } else {
                Q += dogm_oracle_quantize((double)(REAL)f->meas[4 * (size_t)k + 1], S);
                hi = dogm_oracle_alloc_boundary(Q, T0, N);
            }
            for (int s = lo; s < hi; ++s) {
                REAL* st = P_state + 4 * (size_t)s;
                st[0] = (REAL)(k % gs) + (REAL)0.5;
                st[1] = (REAL)(k / gs) + (REAL)0.5;
                st[2] = RFMA(span, (REAL)1 - (REAL)f->init_u[2 * (size_t)s + 0], -vmax);
                st[3] = RFMA(span, (REAL)1 - (REAL)f->init_u[2 * (size_t)s + 1], -vmax);
                P_key[s] = (uint32_t)k;
            }
            lo = hi;
        }
        *w_res = (REAL)1 / (REAL)N;
    }

    /* ---- ego shift of the particles, then prediction --------------------------------- */
    if (f->shifted) {
        for (int i = 0; i < N; ++i) {
            P_state[4 * (size_t)i + 0] = P_state[4 * (size_t)i + 0] - (REAL)f->shift_x;
            P_state[4 * (size_t)i + 1] = P_state[4 * (size_t)i + 1] - (REAL)f->shift_y;
        }
    }
    FN(dogm_oracle_predict)(p, f->dt, f->predict_z, P_state, P_key, NULL, N);

    /* ---- stable counting sort by cell ------------------------------------------------ */
    int* cnt = (int*)calloc((size_t)C + 1, sizeof(int));
    int* perm = (int*)malloc(sizeof(int) * (size_t)N);
    REAL* S_state = (REAL*)malloc(sizeof(REAL) * 4 * (size_t)N);
    uint32_t* S_key = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)N);
    REAL* cells = (REAL*)malloc(sizeof(REAL) * 16 * (size_t)C);
    REAL* rho_b = (REAL*)malloc(sizeof(REAL) * (size_t)C);
    REAL* w_cell = (REAL*)malloc(sizeof(REAL) * (size_t)C);
    REAL* free_new = (REAL*)malloc(sizeof(REAL) * (size_t)C);
    if (!cnt || !perm || !S_state || !S_key || !cells || !rho_b || !w_cell || !free_new) { rc = -1; goto done; }
    for (int i = 0; i < N; ++i) cnt[(P_key[i] & CELL_MASK) + 1]++;
    for (int k = 0; k < C; ++k) cnt[k + 1] += cnt[k];
    {
        int* pos = (int*)malloc(sizeof(int) * (size_t)C);
        if (!pos) { rc = -1; goto done; }
        memcpy(pos, cnt, sizeof(int) * (size_t)C);
        for (int i = 0; i < N; ++i) {
            const int d = pos[P_key[i] & CELL_MASK]++;
            perm[d] = i;
            S_key[d] = P_key[i];
            memcpy(S_state + 4 * (size_t)d, P_state + 4 * (size_t)i, 4 * sizeof(REAL));
        }
        free(pos);
    }

    /* ---- per-cell update -------------------------------------------------------------- */
    {
        const REAL c_pred = (REAL)p->p_S * *w_res;
        const REAL alpha = (REAL)powf(p->freespace_discount, f->dt);
        uint64_t qb = 0, jq = 0;
        for (int k = 0; k < C; ++k) {
            const int x = k % gs, y = k / gs;
            const int start = cnt[k], end = cnt[k + 1] - 1;
            const int occupied = end >= start;
            int n_in = 0;
            REAL svx = 0, svy = 0, svxx = 0, svyy = 0, svxy = 0;
            for (int j = start; j <= end; ++j) {
                if (S_key[j] & OUT_BIT) continue;
                const REAL vx = S_state[4 * (size_t)j + 2], vy = S_state[4 * (size_t)j + 3];
                n_in++;
                svx += vx; svy += vy; svxx += vx * vx; svyy += vy * vy; svxy += vx * vy;
            }
            REAL free_prev;
            if (f->shifted) {
                const int sx = x + f->shift_x, sy = y + f->shift_y;
                free_prev = (sx > 0 && sx < gs && sy > 0 && sy < gs) ? free_mass[sx + gs * sy] : (REAL)0;
            } else {
                free_prev = free_mass[k];
            }
            const float* m = f->meas + 4 * (size_t)k;
            const REAL mfree = (REAL)m[0], mocc = (REAL)m[1], lik = (REAL)m[2], pA = (REAL)m[3];
            const FN(cell_out) o = FN(cell_masses)(n_in, c_pred, free_prev, alpha, (REAL)p->p_B, mfree, mocc);
            REAL muA = 0, muUA = 0, wp = 0, mx = 0, my = 0, vx = 0, vy = 0, cxy = 0;
            if (occupied) {
                const REAL wu = lik * o.w_norm;
                const REAL swu = (REAL)n_in * wu;
                muA = swu > (REAL)0 ? o.rho_p / swu : (REAL)0;
                muUA = o.m_occ_pred > (REAL)0 ? o.rho_p / o.m_occ_pred : (REAL)0;
                wp = (pA * muA) * wu + (((REAL)1 - pA) * muUA) * o.w_norm;
                if (o.rho_p > (REAL)0) {
                    const REAL inv = (REAL)1 / o.rho_p;
                    mx = inv * (wp * svx);
                    my = inv * (wp * svy);
                    vx = inv * (wp * svxx) - mx * mx;
                    vy = inv * (wp * svyy) - my * my;
                    cxy = inv * (wp * svxy) - mx * my;
                }
            }
            REAL* rec = cells + 16 * (size_t)k;
            rec[0] = occupied ? (REAL)start : (REAL)-1;
            rec[1] = occupied ? (REAL)end : (REAL)-1;
            rec[2] = o.rho_b; rec[3] = o.rho_p; rec[4] = o.free_up; rec[5] = o.occ_up; rec[6] = o.m_occ_pred;
            rec[7] = muA; rec[8] = muUA; rec[9] = 0; rec[10] = 0;
            rec[11] = mx; rec[12] = my; rec[13] = vx; rec[14] = vy; rec[15] = cxy;
            free_new[k] = o.free_up;
            rho_b[k] = o.rho_b;
            w_cell[k] = wp;
            qb += dogm_oracle_quantize((double)o.rho_b, S);
            jq += (uint64_t)n_in * dogm_oracle_quantize((double)wp, S);
        }

        /* ---- newborns: slots over the exact scan of quantised newborn masses ----------- */
        const uint64_t T = qb;
        const int n_birth = (T > 0) ? B : 0;
        REAL* B_state = (REAL*)calloc((size_t)(B > 0 ? B : 1) * 4, sizeof(REAL));
        uint32_t* B_key = (uint32_t*)calloc((size_t)(B > 0 ? B : 1), sizeof(uint32_t));
        REAL* B_w = (REAL*)calloc((size_t)(B > 0 ? B : 1), sizeof(REAL));
        if (!B_state || !B_key || !B_w) { rc = -1; goto done; }
        {
            uint64_t Q = 0;
            int lo = 0;
            for (int k = 0; k < C; ++k) {
                Q += dogm_oracle_quantize((double)rho_b[k], S);
                const int hi = dogm_oracle_alloc_boundary(Q, T, B);
                const int nnew = hi - lo;
                if (nnew > 0) {
                    const REAL pA = (REAL)f->meas[4 * (size_t)k + 3];
                    const int nuA = (int)RROUND((REAL)nnew * pA);
                    const int nuUA = nnew - nuA;
                    const REAL wA = nuA > 0 ? (pA * rho_b[k]) / (REAL)nuA : (REAL)0;
                    const REAL wUA = nuUA > 0 ? (((REAL)1 - pA) * rho_b[k]) / (REAL)nuUA : (REAL)0;
                    cells[16 * (size_t)k + 9] = wA;
                    cells[16 * (size_t)k + 10] = wUA;
                    jq += (uint64_t)(nuA > 0 ? nuA : 0) * dogm_oracle_quantize((double)wA, S) +
                          (uint64_t)(nuUA > 0 ? nuUA : 0) * dogm_oracle_quantize((double)wUA, S);
                    for (int s = lo; s < hi; ++s) {
                        const int assoc = (s - lo) < nuA;
                        REAL* st = B_state + 4 * (size_t)s;
                        st[0] = (REAL)(k % gs) + (REAL)0.5;
                        st[1] = (REAL)k / (REAL)gs + (REAL)0.5;
                        st[2] = RFMA((REAL)f->birth_z[2 * (size_t)s + 0], (REAL)p->sigma_birth, (REAL)0);
                        st[3] = RFMA((REAL)f->birth_z[2 * (size_t)s + 1], (REAL)p->sigma_birth, (REAL)0);
                        B_key[s] = (uint32_t)k | (assoc ? ASSOC_BIT : 0u);
                        B_w[s] = assoc ? wA : wUA;
                    }
                }
                lo = hi;
            }
        }

        /* ---- systematic resampling over the exact joint scan ---------------------------- */
        {
            const uint64_t TJ = jq;
            const uint64_t U = (uint64_t)(((unsigned __int128)f->resample_r * TJ) >> 64);
            const int M = N + n_birth;
            uint64_t A = 0;
            int lo = 0;
            for (int j = 0; j < M; ++j) {
                REAL w;
                const REAL* src;
                uint32_t kw;
                if (j < N) {
                    kw = S_key[j];
                    w = (kw & OUT_BIT) ? (REAL)0 : w_cell[kw & CELL_MASK];
                    src = S_state + 4 * (size_t)j;
                } else {
                    kw = B_key[j - N];
                    w = B_w[j - N];
                    src = B_state + 4 * (size_t)(j - N);
                }
                A += dogm_oracle_quantize((double)w, S);
                const int hi = dogm_oracle_comb_count(A, TJ, U, N);
                for (int s = (j == 0 ? 0 : lo); s < hi; ++s) {
                    memcpy(P_state + 4 * (size_t)s, src, 4 * sizeof(REAL));
                    P_key[s] = kw & ~OUT_BIT;
                    if (out && out->res_src) out->res_src[s] = j;
                }
                lo = hi;
            }
            /* w_res = T / N in the arithmetic of the instantiation */
            *w_res = (REAL)LDEXP((REAL)TJ, -S) / (REAL)N;
            if (out) {
                out->joint_total = TJ;
                out->qb_total = T;
                out->n_birth = n_birth;
                if (out->B_state) memcpy(out->B_state, B_state, sizeof(REAL) * 4 * (size_t)B);
                if (out->B_key) memcpy(out->B_key, B_key, sizeof(uint32_t) * (size_t)B);
                if (out->B_w) memcpy(out->B_w, B_w, sizeof(REAL) * (size_t)B);
            }
        }
        free(B_state);
        free(B_key);
        free(B_w);
    }
    memcpy(free_mass, free_new, sizeof(REAL) * (size_t)C);
    if (out) {
        if (out->cells) memcpy(out->cells, cells, sizeof(REAL) * 16 * (size_t)C);
        if (out->S_state) memcpy(out->S_state, S_state, sizeof(REAL) * 4 * (size_t)N);
        if (out->S_key) memcpy(out->S_key, S_key, sizeof(uint32_t) * (size_t)N);
        if (out->perm) memcpy(out->perm, perm, sizeof(int) * (size_t)N);
    }
done:
    free(cnt); free(perm); free(S_state); free(S_key); free(cells); free(rho_b); free(w_cell); free(free_new);
    return rc;
}

#undef FN
#undef CAT
#undef CAT2
