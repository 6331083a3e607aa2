// ref_harness.cu -- TEST INFRASTRUCTURE ONLY: runs the reference's own CUDA build so that the
// tests can pin the GB300 path against it and the bench can time it.  Never part of the
// product path.
//
// The reference's device code comes from its own sources: oracle/ref/build_ref.py compiles
// every file of dogm/src/kernel/ into an sm_103a cubin under oracle/_ref/, loaded here with
// the CUDA driver API.  Kernels are found by enumerating each module's functions
// (cuModuleEnumerateFunctions / cuFuncGetName) and matching the mangled name of
// dogm::<kernel>.  The reference's host code (class dogm::DOGM, dogm/src/dogm.cu) cannot be
// built without its sources, so its sequence is restated below, stage by stage, with the
// same launch geometry, the same Thrust calls (the CUDA toolkit's Thrust, as the reference
// uses), the same device temporaries, host synchronisations and legacy default stream.
//
// Random draws: the reference draws from curand XORWOW states (seed 123456, subsequence =
// thread, dogm/src/dogm.cu:101).  For replay, a capture kernel copies the states and calls
// curand in the same thread / grid-stride order as the reference kernel that is about to
// run, recording the raw draws without advancing the reference's states.
#include <cuda.h>
#include <cuda_runtime.h>
#include <curand_kernel.h>
#include <thrust/binary_search.h>
#include <thrust/device_ptr.h>
#include <thrust/device_vector.h>
#include <thrust/iterator/zip_iterator.h>
#include <thrust/scan.h>
#include <thrust/sort.h>
#include <thrust/transform.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace dogm_ref_types {

// ---- the reference's types, ABI-identical (dogm/include/dogm/dogm_types.h:13-144) ----------
struct RVec4 { float x, y, z, w; };
struct RGridCell {
    int start_idx, end_idx;
    float new_born_occ_mass, pers_occ_mass, free_mass, occ_mass, pred_occ_mass, mu_A, mu_UA, w_A, w_UA;
    float mean_x_vel, mean_y_vel, var_x_vel, var_y_vel, covar_xy_vel;
};
struct RMeas { float free_mass, occ_mass, likelihood, p_A; };
struct RParticle { int grid_cell_idx; float weight; bool associated; RVec4 state; };  // sizeof 28
struct RSoA {  // ParticlesSoA: the pointer block, then memory_block, size, device
    RVec4* state;
    int* grid_cell_idx;
    float* weight;
    bool* associated;
    void* memory_block;
    int size;
    bool device;
};
struct RMat4 { float v[16]; };  // glm::mat4x4: four columns
static_assert(sizeof(RParticle) == 28, "Particle layout");
static_assert(sizeof(RSoA) == 48, "ParticlesSoA layout");
static_assert(sizeof(RGridCell) == 64 && sizeof(RMeas) == 16, "cell layouts");

struct RParams {  // dogm::DOGM::Params (dogm/include/dogm/dogm.h:26-60)
    float size, resolution;
    int particle_count, new_born_particle_count;
    float persistence_prob, stddev_process_noise_position, stddev_process_noise_velocity, birth_prob,
        stddev_velocity, init_max_velocity, freespace_discount;
};

}  // namespace dogm_ref_types

using namespace dogm_ref_types;

namespace {

// ---- kernel table --------------------------------------------------------------------------
enum Kern {
    kSetupRng, kInitGrid, kInitBirth, kReinitIdx, kMoveParticles, kMoveMap, kPredict, kP2G, kMassUpdate, kUpd1,
    kUpd2, kUpd3, kCopyMasses, kInit1, kInit2, kNew1, kNew2, kMom1, kMom2, kResRand, kResample, kNumKern
};
const char* const kKernName[kNumKern] = {
    "setupRandomStatesKernel", "initGridCellsKernel", "initBirthParticlesKernel", "reinitGridParticleIndices",
    "moveParticlesKernel", "moveMapKernel", "predictKernel", "particleToGridKernel", "gridCellPredictionUpdateKernel",
    "updatePersistentParticlesKernel1", "updatePersistentParticlesKernel2", "updatePersistentParticlesKernel3",
    "copyMassesKernel", "initParticlesKernel1", "initParticlesKernel2", "initNewParticlesKernel1",
    "initNewParticlesKernel2", "statisticalMomentsKernel1", "statisticalMomentsKernel2",
    "resamplingGenerateRandomNumbersKernel", "resamplingKernel"};
const char* const kKernFile[kNumKern] = {
    "init", "init", "init", "init", "ego_motion_compensation", "ego_motion_compensation", "predict",
    "particle_to_grid", "mass_update", "update_persistent_particles", "update_persistent_particles",
    "update_persistent_particles", "init_new_particles", "init_new_particles", "init_new_particles",
    "init_new_particles", "init_new_particles", "statistical_moments", "statistical_moments", "resampling",
    "resampling"};

CUfunction g_fn[kNumKern] = {};
bool g_loaded = false;
std::string g_err;

int fail(const std::string& m) {
    g_err = m;
    return 1;
}

#define RCU(call)                                                                                   \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) return fail(std::string(#call) + ": " + cudaGetErrorString(e_));     \
    } while (0)
#define RDRV(call)                                                                                  \
    do {                                                                                            \
        CUresult r_ = (call);                                                                       \
        if (r_ != CUDA_SUCCESS) {                                                                   \
            const char* s_ = nullptr;                                                               \
            cuGetErrorString(r_, &s_);                                                              \
            return fail(std::string(#call) + ": " + (s_ ? s_ : "driver error"));                   \
        }                                                                                           \
    } while (0)

// Launch on the legacy default stream (the reference launches with <<<grid, block>>>).
template <class... A>
int launch(Kern k, dim3 grid, dim3 block, A... args) {
    void* p[] = {(void*)&args...};
    RDRV(cuLaunchKernel(g_fn[k], grid.x, grid.y, grid.z, block.x, block.y, block.z, 0, nullptr, p, nullptr));
    return 0;
}
#define LAUNCH(...) do { if (launch(__VA_ARGS__)) return 1; } while (0)

int div_up(int a, int b) { return (a + b - 1) / b; }

// ---- draw capture (own kernels; curand is called, not re-implemented) ----------------------
// kind 0: n x 4 normals (predictKernel), 1: n x 2 normals (initNewParticlesKernel2),
// 2: n x 2 uniforms (initParticlesKernel2), 3: n uniforms (resamplingGenerateRandomNumbersKernel)
__global__ void capture_draws(const curandState* __restrict__ states, int kind, int count, float* __restrict__ out) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = blockDim.x * gridDim.x;
    curandState s = states[tid];
    for (int i = tid; i < count; i += stride) {
        if (kind == 0) {
            for (int j = 0; j < 4; ++j) out[4 * (size_t)i + j] = curand_normal(&s);
        } else if (kind == 1) {
            for (int j = 0; j < 2; ++j) out[2 * (size_t)i + j] = curand_normal(&s);
        } else if (kind == 2) {
            for (int j = 0; j < 2; ++j) out[2 * (size_t)i + j] = curand_uniform(&s);
        } else {
            out[i] = curand_uniform(&s);
        }
    }
}

// normalize_particle_orders (init_new_particles.cu:66-74): x * (v_B / max)
struct ScaleOrders {
    int v_B;
    float max;
    __host__ __device__ float operator()(float x) const { return x * (v_B / max); }
};

}  // namespace

// Per-update trace for the parity tests (host buffers; NULL skips an item).
struct dogm_ref_trace {
    float* predict_z;     // N x 4 raw normals the predict step draws
    float* birth_z;       // B x 2 raw normals of the newborn velocities
    float* init_u;        // N x 2 raw uniforms of the first-frame velocities
    float* resample_u;    // N raw uniforms of the resampling draws
    float* sorted_state;  // N x 4 after the sort by cell
    int* sorted_idx;      // N cell index after the sort
    float* joint_accum;   // N + B inclusive scan of the joint weights (before the last-value clamp)
    float* rand_sorted;   // N sorted resampling numbers
    int* resample_idx;    // N lower_bound indices
    float* weight_array;  // N reweighted persistent weights (after updatePersistentParticlesKernel3)
};

struct dogm_ref {
    RParams p{};
    int gs = 0, N = 0, B = 0, C = 0;
    dim3 pgrid, block{256};
    RSoA P{}, Pn{}, Bp{};
    RGridCell* cells = nullptr;
    RMeas* meas = nullptr;
    float *weight_array = nullptr, *birth_weight_array = nullptr, *born_masses = nullptr, *rand_array = nullptr;
    float* vel[5] = {};
    curandState* rng = nullptr;
    curandState* rng_copy = nullptr;
    float* capture = nullptr;
    bool first_pose = false, first_meas = false;
    float px = 0.f, py = 0.f, yaw = 0.f;
    dogm_ref_trace* tr = nullptr;
};

namespace {

int soa_init(RSoA& s, int n) {  // ParticlesSoA::init + assignPointers (dogm_types.h:69-85,137-143)
    s.size = n;
    s.device = true;
    RCU(cudaMalloc(&s.memory_block, (size_t)n * sizeof(RParticle)));
    s.state = reinterpret_cast<RVec4*>(s.memory_block);
    s.grid_cell_idx = reinterpret_cast<int*>(s.state + n);
    s.weight = reinterpret_cast<float*>(s.grid_cell_idx + n);
    s.associated = reinterpret_cast<bool*>(s.weight + n);
    return 0;
}

int capture(dogm_ref* d, int kind, int count, float* host_out) {
    if (!host_out || count <= 0) return 0;
    const int per = kind == 0 ? 4 : (kind == 3 ? 1 : 2);
    const size_t T = (size_t)d->pgrid.x * d->block.x;
    RCU(cudaMemcpy(d->rng_copy, d->rng, T * sizeof(curandState), cudaMemcpyDeviceToDevice));
    capture_draws<<<d->pgrid, d->block>>>(d->rng_copy, kind, count, d->capture);
    RCU(cudaGetLastError());
    RCU(cudaMemcpy(host_out, d->capture, (size_t)count * per * sizeof(float), cudaMemcpyDeviceToHost));
    return 0;
}

int normalize_orders(float* acc, int count, int v_B) {  // init_new_particles.cu:66-74
    thrust::device_ptr<float> a(acc);
    float mx = 1.0f;
    RCU(cudaMemcpy(&mx, acc + count - 1, sizeof(float), cudaMemcpyDeviceToHost));
    thrust::transform(a, a + count, a, ScaleOrders{v_B, mx});
    return 0;
}

// DOGM::initializeParticles (dogm.cu:217-241)
int initialize_particles(dogm_ref* d) {
    LAUNCH(kCopyMasses, d->pgrid, d->block, (const RMeas*)d->meas, d->born_masses, d->C);
    RCU(cudaDeviceSynchronize());
    thrust::device_vector<float> acc(d->C);
    thrust::inclusive_scan(thrust::device_ptr<float>(d->born_masses), thrust::device_ptr<float>(d->born_masses) + d->C,
                           acc.begin());
    float* accp = thrust::raw_pointer_cast(acc.data());
    const float new_weight = 1.0f / d->N;
    if (normalize_orders(accp, d->C, d->N)) return 1;
    LAUNCH(kInit1, d->pgrid, d->block, d->cells, (const RMeas*)d->meas, d->P, (const float*)accp, d->C);
    if (d->tr && capture(d, 2, d->N, d->tr->init_u)) return 1;
    LAUNCH(kInit2, d->pgrid, d->block, d->P, (const RGridCell*)d->cells, d->rng, d->p.init_max_velocity, d->gs,
           new_weight, d->N);
    return 0;
}

// DOGM::updatePose (dogm.cu:161-203)
int update_pose(dogm_ref* d, float x, float y, float yaw) {
    if (!d->first_pose) {
        d->px = x; d->py = y; d->yaw = yaw;
        d->first_pose = true;
        return 0;
    }
    const float dx = x - d->px, dy = y - d->py;
    if (fabsf(dx) > d->p.resolution || fabsf(dy) > d->p.resolution) {
        const int xm = -static_cast<int>(dx / d->p.resolution);
        const int ym = -static_cast<int>(dy / d->p.resolution);
        RGridCell* old = nullptr;
        RCU(cudaMalloc(&old, (size_t)d->C * sizeof(RGridCell)));
        RCU(cudaMemcpy(old, d->cells, (size_t)d->C * sizeof(RGridCell), cudaMemcpyDeviceToDevice));
        RCU(cudaMemset(d->cells, 0, (size_t)d->C * sizeof(RGridCell)));
        const dim3 b2(32, 32), g2(div_up(d->gs, 32), div_up(d->gs, 32));
        LAUNCH(kMoveParticles, d->pgrid, d->block, d->P, xm, ym, d->N);
        LAUNCH(kMoveMap, g2, b2, d->cells, (const RGridCell*)old, xm, ym, d->gs);
        RCU(cudaFree(old));
        d->px = x; d->py = y; d->yaw = yaw;
    }
    return 0;
}

// DOGM::particlePrediction (dogm.cu:243-260): transpose of the column-major constructor
// (1,0,dt,0, 0,1,0,dt, 0,0,1,0, 0,0,0,1) -> columns (1,0,0,0) (0,1,0,0) (dt,0,1,0) (0,dt,0,1)
int predict(dogm_ref* d, float dt) {
    RMat4 F{{1, 0, 0, 0, 0, 1, 0, 0, dt, 0, 1, 0, 0, dt, 0, 1}};
    if (d->tr && capture(d, 0, d->N, d->tr->predict_z)) return 1;
    LAUNCH(kPredict, d->pgrid, d->block, d->P, d->rng, d->p.stddev_velocity, d->gs, d->p.persistence_prob, F,
           d->p.stddev_process_noise_position, d->p.stddev_process_noise_velocity, d->N);
    return 0;
}

// DOGM::particleAssignment (dogm.cu:262-281)
int assignment(dogm_ref* d) {
    LAUNCH(kReinitIdx, d->pgrid, d->block, d->cells, d->C);
    thrust::device_ptr<int> key(d->P.grid_cell_idx);
    auto payload = thrust::make_zip_iterator(thrust::make_tuple(thrust::device_ptr<float>(d->P.weight),
                                                                thrust::device_ptr<bool>(d->P.associated),
                                                                thrust::device_ptr<RVec4>(d->P.state)));
    thrust::sort_by_key(key, key + d->N, payload);
    LAUNCH(kP2G, d->pgrid, d->block, d->P, d->cells, d->weight_array, d->N);
    if (d->tr && d->tr->sorted_state)
        RCU(cudaMemcpy(d->tr->sorted_state, d->P.state, (size_t)d->N * 16, cudaMemcpyDeviceToHost));
    if (d->tr && d->tr->sorted_idx)
        RCU(cudaMemcpy(d->tr->sorted_idx, d->P.grid_cell_idx, (size_t)d->N * 4, cudaMemcpyDeviceToHost));
    return 0;
}

// DOGM::gridCellOccupancyUpdate (dogm.cu:283-298)
int occupancy_update(dogm_ref* d, float dt) {
    thrust::device_vector<float> acc(d->N);
    thrust::inclusive_scan(thrust::device_ptr<float>(d->weight_array), thrust::device_ptr<float>(d->weight_array) + d->N,
                           acc.begin());
    const float* accp = thrust::raw_pointer_cast(acc.data());
    const float discount = std::pow(d->p.freespace_discount, dt);
    LAUNCH(kMassUpdate, d->pgrid, d->block, d->cells, d->P, d->weight_array, accp, (const RMeas*)d->meas,
           d->born_masses, d->p.birth_prob, discount, d->C);
    return 0;
}

// DOGM::updatePersistentParticles (dogm.cu:300-321)
int persistent_update(dogm_ref* d) {
    LAUNCH(kUpd1, d->pgrid, d->block, d->P, (const RMeas*)d->meas, d->weight_array, d->N);
    thrust::device_vector<float> acc(d->N);
    thrust::inclusive_scan(thrust::device_ptr<float>(d->weight_array), thrust::device_ptr<float>(d->weight_array) + d->N,
                           acc.begin());
    const float* accp = thrust::raw_pointer_cast(acc.data());
    LAUNCH(kUpd2, dim3(div_up(d->C, 256)), dim3(256), d->cells, accp, d->C);
    LAUNCH(kUpd3, d->pgrid, d->block, d->P, (const RMeas*)d->meas, (const RGridCell*)d->cells, d->weight_array, d->N);
    if (d->tr && d->tr->weight_array)
        RCU(cudaMemcpy(d->tr->weight_array, d->weight_array, (size_t)d->N * 4, cudaMemcpyDeviceToHost));
    return 0;
}

// DOGM::initializeNewParticles (dogm.cu:323-348)
int new_particles(dogm_ref* d) {
    if (d->B <= 0) return fail("new_born_particle_count must be > 0");
    LAUNCH(kInitBirth, d->pgrid, d->block, d->Bp, d->rng, d->p.stddev_velocity, d->gs, d->B);
    thrust::device_vector<float> acc(d->C);
    thrust::inclusive_scan(thrust::device_ptr<float>(d->born_masses), thrust::device_ptr<float>(d->born_masses) + d->C,
                           acc.begin());
    float* accp = thrust::raw_pointer_cast(acc.data());
    if (normalize_orders(accp, d->C, d->B)) return 1;
    LAUNCH(kNew1, d->pgrid, d->block, d->cells, (const RMeas*)d->meas, (const float*)d->weight_array,
           (const float*)d->born_masses, d->Bp, (const float*)accp, d->C);
    if (d->tr && capture(d, 1, d->B, d->tr->birth_z)) return 1;
    LAUNCH(kNew2, d->pgrid, d->block, d->Bp, (const RGridCell*)d->cells, d->rng, d->p.stddev_velocity,
           d->p.init_max_velocity, d->gs, d->B);
    return 0;
}

// DOGM::statisticalMoments (dogm.cu:350-384)
int moments(dogm_ref* d) {
    LAUNCH(kMom1, d->pgrid, d->block, d->P, (const float*)d->weight_array, d->vel[0], d->vel[1], d->vel[2],
           d->vel[3], d->vel[4], d->N);
    thrust::device_vector<float> acc[5];
    const float* accp[5];
    for (int i = 0; i < 5; ++i) {
        acc[i].resize(d->N);
        thrust::inclusive_scan(thrust::device_ptr<float>(d->vel[i]), thrust::device_ptr<float>(d->vel[i]) + d->N,
                               acc[i].begin());
        accp[i] = thrust::raw_pointer_cast(acc[i].data());
    }
    LAUNCH(kMom2, d->pgrid, d->block, d->cells, accp[0], accp[1], accp[2], accp[3], accp[4], d->C);
    return 0;
}

// DOGM::resampling (dogm.cu:386-423) with calc_resampled_indices (resampling.cu:34-47)
int resampling(dogm_ref* d) {
    thrust::device_ptr<float> pw(d->weight_array), bw(d->Bp.weight);
    thrust::device_vector<float> joint;
    joint.insert(joint.end(), pw, pw + d->N);
    joint.insert(joint.end(), bw, bw + d->B);
    thrust::device_vector<float> jacc(joint.size());
    thrust::inclusive_scan(joint.begin(), joint.end(), jacc.begin());
    const float joint_max = jacc.back();
    if (d->tr && d->tr->joint_accum)
        RCU(cudaMemcpy(d->tr->joint_accum, thrust::raw_pointer_cast(jacc.data()), jacc.size() * 4,
                       cudaMemcpyDeviceToHost));
    if (d->tr && capture(d, 3, d->N, d->tr->resample_u)) return 1;
    LAUNCH(kResRand, d->pgrid, d->block, d->rand_array, d->rng, joint_max, d->N);
    thrust::device_ptr<float> rp(d->rand_array);
    thrust::device_vector<float> rv(rp, rp + d->N);
    thrust::sort(rv.begin(), rv.end());
    thrust::device_vector<int> idx(d->N);
    const float rand_max = rv.back();
    if (joint_max != rand_max) jacc.back() = rand_max;
    thrust::lower_bound(jacc.begin(), jacc.end(), rv.begin(), rv.end(), idx.begin());
    if (d->tr && d->tr->rand_sorted)
        RCU(cudaMemcpy(d->tr->rand_sorted, thrust::raw_pointer_cast(rv.data()), (size_t)d->N * 4,
                       cudaMemcpyDeviceToHost));
    if (d->tr && d->tr->resample_idx)
        RCU(cudaMemcpy(d->tr->resample_idx, thrust::raw_pointer_cast(idx.data()), (size_t)d->N * 4,
                       cudaMemcpyDeviceToHost));
    const float new_weight = joint_max / d->N;
    LAUNCH(kResample, d->pgrid, d->block, d->P, d->Pn, d->Bp, (const int*)thrust::raw_pointer_cast(idx.data()),
           new_weight, d->N);
    return 0;
}

}  // namespace

extern "C" {

const char* dogm_ref_last_error(void) { return g_err.c_str(); }

// Loads the nine reference modules from cubin_dir and resolves every kernel.
int dogm_ref_load(const char* cubin_dir) {
    if (g_loaded) return 0;
    RCU(cudaFree(0));  // the primary context the runtime calls below use as well
    RDRV(cuInit(0));
    for (int k = 0; k < kNumKern; ++k) {
        const std::string path = std::string(cubin_dir) + "/" + kKernFile[k] + ".cubin";
        CUmodule mod;
        RDRV(cuModuleLoad(&mod, path.c_str()));
        unsigned int n = 0;
        RDRV(cuModuleGetFunctionCount(&n, mod));
        std::vector<CUfunction> fns(n);
        RDRV(cuModuleEnumerateFunctions(fns.data(), n, mod));
        // Itanium mangling of dogm::<name>(...): "4dogm" <length> <name> "E"
        const std::string want = "4dogm" + std::to_string(std::strlen(kKernName[k])) + kKernName[k] + "E";
        for (CUfunction f : fns) {
            const char* name = nullptr;
            if (cuFuncGetName(&name, f) == CUDA_SUCCESS && name && std::strstr(name, want.c_str())) g_fn[k] = f;
        }
        if (!g_fn[k]) return fail(std::string("kernel ") + kKernName[k] + " not found in " + path);
    }
    g_loaded = true;
    return 0;
}

// DOGM::DOGM + initialize (dogm.cu:33-71, 95-113).  params: the 11 fields of Params.
int dogm_ref_create(const RParams* params, dogm_ref** out) {
    if (!g_loaded) return fail("dogm_ref_load first");
    dogm_ref* d = new dogm_ref();
    *out = nullptr;
    d->p = *params;
    d->gs = static_cast<int>(d->p.size / d->p.resolution);
    d->N = d->p.particle_count;
    d->B = d->p.new_born_particle_count;
    d->C = d->gs * d->gs;
    int dev = 0;
    RCU(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    RCU(cudaGetDeviceProperties(&prop, dev));
    d->pgrid = dim3(prop.multiProcessorCount * (prop.maxThreadsPerMultiProcessor / 256));
    if (soa_init(d->P, d->N) || soa_init(d->Pn, d->N) || soa_init(d->Bp, std::max(d->B, 1))) return 1;
    RCU(cudaMalloc(&d->cells, (size_t)d->C * sizeof(RGridCell)));
    RCU(cudaMalloc(&d->meas, (size_t)d->C * sizeof(RMeas)));
    RCU(cudaMalloc(&d->weight_array, (size_t)d->N * 4));
    RCU(cudaMalloc(&d->birth_weight_array, (size_t)std::max(d->B, 1) * 4));
    RCU(cudaMalloc(&d->born_masses, (size_t)d->C * 4));
    for (auto& v : d->vel) RCU(cudaMalloc(&v, (size_t)d->N * 4));
    RCU(cudaMalloc(&d->rand_array, (size_t)d->N * 4));
    const size_t T = (size_t)d->pgrid.x * d->block.x;
    RCU(cudaMalloc(&d->rng, T * sizeof(curandState)));
    RCU(cudaMalloc(&d->rng_copy, T * sizeof(curandState)));
    RCU(cudaMalloc(&d->capture, (size_t)std::max(4 * d->N, 2 * std::max(d->B, 1)) * 4));
    // Zeroed here (the reference leaves cudaMalloc's contents): initNewParticlesKernel2 reads
    // grid_cell_idx of every newborn slot (init_new_particles.cu:167-168), and a slot that the
    // float allocation leaves unassigned would otherwise index the cells with whatever the
    // allocation held.  With zeroed blocks such a slot reads cell 0 (or last frame's cell).
    for (RSoA* s : {&d->P, &d->Pn, &d->Bp})
        RCU(cudaMemset(s->memory_block, 0, (size_t)std::max(s->size, 1) * sizeof(RParticle)));
    RCU(cudaMemset(d->cells, 0, (size_t)d->C * sizeof(RGridCell)));
    RCU(cudaMemset(d->born_masses, 0, (size_t)d->C * 4));
    RCU(cudaMemset(d->weight_array, 0, (size_t)d->N * 4));
    LAUNCH(kSetupRng, d->pgrid, d->block, d->rng, 123456ull, (int)T);
    RCU(cudaDeviceSynchronize());
    LAUNCH(kInitGrid, d->pgrid, d->block, d->cells, d->meas, d->gs, d->C);
    RCU(cudaDeviceSynchronize());
    *out = d;
    return 0;
}

int dogm_ref_destroy(dogm_ref* d) {
    if (!d) return 0;
    cudaDeviceSynchronize();
    for (void* q : {d->P.memory_block, d->Pn.memory_block, d->Bp.memory_block, (void*)d->cells, (void*)d->meas,
                    (void*)d->weight_array, (void*)d->birth_weight_array, (void*)d->born_masses, (void*)d->rand_array,
                    (void*)d->rng, (void*)d->rng_copy, (void*)d->capture})
        cudaFree(q);
    for (auto v : d->vel) cudaFree(v);
    delete d;
    return 0;
}

// DOGM::updateGrid (dogm.cu:115-131).  meas: grid_size^2 cells, device pointer if device != 0.
// trace may be NULL.
int dogm_ref_update(dogm_ref* d, const RMeas* meas, float x, float y, float yaw, float dt, int device,
                    dogm_ref_trace* trace) {
    d->tr = trace;
    RCU(cudaMemcpy(d->meas, meas, (size_t)d->C * sizeof(RMeas),
                   device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
    if (!d->first_meas) {
        if (initialize_particles(d)) return 1;
        d->first_meas = true;
    }
    if (update_pose(d, x, y, yaw) || predict(d, dt) || assignment(d) || occupancy_update(d, dt) ||
        persistent_update(d) || new_particles(d) || moments(d) || resampling(d))
        return 1;
    // particle_array = particle_array_next (dogm.cu:128): a copy of the whole block
    RCU(cudaMemcpy(d->P.memory_block, d->Pn.memory_block, (size_t)d->N * sizeof(RParticle), cudaMemcpyDeviceToDevice));
    RCU(cudaDeviceSynchronize());
    d->tr = nullptr;
    return 0;
}

// Test hooks: overwrite the particles (skips the first-measurement initialisation from now
// on) and read the state back.
int dogm_ref_set_particles(dogm_ref* d, const float* state, const int* idx, const float* weight,
                           const unsigned char* assoc) {
    const size_t n = (size_t)d->N;
    RCU(cudaMemcpy(d->P.state, state, n * 16, cudaMemcpyHostToDevice));
    RCU(cudaMemcpy(d->P.grid_cell_idx, idx, n * 4, cudaMemcpyHostToDevice));
    RCU(cudaMemcpy(d->P.weight, weight, n * 4, cudaMemcpyHostToDevice));
    std::vector<char> a(n);
    for (size_t i = 0; i < n; ++i) a[i] = assoc[i] ? 1 : 0;
    RCU(cudaMemcpy(d->P.associated, a.data(), n, cudaMemcpyHostToDevice));
    d->first_meas = true;
    return 0;
}

int dogm_ref_get_particles(dogm_ref* d, float* state, int* idx, float* weight, unsigned char* assoc) {
    const size_t n = (size_t)d->N;
    if (state) RCU(cudaMemcpy(state, d->P.state, n * 16, cudaMemcpyDeviceToHost));
    if (idx) RCU(cudaMemcpy(idx, d->P.grid_cell_idx, n * 4, cudaMemcpyDeviceToHost));
    if (weight) RCU(cudaMemcpy(weight, d->P.weight, n * 4, cudaMemcpyDeviceToHost));
    if (assoc) {
        std::vector<char> a(n);
        RCU(cudaMemcpy(a.data(), d->P.associated, n, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; ++i) assoc[i] = a[i] ? 1 : 0;
    }
    return 0;
}

int dogm_ref_get_cells(dogm_ref* d, RGridCell* out) {
    RCU(cudaMemcpy(out, d->cells, (size_t)d->C * sizeof(RGridCell), cudaMemcpyDeviceToHost));
    return 0;
}

int dogm_ref_get_birth(dogm_ref* d, float* state, int* idx, float* weight, unsigned char* assoc) {
    const size_t n = (size_t)d->B;
    if (state) RCU(cudaMemcpy(state, d->Bp.state, n * 16, cudaMemcpyDeviceToHost));
    if (idx) RCU(cudaMemcpy(idx, d->Bp.grid_cell_idx, n * 4, cudaMemcpyDeviceToHost));
    if (weight) RCU(cudaMemcpy(weight, d->Bp.weight, n * 4, cudaMemcpyDeviceToHost));
    if (assoc) {
        std::vector<char> a(n);
        RCU(cudaMemcpy(a.data(), d->Bp.associated, n, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; ++i) assoc[i] = a[i] ? 1 : 0;
    }
    return 0;
}

int dogm_ref_grid_size(const dogm_ref* d) { return d->gs; }
int dogm_ref_rng_threads(const dogm_ref* d) { return (int)(d->pgrid.x * d->block.x); }

// ---- the demo's measurement-grid kernels (dogm/demo/simulator/mapping/kernel/
// measurement_grid.cu), compiled from their source into oracle/_ref/measurement_grid.cubin ----
static CUfunction g_meas_fn[3] = {};  // createPolarGridTexture, fusePolarGridTexture, cartesianGridToMeasurementGrid

int dogm_ref_meas_load(const char* cubin_path) {
    if (g_meas_fn[0]) return 0;
    RCU(cudaFree(0));
    RDRV(cuInit(0));
    CUmodule mod;
    RDRV(cuModuleLoad(&mod, cubin_path));
    unsigned int n = 0;
    RDRV(cuModuleGetFunctionCount(&n, mod));
    std::vector<CUfunction> fns(n);
    RDRV(cuModuleEnumerateFunctions(fns.data(), n, mod));
    const char* want[3] = {"createPolarGridTextureKernel", "fusePolarGridTextureKernel",
                           "cartesianGridToMeasurementGridKernel"};
    for (CUfunction f : fns) {
        const char* name = nullptr;
        if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name) continue;
        for (int k = 0; k < 3; ++k)
            if (std::strstr(name, want[k])) g_meas_fn[k] = f;
    }
    for (int k = 0; k < 3; ++k)
        if (!g_meas_fn[k]) return fail(std::string("kernel ") + want[k] + " not found in " + cubin_path);
    return 0;
}

// The polar grid of one scan as the demo builds it (laser_to_meas_grid.cu:40-48): a float2
// cudaArray of width = beams, height = range bins, bound as a surface; createPolarGridTexture
// writes it, or, with prior (bins x beams float2) uploaded first, fusePolarGridTexture
// combines the scan into it.  out: bins x beams float2.
int dogm_ref_polar_ism(const float* ranges, int beams, int bins, float resolution, float stddev_range,
                       const float* prior, float* out) {
    if (!g_meas_fn[0]) return fail("dogm_ref_meas_load first");
    if (beams <= 0 || bins <= 0) return fail("bad polar grid size");
    cudaChannelFormatDesc desc = cudaCreateChannelDesc(32, 32, 0, 0, cudaChannelFormatKindFloat);
    cudaArray_t arr = nullptr;
    RCU(cudaMallocArray(&arr, &desc, (size_t)beams, (size_t)bins, cudaArraySurfaceLoadStore));
    const size_t pitch = sizeof(float) * 2 * (size_t)beams;
    if (prior) RCU(cudaMemcpy2DToArray(arr, 0, 0, prior, pitch, pitch, (size_t)bins, cudaMemcpyHostToDevice));
    cudaResourceDesc res;
    std::memset(&res, 0, sizeof(res));
    res.resType = cudaResourceTypeArray;
    res.res.array.array = arr;
    cudaSurfaceObject_t surf = 0;
    RCU(cudaCreateSurfaceObject(&surf, &res));
    float* d_ranges = nullptr;
    RCU(cudaMalloc(&d_ranges, sizeof(float) * (size_t)beams));
    RCU(cudaMemcpy(d_ranges, ranges, sizeof(float) * (size_t)beams, cudaMemcpyHostToDevice));
    unsigned long long s = (unsigned long long)surf;
    int w = beams, h = bins;
    void* p[] = {&s, &d_ranges, &w, &h, &resolution, &stddev_range};
    // 32 x 32 blocks over (beam, bin), as laser_to_meas_grid.cu:45-47
    RDRV(cuLaunchKernel(g_meas_fn[prior ? 1 : 0], (unsigned)(beams + 31) / 32, (unsigned)(bins + 31) / 32, 1, 32, 32, 1,
                        0, nullptr, p, nullptr));
    RCU(cudaDeviceSynchronize());
    RCU(cudaMemcpy2DFromArray(out, pitch, arr, 0, 0, pitch, (size_t)bins, cudaMemcpyDeviceToHost));
    cudaDestroySurfaceObject(surf);
    cudaFreeArray(arr);
    cudaFree(d_ranges);
    return 0;
}

// cartesianGridToMeasurementGridKernel (measurement_grid.cu:115-132) on an RGBA float image
// (gs x gs, row y = framebuffer row, y up) bound as a surface; out: gs x gs MeasurementCells.
int dogm_ref_cart_to_meas(const float* rgba, int gs, float* out) {
    if (!g_meas_fn[2]) return fail("dogm_ref_meas_load first");
    if (gs <= 0) return fail("bad grid size");
    cudaChannelFormatDesc desc = cudaCreateChannelDesc(32, 32, 32, 32, cudaChannelFormatKindFloat);
    cudaArray_t arr = nullptr;
    RCU(cudaMallocArray(&arr, &desc, (size_t)gs, (size_t)gs, cudaArraySurfaceLoadStore));
    const size_t pitch = sizeof(float) * 4 * (size_t)gs;
    RCU(cudaMemcpy2DToArray(arr, 0, 0, rgba, pitch, pitch, (size_t)gs, cudaMemcpyHostToDevice));
    cudaResourceDesc res;
    std::memset(&res, 0, sizeof(res));
    res.resType = cudaResourceTypeArray;
    res.res.array.array = arr;
    cudaSurfaceObject_t surf = 0;
    RCU(cudaCreateSurfaceObject(&surf, &res));
    RMeas* d_out = nullptr;
    RCU(cudaMalloc(&d_out, sizeof(RMeas) * (size_t)gs * gs));
    RCU(cudaMemset(d_out, 0, sizeof(RMeas) * (size_t)gs * gs));
    unsigned long long s = (unsigned long long)surf;
    void* p[] = {&d_out, &s, &gs};
    RDRV(cuLaunchKernel(g_meas_fn[2], (unsigned)(gs + 31) / 32, (unsigned)(gs + 31) / 32, 1, 32, 32, 1, 0, nullptr, p,
                        nullptr));
    RCU(cudaDeviceSynchronize());
    RCU(cudaMemcpy(out, d_out, sizeof(RMeas) * (size_t)gs * gs, cudaMemcpyDeviceToHost));
    cudaDestroySurfaceObject(surf);
    cudaFreeArray(arr);
    cudaFree(d_out);
    return 0;
}

}  // extern "C"
