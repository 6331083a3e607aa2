// dogm::DOGM — header-only C++ drop-in for the reference's class of the same name
// (dogm/include/dogm/dogm.h:20-199), implemented over the C ABI in dogm_gb300.h.
//
// Same constructor, updateGrid, getters and public stage methods (initializeParticles,
// particlePrediction, particleAssignment, gridCellOccupancyUpdate, updatePersistentParticles,
// initializeNewParticles, statisticalMoments, resampling; dogm.h:150-157).  updateGrid runs the
// stages fused; called one by one in the reference's order (dogm.cu:119-127) after
// updatePose, they compute the same bits as updateGrid.
// Error behaviour matches the reference's CHECK_ERROR (cuda_utils.h:13-24): print and
// continue; define DOGM_GB300_THROW to throw std::runtime_error instead.
#pragma once

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "../dogm_gb300.h"
#include "dogm_types.h"

namespace dogm
{

inline void checkStatus(dogm_status s, const char* what)
{
    if (s == DOGM_OK)
    {
        return;
    }
#ifdef DOGM_GB300_THROW
    throw std::runtime_error(std::string(what) + ": " + dogm_status_string(s) + " (" + dogm_last_error() + ")");
#else
    std::printf("GPU Kernel Error: %s %s (%s)\n", what, dogm_status_string(s), dogm_last_error());
#endif
}

class DOGM
{
public:
    // dogm.h:26-60 (same field order; layout-compatible with dogm_params)
    struct Params
    {
        float size;
        float resolution;
        int particle_count;
        int new_born_particle_count;
        float persistence_prob;
        float stddev_process_noise_position;
        float stddev_process_noise_velocity;
        float birth_prob;
        float stddev_velocity;
        float init_max_velocity;
        float freespace_discount;
    };
    static_assert(sizeof(Params) == sizeof(dogm_params), "Params layout");

    explicit DOGM(const Params& p, const dogm_options* opt = nullptr) : params(p), handle(nullptr)
    {
        checkStatus(dogm_create(reinterpret_cast<const dogm_params*>(&params), opt, &handle), "DOGM::DOGM");
    }

    ~DOGM() { dogm_destroy(handle); }

    DOGM(const DOGM&) = delete;
    DOGM& operator=(const DOGM&) = delete;

    // dogm.h:80-81
    void updateGrid(MeasurementCell* measurement_grid, float new_x, float new_y, float new_yaw, float dt,
                    bool device = true)
    {
        checkStatus(dogm_update(handle, reinterpret_cast<const dogm_measurement_cell*>(measurement_grid), new_x, new_y,
                                new_yaw, dt, device ? 1 : 0),
                    "DOGM::updateGrid");
    }

    // dogm.h:88
    std::vector<GridCell> getGridCells() const
    {
        std::vector<GridCell> cells(static_cast<size_t>(getGridSize()) * static_cast<size_t>(getGridSize()));
        checkStatus(dogm_get_grid_cells(handle, reinterpret_cast<dogm_grid_cell*>(cells.data()), cells.size()),
                    "DOGM::getGridCells");
        return cells;
    }

    // Not in the reference: queues the copy of the current grid into `out` (grid_size^2 cells,
    // pinned host memory for a real overlap) and returns; the copy overlaps the next
    // updateGrid.  `out` holds the grid once synchronize() returns.
    void getGridCellsAsync(GridCell* out) const
    {
        const size_t n = static_cast<size_t>(getGridSize()) * static_cast<size_t>(getGridSize());
        checkStatus(dogm_get_grid_cells_async(handle, reinterpret_cast<dogm_grid_cell*>(out), n),
                    "DOGM::getGridCellsAsync");
    }

    // Not in the reference: waits for queued updates and asynchronous copies.
    void synchronize() const { checkStatus(dogm_synchronize(handle), "DOGM::synchronize"); }

    // dogm.h:95
    std::vector<MeasurementCell> getMeasurementCells() const
    {
        std::vector<MeasurementCell> cells(static_cast<size_t>(getGridSize()) * static_cast<size_t>(getGridSize()));
        checkStatus(
            dogm_get_measurement_cells(handle, reinterpret_cast<dogm_measurement_cell*>(cells.data()), cells.size()),
            "DOGM::getMeasurementCells");
        return cells;
    }

    // dogm.h:102: a host ParticlesSoA the caller releases with .free()
    ParticlesSoA getParticles() const
    {
        const int n = dogm_get_particle_count(handle);
        ParticlesSoA particles(n, false);
        std::vector<unsigned char> assoc(static_cast<size_t>(n));
        checkStatus(dogm_get_particles(handle, reinterpret_cast<float*>(particles.state), particles.grid_cell_idx,
                                       particles.weight, assoc.data(), static_cast<size_t>(n)),
                    "DOGM::getParticles");
        for (int i = 0; i < n; ++i)
        {
            particles.associated[i] = assoc[static_cast<size_t>(i)] != 0;
        }
        return particles;
    }

    int getGridSize() const { return dogm_get_grid_size(handle); }
    float getResolution() const { return dogm_get_resolution(handle); }
    float getPositionX() const { return dogm_get_position_x(handle); }
    float getYaw() const { return dogm_get_yaw(handle); }
    float getPositionY() const { return dogm_get_position_y(handle); }
    int getIteration() const { return dogm_get_iteration(handle); }

    // public stage methods (dogm.h:150-157), in the order updateGrid runs them (dogm.cu:119-127)
    void initializeParticles() { checkStatus(dogm_initialize_particles(handle), "DOGM::initializeParticles"); }
    void particlePrediction(float dt) { checkStatus(dogm_particle_prediction(handle, dt), "DOGM::particlePrediction"); }
    void particleAssignment() { checkStatus(dogm_particle_assignment(handle), "DOGM::particleAssignment"); }
    void gridCellOccupancyUpdate(float dt)
    {
        checkStatus(dogm_grid_cell_occupancy_update(handle, dt), "DOGM::gridCellOccupancyUpdate");
    }
    void updatePersistentParticles()
    {
        checkStatus(dogm_update_persistent_particles(handle), "DOGM::updatePersistentParticles");
    }
    void initializeNewParticles() { checkStatus(dogm_initialize_new_particles(handle), "DOGM::initializeNewParticles"); }
    void statisticalMoments() { checkStatus(dogm_statistical_moments(handle), "DOGM::statisticalMoments"); }
    // also makes the resampled particles the current ones, which the reference leaves to
    // updateGrid's particle_array = particle_array_next (dogm.cu:128)
    void resampling() { checkStatus(dogm_resampling(handle), "DOGM::resampling"); }

    // private in the reference (dogm.h:145); public here so that a caller can run a whole
    // update stage by stage from a host measurement grid
    void updateMeasurementGrid(const MeasurementCell* measurement_grid)
    {
        const size_t n = static_cast<size_t>(getGridSize()) * static_cast<size_t>(getGridSize());
        checkStatus(dogm_set_measurement_cells(handle, reinterpret_cast<const dogm_measurement_cell*>(measurement_grid), n),
                    "DOGM::updateMeasurementGrid");
    }

    // private in the reference (dogm.h:144); public here so stage tests can drive it
    void updatePose(float new_x, float new_y, float new_yaw)
    {
        checkStatus(dogm_update_pose(handle, new_x, new_y, new_yaw), "DOGM::updatePose");
    }

    Params params;
    dogm_handle* handle;
};

} /* namespace dogm */
