"""GPU: the reference's public stage methods as separate calls (dogm/include/dogm/dogm.h:150-157).

One handle runs dogm_update (updateGrid, dogm/src/dogm.cu:115-131); a twin with the same seed
runs the same frames stage by stage in the reference's order -- measurement copy (and particle
initialisation on the first frame), pose, particlePrediction, particleAssignment,
gridCellOccupancyUpdate, updatePersistentParticles, initializeNewParticles, statisticalMoments,
resampling (dogm.cu:116-128).  Cells, particles, pose and iteration must agree bit for bit
after every frame, the ego moving so that frames shift the grid."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stage_frame(g, meas, x, y, yaw, dt, first):
    g.set_measurement_cells(meas)
    if first:
        g.initialize_particles()
    g.update_pose(x, y, yaw)
    g.particle_prediction(dt)
    g.particle_assignment()
    g.grid_cell_occupancy_update(dt)
    g.update_persistent_particles()
    g.initialize_new_particles()
    g.statistical_moments()
    g.resampling()


def _same(a, b, label):
    ca, cb = a.get_grid_cells(), b.get_grid_cells()
    for f in ca.dtype.names:
        assert ca[f].tobytes() == cb[f].tobytes(), "%s: cells.%s" % (label, f)
    pa, pb = a.get_particles(), b.get_particles()
    for key in ("state", "grid_cell_idx", "weight", "associated"):
        assert pa[key].tobytes() == pb[key].tobytes(), "%s: particles.%s" % (label, key)
    assert (a.get_position_x(), a.get_position_y(), a.get_iteration()) == \
        (b.get_position_x(), b.get_position_y(), b.get_iteration()), label


@pytest.mark.parametrize("workload", ["scene", "random"])
def test_stage_calls_compose_to_update_grid(dogm, scene, workload):
    if workload == "scene":
        cfg = dict(scene.CONFIGS["small"])
        sc = scene.Scene(cfg, seed=3)
        p = dogm.make_params(**scene.params_dict(cfg))
        frames = [sc.frame(k) for k in range(5)]
    else:  # particles spread over a small grid, moving by several cells per frame
        p = dogm.make_params(size=25.6, resolution=0.2, particle_count=40000, new_born_particle_count=4000)
        gs = int(np.float32(25.6) / np.float32(0.2))
        frames = [(scene.random_measurements(gs, seed=40 + k), 0.35 * k, -0.25 * k, 0.0) for k in range(5)]
    a, b = dogm.DOGM(p, seed=77), dogm.DOGM(p, seed=77)
    try:
        for k, (m, x, y, yaw) in enumerate(frames):
            a.update_grid(m, x, y, yaw, 0.1)
            _stage_frame(b, m, x, y, yaw, 0.1, first=(k == 0))
            _same(a, b, "%s frame %d" % (workload, k))
        assert b.last_launch_count() == 1  # resampling alone
        # a stage-driven frame leaves the handle ready for the fused update, and the reverse
        m, x, y, yaw = frames[-1]
        a.update_grid(m, x + 0.3, y, yaw, 0.1)
        b.update_grid(m, x + 0.3, y, yaw, 0.1)
        _same(a, b, "%s fused after stages" % workload)
        _stage_frame(a, m, x + 0.6, y, yaw, 0.1, first=False)
        _stage_frame(b, m, x + 0.6, y, yaw, 0.1, first=False)
        _same(a, b, "%s stages after fused" % workload)
    finally:
        a.close()
        b.close()
