"""GPU: device-side index checks surface as a status code, and the handle recovers.

Injected particles whose cell index lies past the grid's last bucket cannot be placed by the
bucket scatter: the kernel records a status bit instead of writing out of range, the call
returns DOGM_ERR_CUDA with the bounds message, and the next full update starts from a full
counter reset and runs clean."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_out_of_grid_keys_are_reported(dogm, scene):
    p = dogm.make_params(size=10.3, resolution=0.1, particle_count=30001, new_born_particle_count=3001)
    g = dogm.DOGM(p, seed=5)
    gs, n = g.grid_size, g.particle_count   # 103 x 103 cells: 11 buckets of 1024 cells
    meas = scene.random_measurements(gs, seed=1)
    g.update_grid(meas, 0.0, 0.0, 0.0, 0.1)
    g.synchronize()
    parts = g.get_particles()
    state = np.ascontiguousarray(parts["state"], np.float32).reshape(n, 4)
    idx = (np.clip(state[:, 0], 0, gs - 1).astype(np.int64) + gs * np.clip(state[:, 1], 0, gs - 1).astype(np.int64))
    idx = idx.astype(np.int32)
    idx[::97] = 11 * 1024 + 3   # past the last bucket
    g.set_particles(state, idx, np.zeros(n, np.uint8), 1.0 / n)
    with pytest.raises(dogm.DogmError, match="out-of-range"):
        g.particle_assignment()
        g.synchronize()
    # the next update resets every counter and runs clean, twice (the second as a graph)
    for k in range(2):
        g.update_grid(scene.random_measurements(gs, seed=2 + k), 0.0, 0.0, 0.0, 0.1)
        g.synchronize()
    cells = g.get_grid_cells()
    assert np.isfinite(cells["occ_mass"]).all() and (cells["occ_mass"] >= 0).all()
    g.close()
