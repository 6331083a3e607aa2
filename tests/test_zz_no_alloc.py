"""GPU: dogm_update_pose_noalloc (the pose update that allocates no device memory) against
dogm_update_pose, through the C ABI.  Each pair of handles starts from identical state; one
takes the allocating call, the other the allocation-free one, two calls in a row, and the cells,
particles and pose must agree bit for bit (the shift moves records, it computes nothing).
The two grid sizes are interleaved so the shared shift array holds a previous call's records
when the next call starts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pair(dogm, scene, size, res, n, b, seed):
    p = dogm.make_params(size=size, resolution=res, particle_count=n, new_born_particle_count=b)
    a, c = dogm.DOGM(p, seed=seed), dogm.DOGM(p, seed=seed)
    for k in range(2):
        meas = scene.random_measurements(a.grid_size, seed=seed + k)
        a.update_grid(meas, 0.0, 0.0, 0.0, 0.1)
        c.update_grid(meas, 0.0, 0.0, 0.0, 0.1)
    return a, c


def _assert_same(a, c, label):
    assert a.get_grid_cells().tobytes() == c.get_grid_cells().tobytes(), label + " cells"
    pa, pc = a.get_particles(), c.get_particles()
    for key in ("state", "grid_cell_idx", "weight", "associated"):
        assert pa[key].tobytes() == pc[key].tobytes(), label + " particles " + key
    assert (a.get_position_x(), a.get_position_y(), a.get_yaw()) == \
        (c.get_position_x(), c.get_position_y(), c.get_yaw()), label + " pose"


def test_noalloc_pose_update_matches_allocating_one(dogm, scene):
    small = _pair(dogm, scene, 12.8, 0.2, 20000, 2000, 301)    # 64 x 64 cells
    large = _pair(dogm, scene, 50.0, 0.2, 100000, 10000, 401)  # 250 x 250 cells
    plan = [(small, [(0.65, -0.45), (1.1, 0.5)]), (large, [(-0.9, 0.7), (0.3, -1.5)])]
    for call in range(2):
        for (a, c), poses in plan:
            x, y = poses[call]
            a.update_pose(x, y, 0.0)
            c.update_pose_noalloc(x, y, 0.0)
            _assert_same(a, c, "call %d, grid %d" % (call, a.grid_size))
    # the next update starts from the shifted state (including the free-mass buffers)
    for a, c in (small, large):
        meas = scene.random_measurements(a.grid_size, seed=77)
        x, y = a.get_position_x() + 0.1, a.get_position_y()
        a.update_grid(meas, x, y, 0.0, 0.1)
        c.update_grid(meas, x, y, 0.0, 0.1)
        _assert_same(a, c, "update after shifts, grid %d" % a.grid_size)
    for g in small + large:
        g.close()


@pytest.mark.parametrize("call", ["update_pose_noalloc", "update_pose"])
def test_pose_shift_waits_for_queued_grid_readback(dogm, scene, call):
    """A grid copy queued by get_grid_cells_async before a shift must deliver the grid as it
    was before the shift: the shift rewrites the cell records in place, so it has to wait for
    the copy (a torn copy would mix pre- and post-shift records)."""
    p = dogm.make_params(size=50.0, resolution=0.2, particle_count=100000, new_born_particle_count=10000)
    g = dogm.DOGM(p, seed=501)   # 250 x 250 cells: 4 MB of records per copy
    for k in range(2):
        g.update_grid(scene.random_measurements(g.grid_size, seed=600 + k), 0.0, 0.0, 0.0, 0.1)
    before = g.get_grid_cells()
    outs = [dogm.PinnedArray(before.shape, dogm.GRID_CELL_DTYPE) for _ in range(2)]
    try:
        for i, (x, y) in enumerate([(1.3, -0.9), (2.9, 0.7)]):
            g.get_grid_cells_async(outs[i].array)
            getattr(g, call)(x, y, 0.0)
            g.synchronize()
            assert outs[i].array.tobytes() == before.tobytes(), "copy %d torn by the shift" % i
            after = g.get_grid_cells()
            assert after.tobytes() != before.tobytes()   # the shift did move the records
            before = after
    finally:
        for o in outs:
            o.free()
        g.close()


def test_noalloc_pose_update_refuses_grids_over_its_limit(dogm):
    p = dogm.make_params(size=60.0, resolution=0.1, particle_count=1000, new_born_particle_count=100)
    g = dogm.DOGM(p, seed=1)   # 600 x 600 = 360,000 cells > 262,144
    with pytest.raises(dogm.DogmError, match="invalid argument"):
        g.update_pose_noalloc(1.0, 1.0, 0.0)
    assert (g.get_position_x(), g.get_position_y()) == (0.0, 0.0)
    g.update_pose(1.0, 1.0, 0.0)   # the allocating call still serves this grid
    g.close()
