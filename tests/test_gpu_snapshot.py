"""GPU: snapshot and restore (dogm_snapshot / dogm_restore).  A handle restored from a snapshot
continues bit-identically to the handle it was taken from -- the snapshot carries the random
identity, so even a handle created with another seed resumes the same stream -- and a snapshot
of a handle with other parameters is refused with the target left as it was."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_restored_handle_continues_bit_identically(dogm, scene):
    cfg = dict(scene.CONFIGS["small"])
    cfg.update(size=25.6, resolution=0.1, particle_count=150000, new_born_particle_count=15000, ego_speed=8.0)
    sc = scene.Scene(cfg, seed=6)
    frames = [sc.frame(k) for k in range(6)]
    p = dogm.make_params(**scene.params_dict(cfg))
    a = dogm.DOGM(p, seed=77, stream_id=3)
    for m, x, y, yaw in frames[:3]:
        a.update_grid(m, x, y, yaw, 0.1)
    snap = a.snapshot()
    b = dogm.DOGM(p, seed=1)  # another seed: the snapshot carries the random identity
    b.restore(snap)
    assert b.get_iteration() == 3
    assert b.get_grid_cells().tobytes() == a.get_grid_cells().tobytes()
    assert (b.get_position_x(), b.get_position_y()) == (a.get_position_x(), a.get_position_y())
    for m, x, y, yaw in frames[3:]:  # the ego keeps moving: the grid shifts in these frames
        a.update_grid(m, x, y, yaw, 0.1)
        b.update_grid(m, x, y, yaw, 0.1)
        assert a.get_grid_cells().tobytes() == b.get_grid_cells().tobytes()
        pa, pb = a.get_particles(), b.get_particles()
        for key in ("state", "grid_cell_idx", "weight", "associated"):
            assert pa[key].tobytes() == pb[key].tobytes(), key
    other = dogm.DOGM(dogm.make_params(**dict(scene.params_dict(cfg), particle_count=100000)), seed=1)
    before = other.get_grid_cells().tobytes()
    with pytest.raises(dogm.DogmError, match="other parameters"):
        other.restore(snap)
    assert other.get_grid_cells().tobytes() == before and other.get_iteration() == 0
    with pytest.raises(dogm.DogmError):
        b.restore(snap[:100])
    for g in (a, b, other):
        g.close()
