"""GPU: asynchronous grid readback (dogm_get_grid_cells_async).  A handle that reads every
grid back asynchronously (copies overlapping the next update, cell records alternating
between two buffers) produces, frame by frame, the same bits as a handle with the same seed
read back synchronously; synchronous readback, the batched update and further asynchronous
frames interleave with it freely."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_async_readback_matches_sync(dogm, scene):
    cfg = dict(scene.CONFIGS["small"])
    cfg.update(size=25.6, resolution=0.1, particle_count=200000, new_born_particle_count=20000, vehicles=8)
    sc = scene.Scene(cfg, seed=11)
    p = dogm.make_params(**scene.params_dict(cfg))
    a = dogm.DOGM(p, seed=5)
    b = dogm.DOGM(p, seed=5, sync_each_update=False)
    frames = [sc.frame(k) for k in range(8)]
    pins = [dogm.PinnedArray((a.cell_count, 4), np.float32) for _ in range(2)]
    outs = [dogm.PinnedArray((a.cell_count,), dogm.GRID_CELL_DTYPE) for _ in range(len(frames))]
    want = []
    for k, (m, x, y, yaw) in enumerate(frames):
        a.update_grid(m, x, y, yaw, 0.1)
        want.append(a.get_grid_cells())
        pins[k % 2].array[:] = m  # the copy in of frame k - 2 from this buffer has run: see below
        b.update_grid(pins[k % 2].array, x, y, yaw, 0.1, device=False)
        b.get_grid_cells_async(outs[k].array)
        if k % 2 == 1:
            b.synchronize()  # frees the measurement buffers for reuse
    b.synchronize()
    for k in range(len(frames)):
        assert outs[k].array.tobytes() == want[k].tobytes(), "frame %d differs" % k
    # a synchronous readback of the same state, then a batched update, then async again
    assert b.get_grid_cells().tobytes() == want[-1].tobytes()
    m, x, y, yaw = sc.frame(len(frames))
    a.update_grid(m, x, y, yaw, 0.1)
    dogm.update_batch([b], [m], [x], [y], [yaw], [0.1])
    assert b.get_grid_cells().tobytes() == a.get_grid_cells().tobytes()
    m, x, y, yaw = sc.frame(len(frames) + 1)
    a.update_grid(m, x, y, yaw, 0.1)
    b.update_grid(m, x, y, yaw, 0.1)
    b.get_grid_cells_async(outs[0].array)
    b.synchronize()
    assert outs[0].array.tobytes() == a.get_grid_cells().tobytes()
    pa, pb = a.get_particles(), b.get_particles()
    assert all(np.array_equal(pa[f], pb[f]) for f in pa)
    for o in pins + outs:
        o.free()
    a.close()
    b.close()
