"""GPU: the three launch modes of a handle's updates (chained, one CUDA graph per update, plain
launches) compute the same bits, frame after frame, with the ego moving, and switching modes
between updates keeps them identical."""
import pytest

pytestmark = pytest.mark.gpu


def _same(a, b, what):
    assert a.get_grid_cells().tobytes() == b.get_grid_cells().tobytes(), what
    pa, pb = a.get_particles(), b.get_particles()
    assert pa["state"].tobytes() == pb["state"].tobytes(), what
    assert pa["grid_cell_idx"].tobytes() == pb["grid_cell_idx"].tobytes(), what


def test_launch_modes_agree(dogm, scene):
    p = dogm.make_params(size=51.2, resolution=0.1, particle_count=300000, new_born_particle_count=30000)
    chained, graph, plain = (dogm.DOGM(p, seed=31, sync_each_update=False) for _ in range(3))
    graph.set_launch_mode(graph=True)
    plain.set_launch_mode(plain=True)
    gs = chained.grid_size
    for k in range(6):
        m = scene.random_measurements(gs, seed=70 + k)
        for g in (chained, graph, plain):
            g.update_grid(m, 0.4 * k, -0.2 * k, 0.0, 0.1)
        for g in (chained, graph, plain):
            g.synchronize()
        _same(chained, graph, "frame %d (graph)" % k)
        _same(chained, plain, "frame %d (plain)" % k)
        if k == 2:  # switch modes mid-run: chained <-> graph
            chained.set_launch_mode(graph=True)
            graph.set_launch_mode()
    with pytest.raises(dogm.DogmError):
        dogm.check(dogm.load().dogm_set_launch_mode(chained.h, 3), "dogm_set_launch_mode")
    for g in (chained, graph, plain):
        g.close()
