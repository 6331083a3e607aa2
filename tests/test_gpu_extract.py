"""GPU: dynamic-cell extraction (dogm_extract_dynamic_cells) against its restatement of
computeCellsWithVelocity (oracle/pymeas.py dynamic_cells): the same cells in the same row-major
order with bit-identical occupancy, Mahalanobis length and records (the filter is a fixed FP32
expression of the cell record, so the tolerance is zero)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("min_occ,min_vel", [(0.7, 4.0), (0.5, 0.5), (0.0, -1e30)])  # main.cpp:47-48, looser
def test_extract_matches_restatement(dogm, scene, min_occ, min_vel):
    import pymeas
    cfg = dict(scene.CONFIGS["small"])
    cfg.update(size=25.6, resolution=0.1, particle_count=200000, new_born_particle_count=20000, vehicles=8)
    sc = scene.Scene(cfg, seed=4)
    g = dogm.DOGM(dogm.make_params(**scene.params_dict(cfg)), seed=2)
    for k in range(6):
        m, x, y, yaw = sc.frame(k)
        g.update_grid(m, x, y, yaw, 0.1)
    cells = g.get_grid_cells()
    exp = pymeas.dynamic_cells(cells, g.grid_size, min_occ, min_vel)
    got = g.extract_dynamic_cells(min_occ, min_vel, max_out=g.cell_count)
    assert got.size == exp["index"].size
    assert np.array_equal(got["index"], exp["index"])
    assert np.array_equal(got["x"], exp["x"]) and np.array_equal(got["y"], exp["y"])
    assert got["occupancy"].tobytes() == exp["occupancy"].tobytes()
    assert got["mahalanobis"].tobytes() == exp["mahalanobis"].tobytes()
    assert got["cell"].tobytes() == cells[exp["index"]].tobytes()
    # a short output buffer keeps the first cells in row-major order and still counts all
    if got.size > 3:
        part = g.extract_dynamic_cells(min_occ, min_vel, max_out=3)
        assert np.array_equal(part["index"], exp["index"][:3])
    g.close()
