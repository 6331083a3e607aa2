"""GPU: the demo's evaluation chain end to end -- update the grid on the GPU, extract the
dynamic cells (dogm_extract_dynamic_cells), cluster them and score the clusters against the
scene's ground truth (dogm_evaluator_*) -- checked against the evaluator oracle
(oracle/pyeval.py, pinned to the reference evaluator) on the same extracted cells: identical
clusters, matches and error sums.  The scene's objects move in world coordinates; cell indices
run against both world axes (scene.Scene), which fixes the ground truth in the evaluator's frame
(x right, y up, metres from the grid's corner)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def truth_in_grid(sc, k, ex, ey):
    half = float(sc.cfg["size"]) / 2.0
    res = float(sc.cfg["resolution"])
    c = sc.pos0 + sc.vel * (k * 0.1) - np.array([ex, ey])[None, :]
    t = np.empty((len(c), 4), np.float32)
    t[:, 0] = half - c[:, 0] - res / 2  # column * res
    t[:, 1] = half + c[:, 1] + res / 2  # grid length - row * res
    t[:, 2] = -sc.vel[:, 0]
    t[:, 3] = sc.vel[:, 1]
    return t


@pytest.mark.parametrize("mode", ["reference", "standard"])
def test_evaluation_chain_matches_oracle(dogm, scene, mode):
    import pyeval
    cfg = dict(scene.CONFIGS["small"])
    sc = scene.Scene(cfg, seed=7)
    g = dogm.DOGM(dogm.make_params(**scene.params_dict(cfg)), seed=3)
    res, glen = float(cfg["resolution"]), float(g.grid_size) * float(cfg["resolution"])
    ev = dogm.Evaluator(res, glen, mode)
    pe = pyeval.Evaluator(res, glen, mode)
    frames = 0
    for k in range(16):
        m, x, y, yaw = sc.frame(k)
        g.update_grid(m, x, y, yaw, 0.1)
        if k < 8:
            continue
        cells = g.extract_dynamic_cells(0.7, 4.0, max_out=g.cell_count)  # main.cpp:47-48
        t = truth_in_grid(sc, k, x, y)
        got = ev.add_step(cells, t)
        want = pe.add_step(cells["x"], cells["y"], cells["cell"]["mean_x_vel"], cells["cell"]["mean_y_vel"], t)
        assert len(got) == len(want)
        for a, b in zip(got, want):
            assert a["cells"] == b["cells"] and a["truth"] == b["truth"]
            assert np.array_equal(np.array([a["x"], a["y"], a["vx"], a["vy"]], np.float32),
                                  np.array([b["x"], b["y"], b["vx"], b["vy"]], np.float32), equal_nan=True)
        frames += 1
    s = ev.summary()
    mae, rmse, det, una = pe.summary()
    assert np.array_equal(s["mae"], mae) and np.array_equal(s["rmse"], rmse)
    assert (s["detections"], s["unassigned"]) == (det, una)
    # the filter tracks the scene: most clusters are matched and the matched velocities are close
    assert det >= frames
    assert np.all(np.isfinite(s["rmse"]))
    assert s["mae"][2] < 4.0 and s["mae"][3] < 4.0, s
    print(mode, "frames", frames, "detections", det, "unassigned", una, "MAE", s["mae"], "RMSE", s["rmse"])
    g.close()
