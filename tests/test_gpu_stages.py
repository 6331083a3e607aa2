"""GPU: the reference's own known-answer tests (dogm/test/dogm_spec.cpp) against the CUDA path,
through the C++ drop-in (tests/cpp/dogm_spec.cpp) and through the C ABI with the golden
vectors of tests/golden/kat.json."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def kat():
    with open(os.path.join(HERE, "golden", "kat.json")) as f:
        return json.load(f)


def test_cpp_dogm_spec(dogm, tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "dogm_spec")
    lib_dir = os.path.dirname(dogm.LIB_PATH)
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(REPO, "include"),
                        os.path.join(HERE, "cpp", "dogm_spec.cpp"), "-o", exe, "-L" + lib_dir, "-ldogm_gb300",
                        "-Wl,-rpath," + lib_dir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failure(s)" in r.stdout


def _grid(dogm, k, n):
    return dogm.DOGM(dogm.make_params(size=k["size"], resolution=k["resolution"], particle_count=n,
                                      new_born_particle_count=1, persistence_prob=k.get("persistence_prob", 0.5),
                                      stddev_process_noise_position=0.0, stddev_process_noise_velocity=0.0))


def test_stage_predict_known_answer(dogm, kat):
    """DOGM.Predict: zero noise -> state + dt*(vx, vy, 0, 0) and weight * p_S, bit for bit."""
    k = kat["predict"]
    st = np.array(k["state_bits"], np.uint32).view(np.float32)
    n = st.shape[0]
    g = _grid(dogm, k, n)
    w0 = np.float32(0.25)
    g.set_particles(st, np.zeros(n, np.int32), np.zeros(n, np.uint8), float(w0))
    g.particle_prediction(k["dt"])
    parts = g.get_particles()
    assert np.array_equal(parts["state"].view(np.uint32), np.array(k["pred_state_bits"], np.uint32))
    assert np.all(parts["weight"] == np.float32(k["persistence_prob"]) * w0)
    g.close()


def test_stage_ego_shift_known_answer(dogm, kat):
    """DOGM.EgoMotionCompensation: sub-cell moves shift nothing; +3 m moves particles +3 cells."""
    k = kat["ego_shift"]
    st = np.array(k["state_bits"], np.uint32).view(np.float32)
    n = st.shape[0]
    g = _grid(dogm, k, n)
    g.set_particles(st, np.zeros(n, np.int32), np.zeros(n, np.uint8), 0.5)
    for step in k["steps"]:
        g.update_pose(step["pose"][0], step["pose"][1], 0.0)
        assert [g.get_position_x(), g.get_position_y()] == step["expect_pose"]
    parts = g.get_particles()
    assert np.array_equal(parts["state"].view(np.uint32), np.array(k["moved_state_bits"], np.uint32))
    g.close()


def test_iteration_and_readback(dogm, scene):
    p = dogm.make_params(size=12.8, resolution=0.2, particle_count=10000, new_born_particle_count=1000)
    g = dogm.DOGM(p)
    meas = scene.random_measurements(g.grid_size, seed=1)
    for _ in range(3):
        g.update_grid(meas, 0.0, 0.0, 0.0, 0.1)
    assert g.get_iteration() == 3
    back = g.get_measurement_cells()
    assert np.array_equal(back.view(np.float32).reshape(-1, 4), meas)
    cells = g.get_grid_cells()
    occ = cells["start_idx"] >= 0
    assert np.all(cells["end_idx"][occ] >= cells["start_idx"][occ])
    assert g.last_launch_count() == 6  # steady state: predict, bucket scan, scatter, cells, newborn, resample
    g.close()
