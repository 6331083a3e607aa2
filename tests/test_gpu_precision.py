"""GPU: the precision study (tests/precision_study.py) on a reduced workload -- 512 x 512 cells,
4e5 + 4e4 particles, heavy-tailed occupied masses, 4 frames.  Tolerances stated here:
  * resampling indices of the GB300 path (exact fixed-point scan) and of a compensated FP32
    scan differ from an FP64 scan's on at most 1e-4 of the slots; a plain FP32 scan does worse
    than the GB300 path (its 24-bit prefix cannot resolve 4.4e5 items);
  * occupied / free / persistent / newborn masses within 5e-7 of FP64, velocity moments within
    2e-6 of the cell's second moment (the 30-frame run at 2048^2, tests/precision_study_2048.json,
    stays below 2.5e-7 and 6.1e-7)."""
import pytest

pytestmark = pytest.mark.gpu


def test_precision_study_small(dogm, oracle, scene):
    import precision_study
    rep = precision_study.run(dogm, oracle, scene, frames=4, size=51.2, resolution=0.1, particles=400_000,
                              newborn=40_000, seed=3)
    s = rep["summary"]
    print("\n", s)
    mm = s["resample_mismatch_vs_fp64"]
    assert mm["gb300_exact_fixed_point"]["max"] <= 1e-4
    assert mm["compensated_fp32"]["max"] <= 1e-4
    assert mm["fp32"]["mean"] > mm["gb300_exact_fixed_point"]["mean"]
    err = s["cell_error_vs_fp64_max"]
    for k in ("occ_mass", "free_mass", "pers_occ_mass", "new_born_occ_mass"):
        assert err[k] <= 5e-7, (k, err[k])
    for k in ("mean_x_vel", "mean_y_vel", "var_x_vel", "var_y_vel", "covar_xy_vel"):
        assert err[k] <= 2e-6, (k, err[k])
    assert s["cells_compared_min"] > 0.995
