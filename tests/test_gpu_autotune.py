"""GPU: the autotuner (dogm_autotune / dogm_set_tune).  Launch widths and the resampling tile shape
change only how the work is laid out, never a result: a tuned handle and a default one fed the
same frames end bit-identical.  The cache file round-trips; invalid settings are refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tuned_equals_default_and_cache(dogm, scene, tmp_path):
    p = dogm.make_params(size=25.6, resolution=0.1, particle_count=150000, new_born_particle_count=15000)
    a, b = dogm.DOGM(p, seed=9), dogm.DOGM(p, seed=9)
    m0 = scene.random_measurements(a.grid_size, seed=1)
    cache = str(tmp_path / "tune.txt")
    t = a.autotune(m0, reps=3, cache_path=cache)
    assert t.ms_default > 0 and t.ms_tuned <= t.ms_default * 1.05
    t2 = a.autotune(m0, reps=3, cache_path=cache)  # read from the cache, not re-timed
    assert list(t2.blocks_per_sm) == list(t.blocks_per_sm) and t2.resample_tile_bits == t.resample_tile_bits
    assert open(cache).read().count(" : ") == 1
    # a deliberately different shape still computes the same bits
    forced = dogm.Tune()
    for i in range(6):  # the six stages in dogm_stage_name order
        forced.blocks_per_sm[i] = (1, 3, 1, 1, 8, 2)[i]
    forced.resample_tile_bits = 11  # 2048-particle resampling tiles
    b.set_tune(forced)
    got = b.get_tune()
    assert list(got.blocks_per_sm) == list(forced.blocks_per_sm) and got.resample_tile_bits == 11
    for k in range(4):
        m = scene.random_measurements(a.grid_size, seed=10 + k)
        a.update_grid(m, 0.1 * k, 0.0, 0.0, 0.1)
        b.update_grid(m, 0.1 * k, 0.0, 0.0, 0.1)
        assert a.get_grid_cells().tobytes() == b.get_grid_cells().tobytes(), "frame %d" % k
        assert a.get_particles()["state"].tobytes() == b.get_particles()["state"].tobytes()
        if k == 1:  # and the finest tiling
            forced.resample_tile_bits = 9
            b.set_tune(forced)
    bad = dogm.Tune()
    bad.resample_tile_bits = 12
    with pytest.raises(dogm.DogmError):
        b.set_tune(bad)
    bad.resample_tile_bits = 0
    bad.blocks_per_sm[0] = 99
    with pytest.raises(dogm.DogmError):
        b.set_tune(bad)
    bad.blocks_per_sm[0] = 0
    bad.blocks_per_sm[7] = 2  # only six stages
    with pytest.raises(dogm.DogmError):
        b.set_tune(bad)
    got = b.get_tune()  # refused settings leave the handle as it was
    assert list(got.blocks_per_sm) == list(forced.blocks_per_sm) and got.resample_tile_bits == 9
    a.close()
    b.close()
