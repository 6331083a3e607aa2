"""GPU: the particle sort (bucket scatter by cell tile + counting sort of each bucket inside the
cell pass) on inputs that stress its structure, against the FP32 oracle with the GPU's own
draws replayed: keys, the permutation, the sorted states, ranges, masses and resample indices
bit for bit, moments within 4e-6 of the cell's second moment (tests/test_gpu_parity.py).

  * every particle in one cell: one bucket of many 4096-particle chunks, one segment spanning
    every thread of the segmented reduction;
  * particles uniformly random over the grid: every scatter tile holds nearly every bucket;
  * particles in reverse cell order;
  * a grid whose cell count is not a multiple of the 1024-cell tile, with particles on the last,
    partial tile and outside the grid;
  * small dense grids, which sort by buckets finer than a cell tile and split a crowded tile into
    several jobs of the cell pass: every particle in one cell (one bucket far above a job), and
    particles uniformly random (buckets merged into whole-tile jobs)."""
import numpy as np
import pytest

from test_gpu_parity import compare_frame

pytestmark = pytest.mark.gpu


def _run(dogm, oracle, scene, p, state, assoc, frames=2, seed=11):
    g = dogm.DOGM(p, seed=seed)
    g.debug_enable(True)
    gs, n = g.grid_size, g.particle_count
    meas0 = scene.random_measurements(gs, seed=seed)
    # a first update initialises the handle (and the oracle's pose); then the injected state
    d = g.generate_draws(0)
    g.set_replay(d["init_u"], d["predict_z"], d["birth_z"], d["resample_r"])
    g.update_grid(meas0, 0.0, 0.0, 0.0, 0.1)
    o = oracle.OracleDOGM(p, np.float32)
    o.update(meas0, 0.0, 0.0, 0.0, 0.1, d)
    idx = np.clip(state[:, 0].astype(np.int64), 0, gs - 1) + gs * np.clip(state[:, 1].astype(np.int64), 0, gs - 1)
    w = np.float32(1.0 / n)
    g.set_particles(state, idx.astype(np.int32), assoc, float(w))
    o.P_state[:] = state
    o.P_key[:] = idx.astype(np.uint32) | (assoc.astype(np.uint32) << np.uint32(31))
    o.w_res[0] = w
    for k in range(1, frames + 1):
        meas = scene.random_measurements(gs, seed=seed + k)
        d = g.generate_draws(k)
        g.set_replay(d["init_u"], d["predict_z"], d["birth_z"], d["resample_r"])
        g.update_grid(meas, 0.0, 0.0, 0.0, 0.1)
        out = o.update(meas, 0.0, 0.0, 0.0, 0.1, d)
        out["P_state_after"] = o.P_state.copy()
        compare_frame(dogm, oracle, g, out, "frame %d" % k)
    g.close()


def _params(dogm, size, res, n, b):
    # zero position noise keeps an all-in-one-cell start in one cell through the first predict
    return dogm.make_params(size=size, resolution=res, particle_count=n, new_born_particle_count=b)


def test_all_particles_in_one_cell(dogm, oracle, scene):
    p = _params(dogm, 25.6, 0.1, 60000, 6000)   # 256 x 256 cells
    n = p.particle_count
    rng = np.random.default_rng(1)
    state = np.zeros((n, 4), np.float32)
    state[:, 0] = 100.5
    state[:, 1] = 77.5
    state[:, 2:] = rng.normal(0.0, 0.01, (n, 2)).astype(np.float32)
    _run(dogm, oracle, scene, p, state, (rng.random(n) < 0.5).astype(np.uint8))


def test_particles_uniform_over_the_grid(dogm, oracle, scene):
    p = _params(dogm, 51.2, 0.1, 200000, 20000)   # 512 x 512 cells, 256 buckets
    n, gs = p.particle_count, 512
    rng = np.random.default_rng(2)
    state = np.zeros((n, 4), np.float32)
    state[:, 0:2] = rng.uniform(0.0, gs, (n, 2)).astype(np.float32)
    state[:, 2:] = rng.normal(0.0, 3.0, (n, 2)).astype(np.float32)
    _run(dogm, oracle, scene, p, state, np.zeros(n, np.uint8))


def test_particles_in_reverse_cell_order(dogm, oracle, scene):
    p = _params(dogm, 51.2, 0.1, 150000, 15000)
    n, gs = p.particle_count, 512
    rng = np.random.default_rng(3)
    state = np.zeros((n, 4), np.float32)
    state[:, 0:2] = rng.uniform(0.0, gs, (n, 2)).astype(np.float32)
    key = np.floor(state[:, 0]) + gs * np.floor(state[:, 1])
    state = state[np.argsort(-key, kind="stable")]
    state[:, 2:] = rng.normal(0.0, 1.0, (n, 2)).astype(np.float32)
    _run(dogm, oracle, scene, p, state, np.ones(n, np.uint8))


def test_partial_last_tile_and_outside_particles(dogm, oracle, scene):
    p = _params(dogm, 10.3, 0.1, 30001, 3001)   # 103 x 103 = 10,609 cells: 11 tiles, the last partial
    n, gs = p.particle_count, 103
    rng = np.random.default_rng(4)
    state = np.zeros((n, 4), np.float32)
    state[:, 0] = rng.uniform(-3.0, gs + 3.0, n).astype(np.float32)   # some outside the grid
    state[:, 1] = rng.uniform(gs - 12.0, gs + 2.0, n).astype(np.float32)   # most on the last rows
    state[:, 2:] = rng.normal(0.0, 2.0, (n, 2)).astype(np.float32)
    _run(dogm, oracle, scene, p, state, (rng.random(n) < 0.3).astype(np.uint8))


def test_fine_buckets_all_particles_in_one_cell(dogm, oracle, scene):
    # 100 x 100 cells = 10 cell tiles and 60,000 particles (> 2048 per tile): buckets of 64 cells
    p = _params(dogm, 10.0, 0.1, 60000, 6000)
    n = p.particle_count
    rng = np.random.default_rng(5)
    state = np.zeros((n, 4), np.float32)
    state[:, 0] = 40.5
    state[:, 1] = 61.5
    state[:, 2:] = rng.normal(0.0, 0.01, (n, 2)).astype(np.float32)
    _run(dogm, oracle, scene, p, state, (rng.random(n) < 0.5).astype(np.uint8))


def test_fine_buckets_particles_uniform(dogm, oracle, scene):
    # 128 x 128 cells = 16 cell tiles, 100,000 particles: every tile is split into several jobs
    p = _params(dogm, 12.8, 0.1, 100000, 10000)
    n, gs = p.particle_count, 128
    rng = np.random.default_rng(6)
    state = np.zeros((n, 4), np.float32)
    state[:, 0:2] = rng.uniform(0.0, gs, (n, 2)).astype(np.float32)
    state[:, 2:] = rng.normal(0.0, 3.0, (n, 2)).astype(np.float32)
    _run(dogm, oracle, scene, p, state, np.zeros(n, np.uint8))
