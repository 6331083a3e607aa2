"""GPU: distribution tests of unreplayed runs (the kernels' own Philox draws).

Replayed runs are compared bit for bit elsewhere; here the random parts are checked by
their distributions, as the method prescribes them:
  * prediction noise: (x' - x - dt vx) / sigma_pos and (vx' - vx) / sigma_vel ~ N(0, 1)
    (predict.cu:27-35 with cuda_utils.h:37-40), independent components;
  * first-frame velocities ~ U(-v_max, v_max) (init_new_particles.cu:110-113);
  * newborn velocities ~ N(0, sigma_v) at the cell centre (init_new_particles.cu:168-177);
  * systematic resampling: the number of copies of every cell's persistent and newborn
    weight is within 1 of N * weight / total each (both are contiguous runs of the joint
    sequence), so the per-cell count differs from N * W_k / J by less than 2;
  * an unreplayed update against the FP64 oracle fed independent draws: occupancy masses
    agree within the spread of the particle estimate, particle velocity moments within
    sampling error.
KS p-values are taken against alpha = 1e-4 on fixed seeds (deterministic outcomes)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
stats = pytest.importorskip("scipy.stats")
ALPHA = 1e-4


def test_prediction_noise_is_standard_normal(dogm):
    n, dt = 400000, 0.1
    p = dogm.make_params(size=25.6, resolution=0.1, particle_count=n, new_born_particle_count=0,
                         stddev_process_noise_position=0.1, stddev_process_noise_velocity=2.0)
    g = dogm.DOGM(p, seed=77)
    rng = np.random.default_rng(0)
    st = np.empty((n, 4), np.float32)
    st[:, 0:2] = rng.uniform(5.0, 20.0, (n, 2))
    st[:, 2:4] = rng.uniform(-3.0, 3.0, (n, 2))
    g.set_particles(st, np.zeros(n, np.int32), np.zeros(n, np.uint8), 1.0 / n)
    g.particle_prediction(dt)
    s2 = g.get_particles()["state"].astype(np.float64)
    s1 = st.astype(np.float64)
    z = np.empty((n, 4))
    z[:, 0:2] = (s2[:, 0:2] - s1[:, 0:2] - np.float32(dt) * s1[:, 2:4]) / 0.1
    z[:, 2:4] = (s2[:, 2:4] - s1[:, 2:4]) / 2.0
    for j in range(4):
        assert stats.kstest(z[:, j], "norm").pvalue > ALPHA, "component %d is not N(0,1)" % j
        assert abs(z[:, j].mean()) < 5 / np.sqrt(n)
        assert abs(z[:, j].var() - 1.0) < 5 * np.sqrt(2.0 / n)
    c = np.corrcoef(z.T)
    assert np.abs(c - np.eye(4)).max() < 5 / np.sqrt(n), "noise components are correlated"
    g.close()


def test_first_frame_velocities_uniform_and_cell_centres(dogm, scene):
    n = 300000
    p = dogm.make_params(size=25.6, resolution=0.1, particle_count=n, new_born_particle_count=0,
                         init_max_velocity=12.0)
    g = dogm.DOGM(p, seed=5)
    meas = scene.random_measurements(g.grid_size, seed=4, occ_fraction=0.05)
    g.set_measurement_cells(meas)
    g.initialize_particles()
    parts = g.get_particles()
    v = parts["state"][:, 2:4].astype(np.float64)
    for j in range(2):
        assert stats.kstest(v[:, j], "uniform", args=(-12.0, 24.0)).pvalue > ALPHA
        assert v[:, j].min() >= -12.0 and v[:, j].max() <= 12.0
    gs = g.grid_size
    idx = parts["grid_cell_idx"]
    assert np.array_equal(parts["state"][:, 0], (idx % gs).astype(np.float32) + np.float32(0.5))
    assert np.array_equal(parts["state"][:, 1], (idx // gs).astype(np.float32) + np.float32(0.5))
    # particles per cell follow the measured occupied mass (exact allocation: within 1)
    occ = meas[:, 1].astype(np.float64)
    expect = n * occ / occ.sum()
    got = np.bincount(idx, minlength=gs * gs)
    assert np.abs(got - expect).max() < 1.0 + 1e-6 * n
    g.close()


def _full_update(dogm, scene, seed, frames=3):
    p = dogm.make_params(size=25.6, resolution=0.1, particle_count=300000, new_born_particle_count=60000)
    g = dogm.DOGM(p, seed=seed)
    g.debug_enable(True)
    for k in range(frames):
        g.update_grid(scene.random_measurements(g.grid_size, seed=200 + k, occ_fraction=0.05), 0.0, 0.0, 0.0, 0.1)
    return g, p


def test_newborn_velocities_normal_at_cell_centres(dogm, scene):
    g, p = _full_update(dogm, scene, seed=31)
    dbg = g.debug_export()
    nb = dbg["n_birth"]
    assert nb == p.new_born_particle_count
    bs = dbg["birth_state"][:nb].astype(np.float64)
    for j in (2, 3):
        assert stats.kstest(bs[:, j] / 30.0, "norm").pvalue > ALPHA
    gs = g.grid_size
    cell = dbg["birth_cell"][:nb]
    assert np.array_equal(dbg["birth_state"][:nb, 0], (cell % gs).astype(np.float32) + np.float32(0.5))
    # y of a newborn uses float division (init_new_particles.cu:173)
    assert np.array_equal(dbg["birth_state"][:nb, 1],
                          cell.astype(np.float32) / np.float32(gs) + np.float32(0.5))
    g.close()


def test_systematic_resampling_multiplicity(dogm, scene):
    g, p = _full_update(dogm, scene, seed=41)
    n = p.particle_count
    gs = g.grid_size
    cells = g.get_grid_cells()
    dbg = g.debug_export()
    J = dbg["joint_total"] * 2.0 ** -dbg["q_shift"]
    nb = dbg["n_birth"]
    w_birth = np.bincount(dbg["birth_cell"][:nb], weights=dbg["birth_weight"][:nb].astype(np.float64),
                          minlength=gs * gs)
    # persistent weight of a cell after reweighting = rho_p (mu_A normalises it), when the cell
    # holds in-grid particles; border cells also hold clamped out-of-grid particles (weight 0)
    x, y = np.arange(gs * gs) % gs, np.arange(gs * gs) // gs
    interior = (x > 0) & (x < gs - 1) & (y > 0) & (y < gs - 1)
    occupied = cells["start_idx"] >= 0
    w_pers = np.where(occupied, cells["pers_occ_mass"].astype(np.float64), 0.0)
    expect = n * (w_pers + w_birth) / J
    got = np.bincount(g.get_particles()["grid_cell_idx"], minlength=gs * gs)
    dev = np.abs(got - expect)[interior]
    assert dev.max() < 2.0 + 1e-5 * expect[interior].max(), "copies per cell off by %g" % dev.max()
    assert got.sum() == n
    g.close()


def test_unreplayed_update_against_fp64_oracle(dogm, oracle, scene):
    """Same scene, independent random numbers: the GPU with its own Philox stream, the FP64
    oracle with draws of another seed.  Occupancy masses do not depend on the draws except
    through the predicted occupancy, and the velocity moments are sample statistics."""
    cfg = dict(scene.CONFIGS["small"])
    cfg.update(size=25.6, resolution=0.1, particle_count=300000, new_born_particle_count=30000, vehicles=6)
    sc = scene.Scene(cfg, seed=12)
    p = dogm.make_params(**scene.params_dict(cfg))
    g = dogm.DOGM(p, seed=3)
    o = oracle.OracleDOGM(p, np.float64)
    frames = 5
    for k in range(frames):
        m, x, y, yaw = sc.frame(k)
        g.update_grid(m, x, y, yaw, 0.1)
        out = o.update(m, x, y, yaw, 0.1, oracle.draws(999, 7, p.particle_count, p.new_born_particle_count, k))
    cg = g.get_grid_cells()
    co = out["cells"]
    occ_g, occ_o = cg["occ_mass"].astype(np.float64), co[:, 5]
    free_g, free_o = cg["free_mass"].astype(np.float64), co[:, 4]
    # the measurement dominates the combined masses: totals agree within 1 %
    assert abs(occ_g.sum() - occ_o.sum()) < 0.01 * occ_o.sum()
    assert abs(free_g.sum() - free_o.sum()) < 0.01 * free_o.sum()
    # particle velocity moments: two independent particle clouds of the same filter
    vg = g.get_particles()["state"][:, 2:4].astype(np.float64)
    vo = o.P_state[:, 2:4].astype(np.float64)
    for j in range(2):
        sd = np.sqrt(0.5 * (vg[:, j].var() + vo[:, j].var()))
        # resampling duplicates particles: allow 10 x the iid standard error
        assert abs(vg[:, j].mean() - vo[:, j].mean()) < 10 * sd * np.sqrt(2.0 / len(vg))
        assert abs(vg[:, j].std() / vo[:, j].std() - 1.0) < 0.05
    g.close()
