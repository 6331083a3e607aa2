"""GPU: the CUDA path against the reference's own CUDA build.

The reference's kernels are compiled from its sources (dogm/src/kernel/) into sm_103a cubins
by oracle/ref/build_ref.py and run in the restated host sequence of dogm::DOGM::updateGrid
(oracle/ref/ref_harness.cu).  Both implementations start from the same particles; the
reference's own curand draws (captured from its XORWOW states just before each random stage)
are replayed into the GB300 path, so:
  * predicted states, cell keys, the stable sort by cell and the cell ranges are bit-exact,
    with and without an ego shift (dogm.cu:161-203, predict.cu:16-52, dogm.cu:262-281);
  * the reference's multinomial index search (resampling.cu:34-47) reproduced by
    dogm_lower_bound_f32 on the reference's own accumulator and sorted draws is bit-exact;
  * newborn velocities (z * sigma_v per slot) are bit-exact, newborn slots per cell agree
    except where the reference's float allocation rounds a boundary differently;
  * masses and velocity moments of both builds are compared with the FP64 oracle on the same
    inputs: per-field error versus FP64 is reported, the GB300 path's must stay within the
    stated FP32 tolerances (5e-7 on masses, 2e-6 of the second moment on moments) and be no
    larger than the reference build's (whose float prefix-sum differences lose precision as the
    total particle weight grows, quirk Q4).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
MASS_FIELDS = ["new_born_occ_mass", "pers_occ_mass", "free_mass", "occ_mass", "pred_occ_mass"]
MOMENT_FIELDS = ["mean_x_vel", "mean_y_vel", "var_x_vel", "var_y_vel", "covar_xy_vel"]


def _particles(gs, n, seed):
    rng = np.random.default_rng(seed)
    st = np.empty((n, 4), np.float32)
    st[:, 0:2] = rng.uniform(0.0, gs, (n, 2))
    st[:, 2:4] = rng.normal(0.0, 4.0, (n, 2))
    idx = (np.clip(st[:, 0].astype(np.int32), 0, gs - 1) + gs * np.clip(st[:, 1].astype(np.int32), 0, gs - 1))
    return st, idx.astype(np.int32)


def _oracle_from(oracle, p, state, idx, assoc, weight, pose):
    o = oracle.OracleDOGM(p, np.float64)
    o.P_state[:] = state
    o.P_key[:] = idx.astype(np.uint32) | (assoc.astype(np.uint32) << np.uint32(31))
    o.w_res[0] = weight
    o.first_measurement = False
    if pose is not None:
        o.pose_update(*pose)
    return o


def _check_frame(dogm, pyref_build, ours, tr, label):
    dbg = ours.debug_export()
    assert np.array_equal(dbg["sorted_cell"], tr["sorted_idx"]), label + ": sorted cell keys differ"
    bad = np.flatnonzero((dbg["sorted_state"].view(np.uint32) != tr["sorted_state"].view(np.uint32)).any(1))
    assert bad.size == 0, "%s: %d predicted states differ, first %s: %r vs %r" % (
        label, bad.size, bad[:3], dbg["sorted_state"][bad[:3]], tr["sorted_state"][bad[:3]])
    co = ours.get_grid_cells()
    cr = pyref_build.get_grid_cells(dogm.GRID_CELL_DTYPE)
    assert np.array_equal(co["start_idx"], cr["start_idx"]), label + ": start_idx"
    assert np.array_equal(co["end_idx"], cr["end_idx"]), label + ": end_idx"
    # the reference's multinomial search on its own accumulator and sorted draws
    got = dogm.lower_bound_f32(tr["joint_accum"], tr["rand_sorted"], clamp_last=True)
    assert np.array_equal(got, tr["resample_idx"]), label + ": lower_bound"
    return co, cr, dbg


@pytest.mark.parametrize("size,res,n,b", [(25.6, 0.1, 150000, 15000),
                                          (120.0, 0.1, 2_000_000, 200_000)])  # the benchmark's shape
def test_against_reference_build(dogm, oracle, pyref, scene, size, res, n, b):
    p = dogm.make_params(size=size, resolution=res, particle_count=n, new_born_particle_count=b)
    ref = pyref.ReferenceDOGM(p)
    gs = ref.grid_size
    ours = dogm.DOGM(p, seed=1)
    ours.debug_enable(True)
    n = p.particle_count
    state, idx = _particles(gs, n, 5)
    assoc = np.zeros(n, np.uint8)
    w0 = np.float32(1.0) / np.float32(n)
    ref.set_particles(state, idx, np.full(n, w0, np.float32), assoc)
    ours.set_particles(state, idx, assoc, float(w0))
    o = _oracle_from(oracle, p, state, idx, assoc, w0, None)
    report = {}
    poses = [(0.0, 0.0), (0.35, -0.27)]  # the second frame shifts the grid by (-3, +2) cells
    for k, (x, y) in enumerate(poses):
        meas = scene.random_measurements(gs, seed=60 + k, occ_fraction=0.05)
        tr = ref.update(meas, x, y, 0.0, 0.1, trace=True)
        ours.set_replay(None, tr["predict_z"], tr["birth_z"], None)
        ours.update_grid(meas, x, y, 0.0, 0.1)
        draws = {"predict_z": tr["predict_z"], "birth_z": tr["birth_z"], "resample_r": 0}
        out = o.update(meas, x, y, 0.0, 0.1, draws)
        co, cr, dbg = _check_frame(dogm, ref, ours, tr, "frame %d" % k)

        # newborns: velocities are z * sigma per slot in both builds
        rb = ref.get_birth()
        nb = dbg["n_birth"]
        assert nb == p.new_born_particle_count
        assert np.array_equal(dbg["birth_state"][:nb, 2:4].view(np.uint32), rb["state"][:, 2:4].view(np.uint32)), \
            "frame %d: newborn velocities" % k
        # newborns per cell: the reference's slot boundaries int(float scan * B / max) drift from
        # the exact ones by a fraction of a slot (float accumulation over all cells), and its
        # per-slot cell index races at cell starts (nu_A + 1 slots marked, Q5), so the counts
        # are recovered from its cell records (w_A = rho_b / nu_A with p_A = 1) and compared as
        # cumulative slot boundaries
        rho_b, w_a = cr["new_born_occ_mass"].astype(np.float64), cr["w_A"].astype(np.float64)
        n_ref = np.where(w_a > 0, np.rint(rho_b / np.where(w_a > 0, w_a, 1.0)), 0.0)
        n_ours = np.bincount(dbg["birth_cell"][:nb], minlength=gs * gs)
        drift = np.abs(np.cumsum(n_ref) - np.cumsum(n_ours)).max()
        report["frame %d newborn slot drift" % k] = (0.0, drift)
        # (the reference's frame-1 input varies run to run: its Q5 race moves newborns between
        # cells before they are resampled; observed drift 1-3 slots of 15000.  At 2e5 slots over
        # 1.44e6 cells its float scan moves 46-47 slots on the first frame and ~250 after its
        # resampling, totals included)
        tol = max(2, (1e-3 if k == 0 else 5e-3) * nb)
        assert abs(n_ref.sum() - nb) <= tol and drift <= tol, \
            "frame %d: newborn slot boundaries drift by %g" % (k, drift)

        # masses and moments versus FP64 (cells whose particle ranges agree with the double run)
        f64 = out["cells"]
        ok = (co["start_idx"] == f64[:, 0].astype(np.int32)) & (co["end_idx"] == f64[:, 1].astype(np.int32))
        # a particle within float rounding of a border may change cell in double, which moves the
        # ranges of every cell between its two keys (up to a grid row): > 99.5 % of the cells
        # agree at 256^2 / 1.5e5 particles, 96 % at 1200^2 / 2e6
        report["frame %d cells with FP64 ranges" % k] = (float(ok.mean()), 0.0)
        assert ok.mean() > (0.995 if gs < 1000 else 0.94)
        # the outermost ring of cells holds the particles just outside the grid (keys clamped,
        # weight 0, predict.cu:41-48); a particle within rounding of the edge is in the grid in
        # one precision and out in the other, which moves a light cell's newborn mass by half its
        # occupancy with the range unchanged, so the ring is left out of the FP64 comparison
        inner = np.zeros((gs, gs), bool)
        inner[1:-1, 1:-1] = True
        ok &= inner.ravel()
        names = dogm.GRID_CELL_FIELDS
        for name in MASS_FIELDS:
            j = names.index(name)
            e_ours = np.abs(co[name].astype(np.float64) - f64[:, j])[ok].max()
            e_ref = np.abs(cr[name].astype(np.float64) - f64[:, j])[ok].max()
            report["frame %d %s" % (k, name)] = (e_ours, e_ref)
            assert e_ours <= 5e-7, "frame %d %s: GB300 vs FP64 %g" % (k, name, e_ours)
            # the reference's per-cell sums are differences of a float prefix sum over all
            # particles (common.h:24-32): their error grows with the total weight, which is ~1 on
            # the first frame and J (thousands) after a resampling; it is never more accurate
            assert e_ours <= max(e_ref, 5e-7), "frame %d %s: reference closer to FP64" % (k, name)
            # sanity bound that the reference build ran at all (observed up to 1.02e-2 at 256^2: its
            # frame-1 input varies run to run through the Q5 race).  At 1200^2 / 2e6 its prefix-sum
            # differences after a resampling are off by more than 1 (masses leave [0, 1]), so there
            # the error is only reported.
            if gs < 1000:
                assert e_ref <= 5e-2, "frame %d %s: reference build vs FP64 %g" % (k, name, e_ref)
        # moments divide by rho_p = occ - rho_b; where that difference cancels (FP64 can reach
        # exactly 0 and take the zero-moment branch while FP32 keeps 1e-10) the comparison says
        # nothing about the path, so only cells whose FP32 rho_p is within 1e-3 of FP64 count
        # (at 1200^2 one cell of ~1e6 is left out; the reference build, with the same formula,
        # is off there too)
        rp64 = f64[:, names.index("pers_occ_mass")]
        well = np.abs(co["pers_occ_mass"].astype(np.float64) - rp64) <= 1e-3 * np.abs(rp64)
        occ = ok & (co["start_idx"] >= 0) & well
        scale = 1.0 + f64[:, 11] ** 2 + f64[:, 12] ** 2 + np.abs(f64[:, 13]) + np.abs(f64[:, 14])
        for name in MOMENT_FIELDS:
            j = names.index(name)
            e_ours = (np.abs(co[name].astype(np.float64) - f64[:, j]) / scale)[occ].max()
            e_ref = (np.abs(cr[name].astype(np.float64) - f64[:, j]) / scale)[occ].max()
            report["frame %d %s" % (k, name)] = (e_ours, e_ref)
            assert e_ours <= 2e-6, "frame %d %s: GB300 vs FP64 %g" % (k, name, e_ours)

        # both continue from the reference's resampled particles (multinomial there,
        # systematic here), so the next frame starts from identical inputs again
        rp = ref.get_particles()
        assert np.all(rp["weight"] == rp["weight"][0])
        ours.set_particles(rp["state"], rp["grid_cell_idx"], rp["associated"], float(rp["weight"][0]))
        o = _oracle_from(oracle, p, rp["state"], rp["grid_cell_idx"], rp["associated"], rp["weight"][0], (x, y, 0.0))
        o.free_mass[:] = co["free_mass"]  # the free mass the GB300 path carries into the next frame
    print("\nper-field max error versus FP64 (GB300, reference build):")
    for k, (a, b) in report.items():
        print("  %-26s %.3e  %.3e" % (k, a, b))
    ours.close()
    ref.close()


def test_reference_build_runs_the_large_workload_shape(dogm, pyref, scene):
    """The reference build at the benchmark's grid shape completes and conserves its counts."""
    p = dogm.make_params(size=120.0, resolution=0.1, particle_count=2_000_000, new_born_particle_count=200_000)
    ref = pyref.ReferenceDOGM(p)
    assert ref.grid_size == 1200
    for k in range(2):
        ref.update(scene.random_measurements(1200, seed=k, occ_fraction=0.02), 0.0, 0.0, 0.0, 0.1)
    cells = ref.get_grid_cells(dogm.GRID_CELL_DTYPE)
    occupied = cells["start_idx"] >= 0
    assert (cells["end_idx"][occupied] - cells["start_idx"][occupied] + 1).sum() == p.particle_count
    ref.close()
