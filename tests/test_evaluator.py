"""CPU: the accuracy evaluator (dogm_cluster_cells, dogm_evaluator_*) against the reference's own
DBSCAN / PrecisionEvaluator (dogm/demo/utils/dbscan.cpp, precision_evaluator.cpp, metrics.cpp).

Pins: oracle/pyeval.py and the C ABI both reproduce tests/golden/eval_golden.npz (outputs of the
reference evaluator compiled from its sources) bit for bit; where oracle/_ref/libref_eval.so is
present the C ABI is also run beside the reference on larger seeded frames.  The evaluator is
host code: nothing here needs a GPU."""
import ctypes as C
import os

import numpy as np
import pytest

import pyeval

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "eval_golden.npz")
REF_LIB = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libref_eval.so")


def golden():
    d = np.load(GOLDEN)
    out = []
    for k in range(int(d["n_cases"])):
        coff, toff = d["c%d_cell_off" % k], d["c%d_truth_off" % k]
        cells, truth = d["c%d_cells" % k], d["c%d_truth" % k]
        frames = [(cells[coff[s]:coff[s + 1]], truth[toff[s]:toff[s + 1]]) for s in range(len(coff) - 1)]
        out.append({"frames": frames, "labels": d["c%d_labels" % k], "counts": d["c%d_counts" % k],
                    "mae": d["c%d_mae" % k], "rmse": d["c%d_rmse" % k], "unassigned": int(d["c%d_unassigned" % k])})
    return out, float(d["resolution"]), float(d["grid_length"])


def as_cells(dogm, c):
    out = np.zeros(len(c), dogm.DYNAMIC_CELL_DTYPE)
    out["x"], out["y"] = c[:, 0], c[:, 1]
    out["index"] = (c[:, 1] * 500 + c[:, 0]).astype(np.int32)
    out["cell"]["mean_x_vel"], out["cell"]["mean_y_vel"] = c[:, 2], c[:, 3]
    return out


def same_bits(a, b):
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


def test_golden_fixture_exercises_the_reference_quirk():
    cases, _, _ = golden()
    differs = 0
    for case in cases:
        off = 0
        for c, _ in case["frames"]:
            ref = case["labels"][off:off + len(c)]
            std, _ = pyeval.dbscan(c[:, 0], c[:, 1], mode="standard")
            differs += int(np.any(ref != std))
            off += len(c)
    assert differs > 0, "fixtures never hit the labelling slip of dbscan.cpp:64-67"


@pytest.mark.parametrize("k", range(8))
def test_oracle_matches_reference_golden(k):
    cases, res, glen = golden()
    case = cases[k]
    ev = pyeval.Evaluator(res, glen, "reference")
    off = 0
    for s, (c, t) in enumerate(case["frames"]):
        lab, n = pyeval.dbscan(c[:, 0], c[:, 1], mode="reference")
        assert n == case["counts"][s]
        assert np.array_equal(lab, case["labels"][off:off + len(c)])
        off += len(c)
        ev.add_step(c[:, 0], c[:, 1], c[:, 2], c[:, 3], t)
    mae, rmse, _, una = ev.summary()
    assert same_bits(mae, case["mae"]) and same_bits(rmse, case["rmse"])
    assert una == case["unassigned"]


@pytest.mark.parametrize("k", range(8))
def test_abi_matches_reference_golden(dogm, k):
    cases, res, glen = golden()
    case = cases[k]
    ev = dogm.Evaluator(res, glen, "reference")
    off = 0
    for s, (c, t) in enumerate(case["frames"]):
        cells = as_cells(dogm, c)
        lab, n = dogm.cluster_cells(cells, 3.0, 5, "reference")
        assert n == case["counts"][s]
        assert np.array_equal(lab, case["labels"][off:off + len(c)])
        off += len(c)
        ev.add_step(cells, t)
    s = ev.summary()
    assert same_bits(s["mae"], case["mae"]) and same_bits(s["rmse"], case["rmse"])
    assert s["unassigned"] == case["unassigned"]
    ev.close()


@pytest.mark.parametrize("k", range(8))
def test_abi_standard_mode_matches_oracle(dogm, k):
    cases, res, glen = golden()
    ev = dogm.Evaluator(res, glen, "standard")
    pe = pyeval.Evaluator(res, glen, "standard")
    for c, t in cases[k]["frames"]:
        cells = as_cells(dogm, c)
        lab, n = dogm.cluster_cells(cells, 3.0, 5, "standard")
        ref, rn = pyeval.dbscan(c[:, 0], c[:, 1], mode="standard")
        assert n == rn and np.array_equal(lab, ref)
        got = ev.add_step(cells, t)
        want = pe.add_step(c[:, 0], c[:, 1], c[:, 2], c[:, 3], t)
        assert len(got) == len(want)
        for g, w in zip(got, want):
            assert g["cells"] == w["cells"] and g["truth"] == w["truth"]
            assert same_bits([g["x"], g["y"], g["vx"], g["vy"]], [w["x"], w["y"], w["vx"], w["vy"]])
    a, b = ev.summary(), pe.summary()
    assert same_bits(a["mae"], b[0]) and same_bits(a["rmse"], b[1])
    assert (a["detections"], a["unassigned"]) == (b[2], b[3])


def test_standard_mode_clusters_are_density_connected(dogm):
    rng = np.random.default_rng(3)
    pts = set()
    for _ in range(12):
        x0, y0 = rng.integers(0, 120, 2)
        for _ in range(40):
            pts.add((int(x0 + rng.integers(0, 7)), int(y0 + rng.integers(0, 7))))
    xy = np.array(sorted(pts, key=lambda p: (p[1], p[0])), np.float32)
    cells = as_cells(dogm, np.concatenate([xy, np.zeros_like(xy)], 1))
    lab, n = dogm.cluster_cells(cells, 3.0, 5, "standard")
    d2 = ((xy[:, None, :] - xy[None, :, :]) ** 2).sum(-1)
    nbr = np.sqrt(d2.astype(np.float32)) <= 3.0
    core = nbr.sum(1) >= 5
    # core cells within eps share a cluster; every core cell is labelled; border cells sit next to a core
    i, j = np.nonzero(nbr & core[:, None] & core[None, :])
    assert np.all(lab[i] == lab[j])
    assert np.all(lab[core] >= 0)
    for p in np.nonzero((lab >= 0) & ~core)[0]:
        assert np.any(nbr[p] & core & (lab == lab[p]))
    assert np.all(nbr[lab < 0][:, core].sum(1) == 0)
    assert set(np.unique(lab[lab >= 0])) == set(range(n))


def test_empty_inputs_and_argument_checks(dogm):
    ev = dogm.Evaluator(0.1, 50.0)
    empty = np.zeros(0, dogm.DYNAMIC_CELL_DTYPE)
    assert len(ev.add_step(empty, [(1, 2, 3, 4)])) == 0
    one = as_cells(dogm, np.array([[10, 10, 1, 1]] * 1, np.float32))
    assert len(ev.add_step(one, np.zeros((0, 4), np.float32))) == 0
    s = ev.summary()
    assert s["detections"] == 0 and s["unassigned"] == 0 and np.all(np.isnan(s["mae"]))
    lab, n = dogm.cluster_cells(empty)
    assert n == 0 and len(lab) == 0
    lib = dogm.load()
    nc = C.c_int(0)
    assert lib.dogm_cluster_cells(None, 3, 3.0, 5, 0, None, C.byref(nc)) == 1
    assert lib.dogm_cluster_cells(None, 0, 0.0, 5, 0, None, C.byref(nc)) == 1
    assert lib.dogm_cluster_cells(None, 0, 3.0, 5, 7, None, C.byref(nc)) == 1
    e = C.c_void_p()
    assert lib.dogm_evaluator_create(0.0, 50.0, 0, C.byref(e)) == 1
    assert lib.dogm_evaluator_create(0.1, 50.0, 2, C.byref(e)) == 1
    assert lib.dogm_evaluator_summary(None, None, None, None, None) == 1
    ev.close()


def _ref_lib():
    if not os.path.exists(REF_LIB):
        pytest.skip("oracle/_ref/libref_eval.so is not built here (the reference sources are absent)")
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_eval_golden", os.path.join(HERE, "golden",
                                                                                   "make_eval_golden.py"))
    g = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(g)
    return g, g.load_ref()


@pytest.mark.parametrize("seed", [101, 102, 103])
def test_abi_matches_reference_build_on_crowded_frames(dogm, seed):
    g, lib = _ref_lib()
    rng = np.random.default_rng(seed)
    frames = [g.frame(rng, int(rng.integers(20, 40)), int(rng.integers(50, 200))) for _ in range(3)]
    labels, counts, _, _, _, _, mae, rmse, una = g.reference(lib, frames)
    ev = dogm.Evaluator(g.RESOLUTION, g.GRID_LENGTH, "reference")
    for s, (c, t) in enumerate(frames):
        cells = as_cells(dogm, c)
        lab, n = dogm.cluster_cells(cells, 3.0, 5, "reference")
        assert n == counts[s] and np.array_equal(lab, labels[s])
        ev.add_step(cells, t)
    got = ev.summary()
    assert same_bits(got["mae"], mae) and same_bits(got["rmse"], rmse) and got["unassigned"] == una
