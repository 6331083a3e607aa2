"""Generates tests/golden/eval_golden.npz: outputs of the reference's own accuracy evaluator.

Feeds seeded synthetic frames of dynamic cells (blobs of moving cells in row-major order, some
touching, scattered single cells, ground-truth objects near most blobs plus distractors, a frame
without cells and one without objects) to the reference's DBSCAN and PrecisionEvaluator
(dogm/demo/utils/dbscan.cpp, precision_evaluator.cpp, metrics.cpp), compiled from the reference
sources into oracle/_ref/libref_eval.so by oracle/ref/build_ref.py, and stores inputs and
outputs: per frame the cluster label of every cell, per case the MAE and RMSE of
(x, y, vx, vy) and the unassigned-detection count.

    python oracle/ref/build_ref.py && python tests/golden/make_eval_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(REPO, "oracle", "_ref", "libref_eval.so")
OUT = os.path.join(HERE, "eval_golden.npz")

GRID_CELLS, RESOLUTION = 500, 0.1  # the demo's 50 m grid at 0.1 m
GRID_LENGTH = GRID_CELLS * RESOLUTION


def frame(rng: np.random.Generator, n_blobs: int, n_noise: int):
    """One frame: cells (x, y, vx, vy; row-major, distinct) and objects (x, y, vx, vy, metres)."""
    cells = {}
    truth = []
    for b in range(n_blobs):
        w, h = int(rng.integers(1, 9)), int(rng.integers(1, 6))
        x0, y0 = int(rng.integers(0, GRID_CELLS - w)), int(rng.integers(0, GRID_CELLS - h))
        if b > 0 and rng.random() < 0.25:  # touch the previous blob
            x0 = min(max(px + pw + int(rng.integers(-1, 3)), 0), GRID_CELLS - w)
            y0 = min(max(py + int(rng.integers(-2, 3)), 0), GRID_CELLS - h)
        px, py, pw = x0, y0, w
        vx, vy = rng.normal(0, 60), rng.normal(0, 60)  # cells per second
        for y in range(y0, y0 + h):
            for x in range(x0, x0 + w):
                if rng.random() < 0.9:
                    cells[(x, y)] = (vx + rng.normal(0, 8), vy + rng.normal(0, 8))
        if rng.random() < 0.8:
            cx, cy = (x0 + (w - 1) / 2) * RESOLUTION, GRID_LENGTH - (y0 + (h - 1) / 2) * RESOLUTION
            truth.append((cx + rng.normal(0, 0.8), cy + rng.normal(0, 0.8), vx * RESOLUTION + rng.normal(0, 1),
                          -vy * RESOLUTION + rng.normal(0, 1)))
    for _ in range(n_noise):
        x, y = int(rng.integers(0, GRID_CELLS)), int(rng.integers(0, GRID_CELLS))
        cells.setdefault((x, y), (rng.normal(0, 60), rng.normal(0, 60)))
    for _ in range(int(rng.integers(0, 3))):  # distractors
        truth.append((rng.uniform(0, GRID_LENGTH), rng.uniform(0, GRID_LENGTH), rng.normal(0, 5), rng.normal(0, 5)))
    keys = sorted(cells, key=lambda k: (k[1], k[0]))
    c = np.array([(k[0], k[1], cells[k][0], cells[k][1]) for k in keys], np.float32).reshape(-1, 4)
    t = np.array(truth, np.float32).reshape(-1, 4)
    return c, t


def case(seed: int, steps: int):
    rng = np.random.default_rng(seed)
    frames = []
    for s in range(steps):
        c, t = frame(rng, int(rng.integers(2, 8)), int(rng.integers(0, 30)))
        if s == 2 and seed % 2 == 0:
            c = c[:0]
        if s == 3 and seed % 3 == 0:
            t = t[:0]
        frames.append((c, t))
    return frames


def dense_frame(seed: int):
    """A crowded frame (long row-major runs) where the reference's labelling slip shows most."""
    rng = np.random.default_rng(seed)
    return frame(rng, 14, 60)


def reference(lib, frames):
    labels, counts = [], []
    for c, _ in frames:
        n = len(c)
        lab = np.empty(max(n, 1), np.int32)
        x, y = np.ascontiguousarray(c[:, 0]), np.ascontiguousarray(c[:, 1])
        counts.append(lib.ref_dbscan(x.ctypes.data, y.ctypes.data, n, C.c_float(3.0), 5, lab.ctypes.data))
        labels.append(lab[:n])
    steps = len(frames)
    coff = np.zeros(steps + 1, np.int32)
    toff = np.zeros(steps + 1, np.int32)
    for s, (c, t) in enumerate(frames):
        coff[s + 1] = coff[s] + len(c)
        toff[s + 1] = toff[s] + len(t)
    cc = np.concatenate([c for c, _ in frames]).reshape(-1, 4)
    tt = np.concatenate([t for _, t in frames]).reshape(-1, 4)
    cols = [np.ascontiguousarray(cc[:, j]) for j in range(4)] + [np.ascontiguousarray(tt[:, j]) for j in range(4)]
    mae, rmse = np.empty(4, np.float32), np.empty(4, np.float32)
    una = C.c_int(0)
    lib.ref_evaluate(steps, coff.ctypes.data, *[a.ctypes.data for a in cols[:4]], toff.ctypes.data,
                     *[a.ctypes.data for a in cols[4:]], C.c_float(RESOLUTION), C.c_float(GRID_LENGTH),
                     mae.ctypes.data, rmse.ctypes.data, C.byref(una))
    return labels, np.array(counts, np.int32), coff, toff, cc, tt, mae, rmse, una.value


def load_ref():
    lib = C.CDLL(LIB)
    lib.ref_dbscan.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_int, C.c_void_p]
    lib.ref_dbscan.restype = C.c_int
    lib.ref_evaluate.argtypes = [C.c_int, C.c_void_p] + [C.c_void_p] * 4 + [C.c_void_p] + [C.c_void_p] * 4 + \
        [C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.ref_evaluate.restype = C.c_int
    return lib


CASES = [(11, 6), (12, 6), (13, 6), (14, 4), (15, 4), (16, 8)]


def main() -> int:
    if not os.path.exists(LIB):
        print("oracle/_ref/libref_eval.so is missing: run oracle/ref/build_ref.py first", file=sys.stderr)
        return 1
    lib = load_ref()
    data = {"resolution": np.float32(RESOLUTION), "grid_length": np.float32(GRID_LENGTH)}
    all_cases = [case(seed, steps) for seed, steps in CASES] + [[dense_frame(seed)] for seed in (21, 22)]
    for k, frames in enumerate(all_cases):
        labels, counts, coff, toff, cc, tt, mae, rmse, una = reference(lib, frames)
        data["c%d_cell_off" % k] = coff
        data["c%d_truth_off" % k] = toff
        data["c%d_cells" % k] = cc
        data["c%d_truth" % k] = tt
        data["c%d_labels" % k] = np.concatenate(labels).astype(np.int32) if labels else np.zeros(0, np.int32)
        data["c%d_counts" % k] = counts
        data["c%d_mae" % k] = mae
        data["c%d_rmse" % k] = rmse
        data["c%d_unassigned" % k] = np.int32(una)
    data["n_cases"] = np.int32(len(all_cases))
    np.savez_compressed(OUT, **data)
    print("wrote", OUT, "cases", len(all_cases), "cells", sum(len(data["c%d_cells" % k]) for k in range(len(all_cases))))
    return 0


if __name__ == "__main__":
    sys.exit(main())
