"""Accuracy-evaluator oracle (test infrastructure: the checker, not the product).

Pure-Python / numpy-float32 restatement of the demo's evaluator: DBSCAN
(dogm/demo/utils/dbscan.cpp:24-114), the cluster mean in metres with y up
(precision_evaluator.cpp:98-121), nearest-object assignment within 5 m
(precision_evaluator.cpp:38-94) and the MAE / RMSE metrics (metrics.cpp:8-56).  Region queries
scan every point (O(n^2)), as the reference does, so keep inputs to a few thousand cells.

mode "reference" follows dbscan.cpp:55-98 step by step, including its labelling of the first
|seeds| points of the input (dbscan.cpp:64-67) and its seed list with erase-all-equal;
mode "standard" is the published DBSCAN with the same visiting order.  Pinned against the
reference's own evaluator, compiled here by oracle/ref/build_ref.py, through the fixtures of
tests/golden/make_eval_golden.py.
"""
from __future__ import annotations

import numpy as np

UNCLASSIFIED, NOISE = -2, -1
MAX_ASSIGN, EPS, MIN_CELLS = np.float32(5.0), np.float32(3.0), 5

f32 = np.float32


def _dist(ax, ay, bx, by) -> np.float32:
    dx = f32(f32(ax) - f32(bx))
    dy = f32(f32(ay) - f32(by))
    return np.sqrt(f32(f32(dx * dx) + f32(dy * dy)))


def _region(x, y, q, eps):
    # float32 array arithmetic rounds each operation like the scalar expression in dbscan.cpp:19-22
    dx = x[q] - x
    dy = y[q] - y
    return np.nonzero(np.sqrt(dx * dx + dy * dy) <= eps)[0].tolist()


def dbscan(x, y, eps=EPS, min_cells=MIN_CELLS, mode="reference"):
    """Labels (cluster index or -1) and cluster count; x, y float32 sequences."""
    x = np.asarray(x, np.float32)
    y = np.asarray(y, np.float32)
    n = len(x)
    label = [UNCLASSIFIED] * n
    eps = f32(eps)
    cid = 0
    for i in range(n):
        if label[i] != UNCLASSIFIED:
            continue
        seeds = _region(x, y, i, eps)
        if len(seeds) < min_cells:
            label[i] = NOISE
            continue
        if mode == "reference":
            for k in range(len(seeds)):  # dbscan.cpp:64-67: the first |seeds| points
                label[k] = cid
            seeds = [s for s in seeds if s != i]
            while seeds:
                cur = seeds[0]
                res = _region(x, y, cur, eps)
                if len(res) >= min_cells:
                    for p in res:
                        if label[p] in (UNCLASSIFIED, NOISE):
                            if label[p] == UNCLASSIFIED:
                                seeds.append(p)
                            label[p] = cid
                seeds = [s for s in seeds if s != cur]
        else:
            label[i] = cid
            queue = []
            for p in seeds:
                if p != i and label[p] in (UNCLASSIFIED, NOISE):
                    if label[p] == UNCLASSIFIED:
                        queue.append(p)
                    label[p] = cid
            while queue:
                cur = queue.pop(0)
                res = _region(x, y, cur, eps)
                if len(res) >= min_cells:
                    for p in res:
                        if label[p] in (UNCLASSIFIED, NOISE):
                            if label[p] == UNCLASSIFIED:
                                queue.append(p)
                            label[p] = cid
        cid += 1
    return np.array([l if l >= 0 else -1 for l in label], np.int32), cid


class Evaluator:
    """PrecisionEvaluator with an MAE and an RMSE metric (float32 accumulators)."""

    def __init__(self, resolution: float, grid_length: float, mode: str = "reference"):
        self.r = f32(resolution)
        self.g = f32(grid_length)
        self.mode = mode
        self.abs = [f32(0)] * 4
        self.sq = [f32(0)] * 4
        self.detections = 0
        self.unassigned = 0

    def add_step(self, x, y, vx, vy, truth):
        """truth: rows (x, y, vx, vy) in metres, y up.  Returns the frame's cluster records."""
        out = []
        if len(x) == 0 or len(truth) == 0:
            return out
        label, nc = dbscan(x, y, mode=self.mode)
        with np.errstate(invalid="ignore", divide="ignore"):
            for c in range(nc):
                s = [f32(0)] * 4
                k = 0
                for i in np.nonzero(label == c)[0]:
                    s[0] = f32(s[0] + f32(x[i]))
                    s[1] = f32(s[1] + f32(y[i]))
                    s[2] = f32(s[2] + f32(vx[i]))
                    s[3] = f32(s[3] + f32(vy[i]))
                    k += 1
                kf = f32(k)
                mx = f32(f32(s[0] / kf) * self.r)
                my = f32(self.g - f32(f32(s[1] / kf) * self.r))
                mvx = f32(f32(s[2] / kf) * self.r)
                mvy = f32(-f32(f32(s[3] / kf) * self.r))
                best, bi = None, -1
                for t, v in enumerate(truth):
                    d = _dist(mx, my, v[0], v[1])
                    if d < MAX_ASSIGN and (bi < 0 or d < best):
                        best, bi = d, t
                rec = {"x": mx, "y": my, "vx": mvx, "vy": mvy, "cells": k, "truth": bi}
                if bi < 0:
                    self.unassigned += 1
                else:
                    v = truth[bi]
                    err = [f32(mx - f32(v[0])), f32(my - f32(v[1])), f32(mvx - f32(v[2])), f32(mvy - f32(v[3]))]
                    for j in range(4):
                        self.abs[j] = f32(self.abs[j] + abs(err[j]))
                        self.sq[j] = f32(self.sq[j] + f32(err[j] * err[j]))
                    self.detections += 1
                    rec["err"] = err
                out.append(rec)
        return out

    def summary(self):
        with np.errstate(invalid="ignore", divide="ignore"):
            n = f32(self.detections)
            mae = np.array([f32(a / n) for a in self.abs], np.float32)
            rmse = np.array([np.sqrt(f32(s / n)) for s in self.sq], np.float32)
        return mae, rmse, self.detections, self.unassigned
