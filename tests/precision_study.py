"""Precision study of the update (the precision workload: 2048 x 2048 cells at 0.1 m, 8e6
persistent and 8e5 newborn particles, heavy-tailed occupied masses Beta(0.5, 0.5), 30 frames).

Per frame, the GB300 path (FP32 state, exact fixed-point scans) and the FP64 oracle run on the
same inputs: the oracle is reset to the GPU's particles, weight and free mass before every
frame, and both take the GPU's own random draws, so every frame measures one update's error
and no divergence accumulates.  Reported per frame and over all frames:

  * resampling-index mismatch against FP64: the systematic comb over the frame's joint weights
    (dogm_debug_joint_weights) with the prefix in plain FP32, compensated FP32 (float pair) and
    FP64 (the oracle's comb_indices), and the GB300 path's own assignment (exact 64-bit
    fixed-point scan, dogm_debug_export resample_src), each compared slot by slot with FP64;
  * per-cell error against FP64 of occupied / free mass and velocity mean and variance (cells
    whose particle ranges agree with the double run; moments relative to the cell's second
    moment 1 + mx^2 + my^2 + |var_x| + |var_y|).

    python tests/precision_study.py [--frames 30] [--out report.json]   (needs the GPU)

The record of the full 30-frame run is tests/precision_study_2048.json.
Test infrastructure: imports the oracle; tests/test_gpu_precision.py runs a small case.
"""
from __future__ import annotations

import argparse
import importlib
import importlib.util
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
PKG = "dynamic-occupancy-grid-map_gb300"
COMB_MODES = ("fp32", "compensated_fp32", "fp64")


def heavy_tailed(m: np.ndarray, rng: np.random.Generator, eps: float = 1e-5) -> np.ndarray:
    """Occupied mass Beta(0.5, 0.5) wherever the inverse sensor model saw a hit."""
    out = m.copy()
    hit = out[:, 1] > 0.5
    occ = rng.beta(0.5, 0.5, int(hit.sum()))
    out[hit, 1] = np.clip(occ, eps, 1.0 - eps).astype(np.float32)
    out[hit, 0] = np.float32(eps)
    return out


def run(dogm, oracle, scene, frames: int = 30, size: float = 204.8, resolution: float = 0.1,
        particles: int = 8_000_000, newborn: int = 800_000, seed: int = 5, log=None) -> dict:
    cfg = dict(scene.CONFIGS["precision"])
    cfg.update(size=size, resolution=resolution, particle_count=particles, new_born_particle_count=newborn)
    sc = scene.Scene(cfg, seed=seed)
    p = dogm.make_params(**scene.params_dict(cfg))
    g = dogm.DOGM(p, seed=seed)
    g.debug_enable(True)
    o = oracle.OracleDOGM(p, np.float64)
    rng = np.random.default_rng(seed)
    names = dogm.GRID_CELL_FIELDS
    per_frame = []
    prev_cells = None
    n = p.particle_count
    for k in range(frames):
        t0 = time.time()
        m, x, y, yaw = sc.frame(k)
        m = heavy_tailed(m, rng)
        if prev_cells is not None:  # the oracle starts this frame from the GPU's state
            parts = g.get_particles()
            o.P_state[:] = parts["state"]
            o.P_key[:] = parts["grid_cell_idx"].astype(np.uint32) | (parts["associated"].astype(np.uint32) << 31)
            o.w_res[0] = parts["weight"].max()
            o.free_mass[:] = prev_cells["free_mass"]
        d = g.generate_draws(k)
        g.set_replay(d["init_u"], d["predict_z"], d["birth_z"], d["resample_r"])
        g.update_grid(m, x, y, yaw, 0.1)
        out = o.update(m, x, y, yaw, 0.1, d)
        cells = g.get_grid_cells()
        f64 = out["cells"]
        ok = (cells["start_idx"] == f64[:, 0].astype(np.int32)) & (cells["end_idx"] == f64[:, 1].astype(np.int32))
        occupied = ok & (cells["start_idx"] >= 0)
        rec = {"frame": k, "cells_compared": float(ok.mean())}
        for name in ("occ_mass", "free_mass", "pers_occ_mass", "new_born_occ_mass"):
            e = np.abs(cells[name].astype(np.float64) - f64[:, names.index(name)])[ok]
            rec[name] = {"max": float(e.max()), "mean": float(e.mean())}
        scale = 1.0 + f64[:, 11] ** 2 + f64[:, 12] ** 2 + np.abs(f64[:, 13]) + np.abs(f64[:, 14])
        for name in ("mean_x_vel", "mean_y_vel", "var_x_vel", "var_y_vel", "covar_xy_vel"):
            e = (np.abs(cells[name].astype(np.float64) - f64[:, names.index(name)]) / scale)[occupied]
            rec[name] = {"max": float(e.max()) if e.size else 0.0, "mean": float(e.mean()) if e.size else 0.0}
        # resampling indices against FP64
        w = g.debug_joint_weights()
        src = g.debug_export()["resample_src"]
        u = float(d["resample_r"]) / 2.0 ** 64
        idx = {mode: oracle.comb_indices(w, n, u, mode) for mode in COMB_MODES}
        rec["resample_mismatch"] = {
            "fp32": float(np.mean(idx["fp32"] != idx["fp64"])),
            "compensated_fp32": float(np.mean(idx["compensated_fp32"] != idx["fp64"])),
            "gb300_exact_fixed_point": float(np.mean(src != idx["fp64"])),
        }
        rec["joint_items"] = int(w.size)
        rec["seconds"] = round(time.time() - t0, 2)
        per_frame.append(rec)
        prev_cells = cells
        if log:
            log("frame %d: %s" % (k, json.dumps(rec)))
    g.close()

    def worst(key, stat="max"):
        return max(r[key][stat] for r in per_frame)

    summary = {
        "workload": "%d x %d cells at %.2f m, %d + %d particles, occupied mass Beta(0.5, 0.5) at hits, %d frames"
                    % (g.grid_size, g.grid_size, resolution, particles, newborn, frames),
        "resample_mismatch_vs_fp64": {m: {"mean": float(np.mean([r["resample_mismatch"][m] for r in per_frame])),
                                          "max": float(np.max([r["resample_mismatch"][m] for r in per_frame]))}
                                      for m in ("fp32", "compensated_fp32", "gb300_exact_fixed_point")},
        "cell_error_vs_fp64_max": {k: worst(k) for k in ("occ_mass", "free_mass", "pers_occ_mass",
                                                         "new_born_occ_mass", "mean_x_vel", "mean_y_vel",
                                                         "var_x_vel", "var_y_vel", "covar_xy_vel")},
        "cell_error_vs_fp64_mean": {k: float(np.mean([r[k]["mean"] for r in per_frame]))
                                    for k in ("occ_mass", "free_mass", "mean_x_vel", "var_x_vel")},
        "cells_compared_min": min(r["cells_compared"] for r in per_frame),
    }
    return {"summary": summary, "frames": per_frame}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--frames", type=int, default=30)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    for path in (REPO, os.path.join(REPO, "oracle")):
        sys.path.insert(0, path)
    spec = importlib.util.spec_from_file_location("dogm_build", os.path.join(REPO, PKG, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build_cuda()
    b.build_oracle()
    dogm = importlib.import_module(PKG)
    dogm.load()
    scene = importlib.import_module(PKG + ".scene")
    import pyoracle
    pyoracle.load()
    t0 = time.time()
    rep = run(dogm, pyoracle, scene, frames=args.frames, log=lambda s: print(s, flush=True))
    import subprocess
    try:
        gpu = subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader", "-i", "0"],
                             capture_output=True, text=True, timeout=10).stdout.strip()
    except (OSError, subprocess.SubprocessError):
        gpu = "unknown"
    rep["summary"]["provenance"] = {"command": "python tests/precision_study.py --frames %d" % args.frames,
                                    "gpu": gpu, "wall_s": round(time.time() - t0, 1)}
    print(json.dumps(rep["summary"], indent=1))
    if args.out:
        with open(args.out, "w") as f:
            json.dump(rep, f, indent=1)


if __name__ == "__main__":
    main()
