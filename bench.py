#!/usr/bin/env python
"""bench.py — ms per DOGM update on one GB300 at the 2M-particle / 1.44M-cell workload.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

A step is one full update (ego shift, predict, sort, mass update, reweighting, newborns,
moments, resampling) of the 1200 x 1200 grid with 2e6 persistent and 2e5 newborn particles,
driven by a seeded synthetic scene.  Prints one JSON line (rank 0).
  value   device time per update with the measurement grids already in HBM (CUDA events
          on the library's stream over K back-to-back updates; the working set, > 300 MB
          per update, is larger than the 129 MB L2, so no L2 flush is added)
  e2e     the same through the C ABI with host buffers: pinned measurement in, H2D copy,
          update, full grid (GridCell array) copied back to pinned host memory, per step
  --impl reference  the reference's pipeline transcribed to C (oracle/dogm_oracle.c,
          dogm_oracle_reference_f32) on all host cores, one full update per step.
"""
from __future__ import annotations

import argparse
import importlib
import importlib.util
import ctypes as C
import glob
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)
PKG = "dynamic-occupancy-grid-map_gb300"

METRIC = "ms/update and HBM GB/s at 2M particles/1.44M cells; batched frames/s, p50/p99"
# the headline workload, and the reference's own published case (--workload small)
WORKLOADS = {
    "large": "large: 120 x 120 m at 0.1 m (1200^2 = 1.44e6 cells), 2e6 persistent + 2e5 newborn particles, ego 10 m/s",
    "small": "small: 50 x 50 m at 0.2 m (250^2 = 62,500 cells), 3e5 persistent + 3e4 newborn particles, static ego "
             "(the case the reference's README times)",
}
WORKLOAD = "large"
WORKLOAD_DESC = WORKLOADS[WORKLOAD]
# Per-unit algorithmic bytes of the whole update (compulsory traffic of a single-read,
# single-write pipeline): 152 B per particle, 29 B per newborn, 108 B per cell.
ALG_PER_PARTICLE, ALG_PER_NEWBORN, ALG_PER_CELL = 152, 29, 108


def stage_bytes(N: int, B: int, C_: int, n_occ: int, n_birth_cells: int, sort_tiles: int, buckets: int) -> dict:
    """Algorithmic bytes per launch of each kernel (what it must read and write once)."""
    return {
        "predict": 40 * N + 4 * sort_tiles * buckets,  # state R/W 16+16, key R/W 4+4; bucket counts W
        "sort_scan": 8 * sort_tiles * buckets,      # bucket counts R, offsets W
        "sort_scatter": 40 * N + 4 * sort_tiles * buckets,  # state+key R 20, W 20 (bucketed); offsets R
        "cells": 40 * N + 112 * C_,                 # bucketed state+key R 20, sorted W 20; meas 16 + free 4
                                                    # R; record 64 + free 4 + rho_b 4 + w 4 + meas copy 16 W
        "newborn": 4 * C_ + 32 * n_birth_cells,     # newborn mass R; w_A/w_UA + newborn-cell list W
        "resample": 24 * N + 20 * N,                # key 4 + state 16 + weight 4 R; state+key 20 W
                                                    # (newborns are created in registers)
    }


def load_cudart():
    cands = ["libcudart.so", "libcudart.so.13"] + sorted(glob.glob("/usr/local/cuda*/lib64/libcudart.so*"))
    for c in cands:
        try:
            lib = C.CDLL(c)
            lib.cudaEventCreate.argtypes = [C.c_void_p]
            lib.cudaEventRecord.argtypes = [C.c_void_p, C.c_void_p]
            lib.cudaEventSynchronize.argtypes = [C.c_void_p]
            lib.cudaEventElapsedTime.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
            lib.cudaMalloc.argtypes = [C.c_void_p, C.c_size_t]
            lib.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
            lib.cudaFree.argtypes = [C.c_void_p]
            return lib
        except OSError:
            continue
    raise RuntimeError("libcudart not found")


class CudartBuffer:
    """Device buffer through libcudart alone (the reference arm maps nothing of this library)."""

    def __init__(self, rt, nbytes: int):
        self.rt, self.nbytes = rt, int(nbytes)
        p = C.c_void_p()
        assert rt.cudaMalloc(C.byref(p), C.c_size_t(self.nbytes)) == 0, "cudaMalloc"
        self.ptr = p.value

    def upload(self, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr)
        assert a.nbytes <= self.nbytes
        assert self.rt.cudaMemcpy(C.c_void_p(self.ptr), C.c_void_p(a.ctypes.data), C.c_size_t(a.nbytes), 1) == 0

    def free(self) -> None:
        if self.ptr:
            self.rt.cudaFree(C.c_void_p(self.ptr))
            self.ptr = 0


class Events:
    """CUDA events recorded on an explicit stream (the library's own)."""

    def __init__(self, rt, stream: int):
        self.rt, self.stream = rt, C.c_void_p(stream)

    def new(self):
        e = C.c_void_p()
        assert self.rt.cudaEventCreate(C.byref(e)) == 0
        return e

    def record(self, e):
        assert self.rt.cudaEventRecord(e, self.stream) == 0

    def elapsed(self, a, b) -> float:
        assert self.rt.cudaEventSynchronize(b) == 0
        ms = C.c_float()
        assert self.rt.cudaEventElapsedTime(C.byref(ms), a, b) == 0
        return float(ms.value)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.proc = None
        self.lines = []
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "10"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the timed region starts once the sampler is delivering
            t_end = time.perf_counter() + 5.0
            while not self.lines and time.perf_counter() < t_end and self.proc.poll() is None:
                time.sleep(0.01)
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peak_gbs() -> tuple[float, str]:
    """HBM copy bandwidth of this GPU pool: the measured figure when the pool's measurement
    file is present, else the earlier GB300 measurement of 6.8 TB/s."""
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
        v = peaks["hbm_gbs"]
        if isinstance(v, dict):  # a record with its figure under a key of its own
            v = next(v[k] for k in ("value", "gbs", "median", "mean") if k in v)
        return float(v), "measured"
    except (OSError, KeyError, ValueError, TypeError, StopIteration):
        return 6800.0, "fallback"


def make_frames(count: int, seed: int = 0):
    import importlib
    scene = importlib.import_module(PKG + ".scene")
    cfg = scene.CONFIGS[WORKLOAD]
    sc = scene.Scene(cfg, seed=seed)
    return scene, cfg, [sc.frame(k) for k in range(count)]


def pingpong(n: int, pool: int) -> int:
    """Frame index of step n when cycling a pool forth and back (0..P-1, P-2..1, 0, ...):
    the ego drives back and forth, so every step still moves the grid."""
    if pool <= 1:
        return 0
    period = 2 * pool - 2
    m = n % period
    return m if m < pool else period - m


def cpu_baseline(frames, cfg, n_frames: int, threads: int = 0) -> dict:
    """The reference's pipeline on the host cores over a bounded sample of the workload."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import importlib
    import pyoracle
    spec = importlib.util.spec_from_file_location("dogm_build", os.path.join(REPO, PKG, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build_oracle()
    dogm = importlib.import_module(PKG)
    p = dogm.make_params(**importlib.import_module(PKG + ".scene").params_dict(cfg))
    ref = pyoracle.ReferencePipeline(p, threads=threads)
    m, x, y, yaw = frames[0]
    ref.update(m, x, y, yaw, 0.1)  # first measurement: initialisation, not timed
    times = []
    for k in range(1, n_frames + 1):
        m, x, y, yaw = frames[pingpong(k, len(frames))]
        t0 = time.perf_counter()
        ref.update(m, x, y, yaw, 0.1)
        times.append((time.perf_counter() - t0) * 1e3)
    return {"value": statistics.median(times), "unit": "ms/update", "cores": ref.threads_used, "kind": "port",
            "sample": "%d full updates of the %s workload after the first-measurement initialisation "
                      "(dogm_oracle_reference_f32: the reference's stage sequence in float, OpenMP)"
                      % (n_frames, WORKLOAD)}


def run_gb300(args, rank: int, world: int):
    import importlib
    dogm = importlib.import_module(PKG)
    spec = importlib.util.spec_from_file_location("dogm_build", os.path.join(REPO, PKG, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build_cuda()
    dogm.load()
    K, W = args.steps, args.warmup
    P = 24  # profiled updates (event pairs tick coarsely: the stage times are means)
    # steps: [0, W] warm-up, then K timed, K end-to-end, P profiled; measurement grids come
    # from a pool of distinct frames cycled forth and back (pingpong)
    t0_, e0_, p0_ = W + 1, W + 1 + K, W + 1 + 2 * K
    pool = min(W + 1 + 2 * K + P, args.pool)
    scene, cfg, frames = make_frames(pool, seed=rank)
    fr = lambda n: pingpong(n, pool)
    p = dogm.make_params(**scene.params_dict(cfg))
    N, B = p.particle_count, p.new_born_particle_count
    g = dogm.DOGM(p, seed=123456, stream_id=rank, sync_each_update=False)
    C_ = g.cell_count
    rt = load_cudart()
    ev = Events(rt, g.stream())

    # measurement grids resident in HBM
    dbufs = []
    for m, *_ in frames:
        d = dogm.DeviceBuffer(m.nbytes)
        d.upload(m)
        dbufs.append(d)
    # launch widths chosen by the autotuner on this GPU (a scratch handle
    # fed the first frame; kept only when faster than the defaults)
    tune = g.autotune(dbufs[0].ptr, reps=10, device=True) if not args.no_autotune else None
    # first measurement (initialisation) + warm-up (graph capture for both mirrors)
    for k in range(W + 1):
        m, x, y, yaw = frames[fr(k)]
        g.update_grid(dbufs[fr(k)].ptr, x, y, yaw, 0.1, device=True)
    g.synchronize()

    # the timed region: R back-to-back blocks of the same K steps, R chosen so that the region
    # lasts at least --min-seconds (the clock sampler then sees it); value = mean per update
    def timed_block(r):
        # block r continues the forth-and-back frame sequence, so the ego keeps moving
        for k in range(t0_ + r * K, t0_ + (r + 1) * K):
            m, x, y, yaw = frames[fr(k)]
            g.update_grid(dbufs[fr(k)].ptr, x, y, yaw, 0.1, device=True)

    a, b_ = ev.new(), ev.new()
    ev.record(a)
    timed_block(0)
    ev.record(b_)
    block_ms = reduce_max(ev.elapsed(a, b_), world)
    repeats = max(1, int(np.ceil(args.min_seconds * 1e3 / max(block_ms, 1e-3))))
    g.synchronize()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")) if world > 1 else 0)
    clocks.start()
    barrier(world)
    e0, e1 = ev.new(), ev.new()
    wall0 = time.perf_counter()
    ev.record(e0)
    for r in range(repeats):
        timed_block(1 + r)
    ev.record(e1)
    total_ms = ev.elapsed(e0, e1)
    wall_s = time.perf_counter() - wall0
    g.synchronize()
    clk = clocks.stop()
    launches = g.last_launch_count() * K * repeats
    total_ms = reduce_max(total_ms, world)

    # the update at the residency a single persistent kernel per frame would have: every stage
    # limited to what the largest one (the cell pass: 64 registers, 87 KB shared memory) allows,
    # two 512-thread blocks = 1024 threads per SM (predict 2 x 512, bucket scan 1 x 1024,
    # newborn and resampling 4 x 256); same frames, 0.3 s of updates
    saved = g.get_tune()
    single = dogm.Tune()
    for i, m in enumerate((2, 1, 2, 2, 4, 4)):
        single.blocks_per_sm[i] = m
    g.set_tune(single)
    for r in range(3):
        timed_block(1 + repeats + r)
    g.synchronize()
    sr = max(1, repeats * 3 // 10)
    a, b_ = ev.new(), ev.new()
    ev.record(a)
    for r in range(sr):
        timed_block(4 + repeats + r)
    ev.record(b_)
    single_ms = reduce_max(ev.elapsed(a, b_), world) / (sr * K)
    g.set_tune(saved)
    for r in range(3):
        timed_block(4 + repeats + sr + r)
    g.synchronize()

    # synchronous updates, each waited for on the host like the reference's updateGrid
    # (dogm.cu:130): host wall clock per update, measurement grids in HBM
    sync_ms = []
    for k in range(e0_, e0_ + min(K, 100)):
        m, x, y, yaw = frames[fr(k)]
        w0 = time.perf_counter()
        g.update_grid(dbufs[fr(k)].ptr, x, y, yaw, 0.1, device=True)
        g.synchronize()
        sync_ms.append((time.perf_counter() - w0) * 1e3)

    # end to end through the C ABI with host buffers (pinned), grid read back every step
    pins = {}
    for k in range(K):
        i = fr(e0_ + k)
        if i not in pins:
            pa = dogm.PinnedArray((C_, 4), np.float32)
            pa.array[:] = frames[i][0]
            pins[i] = pa
    out = dogm.PinnedArray((C_,), dogm.GRID_CELL_DTYPE)
    g.synchronize()
    barrier(world)
    e2, e3 = ev.new(), ev.new()
    ev.record(e2)
    for k in range(K):
        i = fr(e0_ + k)
        _, x, y, yaw = frames[i]
        g.update_grid(pins[i].array, x, y, yaw, 0.1, device=False)
        g.get_grid_cells(out.array)
    ev.record(e3)
    e2e_sync_ms = reduce_max(ev.elapsed(e2, e3), world)
    # the same steps with the grid read back asynchronously (dogm_get_grid_cells_async): step
    # k's 92 MB copy out overlaps step k+1's measurement copy in and kernels; every step's grid
    # still lands in pinned host memory (two buffers in turn) inside the timed region
    outs = [out, dogm.PinnedArray((C_,), dogm.GRID_CELL_DTYPE)]
    g.synchronize()
    barrier(world)
    e4, e5 = ev.new(), ev.new()
    ev.record(e4)
    for k in range(K):
        i = fr(e0_ + k)
        _, x, y, yaw = frames[i]
        g.update_grid(pins[i].array, x, y, yaw, 0.1, device=False)
        g.get_grid_cells_async(outs[k % 2].array)
    g.synchronize()
    ev.record(e5)
    e2e_ms = reduce_max(ev.elapsed(e4, e5), world)
    for pa in pins.values():
        pa.free()
    for o in outs:
        o.free()

    # per-stage times (plain launches with an event between stages; separate from the timed loop)
    g.profile_enable(True)
    stage_runs = []
    for k in range(p0_, p0_ + P):
        m, x, y, yaw = frames[fr(k)]
        g.update_grid(dbufs[fr(k)].ptr, x, y, yaw, 0.1, device=True)
        g.synchronize()
        stage_runs.append(g.stage_times())
    g.profile_enable(False)
    stages = {k: statistics.fmean(r[k] for r in stage_runs) for k in stage_runs[0]}
    cells = g.get_grid_cells()
    n_occ = int((cells["start_idx"] >= 0).sum())
    n_bcells = int(((cells["w_A"] > 0) | (cells["w_UA"] > 0)).sum())
    sort_tiles = -(-N // 4096)
    sb = stage_bytes(N, B, C_, n_occ, n_bcells, sort_tiles, -(-C_ // 1024))
    dom = max(stages, key=lambda k: stages[k])
    peak, peak_src = peak_gbs()
    achieved = sb[dom] / (stages[dom] * 1e-3) / 1e9

    ms = total_ms / (K * repeats)
    alg = ALG_PER_PARTICLE * N + ALG_PER_NEWBORN * B + ALG_PER_CELL * C_
    line = {
        "metric": METRIC, "value": round(ms, 4), "unit": "ms/update", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": round(ms, 4), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "timed_region": {"repeats_of_k_steps": repeats, "updates": K * repeats, "device_s": round(total_ms / 1e3, 3),
                         "host_wall_s": round(wall_s, 3)},
        "dtype": "f32", "data": "synthetic (seeded scene: 40 vehicles + 30 pedestrians, 2160-beam lidar, "
                                "inverse sensor model; no public dataset exists for this workload)",
        "config": {"workload": WORKLOAD_DESC, "cells": C_, "particles": N, "newborn": B,
                   "l2": "inputs larger than L2 (per-update working set > 300 MB vs 129 MB L2); no flush",
                   "parallelism": "replicas" if world > 1 else "single",
                   "autotune": tune.as_dict() if tune is not None else "off"},
        "hbm_gbs_whole_update": round(alg / (ms * 1e-3) / 1e9, 1),
        "updates_per_s": round(1e3 / ms, 1),
        "single_kernel_residency": {"ms_per_update": round(single_ms, 4), "blocks_per_sm": [2, 1, 2, 2, 4, 4],
                                    "note": "every stage at the residency of one persistent kernel per frame "
                                            "(the cell pass's 2 x 512 threads per SM)"},
        "sync_update_ms": {"median": round(statistics.median(sync_ms), 4), "mean": round(statistics.fmean(sync_ms), 4),
                           "updates": len(sync_ms),
                           "method": "host wall clock around one update and its synchronisation (as the reference's "
                                     "synchronous updateGrid), measurement grid in HBM"},
        "stage_ms": {k: round(v, 4) for k, v in stages.items()},
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 3), "peak_source": peak_src, "traffic": None,
                     "algorithmic_bytes": sb[dom],
                     "traffic_note": "DRAM bytes come from a separate ncu capture, not from this run"},
        "e2e": {"value": round(e2e_ms / K / world, 4), "unit": "ms/update", "h2d_bytes_per_step": C_ * 16,
                "d2h_bytes_per_step": C_ * 64, "readback": "asynchronous (dogm_get_grid_cells_async)",
                "sync_readback_ms": round(e2e_sync_ms / K / world, 4)},
        "gpu_launches": launches,
        "clocks": clk,
    }
    g.close()
    for d in dbufs:
        d.free()
    line["meas_grid"] = run_meas_grid(dogm)
    if not args.no_serving:
        # the latency-sensitive serving leg first: later in a process its tails grew
        line["serving"] = run_serving(dogm, scene, seconds=args.serve_seconds)
        line["batched"] = run_batched(dogm, scene)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(frames, cfg, args.cpu_frames)
    return line


def _stream_pool(dogm, scene, n: int, seed: int, pinned: bool):
    """n uneven streams (scene.stream_configs) with two measurement frames each, in HBM
    (device buffers) or in one pinned host block."""
    cfgs = scene.stream_configs(n, seed=seed)
    params, frames = [], []
    for i, c in enumerate(cfgs):
        params.append(dogm.make_params(**scene.params_dict(c)))
        sc = scene.Scene(c, seed=seed * 1000 + i)
        frames.append([sc.frame(k)[0] for k in range(2)])
    cells = [f[0].shape[0] for f in frames]
    if pinned:
        block = dogm.PinnedArray((2 * sum(cells), 4), np.float32)
        bufs, off = [], 0
        for f in frames:
            pair = []
            for m in f:
                v = block.array[off:off + m.shape[0]]
                v[:] = m
                pair.append(v)
                off += m.shape[0]
            bufs.append(pair)
        return params, cells, bufs, block
    bufs = []
    for f in frames:
        pair = []
        for m in f:
            d = dogm.DeviceBuffer(m.nbytes)
            d.upload(m)
            pair.append(d)
        bufs.append(pair)
    return params, cells, bufs, None


def run_batched(dogm, scene, n_streams: int = 64, rounds: int = 30, warm: int = 3) -> dict:
    """Batched uneven grids: n_streams independent grids updated per frame by one launch per
    stage (dogm_update_batch, CUDA graph) against per-stream baselines: one dogm_update per grid
    on its own CUDA stream with no host wait between grids, as a CUDA graph launch and as chained
    launches (the default launch mode), and per-stream plain launches (every kernel launched one
    by one, each update waited for, as the reference's updateGrid).  Measurement grids resident in HBM;
    host wall clock over `rounds` frames of all grids (synchronised at both ends)."""
    params, cells, bufs, _ = _stream_pool(dogm, scene, n_streams, seed=2, pinned=False)
    grids = [dogm.DOGM(p, seed=1000 + i, stream_id=i, sync_each_update=False) for i, p in enumerate(params)]
    zeros = [0.0] * n_streams
    dts = [0.1] * n_streams

    def batched(r):
        dogm.update_batch(grids, [bufs[i][r % 2].ptr for i in range(n_streams)], zeros, zeros, zeros, dts,
                          device=True)

    def per_stream_graph(r):  # also the chained form: the same calls in another launch mode
        for i, g in enumerate(grids):
            g.update_grid(bufs[i][r % 2].ptr, 0.0, 0.0, 0.0, 0.1, device=True)

    def per_stream_plain(r):
        for i, g in enumerate(grids):
            g.update_grid(bufs[i][r % 2].ptr, 0.0, 0.0, 0.0, 0.1, device=True)
            g.synchronize()

    def sync():
        for g in grids:
            g.synchronize()

    out = {}
    for name, step in (("batched", batched), ("per_stream_graph", per_stream_graph),
                       ("per_stream_chained", per_stream_graph), ("per_stream_plain", per_stream_plain)):
        for g in grids:
            g.set_launch_mode(plain=(name == "per_stream_plain"), graph=(name == "per_stream_graph"))
        for r in range(warm):
            step(r)
        sync()
        t0 = time.perf_counter()
        for r in range(rounds):
            step(r)
        sync()
        dt = time.perf_counter() - t0
        out[name] = n_streams * rounds / dt
    for g in grids:
        g.close()
    for pair in bufs:
        for d in pair:
            d.free()
    total_cells = sum(cells)
    total_particles = sum(p.particle_count for p in params)
    newborn = sum(p.new_born_particle_count for p in params)
    alg = ALG_PER_PARTICLE * total_particles + ALG_PER_NEWBORN * newborn + ALG_PER_CELL * total_cells
    peak = peak_gbs()[0]
    gbs = alg * out["batched"] / n_streams / 1e9
    return {"frames_per_s": round(out["batched"], 1),
            "per_stream_graph_frames_per_s": round(out["per_stream_graph"], 1),
            "per_stream_chained_frames_per_s": round(out["per_stream_chained"], 1),
            "speedup_vs_per_stream_chained": round(out["batched"] / out["per_stream_chained"], 2),
            "per_stream_plain_frames_per_s": round(out["per_stream_plain"], 1),
            "speedup_vs_per_stream_graph": round(out["batched"] / out["per_stream_graph"], 2),
            "speedup_vs_per_stream_plain": round(out["batched"] / out["per_stream_plain"], 2),
            "hbm_gbs": round(gbs, 1), "hbm_frac": round(gbs / peak, 3),
            "streams": n_streams, "rounds": rounds, "cells": total_cells, "particles": total_particles,
            "config": "%d grids, side log-uniform [128, 1024] cells at 0.1-0.2 m, 1.5 particles per cell, "
                      "10%% newborns; measurement grids in HBM; host wall clock; per-stream plain = kernels "
                      "launched one by one and each update waited for (the reference's updateGrid)" % n_streams}


def run_serving(dogm, scene, n_streams: int = 200, rate_hz: float = 10.0, seconds: float = 10.0,
                saturate_frames: int = 24, budget: int = 150 * 10**9) -> dict:
    """Serving: n_streams sensor streams with Poisson frame arrivals (rate_hz each) submitted
    to dogm_server_* under an HBM budget, in batched (continuous batching) and per-stream
    (one dogm_update per frame) mode.  Latency = result ready minus submission; measurement
    grids come from pinned host memory (H2D copy inside the served frame)."""
    params, cells, bufs, block = _stream_pool(dogm, scene, n_streams, seed=4, pinned=True)
    rng = np.random.default_rng(9)
    arrivals = []
    for i in range(n_streams):
        t = rng.exponential(1.0 / rate_hz)
        while t < seconds:
            arrivals.append((t, i))
            t += rng.exponential(1.0 / rate_hz)
    arrivals.sort()
    out = {}
    for mode_name, mode in (("batched", dogm.SERVE_BATCHED), ("per_stream", dogm.SERVE_PER_STREAM),
                            ("per_stream_plain", dogm.SERVE_PER_STREAM_PLAIN)):
        srv = dogm.Server(hbm_budget_bytes=budget, mode=mode, max_batch=64, max_inflight=2)
        sids = [srv.open_stream(p, seed=2000 + i, stream_id=i) for i, p in enumerate(params)]
        frame_no = [0] * n_streams

        def submit(i, tag):
            k = frame_no[i]
            frame_no[i] += 1
            srv.submit(sids[i], bufs[i][k % 2], 0.0, 0.0, 0.0, 0.1, tag=tag)

        # warm-up: first frames (initialisation); the batched slots' CUDA graphs of every
        # batch-size bucket are built when the server is created
        for r in range(3):
            for i in range(n_streams):
                submit(i, 0)
            srv.drain(600000)
        srv.poll_array(1 << 20)
        # saturation: every stream has `saturate_frames` frames queued at once; the median of
        # three such rounds (one round lasts about 0.2 s and a single host hiccup skews it)
        sat_rounds = []
        for rep in range(3):
            t0 = time.perf_counter()
            for r in range(saturate_frames):
                for i in range(n_streams):
                    submit(i, 0)
            srv.drain(600000)
            sat_rounds.append(time.perf_counter() - t0)
            srv.poll_array(1 << 20)
        sat_s = statistics.median(sat_rounds)
        # Poisson arrivals paced on the host clock
        t_start = time.perf_counter()
        for j, (t, i) in enumerate(arrivals):
            delay = t_start + t - time.perf_counter()
            if delay > 2e-4:
                time.sleep(delay - 1e-4)
            submit(i, j + 1)
        srv.drain(600000)
        wall = time.perf_counter() - t_start
        res = srv.poll_array(len(arrivals) + 16)
        st = srv.stats()
        srv.close()
        assert len(res) == len(arrivals) and (res["status"] == 0).all(), "served frames failed"
        lat = (res["t_done_ns"] - res["t_submit_ns"]) / 1e6
        out[mode_name] = {
            "saturated_frames_per_s": round(n_streams * saturate_frames / sat_s, 1),
            "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
            "p999_ms": round(float(np.percentile(lat, 99.9)), 3), "max_ms": round(float(lat.max()), 3),
            "frames": int(len(res)), "served_frames_per_s": round(len(res) / wall, 1),
            "mean_batch": round(float(res["batch_size"].mean()), 2),
            "resident_gb": round(st["resident_bytes"] / 1e9, 2),
        }
    block.free()
    sat = {k: v["saturated_frames_per_s"] for k, v in out.items()}
    return {"batched": out["batched"], "per_stream": out["per_stream"], "per_stream_plain": out["per_stream_plain"],
            "saturated_speedup": round(sat["batched"] / sat["per_stream"], 2),
            "saturated_speedup_vs_plain": round(sat["batched"] / sat["per_stream_plain"], 2),
            "config": "%d streams, Poisson %.0f Hz each (%.0f frames/s offered) for %.0f s, grids as the batched "
                      "workload, %.0f GB HBM budget; latency = submit to result on the device; saturation = %d "
                      "frames queued per stream" % (n_streams, rate_hz, n_streams * rate_hz, seconds, budget / 1e9,
                                                    saturate_frames) + ", median of three rounds"}


def run_meas_grid(dogm, gs_len: float = 120.0, res: float = 0.1, beams: int = 2160, reps: int = 50) -> dict:
    """Lidar scan -> measurement grid on the GPU at the large grid shape (1200 x 1200 cells at
    0.1 m, 2160 beams over a 120-degree field of view, 120 m range): host wall clock per
    synchronous generate call, ranges copied from host memory."""
    g = dogm.MeasurementGridGenerator(max_range=gs_len, resolution=res, fov=120.0, stddev_range=0.5,
                                      grid_length=gs_len, grid_resolution=res, beams=beams)
    rng = np.random.default_rng(1)
    scans = [rng.uniform(2.0, gs_len * 0.9, beams).astype(np.float32) for _ in range(4)]
    for k in range(5):
        g.generate_device(scans[k % 4])
    t0 = time.perf_counter()
    for k in range(reps):
        g.generate_device(scans[k % 4])
    us = (time.perf_counter() - t0) * 1e6 / reps
    out = {"us_per_grid": round(us, 1), "cells": g.cell_count, "polar_bins": int(gs_len / res), "beams": beams,
           "config": "1200 x 1200 cells at 0.1 m, 2160 beams, fov 120 deg, range 120 m; synchronous call, "
                     "ranges from host memory"}
    g.close()
    return out


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return None
    K, W = args.steps, args.warmup
    _, cfg, frames = make_frames(min(K + W + 1, 24), seed=0)
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import importlib
    import pyoracle
    spec = importlib.util.spec_from_file_location("dogm_build", os.path.join(REPO, PKG, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build_oracle()
    b.build_ref_harness()
    # parameters as a plain record: the reference arm loads nothing of this library
    import types
    p = types.SimpleNamespace(**importlib.import_module(PKG + ".scene").params_dict(cfg))
    ref = pyoracle.ReferencePipeline(p, threads=0)
    for k in range(W + 1):
        m, x, y, yaw = frames[pingpong(k, len(frames))]
        ref.update(m, x, y, yaw, 0.1)
    t0 = time.perf_counter()
    for k in range(K):
        m, x, y, yaw = frames[pingpong(W + 1 + k, len(frames))]
        ref.update(m, x, y, yaw, 0.1)
    ms = (time.perf_counter() - t0) * 1e3 / K
    sample = "%d full updates of the %s workload (%d cells, %d + %d particles)" % (
        K, WORKLOAD, int(p.size / p.resolution) ** 2, p.particle_count, p.new_born_particle_count)
    line = {"impl": "reference", "metric": METRIC, "value": round(ms, 3), "unit": "ms/update", "n_gpus": world,
            "steps": K, "warmup": W, "ms_per_step": round(ms, 3), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD_DESC,
                       "implementation": "the reference's pipeline (dogm/src/dogm.cu:115-131) transcribed to C "
                                         "with OpenMP; the reference itself is CUDA-only and has no CPU path"},
            "cpu_baseline": {"value": round(ms, 3), "unit": "ms/update", "cores": ref.threads_used, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(ms, 3), "unit": "ms/update", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    line["reference_cuda"] = reference_cuda(p, frames, W, min(K, 100))
    return line


def reference_cuda(p, frames, warm: int, steps: int) -> dict:
    """The reference's own CUDA build on this GPU: its kernels (cubins compiled from
    dogm/src/kernel/) in the restated updateGrid sequence (oracle/ref/ref_harness.cu).  Each
    update is synchronous, like the reference's (dogm.cu:130): host wall clock per update,
    measurement grids resident in HBM; e2e adds the host measurement copy and the grid readback
    (getGridCells) per update."""
    import pyref
    why = pyref.missing()
    if why:
        return {"unavailable": why}
    rt = load_cudart()
    bufs = []
    for m, *_ in frames:
        d = CudartBuffer(rt, m.nbytes)
        d.upload(m)
        bufs.append(d)
    ref = pyref.ReferenceDOGM(p)
    fr = lambda k: pingpong(k, len(frames))
    for k in range(warm + 1):
        _, x, y, yaw = frames[fr(k)]
        ref.update(bufs[fr(k)].ptr, x, y, yaw, 0.1, device=True)
    times = []
    for k in range(warm + 1, warm + 1 + steps):
        _, x, y, yaw = frames[fr(k)]
        t0 = time.perf_counter()
        ref.update(bufs[fr(k)].ptr, x, y, yaw, 0.1, device=True)
        times.append((time.perf_counter() - t0) * 1e3)
    e2e = []
    for k in range(warm + 1 + steps, warm + 1 + steps + max(steps // 4, 5)):
        m, x, y, yaw = frames[fr(k)]
        t0 = time.perf_counter()
        ref.update(m, x, y, yaw, 0.1, device=False)
        ref.get_grid_cells()
        e2e.append((time.perf_counter() - t0) * 1e3)
    ref.close()
    for d in bufs:
        d.free()
    return {"ms_per_update": round(statistics.median(times), 3), "mean_ms": round(statistics.fmean(times), 3),
            "e2e_ms": round(statistics.median(e2e), 3), "steps": steps,
            "kind": "reference kernels compiled from dogm/src/kernel/*.cu for sm_103a, run in the restated "
                    "dogm::DOGM::updateGrid host sequence (Thrust from the CUDA toolkit, legacy stream, its "
                    "host synchronisations and per-frame temporaries)"}


_dist = None


def barrier(world: int):
    if world > 1 and _dist is not None:
        _dist.barrier()


def reduce_max(v: float, world: int) -> float:
    if world <= 1 or _dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    _dist.all_reduce(t, op=_dist.ReduceOp.MAX)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--pool", type=int, default=40, help="distinct measurement frames resident on the device")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-frames", type=int, default=200)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="skip the batched and serving workloads")
    ap.add_argument("--no-autotune", action="store_true", help="time the built-in launch shape")
    ap.add_argument("--min-seconds", type=float, default=1.0,
                    help="the timed region repeats the K steps until it lasts at least this long")
    ap.add_argument("--workload", default="large", choices=sorted(WORKLOADS),
                    help="the single-grid workload of value, e2e and the baselines (large: the headline)")
    ap.add_argument("--serve-seconds", type=float, default=10.0,
                    help="seconds of Poisson arrivals per serving mode (the serving workload names 60)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    global WORKLOAD, WORKLOAD_DESC
    WORKLOAD, WORKLOAD_DESC = args.workload, WORKLOADS[args.workload]
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    global _dist
    if world > 1:
        # one replica per GPU: the update does not shard, ranks share no data
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ.get("LOCAL_RANK", "0"))
        import torch.distributed as dist
        dist.init_process_group("gloo")
        _dist = dist
    line = run_reference(args, rank, world) if args.impl == "reference" else run_gb300(args, rank, world)
    if rank == 0 and line is not None:
        print(json.dumps(line))
    if _dist is not None:
        _dist.destroy_process_group()


if __name__ == "__main__":
    main()
