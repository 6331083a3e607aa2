"""GB300-native dynamic occupancy grid map (DOGM) update — Python binding of the C ABI.

The product is libdogm_gb300.so (CUDA kernels for sm_103a + the C ABI of
include/dogm_gb300.h).  This module binds it with ctypes and mirrors the reference's
dogm::DOGM class (dogm/include/dogm/dogm.h:20-199) for Python callers, tests and the
bench.  There is no CPU fallback: if the library was not built, loading raises.

The directory name contains hyphens, so import it with
    importlib.import_module("dynamic-occupancy-grid-map_gb300")
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "lib", "libdogm_gb300.so")

# dogm_grid_cell (dogm_types.h:13-33) and dogm_measurement_cell (dogm_types.h:35-41)
GRID_CELL_DTYPE = np.dtype([
    ("start_idx", "<i4"), ("end_idx", "<i4"), ("new_born_occ_mass", "<f4"), ("pers_occ_mass", "<f4"),
    ("free_mass", "<f4"), ("occ_mass", "<f4"), ("pred_occ_mass", "<f4"), ("mu_A", "<f4"), ("mu_UA", "<f4"),
    ("w_A", "<f4"), ("w_UA", "<f4"), ("mean_x_vel", "<f4"), ("mean_y_vel", "<f4"), ("var_x_vel", "<f4"),
    ("var_y_vel", "<f4"), ("covar_xy_vel", "<f4")])
MEAS_DTYPE = np.dtype([("free_mass", "<f4"), ("occ_mass", "<f4"), ("likelihood", "<f4"), ("p_A", "<f4")])
GRID_CELL_FIELDS = GRID_CELL_DTYPE.names
# dogm_dynamic_cell: a kept cell of dogm_extract_dynamic_cells
DYNAMIC_CELL_DTYPE = np.dtype([("index", "<i4"), ("x", "<f4"), ("y", "<f4"), ("occupancy", "<f4"),
                               ("mahalanobis", "<f4"), ("cell", GRID_CELL_DTYPE)])

DOGM_OK = 0
STATUS_NAMES = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "device wait timed out",
                5: "not ready", 6: "unsupported", 7: "over budget"}

# C ABI symbols declared in include/dogm_gb300.h (checked by the CPU test suite).
ABI_SYMBOLS = [
    "dogm_default_options", "dogm_create", "dogm_destroy", "dogm_update", "dogm_update_batch", "dogm_synchronize",
    "dogm_get_grid_cells", "dogm_get_grid_cells_device", "dogm_get_grid_cells_async", "dogm_get_measurement_cells", "dogm_get_particles",
    "dogm_get_grid_size", "dogm_get_resolution", "dogm_get_position_x", "dogm_get_position_y", "dogm_get_yaw",
    "dogm_get_iteration", "dogm_get_particle_count", "dogm_get_new_born_particle_count", "dogm_particle_prediction",
    "dogm_update_pose", "dogm_update_pose_noalloc", "dogm_initialize_particles", "dogm_particle_assignment",
    "dogm_grid_cell_occupancy_update", "dogm_update_persistent_particles", "dogm_initialize_new_particles",
    "dogm_statistical_moments", "dogm_resampling", "dogm_set_measurement_cells", "dogm_set_particles",
    "dogm_set_replay", "dogm_clear_replay", "dogm_generate_draws", "dogm_debug_enable", "dogm_debug_export",
    "dogm_debug_joint_weights",
    "dogm_lower_bound_f32", "dogm_host_alloc", "dogm_host_free", "dogm_device_alloc", "dogm_device_free",
    "dogm_memcpy", "dogm_state_bytes", "dogm_last_launch_count", "dogm_last_error", "dogm_status_string",
    "dogm_abi_version", "dogm_get_stream", "dogm_profile_enable", "dogm_stage_times", "dogm_stage_name",
    "dogm_server_default_config", "dogm_server_create", "dogm_server_destroy", "dogm_server_open_stream",
    "dogm_server_close_stream", "dogm_server_submit", "dogm_server_pause", "dogm_server_poll", "dogm_server_drain",
    "dogm_server_get_stats", "dogm_server_stream_state", "dogm_server_stream_handle", "dogm_server_now_ns",
    "dogm_get_tune", "dogm_set_tune", "dogm_autotune", "dogm_set_launch_mode",
    "dogm_meas_grid_create", "dogm_meas_grid_destroy", "dogm_meas_grid_generate", "dogm_meas_grid_size",
    "dogm_meas_grid_polar", "dogm_meas_grid_fan", "dogm_extract_dynamic_cells", "dogm_extract_dynamic_cells_device",
    "dogm_snapshot_bytes", "dogm_snapshot", "dogm_restore",
    "dogm_cluster_cells", "dogm_evaluator_create", "dogm_evaluator_destroy", "dogm_evaluator_add_step",
    "dogm_evaluator_summary",
]


class Params(C.Structure):
    """dogm::DOGM::Params (dogm.h:26-60), field order = ABI."""
    _fields_ = [("size", C.c_float), ("resolution", C.c_float), ("particle_count", C.c_int),
                ("new_born_particle_count", C.c_int), ("persistence_prob", C.c_float),
                ("stddev_process_noise_position", C.c_float), ("stddev_process_noise_velocity", C.c_float),
                ("birth_prob", C.c_float), ("stddev_velocity", C.c_float), ("init_max_velocity", C.c_float),
                ("freespace_discount", C.c_float)]


class Options(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("stream_id", C.c_uint32), ("resample_mode", C.c_int),
                ("sync_each_update", C.c_int)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("mode", C.c_int), ("max_batch", C.c_int),
                ("max_inflight", C.c_int), ("queue_admission", C.c_int)]


class ServerResult(C.Structure):
    _fields_ = [("stream", C.c_int), ("status", C.c_int), ("tag", C.c_uint64), ("iteration", C.c_int),
                ("batch_size", C.c_int), ("t_submit_ns", C.c_int64), ("t_launch_ns", C.c_int64),
                ("t_done_ns", C.c_int64)]


class ServerStats(C.Structure):
    _fields_ = [("frames_submitted", C.c_uint64), ("frames_done", C.c_uint64), ("launches", C.c_uint64),
                ("streams_active", C.c_int), ("streams_waiting", C.c_int), ("resident_bytes", C.c_size_t),
                ("budget_bytes", C.c_size_t), ("mean_batch", C.c_double)]


class Tune(C.Structure):
    """dogm_tune: blocks per SM per stage (0 = default), resampling tile 2^bits (0 = default 10)."""
    _fields_ = [("blocks_per_sm", C.c_int * 8), ("resample_tile_bits", C.c_int), ("ms_tuned", C.c_float),
                ("ms_default", C.c_float)]

    def as_dict(self) -> dict:
        return {"blocks_per_sm": list(self.blocks_per_sm), "resample_tile_bits": self.resample_tile_bits,
                "ms_tuned": round(self.ms_tuned, 4), "ms_default": round(self.ms_default, 4)}


SERVE_BATCHED, SERVE_PER_STREAM, SERVE_PER_STREAM_PLAIN = 0, 1, 2
LAUNCH_CHAINED, LAUNCH_PLAIN, LAUNCH_GRAPH = 0, 1, 2
STREAM_WAITING, STREAM_ACTIVE, STREAM_CLOSED = 0, 1, 2


class DogmError(RuntimeError):
    pass


_lib = None


def load(path: str | None = None) -> C.CDLL:
    """Load libdogm_gb300.so (build it with __graft_entry__.build()); raises if missing."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise DogmError("libdogm_gb300.so is not built (%s): run __graft_entry__.build(); "
                        "there is no CPU fallback" % p)
    lib = C.CDLL(p)
    vp, f, i, u64, sz = C.c_void_p, C.c_float, C.c_int, C.c_uint64, C.c_size_t
    sig = {
        "dogm_default_options": ([vp], i), "dogm_create": ([vp, vp, vp], i), "dogm_destroy": ([vp], i),
        "dogm_update": ([vp, vp, f, f, f, f, i], i),
        "dogm_update_batch": ([vp, i, vp, vp, vp, vp, vp, i], i), "dogm_synchronize": ([vp], i),
        "dogm_get_grid_cells": ([vp, vp, sz], i), "dogm_get_grid_cells_device": ([vp, vp, sz], i),
        "dogm_get_grid_cells_async": ([vp, vp, sz], i),
        "dogm_get_measurement_cells": ([vp, vp, sz], i), "dogm_get_particles": ([vp, vp, vp, vp, vp, sz], i),
        "dogm_get_grid_size": ([vp], i), "dogm_get_resolution": ([vp], f), "dogm_get_position_x": ([vp], f),
        "dogm_get_position_y": ([vp], f), "dogm_get_yaw": ([vp], f), "dogm_get_iteration": ([vp], i),
        "dogm_get_particle_count": ([vp], i), "dogm_get_new_born_particle_count": ([vp], i),
        "dogm_particle_prediction": ([vp, f], i), "dogm_update_pose": ([vp, f, f, f], i),
        "dogm_update_pose_noalloc": ([vp, f, f, f], i),
        "dogm_initialize_particles": ([vp], i), "dogm_particle_assignment": ([vp], i),
        "dogm_grid_cell_occupancy_update": ([vp, f], i), "dogm_update_persistent_particles": ([vp], i),
        "dogm_initialize_new_particles": ([vp], i), "dogm_statistical_moments": ([vp], i),
        "dogm_resampling": ([vp], i), "dogm_set_measurement_cells": ([vp, vp, sz], i),
        "dogm_set_particles": ([vp, vp, vp, vp, f, sz], i), "dogm_set_replay": ([vp, vp, vp, vp, vp], i),
        "dogm_clear_replay": ([vp], i), "dogm_generate_draws": ([vp, i, vp, vp, vp, vp], i),
        "dogm_debug_enable": ([vp, i], i), "dogm_debug_joint_weights": ([vp, vp, sz, vp], i),
        "dogm_debug_export": ([vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp], i),
        "dogm_lower_bound_f32": ([vp, i, vp, i, vp, i, vp], i), "dogm_host_alloc": ([vp, sz], i),
        "dogm_host_free": ([vp], i), "dogm_device_alloc": ([vp, sz], i), "dogm_device_free": ([vp], i),
        "dogm_memcpy": ([vp, vp, sz, i], i), "dogm_state_bytes": ([vp], sz), "dogm_last_launch_count": ([vp], i),
        "dogm_set_launch_mode": ([vp, i], i),
        "dogm_last_error": ([], C.c_char_p), "dogm_get_stream": ([vp], vp), "dogm_profile_enable": ([vp, i], i),
        "dogm_stage_times": ([vp, vp, i], i), "dogm_stage_name": ([i], C.c_char_p), "dogm_status_string": ([i], C.c_char_p), "dogm_abi_version": ([], i),
        "dogm_server_default_config": ([vp], i), "dogm_server_create": ([vp, vp], i), "dogm_server_destroy": ([vp], i),
        "dogm_server_open_stream": ([vp, vp, vp, vp], i), "dogm_server_close_stream": ([vp, i], i),
        "dogm_server_submit": ([vp, i, vp, i, f, f, f, f, vp, u64], i), "dogm_server_poll": ([vp, vp, i, i, vp], i), "dogm_server_pause": ([vp, i], i),
        "dogm_server_drain": ([vp, i], i), "dogm_server_get_stats": ([vp, vp], i),
        "dogm_server_stream_state": ([vp, i], i), "dogm_server_stream_handle": ([vp, i, vp], i),
        "dogm_server_now_ns": ([], C.c_int64),
        "dogm_get_tune": ([vp, vp], i), "dogm_set_tune": ([vp, vp], i),
        "dogm_autotune": ([vp, vp, i, i, C.c_char_p, vp], i),
        "dogm_meas_grid_create": ([vp, f, f, i, vp], i), "dogm_meas_grid_destroy": ([vp], i),
        "dogm_meas_grid_generate": ([vp, vp, i, i, vp, vp], i), "dogm_meas_grid_size": ([vp], i),
        "dogm_meas_grid_polar": ([vp, vp, sz, vp, vp], i), "dogm_meas_grid_fan": ([vp, vp, vp, vp, i, vp, vp], i),
        "dogm_extract_dynamic_cells": ([vp, f, f, vp, i, vp], i),
        "dogm_extract_dynamic_cells_device": ([vp, i, f, f, vp, i, vp, vp, vp], i),
        "dogm_snapshot_bytes": ([vp], sz), "dogm_snapshot": ([vp, vp, sz], i), "dogm_restore": ([vp, vp, sz], i),
        "dogm_cluster_cells": ([vp, i, f, i, i, vp, vp], i), "dogm_evaluator_create": ([f, f, i, vp], i),
        "dogm_evaluator_destroy": ([vp], i), "dogm_evaluator_add_step": ([vp, vp, i, vp, i, vp, i, vp], i),
        "dogm_evaluator_summary": ([vp, vp, vp, vp, vp], i),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(status: int, what: str = "dogm") -> None:
    if status != DOGM_OK:
        msg = load().dogm_last_error().decode(errors="replace")
        raise DogmError("%s: %s (%s)" % (what, STATUS_NAMES.get(status, status), msg))


def _ptr(a) -> C.c_void_p | None:
    if a is None:
        return None
    if isinstance(a, int):
        return C.c_void_p(a)
    return C.c_void_p(a.ctypes.data)


def make_params(**kw) -> Params:
    p = Params()
    defaults = dict(size=50.0, resolution=0.2, particle_count=300000, new_born_particle_count=30000,
                    persistence_prob=0.99, stddev_process_noise_position=0.1, stddev_process_noise_velocity=2.0,
                    birth_prob=0.02, stddev_velocity=30.0, init_max_velocity=12.0, freespace_discount=0.01)
    defaults.update(kw)
    for k, v in defaults.items():
        setattr(p, k, v)
    return p


class DeviceBuffer:
    """Raw device allocation (cudaMalloc through the C ABI)."""

    def __init__(self, nbytes: int):
        self.nbytes = int(nbytes)
        p = C.c_void_p()
        check(load().dogm_device_alloc(C.byref(p), self.nbytes), "dogm_device_alloc")
        self.ptr = p.value

    def upload(self, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr)
        assert a.nbytes <= self.nbytes
        check(load().dogm_memcpy(C.c_void_p(self.ptr), _ptr(a), a.nbytes, 1), "dogm_memcpy H2D")

    def download(self, arr: np.ndarray) -> np.ndarray:
        check(load().dogm_memcpy(_ptr(arr), C.c_void_p(self.ptr), arr.nbytes, 2), "dogm_memcpy D2H")
        return arr

    def free(self) -> None:
        if self.ptr:
            load().dogm_device_free(C.c_void_p(self.ptr))
            self.ptr = 0

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class PinnedArray:
    """A numpy array over pinned host memory (cudaMallocHost through the C ABI)."""

    def __init__(self, shape, dtype):
        self.dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * self.dtype.itemsize
        p = C.c_void_p()
        check(load().dogm_host_alloc(C.byref(p), max(n, 1)), "dogm_host_alloc")
        self.ptr = p.value
        buf = (C.c_char * max(n, 1)).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=self.dtype, count=int(np.prod(shape))).reshape(shape)

    def free(self) -> None:
        if self.ptr:
            self.array = None
            load().dogm_host_free(C.c_void_p(self.ptr))
            self.ptr = 0


class DOGM:
    """Python mirror of dogm::DOGM over the C ABI (dogm/include/dogm/dogm.h:20-199)."""

    def __init__(self, params: Params, seed: int = 123456, stream_id: int = 0, sync_each_update: bool = True):
        lib = load()
        self.params = params
        opt = Options()
        check(lib.dogm_default_options(C.byref(opt)), "dogm_default_options")
        opt.seed = seed
        opt.stream_id = stream_id
        opt.sync_each_update = 1 if sync_each_update else 0
        h = C.c_void_p()
        check(lib.dogm_create(C.byref(params), C.byref(opt), C.byref(h)), "dogm_create")
        self.h = h
        self.grid_size = lib.dogm_get_grid_size(h)
        self.cell_count = self.grid_size * self.grid_size
        self.particle_count = lib.dogm_get_particle_count(h)
        self.new_born_particle_count = lib.dogm_get_new_born_particle_count(h)

    def close(self) -> None:
        if self.h:
            load().dogm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- the update (dogm.cu:115-131) -----------------------------------------------------
    def update_grid(self, meas, new_x: float, new_y: float, new_yaw: float, dt: float, device: bool = False) -> None:
        """meas: MEAS_DTYPE array (host), an int device pointer (device=True) or None."""
        if meas is None:
            p = None
        elif isinstance(meas, int):
            p = C.c_void_p(meas)
        else:
            a = np.ascontiguousarray(meas)
            assert a.nbytes == self.cell_count * 16, "measurement grid must hold grid_size^2 cells"
            p = _ptr(a)
        check(load().dogm_update(self.h, p, new_x, new_y, new_yaw, dt, 1 if device else 0), "dogm_update")

    def synchronize(self) -> None:
        check(load().dogm_synchronize(self.h), "dogm_synchronize")

    # -- readback -------------------------------------------------------------------------
    def get_grid_cells(self, out: np.ndarray | None = None) -> np.ndarray:
        out = np.empty(self.cell_count, GRID_CELL_DTYPE) if out is None else out
        check(load().dogm_get_grid_cells(self.h, _ptr(out), self.cell_count), "dogm_get_grid_cells")
        return out

    def get_grid_cells_async(self, out: np.ndarray) -> np.ndarray:
        """Queues the copy of the current grid into `out` (GRID_CELL_DTYPE, grid_size^2 entries,
        ideally a PinnedArray's array); it overlaps the next update and is complete after
        synchronize()."""
        if out.dtype != GRID_CELL_DTYPE or out.size != self.cell_count or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous GRID_CELL_DTYPE array of grid_size^2 cells")
        check(load().dogm_get_grid_cells_async(self.h, _ptr(out), self.cell_count), "dogm_get_grid_cells_async")
        return out

    def get_measurement_cells(self) -> np.ndarray:
        out = np.empty(self.cell_count, MEAS_DTYPE)
        check(load().dogm_get_measurement_cells(self.h, _ptr(out), self.cell_count), "dogm_get_measurement_cells")
        return out

    def get_particles(self) -> dict:
        n = self.particle_count
        st = np.empty((n, 4), np.float32)
        idx = np.empty(n, np.int32)
        w = np.empty(n, np.float32)
        a = np.empty(n, np.uint8)
        check(load().dogm_get_particles(self.h, _ptr(st), _ptr(idx), _ptr(w), _ptr(a), n), "dogm_get_particles")
        return {"state": st, "grid_cell_idx": idx, "weight": w, "associated": a}

    def get_grid_size(self) -> int:
        return load().dogm_get_grid_size(self.h)

    def get_resolution(self) -> float:
        return load().dogm_get_resolution(self.h)

    def get_position_x(self) -> float:
        return load().dogm_get_position_x(self.h)

    def get_position_y(self) -> float:
        return load().dogm_get_position_y(self.h)

    def get_yaw(self) -> float:
        return load().dogm_get_yaw(self.h)

    def get_iteration(self) -> int:
        return load().dogm_get_iteration(self.h)

    def set_launch_mode(self, plain: bool = False, graph: bool = False) -> None:
        """Plain kernel launches per update (as the reference), one CUDA graph per update, or
        (neither: the default) chained launches with nothing between two updates."""
        check(load().dogm_set_launch_mode(self.h, LAUNCH_PLAIN if plain else (LAUNCH_GRAPH if graph else LAUNCH_CHAINED)),
              "dogm_set_launch_mode")

    def last_launch_count(self) -> int:
        return load().dogm_last_launch_count(self.h)

    def stream(self) -> int:
        """The cudaStream_t the handle launches on (record CUDA events on it)."""
        return load().dogm_get_stream(self.h) or 0

    def snapshot(self) -> bytes:
        """The state this handle carries into its next update (dogm_snapshot)."""
        n = load().dogm_snapshot_bytes(self.h)
        buf = np.empty(n, np.uint8)
        check(load().dogm_snapshot(self.h, _ptr(buf), n), "dogm_snapshot")
        return buf.tobytes()

    def restore(self, snap: bytes) -> None:
        buf = np.frombuffer(snap, np.uint8)
        check(load().dogm_restore(self.h, _ptr(buf), buf.size), "dogm_restore")

    def extract_dynamic_cells(self, min_occupancy: float = 0.7, min_velocity: float = 4.0,
                              max_out: int = 1 << 16) -> np.ndarray:
        """Cells whose pignistic occupancy and velocity Mahalanobis length reach the thresholds
        (computeCellsWithVelocity, image_creation.cpp:24-66), in row-major order."""
        out = np.empty(max(max_out, 1), DYNAMIC_CELL_DTYPE)
        n = C.c_int(0)
        check(load().dogm_extract_dynamic_cells(self.h, min_occupancy, min_velocity, _ptr(out), max_out, C.byref(n)),
              "dogm_extract_dynamic_cells")
        return out[:min(n.value, max_out)]

    def autotune(self, meas, reps: int = 10, cache_path: str | None = None, device: bool = False) -> Tune:
        """Times the resampling tile and launch widths on a scratch handle fed `meas` (host array
        or int device pointer) and applies the fastest to this handle."""
        t = Tune()
        p = C.c_void_p(meas) if isinstance(meas, int) else _ptr(np.ascontiguousarray(meas))
        check(load().dogm_autotune(self.h, p, 1 if device else 0, reps,
                                   cache_path.encode() if cache_path else None, C.byref(t)), "dogm_autotune")
        return t

    def get_tune(self) -> Tune:
        t = Tune()
        check(load().dogm_get_tune(self.h, C.byref(t)), "dogm_get_tune")
        return t

    def set_tune(self, t: Tune) -> None:
        check(load().dogm_set_tune(self.h, C.byref(t)), "dogm_set_tune")

    def profile_enable(self, enable: bool = True) -> None:
        check(load().dogm_profile_enable(self.h, 1 if enable else 0), "dogm_profile_enable")

    def stage_times(self) -> dict:
        """Per-stage milliseconds of the last update (profiling enabled)."""
        ms = np.zeros(16, np.float32)
        n = load().dogm_stage_times(self.h, _ptr(ms), 16)
        return {load().dogm_stage_name(i).decode(): float(ms[i]) for i in range(n)}

    # -- stages ---------------------------------------------------------------------------
    def particle_prediction(self, dt: float) -> None:
        check(load().dogm_particle_prediction(self.h, dt), "dogm_particle_prediction")

    def update_pose(self, x: float, y: float, yaw: float) -> None:
        check(load().dogm_update_pose(self.h, x, y, yaw), "dogm_update_pose")

    def update_pose_noalloc(self, x: float, y: float, yaw: float) -> None:
        """update_pose without device allocation (grids of at most 262,144 cells)."""
        check(load().dogm_update_pose_noalloc(self.h, x, y, yaw), "dogm_update_pose_noalloc")

    # stage methods after particlePrediction, in updateGrid's order (dogm/src/dogm.cu:119-127)
    def particle_assignment(self) -> None:
        check(load().dogm_particle_assignment(self.h), "dogm_particle_assignment")

    def grid_cell_occupancy_update(self, dt: float) -> None:
        check(load().dogm_grid_cell_occupancy_update(self.h, dt), "dogm_grid_cell_occupancy_update")

    def update_persistent_particles(self) -> None:
        check(load().dogm_update_persistent_particles(self.h), "dogm_update_persistent_particles")

    def initialize_new_particles(self) -> None:
        check(load().dogm_initialize_new_particles(self.h), "dogm_initialize_new_particles")

    def statistical_moments(self) -> None:
        check(load().dogm_statistical_moments(self.h), "dogm_statistical_moments")

    def resampling(self) -> None:
        check(load().dogm_resampling(self.h), "dogm_resampling")

    def initialize_particles(self) -> None:
        check(load().dogm_initialize_particles(self.h), "dogm_initialize_particles")

    # -- state injection, replay, debug ---------------------------------------------------
    def set_measurement_cells(self, meas: np.ndarray) -> None:
        a = np.ascontiguousarray(meas)
        check(load().dogm_set_measurement_cells(self.h, _ptr(a), self.cell_count), "dogm_set_measurement_cells")

    def set_particles(self, state, grid_cell_idx, associated, weight: float) -> None:
        st = np.ascontiguousarray(state, np.float32)
        idx = np.ascontiguousarray(grid_cell_idx, np.int32)
        a = np.ascontiguousarray(associated, np.uint8)
        check(load().dogm_set_particles(self.h, _ptr(st), _ptr(idx), _ptr(a), weight, self.particle_count),
              "dogm_set_particles")

    def set_replay(self, init_u=None, predict_z=None, birth_z=None, resample_r=None) -> None:
        arrs = [None if x is None else np.ascontiguousarray(x, np.float32) for x in (init_u, predict_z, birth_z)]
        r = None if resample_r is None else np.array([resample_r], np.uint64)
        self._replay_keep = arrs + [r]
        check(load().dogm_set_replay(self.h, *[_ptr(x) for x in arrs], _ptr(r)), "dogm_set_replay")

    def clear_replay(self) -> None:
        check(load().dogm_clear_replay(self.h), "dogm_clear_replay")

    def generate_draws(self, iteration: int) -> dict:
        n, b = self.particle_count, self.new_born_particle_count
        init_u = np.empty((n, 2), np.float32)
        pz = np.empty((n, 4), np.float32)
        bz = np.empty((max(b, 1), 2), np.float32)
        r = np.zeros(1, np.uint64)
        check(load().dogm_generate_draws(self.h, iteration, _ptr(init_u), _ptr(pz), _ptr(bz), _ptr(r)),
              "dogm_generate_draws")
        return {"init_u": init_u, "predict_z": pz, "birth_z": bz[:b], "resample_r": int(r[0])}

    def debug_enable(self, enable: bool = True) -> None:
        check(load().dogm_debug_enable(self.h, 1 if enable else 0), "dogm_debug_enable")

    def debug_export(self) -> dict:
        n, b = self.particle_count, self.new_born_particle_count
        sc = np.empty(n, np.int32)
        ss = np.empty((n, 4), np.float32)
        sp = np.empty(n, np.int32)
        bs = np.empty((max(b, 1), 4), np.float32)
        bc = np.empty(max(b, 1), np.int32)
        ba = np.empty(max(b, 1), np.uint8)
        bw = np.empty(max(b, 1), np.float32)
        rs = np.empty(n, np.int32)
        jt = np.zeros(1, np.uint64)
        qs = np.zeros(1, np.int32)
        nb = np.zeros(1, np.int32)
        check(load().dogm_debug_export(self.h, _ptr(sc), _ptr(ss), _ptr(sp), _ptr(bs), _ptr(bc), _ptr(ba), _ptr(bw),
                                       _ptr(rs), _ptr(jt), _ptr(qs), _ptr(nb)), "dogm_debug_export")
        return {"sorted_cell": sc, "sorted_state": ss, "sort_perm": sp, "birth_state": bs[:b], "birth_cell": bc[:b],
                "birth_assoc": ba[:b], "birth_weight": bw[:b], "resample_src": rs, "joint_total": int(jt[0]),
                "q_shift": int(qs[0]), "n_birth": int(nb[0])}

    def debug_joint_weights(self) -> np.ndarray:
        """The last update's joint resampling weights (persistent sorted, then newborns)."""
        n = self.particle_count + self.new_born_particle_count
        w = np.empty(max(n, 1), np.float32)
        m = C.c_int(0)
        check(load().dogm_debug_joint_weights(self.h, _ptr(w), w.size, C.byref(m)), "dogm_debug_joint_weights")
        return w[:m.value]


def update_batch(grids: list[DOGM], meas: list, xs, ys, yaws, dts, device: bool = False) -> None:
    """One batched update of several grids (uneven sizes allowed)."""
    n = len(grids)
    hs = (C.c_void_p * n)(*[g.h.value for g in grids])
    keep = []
    ptrs = (C.c_void_p * n)()
    for i, m in enumerate(meas):
        if m is None:
            ptrs[i] = None
        elif isinstance(m, int):
            ptrs[i] = m
        else:
            a = np.ascontiguousarray(m)
            keep.append(a)
            ptrs[i] = a.ctypes.data
    f = lambda v: np.ascontiguousarray(v, np.float32)
    ax, ay, ayaw, adt = f(xs), f(ys), f(yaws), f(dts)
    check(load().dogm_update_batch(hs, n, ptrs, _ptr(ax), _ptr(ay), _ptr(ayaw), _ptr(adt), 1 if device else 0),
          "dogm_update_batch")


def lower_bound_f32(accum: np.ndarray, queries: np.ndarray, clamp_last: bool = True) -> np.ndarray:
    """Device multinomial index search (the reference's thrust::lower_bound step)."""
    acc = np.ascontiguousarray(accum, np.float32)
    q = np.ascontiguousarray(queries, np.float32)
    da, dq, do = DeviceBuffer(acc.nbytes), DeviceBuffer(max(q.nbytes, 4)), DeviceBuffer(max(q.size * 4, 4))
    da.upload(acc)
    dq.upload(q)
    check(load().dogm_lower_bound_f32(C.c_void_p(da.ptr), acc.size, C.c_void_p(dq.ptr), q.size, C.c_void_p(do.ptr),
                                      1 if clamp_last else 0, None), "dogm_lower_bound_f32")
    out = np.empty(q.size, np.int32)
    do.download(out)
    for b in (da, dq, do):
        b.free()
    return out


def state_bytes(params: Params) -> int:
    return int(load().dogm_state_bytes(C.byref(params)))


class _StreamView(DOGM):
    """Readback view of a server stream's handle (owned by the server; never destroyed here)."""

    def __init__(self, h, params: Params):
        lib = load()
        self.params = params
        self.h = h
        self.grid_size = lib.dogm_get_grid_size(h)
        self.cell_count = self.grid_size * self.grid_size
        self.particle_count = lib.dogm_get_particle_count(h)
        self.new_born_particle_count = lib.dogm_get_new_born_particle_count(h)

    def close(self) -> None:
        self.h = None


class Server:
    """Serving loop over the C ABI (dogm_server_*): resident streams admitted under an HBM
    budget, frames updated by continuous batching (or per stream, for comparison)."""

    def __init__(self, hbm_budget_bytes: int | None = None, mode: int = SERVE_BATCHED, max_batch: int = 64,
                 max_inflight: int = 2, queue_admission: bool = True):
        lib = load()
        cfg = ServerConfig()
        check(lib.dogm_server_default_config(C.byref(cfg)), "dogm_server_default_config")
        if hbm_budget_bytes is not None:
            cfg.hbm_budget_bytes = int(hbm_budget_bytes)
        cfg.mode, cfg.max_batch, cfg.max_inflight = mode, max_batch, max_inflight
        cfg.queue_admission = 1 if queue_admission else 0
        s = C.c_void_p()
        check(lib.dogm_server_create(C.byref(cfg), C.byref(s)), "dogm_server_create")
        self.s = s
        self.params: dict[int, Params] = {}
        self._keep: dict[int, object] = {}

    def close(self) -> None:
        if self.s:
            check(load().dogm_server_destroy(self.s), "dogm_server_destroy")
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def open_stream(self, params: Params, seed: int = 123456, stream_id: int = 0) -> int:
        lib = load()
        opt = Options()
        check(lib.dogm_default_options(C.byref(opt)), "dogm_default_options")
        opt.seed, opt.stream_id = seed, stream_id
        sid = C.c_int(-1)
        check(lib.dogm_server_open_stream(self.s, C.byref(params), C.byref(opt), C.byref(sid)),
              "dogm_server_open_stream")
        self.params[sid.value] = params
        return sid.value

    def close_stream(self, sid: int) -> None:
        check(load().dogm_server_close_stream(self.s, sid), "dogm_server_close_stream")

    def submit(self, sid: int, meas, x: float, y: float, yaw: float, dt: float, cells_out=None, tag: int = 0,
               device: bool = False) -> None:
        """meas: MEAS_DTYPE host array (kept alive until the result), an int device pointer or None."""
        if meas is None:
            p = None
        elif isinstance(meas, int):
            p = C.c_void_p(meas)
        else:
            p = _ptr(meas)
        check(load().dogm_server_submit(self.s, sid, p, 1 if device else 0, x, y, yaw, dt, _ptr(cells_out), tag),
              "dogm_server_submit")

    def pause(self, paused: bool = True) -> None:
        """Hold back new launches (True) or resume (False); submitted frames keep queueing."""
        check(load().dogm_server_pause(self.s, 1 if paused else 0), "dogm_server_pause")

    def poll(self, max_results: int = 1024, timeout_us: int = 0) -> list[dict]:
        buf = (ServerResult * max_results)()
        n = C.c_int(0)
        check(load().dogm_server_poll(self.s, buf, max_results, timeout_us, C.byref(n)), "dogm_server_poll")
        return [{k: getattr(buf[i], k) for k, _ in ServerResult._fields_} for i in range(n.value)]

    def poll_array(self, max_results: int = 65536, timeout_us: int = 0) -> np.ndarray:
        """Like poll, as a structured numpy array (cheap for many results)."""
        dt = np.dtype([("stream", "<i4"), ("status", "<i4"), ("tag", "<u8"), ("iteration", "<i4"),
                       ("batch_size", "<i4"), ("t_submit_ns", "<i8"), ("t_launch_ns", "<i8"), ("t_done_ns", "<i8")])
        assert dt.itemsize == C.sizeof(ServerResult)
        out = np.empty(max_results, dt)
        n = C.c_int(0)
        check(load().dogm_server_poll(self.s, _ptr(out), max_results, timeout_us, C.byref(n)), "dogm_server_poll")
        return out[:n.value]

    def drain(self, timeout_ms: int = 60000) -> None:
        check(load().dogm_server_drain(self.s, timeout_ms), "dogm_server_drain")

    def stats(self) -> dict:
        st = ServerStats()
        check(load().dogm_server_get_stats(self.s, C.byref(st)), "dogm_server_get_stats")
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def stream_state(self, sid: int) -> int:
        return load().dogm_server_stream_state(self.s, sid)

    def stream(self, sid: int) -> DOGM:
        """Readback view (get_grid_cells, get_particles ...) of an admitted stream; drain first."""
        h = C.c_void_p()
        check(load().dogm_server_stream_handle(self.s, sid, C.byref(h)), "dogm_server_stream_handle")
        return _StreamView(h, self.params[sid])


def now_ns() -> int:
    return int(load().dogm_server_now_ns())


class LaserParams(C.Structure):
    """LaserMeasurementGrid::Params (laser_to_meas_grid.h:16-22)."""
    _fields_ = [("max_range", C.c_float), ("resolution", C.c_float), ("fov", C.c_float), ("stddev_range", C.c_float)]


class MeasurementGridGenerator:
    """Lidar scan -> measurement grid on the GPU (dogm_meas_grid_*): the inverse sensor model in
    polar coordinates and the warp over the field of view, replacing the OpenGL path of the
    reference's LaserMeasurementGrid (laser_to_meas_grid.cu:25-70)."""

    def __init__(self, max_range: float, resolution: float, fov: float, stddev_range: float, grid_length: float,
                 grid_resolution: float, beams: int):
        self.params = LaserParams(max_range, resolution, fov, stddev_range)
        self.beams = int(beams)
        m = C.c_void_p()
        check(load().dogm_meas_grid_create(C.byref(self.params), grid_length, grid_resolution, self.beams,
                                           C.byref(m)), "dogm_meas_grid_create")
        self.m = m
        self.grid_size = load().dogm_meas_grid_size(m)
        self.cell_count = self.grid_size ** 2
        self._out = DeviceBuffer(16 * self.cell_count)

    def close(self) -> None:
        if self.m:
            load().dogm_meas_grid_destroy(self.m)
            self.m = None
            self._out.free()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def generate_device(self, ranges, out_ptr: int | None = None, fuse: bool = False, device: bool = False) -> int:
        """Writes the grid to device memory (out_ptr, or an internal buffer); returns the pointer."""
        out = self._out.ptr if out_ptr is None else out_ptr
        r = C.c_void_p(ranges) if isinstance(ranges, int) else _ptr(np.ascontiguousarray(ranges, np.float32))
        check(load().dogm_meas_grid_generate(self.m, r, 1 if device else 0, 1 if fuse else 0, C.c_void_p(out), None),
              "dogm_meas_grid_generate")
        return out

    def generate(self, ranges, fuse: bool = False) -> np.ndarray:
        """The measurement grid of one scan (host ranges) as a MEAS_DTYPE host array."""
        ptr = self.generate_device(ranges, fuse=fuse)
        out = np.empty(self.cell_count, MEAS_DTYPE)
        check(load().dogm_memcpy(_ptr(out), C.c_void_p(ptr), out.nbytes, 2), "dogm_memcpy D2H")
        return out

    def polar(self) -> np.ndarray:
        nb, nr = C.c_int(0), C.c_int(0)
        check(load().dogm_meas_grid_polar(self.m, None, 0, C.byref(nb), C.byref(nr)), "dogm_meas_grid_polar")
        out = np.empty((nr.value, nb.value, 2), np.float32)
        check(load().dogm_meas_grid_polar(self.m, _ptr(out), out.size, None, None), "dogm_meas_grid_polar")
        return out

    def fan(self) -> dict:
        nv, a0 = C.c_int(0), C.c_int(0)
        check(load().dogm_meas_grid_fan(self.m, None, None, None, 0, C.byref(nv), C.byref(a0)), "dogm_meas_grid_fan")
        x = np.empty(nv.value, np.int64)
        y = np.empty(nv.value, np.int64)
        sv = np.empty(nv.value, np.float32)
        check(load().dogm_meas_grid_fan(self.m, _ptr(x), _ptr(y), _ptr(sv), nv.value, None, None),
              "dogm_meas_grid_fan")
        return {"x256": x, "y256": y, "s": sv, "first_angle": a0.value}


# ---- accuracy evaluation (host code: dogm_cluster_cells, dogm_evaluator_*) -------------------
DBSCAN_REFERENCE, DBSCAN_STANDARD = 0, 1
_DBSCAN_MODES = {"reference": DBSCAN_REFERENCE, "standard": DBSCAN_STANDARD}
# dogm_object_truth: a ground-truth vehicle, metres and m/s with y up
OBJECT_TRUTH_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("vx", "<f4"), ("vy", "<f4")])
# dogm_cluster: one DBSCAN cluster of a frame and its match
CLUSTER_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("vx", "<f4"), ("vy", "<f4"), ("cells", "<i4"),
                          ("truth", "<i4"), ("err_x", "<f4"), ("err_y", "<f4"), ("err_vx", "<f4"),
                          ("err_vy", "<f4")])


def _cells(cells) -> np.ndarray:
    return np.ascontiguousarray(cells, DYNAMIC_CELL_DTYPE)


def cluster_cells(cells, eps: float = 3.0, min_cells: int = 5, mode: str = "reference") -> tuple[np.ndarray, int]:
    """DBSCAN over dynamic cells (dbscan.cpp:24-114): per-cell cluster labels (-1: none) and the
    cluster count."""
    c = _cells(cells)
    label = np.empty(max(len(c), 1), np.int32)
    n = C.c_int(0)
    check(load().dogm_cluster_cells(_ptr(c), len(c), eps, min_cells, _DBSCAN_MODES[mode], _ptr(label), C.byref(n)),
          "dogm_cluster_cells")
    return label[:len(c)], n.value


class Evaluator:
    """PrecisionEvaluator with its MAE and RMSE metrics (precision_evaluator.cpp:16-139)."""

    def __init__(self, resolution: float, grid_length: float, mode: str = "reference"):
        e = C.c_void_p()
        check(load().dogm_evaluator_create(resolution, grid_length, _DBSCAN_MODES[mode], C.byref(e)),
              "dogm_evaluator_create")
        self.e = e

    def close(self) -> None:
        if self.e:
            load().dogm_evaluator_destroy(self.e)
            self.e = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_step(self, cells, truth) -> np.ndarray:
        """Clusters one frame's cells, matches them to `truth` (OBJECT_TRUTH_DTYPE or rows of
        x, y, vx, vy) and accumulates the errors; returns the frame's clusters."""
        c = _cells(cells)
        t = np.asarray(truth)
        if t.dtype == OBJECT_TRUTH_DTYPE:
            t = np.ascontiguousarray(t).reshape(-1)
        else:
            t = np.ascontiguousarray(np.asarray(truth, np.float32).reshape(-1, 4)).view(OBJECT_TRUTH_DTYPE).reshape(-1)
        cap = max(len(c), 1)
        out = np.zeros(cap, CLUSTER_DTYPE)
        n = C.c_int(0)
        check(load().dogm_evaluator_add_step(self.e, _ptr(c), len(c), _ptr(t), len(t), _ptr(out), cap,
                                             C.byref(n)), "dogm_evaluator_add_step")
        return out[:n.value]

    def summary(self) -> dict:
        mae = np.empty(4, np.float32)
        rmse = np.empty(4, np.float32)
        det, una = C.c_int(0), C.c_int(0)
        check(load().dogm_evaluator_summary(self.e, _ptr(mae), _ptr(rmse), C.byref(det), C.byref(una)),
              "dogm_evaluator_summary")
        return {"mae": mae, "rmse": rmse, "detections": det.value, "unassigned": una.value}
