"""ctypes binding of oracle/ref/ref_harness.cu -- TEST INFRASTRUCTURE ONLY (the checker, never
the product): the reference's own CUDA kernels (cubins compiled from dogm/src/kernel/ by
oracle/ref/build_ref.py into oracle/_ref/) run in the restated host sequence of
dogm::DOGM::updateGrid (dogm/src/dogm.cu:115-131).  Used by the GPU parity tests and by
bench.py's reference arm."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(HERE, "_build", "libdogm_ref.so")
KERNEL_FILES = ["ego_motion_compensation", "init", "init_new_particles", "mass_update", "particle_to_grid", "predict",
                "resampling", "statistical_moments", "update_persistent_particles"]


class RefParams(C.Structure):
    _fields_ = [("size", C.c_float), ("resolution", C.c_float), ("particle_count", C.c_int),
                ("new_born_particle_count", C.c_int), ("persistence_prob", C.c_float),
                ("stddev_process_noise_position", C.c_float), ("stddev_process_noise_velocity", C.c_float),
                ("birth_prob", C.c_float), ("stddev_velocity", C.c_float), ("init_max_velocity", C.c_float),
                ("freespace_discount", C.c_float)]


class RefTrace(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("predict_z", "birth_z", "init_u", "resample_u", "sorted_state", "sorted_idx",
                                          "joint_accum", "rand_sorted", "resample_idx", "weight_array")]


def missing() -> str | None:
    """Why the reference build cannot run here, or None."""
    absent = [f for f in KERNEL_FILES if not os.path.exists(os.path.join(CUBIN_DIR, f + ".cubin"))]
    if absent:
        return "reference cubins missing in %s (%s): build them with oracle/ref/build_ref.py where the " \
               "reference sources are" % (CUBIN_DIR, ", ".join(absent))
    if not os.path.exists(LIB):
        return "%s not built" % LIB
    return None


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    why = missing()
    if why:
        raise RuntimeError(why)
    lib = C.CDLL(LIB)
    vp = C.c_void_p
    lib.dogm_ref_last_error.restype = C.c_char_p
    lib.dogm_ref_load.argtypes = [C.c_char_p]
    lib.dogm_ref_create.argtypes = [vp, vp]
    lib.dogm_ref_destroy.argtypes = [vp]
    lib.dogm_ref_update.argtypes = [vp, vp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, vp]
    lib.dogm_ref_set_particles.argtypes = [vp, vp, vp, vp, vp]
    lib.dogm_ref_get_particles.argtypes = [vp, vp, vp, vp, vp]
    lib.dogm_ref_get_birth.argtypes = [vp, vp, vp, vp, vp]
    lib.dogm_ref_get_cells.argtypes = [vp, vp]
    lib.dogm_ref_grid_size.argtypes = [vp]
    lib.dogm_ref_rng_threads.argtypes = [vp]
    if lib.dogm_ref_load(CUBIN_DIR.encode()) != 0:
        raise RuntimeError("reference load failed: " + lib.dogm_ref_last_error().decode())
    _lib = lib
    return lib


MEAS_CUBIN = os.path.join(CUBIN_DIR, "measurement_grid.cubin")


def meas_missing() -> str | None:
    """Why the reference's measurement-grid kernels cannot run here, or None."""
    if not os.path.exists(MEAS_CUBIN):
        return "%s missing: build it with oracle/ref/build_ref.py where the reference sources are" % MEAS_CUBIN
    return missing()


def _meas_lib() -> C.CDLL:
    lib = load()
    if not getattr(lib, "_meas_ready", False):
        vp = C.c_void_p
        lib.dogm_ref_meas_load.argtypes = [C.c_char_p]
        lib.dogm_ref_polar_ism.argtypes = [vp, C.c_int, C.c_int, C.c_float, C.c_float, vp, vp]
        lib.dogm_ref_cart_to_meas.argtypes = [vp, C.c_int, vp]
        if lib.dogm_ref_meas_load(MEAS_CUBIN.encode()) != 0:
            raise RuntimeError("reference measurement kernels: " + lib.dogm_ref_last_error().decode())
        lib._meas_ready = True
    return lib


def polar_ism(ranges, bins: int, resolution: float, stddev_range: float, prior=None) -> np.ndarray:
    """The reference's createPolarGridTextureKernel (or, with prior, fusePolarGridTextureKernel)
    on a surface: (bins, beams, 2) float32 {occ, free}."""
    lib = _meas_lib()
    r = np.ascontiguousarray(ranges, np.float32)
    beams = r.shape[0]
    out = np.zeros((bins, beams, 2), np.float32)
    pr = None if prior is None else np.ascontiguousarray(prior, np.float32).reshape(bins, beams, 2)
    _check(lib.dogm_ref_polar_ism(_p(r), beams, bins, resolution, stddev_range, _p(pr), _p(out)), "dogm_ref_polar_ism")
    return out


def cart_to_meas(rgba) -> np.ndarray:
    """The reference's cartesianGridToMeasurementGridKernel on an RGBA float image (gs, gs, 4),
    row y = framebuffer row: (gs * gs, 4) float32 MeasurementCells."""
    lib = _meas_lib()
    img = np.ascontiguousarray(rgba, np.float32)
    gs = img.shape[0]
    out = np.zeros((gs * gs, 4), np.float32)
    _check(lib.dogm_ref_cart_to_meas(_p(img), gs, _p(out)), "dogm_ref_cart_to_meas")
    return out


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError("%s: %s" % (what, load().dogm_ref_last_error().decode()))


def _p(a):
    return None if a is None else C.c_void_p(a if isinstance(a, int) else a.ctypes.data)


class ReferenceDOGM:
    """The reference's dogm::DOGM on the GPU (its own kernels, restated host sequence)."""

    def __init__(self, params):
        lib = load()
        rp = RefParams(**{n: getattr(params, n) for n, _ in RefParams._fields_})
        h = C.c_void_p()
        _check(lib.dogm_ref_create(C.byref(rp), C.byref(h)), "dogm_ref_create")
        self.h = h
        self.N, self.B = params.particle_count, params.new_born_particle_count
        self.grid_size = lib.dogm_ref_grid_size(h)
        self.C = self.grid_size ** 2
        self.rng_threads = lib.dogm_ref_rng_threads(h)

    def close(self) -> None:
        if self.h:
            load().dogm_ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update(self, meas, x: float, y: float, yaw: float, dt: float, device: bool = False,
               trace: bool = False) -> dict | None:
        """One updateGrid.  meas: (C, 4) float32 host array or an int device pointer.  With
        trace, returns the draws the update took and the intermediate arrays."""
        tr, keep = None, {}
        if trace:
            n, b = self.N, self.B
            keep = {"predict_z": np.zeros((n, 4), np.float32), "birth_z": np.zeros((max(b, 1), 2), np.float32),
                    "init_u": np.zeros((n, 2), np.float32), "resample_u": np.zeros(n, np.float32),
                    "sorted_state": np.zeros((n, 4), np.float32), "sorted_idx": np.zeros(n, np.int32),
                    "joint_accum": np.zeros(n + b, np.float32), "rand_sorted": np.zeros(n, np.float32),
                    "resample_idx": np.zeros(n, np.int32), "weight_array": np.zeros(n, np.float32)}
            tr = RefTrace(**{k: v.ctypes.data for k, v in keep.items()})
        if isinstance(meas, int):
            m = meas
        else:
            m = np.ascontiguousarray(np.asarray(meas).view(np.float32).reshape(-1, 4))
            # the reference scales its allocation scans by the total occupied / newborn mass
            # (init_new_particles.cu:66-74): a grid without occupied mass divides by zero and its
            # slot ranges then index out of bounds, so such a grid is refused here
            if not (m[:, 1] > 0).any():
                raise ValueError("the reference build needs some occupied mass in the measurement grid")
        _check(load().dogm_ref_update(self.h, _p(m), x, y, yaw, dt, 1 if device else 0,
                                      C.byref(tr) if tr is not None else None), "dogm_ref_update")
        if trace:
            keep["birth_z"] = keep["birth_z"][:self.B]
            return keep
        return None

    def set_particles(self, state, idx, weight, assoc) -> None:
        st = np.ascontiguousarray(state, np.float32)
        ix = np.ascontiguousarray(idx, np.int32)
        w = np.ascontiguousarray(weight, np.float32)
        a = np.ascontiguousarray(assoc, np.uint8)
        _check(load().dogm_ref_set_particles(self.h, _p(st), _p(ix), _p(w), _p(a)), "dogm_ref_set_particles")

    def get_particles(self) -> dict:
        n = self.N
        st, ix, w, a = np.zeros((n, 4), np.float32), np.zeros(n, np.int32), np.zeros(n, np.float32), np.zeros(n, np.uint8)
        _check(load().dogm_ref_get_particles(self.h, _p(st), _p(ix), _p(w), _p(a)), "dogm_ref_get_particles")
        return {"state": st, "grid_cell_idx": ix, "weight": w, "associated": a}

    def get_birth(self) -> dict:
        b = max(self.B, 1)
        st, ix, w, a = np.zeros((b, 4), np.float32), np.zeros(b, np.int32), np.zeros(b, np.float32), np.zeros(b, np.uint8)
        _check(load().dogm_ref_get_birth(self.h, _p(st), _p(ix), _p(w), _p(a)), "dogm_ref_get_birth")
        return {"state": st[:self.B], "grid_cell_idx": ix[:self.B], "weight": w[:self.B], "associated": a[:self.B]}

    def get_grid_cells(self, dtype=None) -> np.ndarray:
        out = np.zeros((self.C, 16), np.float32)
        _check(load().dogm_ref_get_cells(self.h, _p(out)), "dogm_ref_get_cells")
        return out if dtype is None else out.view(dtype).reshape(-1)
