"""ctypes binding of the C oracle (oracle/_build/libdogm_oracle.so).

TEST INFRASTRUCTURE ONLY: the checker that tests/, __graft_entry__.smoke() and bench.py's CPU
baseline use.  The product (libdogm_gb300.so) never imports or calls anything here.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdogm_oracle.so")

CELL_MASK = 0x3FFFFFFF
OUT_BIT = 1 << 30
ASSOC_BIT = 1 << 31


class OracleParams(C.Structure):
    _fields_ = [("gs", C.c_int), ("N", C.c_int), ("B", C.c_int), ("q_shift", C.c_int),
                ("p_S", C.c_float), ("sigma_pos", C.c_float), ("sigma_vel", C.c_float), ("p_B", C.c_float),
                ("sigma_birth", C.c_float), ("init_max_vel", C.c_float), ("freespace_discount", C.c_float)]


class OracleFrame(C.Structure):
    _fields_ = [("dt", C.c_float), ("shifted", C.c_int), ("shift_x", C.c_int), ("shift_y", C.c_int),
                ("first_frame", C.c_int), ("meas", C.c_void_p), ("init_u", C.c_void_p), ("predict_z", C.c_void_p),
                ("birth_z", C.c_void_p), ("resample_r", C.c_uint64)]


class OracleOut(C.Structure):
    _fields_ = [("cells", C.c_void_p), ("S_state", C.c_void_p), ("S_key", C.c_void_p), ("perm", C.c_void_p),
                ("B_state", C.c_void_p), ("B_key", C.c_void_p), ("B_w", C.c_void_p), ("res_src", C.c_void_p),
                ("joint_total", C.c_uint64), ("qb_total", C.c_uint64), ("n_birth", C.c_int)]


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("oracle not built: run __graft_entry__.build()")
        lib = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        lib.dogm_oracle_update_f32.argtypes = [vp] * 7
        lib.dogm_oracle_update_f64.argtypes = [vp] * 7
        lib.dogm_oracle_philox.argtypes = [vp, vp, vp]
        lib.dogm_oracle_quantize.argtypes = [C.c_double, C.c_int]
        lib.dogm_oracle_quantize.restype = C.c_uint64
        lib.dogm_oracle_alloc_boundary.argtypes = [C.c_uint64, C.c_uint64, C.c_int]
        lib.dogm_oracle_comb_count.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_int]
        lib.dogm_oracle_draws.argtypes = [C.c_uint64, C.c_uint32, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp]
        lib.dogm_oracle_predict_f32.argtypes = [vp, C.c_float, vp, vp, vp, vp, C.c_int]
        lib.dogm_oracle_shift_particles_f32.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        lib.dogm_oracle_pose.argtypes = [C.c_float, vp, vp, vp, vp, C.c_float, C.c_float, C.c_float, vp, vp]
        lib.dogm_oracle_comb_indices.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_int, vp]
        lib.dogm_oracle_reference_f32.argtypes = [vp, vp, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64,
                                                  C.c_uint32, vp, vp, vp, vp, vp, C.c_int]
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def bitlen(v: int) -> int:
    return int(v).bit_length()


def philox(ctr, key) -> np.ndarray:
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    load().dogm_oracle_philox(_p(c), _p(k), _p(o))
    return o


def quantize(w: float, S: int) -> int:
    return int(load().dogm_oracle_quantize(float(w), S))


def alloc_boundary(Q: int, T: int, M: int) -> int:
    return int(load().dogm_oracle_alloc_boundary(Q, T, M))


def comb_count(a: int, T: int, U: int, N: int) -> int:
    return int(load().dogm_oracle_comb_count(a, T, U, N))


def oracle_params(p) -> OracleParams:
    """From a dogm Params-like object (size, resolution, counts, filter parameters)."""
    gs = int(np.float32(p.size) / np.float32(p.resolution))
    C_ = gs * gs
    return OracleParams(gs=gs, N=p.particle_count, B=p.new_born_particle_count, q_shift=61 - bitlen(C_),
                        p_S=p.persistence_prob, sigma_pos=p.stddev_process_noise_position,
                        sigma_vel=p.stddev_process_noise_velocity, p_B=p.birth_prob, sigma_birth=p.stddev_velocity,
                        init_max_vel=p.init_max_velocity, freespace_discount=p.freespace_discount)


class OracleDOGM:
    """The update restatement with the same host bookkeeping as the GPU path's dogm_update
    (first measurement -> particle initialisation, pose -> ego shift).  dtype float32 gives
    the bit-exact restatement, float64 the high-precision one."""

    def __init__(self, params, dtype=np.float32):
        self.op = oracle_params(params)
        self.resolution = float(np.float32(params.resolution))
        self.dtype = np.dtype(dtype)
        n, c = self.op.N, self.op.gs * self.op.gs
        self.P_state = np.zeros((n, 4), self.dtype)
        self.P_key = np.zeros(n, np.uint32)
        self.free_mass = np.zeros(c, self.dtype)
        self.w_res = np.zeros(1, self.dtype)
        self.first_pose = np.zeros(1, np.int32)
        self.pose = np.zeros(3, np.float32)
        self.first_measurement = True
        self.meas = np.zeros((c, 4), np.float32)
        self.meas[:, 2] = 1.0
        self.meas[:, 3] = 1.0
        self.iteration = 0

    def pose_update(self, x, y, yaw):
        xm = np.zeros(1, np.int32)
        ym = np.zeros(1, np.int32)
        px, py, pyaw = (self.pose[i:i + 1] for i in range(3))
        shifted = load().dogm_oracle_pose(self.resolution, _p(self.first_pose), _p(px), _p(py), _p(pyaw), x, y, yaw,
                                          _p(xm), _p(ym))
        return int(shifted), int(xm[0]), int(ym[0])

    def update(self, meas, x, y, yaw, dt, draws: dict) -> dict:
        """meas: (C,4) float32 or a MEAS_DTYPE array or None (keep); draws: dict of
        init_u (N,2), predict_z (N,4), birth_z (B,2), resample_r (int)."""
        if meas is not None:
            self.meas = np.ascontiguousarray(np.asarray(meas).view(np.float32).reshape(-1, 4))
        first = self.first_measurement
        shifted, xm, ym = self.pose_update(x, y, yaw)
        n, b, c = self.op.N, self.op.B, self.op.gs * self.op.gs
        init_u = np.ascontiguousarray(draws.get("init_u", np.full((n, 2), 0.5, np.float32)), np.float32)
        pz = np.ascontiguousarray(draws["predict_z"], np.float32)
        bz = np.ascontiguousarray(draws.get("birth_z", np.zeros((max(b, 1), 2), np.float32)), np.float32)
        fr = OracleFrame(dt=dt, shifted=shifted, shift_x=xm, shift_y=ym, first_frame=1 if first else 0,
                         meas=self.meas.ctypes.data, init_u=init_u.ctypes.data, predict_z=pz.ctypes.data,
                         birth_z=bz.ctypes.data, resample_r=int(draws.get("resample_r", 0)))
        out = {"cells": np.zeros((c, 16), self.dtype), "S_state": np.zeros((n, 4), self.dtype),
               "S_key": np.zeros(n, np.uint32), "perm": np.zeros(n, np.int32),
               "B_state": np.zeros((max(b, 1), 4), self.dtype), "B_key": np.zeros(max(b, 1), np.uint32),
               "B_w": np.zeros(max(b, 1), self.dtype), "res_src": np.zeros(n, np.int32)}
        o = OracleOut(**{k: v.ctypes.data for k, v in out.items()})
        fn = load().dogm_oracle_update_f32 if self.dtype == np.float32 else load().dogm_oracle_update_f64
        rc = fn(C.byref(self.op), C.byref(fr), _p(self.P_state), _p(self.P_key), _p(self.free_mass), _p(self.w_res),
                C.byref(o))
        if rc != 0:
            raise RuntimeError("oracle update failed (%d)" % rc)
        self.first_measurement = False
        self.iteration += 1
        out["joint_total"] = int(o.joint_total)
        out["qb_total"] = int(o.qb_total)
        out["n_birth"] = int(o.n_birth)
        out["B_state"] = out["B_state"][:b]
        out["B_key"] = out["B_key"][:b]
        out["B_w"] = out["B_w"][:b]
        out["shift"] = (shifted, xm, ym)
        return out


def draws(seed: int, stream_id: int, N: int, B: int, iteration: int) -> dict:
    """Philox draws computed on the CPU (uniforms bit-exact with the GPU path; normals use
    the host's libm, so replay the GPU's own draws where bits matter)."""
    init_u = np.empty((N, 2), np.float32)
    pz = np.empty((N, 4), np.float32)
    bz = np.empty((max(B, 1), 2), np.float32)
    r = np.zeros(1, np.uint64)
    load().dogm_oracle_draws(seed, stream_id, N, B, iteration, _p(init_u), _p(pz), _p(bz), _p(r))
    return {"init_u": init_u, "predict_z": pz, "birth_z": bz[:B], "resample_r": int(r[0])}


class ReferencePipeline:
    """The reference's own stage sequence in float on the host cores (the CPU baseline)."""

    def __init__(self, params, seed: int = 123456, threads: int = 0):
        self.op = oracle_params(params)
        self.resolution = float(np.float32(params.resolution))
        n, c = self.op.N, self.op.gs * self.op.gs
        self.P_state = np.zeros((n, 4), np.float32)
        self.P_idx = np.zeros(n, np.int32)
        self.P_w = np.zeros(n, np.float32)
        self.P_assoc = np.zeros(n, np.uint8)
        self.cells = np.zeros((c, 16), np.float32)
        self.cells.view(np.int32)[:, 0:2] = -1
        self.first_pose = np.zeros(1, np.int32)
        self.pose = np.zeros(3, np.float32)
        self.first_measurement = True
        self.seed = seed
        self.threads = threads
        self.frame = 0
        self.threads_used = 0

    def update(self, meas, x, y, yaw, dt) -> None:
        m = np.ascontiguousarray(np.asarray(meas).view(np.float32).reshape(-1, 4))
        xm = np.zeros(1, np.int32)
        ym = np.zeros(1, np.int32)
        px, py, pyaw = (self.pose[i:i + 1] for i in range(3))
        first = self.first_measurement
        shifted = load().dogm_oracle_pose(self.resolution, _p(self.first_pose), _p(px), _p(py), _p(pyaw), x, y, yaw,
                                          _p(xm), _p(ym))
        self.threads_used = load().dogm_oracle_reference_f32(
            C.byref(self.op), _p(m), dt, 1 if first else 0, shifted, int(xm[0]), int(ym[0]), self.seed, self.frame,
            _p(self.P_state), _p(self.P_idx), _p(self.P_w), _p(self.P_assoc), _p(self.cells), self.threads)
        self.first_measurement = False
        self.frame += 1


COMB_MODES = {"fp32": 0, "compensated_fp32": 1, "fp64": 2}


def comb_indices(weights: np.ndarray, n: int, u: float, mode: str) -> np.ndarray:
    """Systematic resampling of n slots over the joint weights with the prefix sum in the given
    precision ("fp32", "compensated_fp32", "fp64"): the joint item of every slot."""
    w = np.ascontiguousarray(weights, np.float32)
    out = np.empty(n, np.int32)
    load().dogm_oracle_comb_indices(_p(w), w.size, n, float(u), COMB_MODES[mode], _p(out))
    return out
