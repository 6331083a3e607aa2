"""CPU: the oracle against the known answers in tests/golden/kat.json (Random123 Philox, the
reference's DOGM.Predict and DOGM.EgoMotionCompensation tests) and the exact-arithmetic
helpers against Python integer arithmetic."""
import json
import os
from fractions import Fraction

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def kat():
    with open(os.path.join(HERE, "golden", "kat.json")) as f:
        return json.load(f)


def test_philox_published_answers(oracle, kat):
    for case in kat["philox"]:
        assert oracle.philox(case["ctr"], case["key"]).tolist() == case["out"]


def test_predict_known_answer(oracle, kat):
    """dogm_spec.cpp:68-103: zero noise -> state + dt*(vx, vy, 0, 0), weight * p_S (bit-exact)."""
    k = kat["predict"]
    st = np.array(k["state_bits"], np.uint32).view(np.float32).copy()
    w = np.array(k["weight_bits"], np.uint32).view(np.float32).copy()
    n = st.shape[0]

    class P:
        size, resolution = k["size"], k["resolution"]
        particle_count, new_born_particle_count = n, 1
        persistence_prob = k["persistence_prob"]
        stddev_process_noise_position = stddev_process_noise_velocity = 0.0
        birth_prob, stddev_velocity, init_max_velocity, freespace_discount = 0.02, 10.0, 30.0, 0.01

    import ctypes
    op = oracle.oracle_params(P)
    key = np.zeros(n, np.uint32)
    z = np.random.default_rng(0).normal(size=(n, 4)).astype(np.float32)  # scaled by sigma = 0
    oracle.load().dogm_oracle_predict_f32(ctypes.byref(op), k["dt"], ctypes.c_void_p(z.ctypes.data),
                                          ctypes.c_void_p(st.ctypes.data), ctypes.c_void_p(key.ctypes.data),
                                          ctypes.c_void_p(w.ctypes.data), n)
    assert np.array_equal(st.view(np.uint32), np.array(k["pred_state_bits"], np.uint32))
    assert np.array_equal(w.view(np.uint32), np.array(k["pred_weight_bits"], np.uint32))
    # keys: clamp(int x) + gs * clamp(int y), gs = 10 (predict.cu:42-44)
    gs = 10
    exp = np.clip(st[:, 0].astype(np.int32), 0, gs - 1) + gs * np.clip(st[:, 1].astype(np.int32), 0, gs - 1)
    assert np.array_equal((key & oracle.CELL_MASK).astype(np.int32), exp)


def test_ego_shift_known_answer(oracle, kat):
    """dogm_spec.cpp:10-66: sub-cell moves shift nothing; +3 m at 1 m/cell adds 3 to x."""
    import ctypes
    k = kat["ego_shift"]
    st = np.array(k["state_bits"], np.uint32).view(np.float32).copy()
    first = np.zeros(1, np.int32)
    pose = np.zeros(3, np.float32)
    for step in k["steps"]:
        xm = np.zeros(1, np.int32)
        ym = np.zeros(1, np.int32)
        ptr = lambda a: ctypes.c_void_p(a.ctypes.data)
        px, py, pyaw = pose[0:1], pose[1:2], pose[2:3]
        shifted = oracle.load().dogm_oracle_pose(k["resolution"], ptr(first), ptr(px), ptr(py), ptr(pyaw),
                                                 step["pose"][0], step["pose"][1], 0.0, ptr(xm), ptr(ym))
        assert (int(xm[0]), int(ym[0])) == (step["x_move"], step["y_move"])
        assert pose[0:2].tolist() == step["expect_pose"]
        if shifted:
            oracle.load().dogm_oracle_shift_particles_f32(ptr(st), st.shape[0], int(xm[0]), int(ym[0]))
    assert np.array_equal(st.view(np.uint32), np.array(k["moved_state_bits"], np.uint32))


def _round_half_even(fr: Fraction) -> int:
    fl = fr.numerator // fr.denominator
    rem = fr - fl
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and fl % 2 == 1):
        return fl + 1
    return fl


def test_quantize_is_round_half_even(oracle):
    rng = np.random.default_rng(1)
    vals = np.concatenate([rng.random(200).astype(np.float32), np.float32([1e-12, 1e-30, 2.5, 0.0, -1.0, 1.0]),
                           (rng.random(50) * 1e-9).astype(np.float32)])
    for S in (20, 33, 40):
        for v in vals:
            w = min(max(float(v), 0.0), 2.0)
            exp = 0 if w <= 0 else _round_half_even(Fraction(w) * (1 << S))
            assert oracle.quantize(float(v), S) == exp


def test_alloc_and_comb_exact(oracle):
    rng = np.random.default_rng(2)
    for _ in range(2000):
        T = int(rng.integers(1, 1 << 61))
        Q = int(rng.integers(0, T + 1))
        M = int(rng.integers(1, 1 << 24))
        assert oracle.alloc_boundary(Q, T, M) == (Q * M) // T
        a = int(rng.integers(0, T + 1))
        U = int(rng.integers(0, T))
        N = int(rng.integers(1, 1 << 24))
        # count of i in [0,N) with i*T + U < a*N
        num = a * N - U
        c = 0 if num <= 0 else min(N, -(-num // T))
        if a >= T:
            c = N
        assert oracle.comb_count(a, T, U, N) == c
    assert oracle.comb_count(5, 0, 0, 7) == 7
    assert oracle.alloc_boundary(3, 0, 9) == 0
