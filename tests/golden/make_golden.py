"""Generates tests/golden/kat.json: the known answers the oracle and the GPU path are pinned to.

Sources (nothing here runs the oracle or the GPU path; answers follow from the cited
relations with plain numpy float32 arithmetic):
  philox      Random123's published Philox4x32-10 answers (Salmon et al., SC'11).
  predict     dogm/test/dogm_spec.cpp:68-103 (DOGM.Predict): with zero process noise,
              state' = state + dt * (vx, vy, 0, 0) and weight' = p_S * weight, for the
              test's grid (10 m at 1 m), p_S = 0.5, dt = 0.1; evaluated on seeded states.
  ego_shift   dogm/test/dogm_spec.cpp:10-66 (DOGM.EgoMotionCompensation): first pose (10,10)
              moves nothing; (+0.5,+0.5) is below one cell and moves nothing; (+3, 0) moves
              every particle by +3 in x and the stored pose to (13, 10).
Run: python tests/golden/make_golden.py
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    out = {}
    out["philox"] = [
        {"ctr": [0, 0, 0, 0], "key": [0, 0], "out": [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]},
        {"ctr": [0xFFFFFFFF] * 4, "key": [0xFFFFFFFF] * 2, "out": [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]},
        {"ctr": [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], "key": [0xA4093822, 0x299F31D0],
         "out": [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]},
    ]
    rng = np.random.default_rng(20200101)
    n = 64
    st = np.empty((n, 4), np.float32)
    st[:, 0:2] = rng.uniform(1.0, 8.0, (n, 2)).astype(np.float32)  # stays inside [0, 9] after the move
    st[:, 2:4] = rng.uniform(-9.0, 9.0, (n, 2)).astype(np.float32)
    w = rng.uniform(0.01, 1.0, n).astype(np.float32)
    dt = np.float32(0.1)
    p_s = np.float32(0.5)
    pred = st.copy()
    pred[:, 0] = st[:, 0] + dt * st[:, 2]
    pred[:, 1] = st[:, 1] + dt * st[:, 3]
    pred[:, 2] = st[:, 2] + dt * np.float32(0)
    pred[:, 3] = st[:, 3] + dt * np.float32(0)
    out["predict"] = {
        "size": 10.0, "resolution": 1.0, "persistence_prob": 0.5, "dt": 0.1,
        "state_bits": st.view(np.uint32).tolist(), "weight_bits": w.view(np.uint32).tolist(),
        "pred_state_bits": pred.view(np.uint32).tolist(), "pred_weight_bits": (p_s * w).view(np.uint32).tolist(),
    }
    moved = st.copy()
    moved[:, 0] = st[:, 0] + np.float32(3.0)
    out["ego_shift"] = {
        "size": 10.0, "resolution": 1.0,
        "steps": [
            {"pose": [10.0, 10.0], "expect_pose": [10.0, 10.0], "x_move": 0, "y_move": 0},
            {"pose": [10.5, 10.5], "expect_pose": [10.0, 10.0], "x_move": 0, "y_move": 0},
            {"pose": [13.0, 10.0], "expect_pose": [13.0, 10.0], "x_move": -3, "y_move": 0},
        ],
        "state_bits": st.view(np.uint32).tolist(), "moved_state_bits": moved.view(np.uint32).tolist(),
    }
    with open(os.path.join(HERE, "kat.json"), "w") as f:
        json.dump(out, f)
    print("wrote", os.path.join(HERE, "kat.json"))


if __name__ == "__main__":
    main()
