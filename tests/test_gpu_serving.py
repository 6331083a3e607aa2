"""GPU: the serving loop (dogm_server_*) through the C ABI.

* Each stream's result is the same alone and in the mix: a stream updated by the server,
  batched with streams of other sizes whose frames arrive at other times, ends in exactly the
  state (every cell field, every particle) of the same stream updated alone with dogm_update
  (tolerance: bit-exact -- a batched launch computes each grid with the same operations).
* Per-stream mode gives the same bits too.
* Admission: a stream that does not fit the HBM budget waits, its frames wait with it, and it
  runs once a closed stream frees the budget; without queued admission it is refused.
* Readback buffers passed to submit receive the grid after the frame's update.
"""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [(12.8, 0.2, 20000, 2000), (25.6, 0.1, 100000, 10000), (6.4, 0.2, 6000, 600), (19.2, 0.15, 40000, 4000)]


def _frames(scene, gs, n, seed):
    return [np.ascontiguousarray(scene.random_measurements(gs, seed=seed + k)) for k in range(n)]


def _pose(k):
    # moves by more than one cell every second frame, so the grid shift runs in the mix
    return 0.35 * (k // 2), -0.2 * (k // 2)


def _alone(dogm, p, frames, seed, sid):
    g = dogm.DOGM(p, seed=seed, stream_id=sid)
    for k, m in enumerate(frames):
        x, y = _pose(k)
        g.update_grid(m, x, y, 0.0, 0.1)
    cells, parts = g.get_grid_cells(), g.get_particles()
    it = g.get_iteration()
    g.close()
    return cells, parts, it


def _assert_same(view, cells, parts, it, label):
    got = view.get_grid_cells()
    assert got.tobytes() == cells.tobytes(), label + ": cells differ"
    gp = view.get_particles()
    for key in ("state", "grid_cell_idx", "weight", "associated"):
        assert gp[key].tobytes() == parts[key].tobytes(), label + ": particles " + key
    assert view.get_iteration() == it, label + ": iteration"


@pytest.mark.parametrize("mode", [0, 1])
def test_alone_equals_in_the_mix(dogm, scene, mode):
    n_frames = 5
    params = [dogm.make_params(size=s, resolution=r, particle_count=n, new_born_particle_count=b)
              for s, r, n, b in SIZES]
    grid = [int(np.float32(s) / np.float32(r)) for s, r, _, _ in SIZES]
    frames = [_frames(scene, gs, n_frames, 100 * i) for i, gs in enumerate(grid)]
    alone = [_alone(dogm, p, frames[i], 11 + i, i) for i, p in enumerate(params)]

    srv = dogm.Server(mode=mode, max_batch=3, max_inflight=2)
    sids = [srv.open_stream(p, seed=11 + i, stream_id=i) for i, p in enumerate(params)]
    # frames 0-2: uneven arrival, stream i submits from its own thread with its own pacing, so
    # launches carry changing subsets of the streams
    paced = 3

    def feed(i):
        rng = np.random.default_rng(i)
        for k in range(paced):
            x, y = _pose(k)
            srv.submit(sids[i], frames[i][k], x, y, 0.0, 0.1, tag=1000 * i + k)
            threading.Event().wait(float(rng.uniform(0, 0.004)))
    ts = [threading.Thread(target=feed, args=(i,)) for i in range(len(params))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    srv.drain()
    # frames 3-4 queue while launches are held back: on resume the first launch takes the
    # oldest frame of max_batch = 3 streams, the second slot the fourth stream's
    srv.pause(True)
    for k in range(paced, n_frames):
        x, y = _pose(k)
        for i in range(len(params)):
            srv.submit(sids[i], frames[i][k], x, y, 0.0, 0.1, tag=1000 * i + k)
    srv.pause(False)
    srv.drain()
    res = srv.poll(1024)
    assert len(res) == n_frames * len(params)
    assert all(r["status"] == 0 for r in res)
    for i in range(len(params)):
        mine = sorted((r for r in res if r["stream"] == sids[i]), key=lambda r: r["iteration"])
        assert [r["tag"] for r in mine] == [1000 * i + k for k in range(n_frames)], "frames ran out of order"
        assert [r["iteration"] for r in mine] == list(range(1, n_frames + 1))
        for r in mine:
            assert r["t_submit_ns"] <= r["t_launch_ns"] <= r["t_done_ns"]
            assert 1 <= r["batch_size"] <= 3
    if mode == 0:
        assert max(r["batch_size"] for r in res) == 3, "the queued frames did not share a launch"
    for i, sid in enumerate(sids):
        _assert_same(srv.stream(sid), *alone[i], label="mode %d stream %d" % (mode, i))
    st = srv.stats()
    assert st["frames_done"] == st["frames_submitted"] == n_frames * len(params)
    srv.close()


def test_admission_waits_for_budget(dogm, scene):
    small = dogm.make_params(size=12.8, resolution=0.2, particle_count=20000, new_born_particle_count=2000)
    one = dogm.state_bytes(small)
    srv = dogm.Server(hbm_budget_bytes=int(2.5 * one), max_batch=8)
    a = srv.open_stream(small, seed=1)
    b = srv.open_stream(small, seed=2)
    c = srv.open_stream(small, seed=3, stream_id=3)
    assert [srv.stream_state(s) for s in (a, b, c)] == [dogm.STREAM_ACTIVE, dogm.STREAM_ACTIVE,
                                                         dogm.STREAM_WAITING]
    st = srv.stats()
    assert st["streams_waiting"] == 1 and st["resident_bytes"] == 2 * one
    frames = _frames(scene, 64, 3, 7)
    for k, m in enumerate(frames):
        srv.submit(c, m, 0.0, 0.0, 0.0, 0.1, tag=k)
        srv.submit(a, m, 0.0, 0.0, 0.0, 0.1, tag=10 + k)
    with pytest.raises(dogm.DogmError, match="not ready"):
        srv.drain(timeout_ms=300)  # c cannot run while a and b hold the budget
    srv.close_stream(b)
    srv.drain()
    assert srv.stream_state(c) == dogm.STREAM_ACTIVE and srv.stream_state(b) == dogm.STREAM_CLOSED
    res = srv.poll(64)
    assert sorted(r["tag"] for r in res if r["stream"] == c) == [0, 1, 2]
    cells, parts, it = _alone_static(dogm, small, frames, 3, 3)
    _assert_same(srv.stream(c), cells, parts, it, "admitted late")
    with pytest.raises(dogm.DogmError, match="closed"):
        srv.submit(b, frames[0], 0.0, 0.0, 0.0, 0.1)
    srv.close()

    strict = dogm.Server(hbm_budget_bytes=int(1.5 * one), queue_admission=False)
    strict.open_stream(small)
    with pytest.raises(dogm.DogmError, match="over budget"):
        strict.open_stream(small)
    with pytest.raises(dogm.DogmError, match="over budget"):
        strict.open_stream(dogm.make_params(size=51.2, resolution=0.1, particle_count=400000,
                                            new_born_particle_count=40000))
    strict.close()


def _alone_static(dogm, p, frames, seed, sid):
    g = dogm.DOGM(p, seed=seed, stream_id=sid)
    for m in frames:
        g.update_grid(m, 0.0, 0.0, 0.0, 0.1)
    out = g.get_grid_cells(), g.get_particles(), g.get_iteration()
    g.close()
    return out


@pytest.mark.parametrize("mode", [0, 1])
def test_readback_buffers(dogm, scene, mode):
    p = dogm.make_params(size=12.8, resolution=0.2, particle_count=20000, new_born_particle_count=2000)
    srv = dogm.Server(mode=mode)
    sid = srv.open_stream(p, seed=5)
    frames = _frames(scene, 64, 3, 21)
    outs = [np.zeros(64 * 64, dogm.GRID_CELL_DTYPE) for _ in frames]
    for k, m in enumerate(frames):
        srv.submit(sid, m, 0.0, 0.0, 0.0, 0.1, cells_out=outs[k], tag=k)
        srv.drain()
        assert outs[k].tobytes() == srv.stream(sid).get_grid_cells().tobytes(), "readback of frame %d" % k
    assert outs[0].tobytes() != outs[2].tobytes()
    srv.close()
