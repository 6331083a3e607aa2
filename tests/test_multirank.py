"""CPU: the multi-rank path of bench.py, world size 2 over gloo.  The update does not shard
(one grid is one update with global dependencies), so N GPUs run N independent replicas; the
only cross-rank steps are the barrier around the timed region and the max of the ranks'
times, and the reference arm runs on rank 0 alone."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out: str) -> None:
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    bench._dist = dist
    bench.barrier(world)
    mx = bench.reduce_max(1.5 + rank, world)
    args = type("A", (), {"steps": 1, "warmup": 1})()
    ref = bench.run_reference(args, rank, world) if rank != 0 else "rank0"
    with open(os.path.join(out, "rank%d.txt" % rank), "w") as f:
        f.write("%r %r\n" % (mx, ref))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.spawn(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        got = open(tmp_path / ("rank%d.txt" % r)).read().split()
        assert float(got[0]) == 2.5, "max over ranks"
    # a rank other than 0 returns without work in the reference arm
    assert open(tmp_path / "rank1.txt").read().split()[1] == "None"
