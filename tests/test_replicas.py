"""Several GPUs run independent replicas of the bed (the path does not shard):
the whole-job rate is every rank's particle-steps over the slowest rank's time.
Two gloo ranks on the CPU check the aggregation bench.py uses."""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank: int, ws: int, port: int, q) -> None:
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=ws)
    try:
        local = [0.5, 2.0][rank]  # the second replica is slower
        rate, slow = bench.replica_rate(local, 1000, 10, ws, device="cpu")
        q.put((rank, rate, slow))
    finally:
        dist.destroy_process_group()


def test_replica_rate_uses_the_slowest_rank():
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=10) for _ in range(ws))
    for rank, rate, slow in got:
        assert slow == 2.0
        assert rate == pytest.approx(2 * 1000 * 10 / 2.0)


def test_one_rank_is_its_own_rate():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.replica_rate(0.25, 200, 4, 1) == (200 * 4 / 0.25, 0.25)


def test_algorithmic_bytes_model():
    """the byte model of the roofline: 152 per particle, 4 per list entry, 128
    per contact or wall contact, 16 per bridge"""
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.algorithmic_bytes(0, 0, 0, 0) == 152
    assert bench.algorithmic_bytes(8.66, 6.42, 0.84, 0.066) == pytest.approx(
        152 + 4 * 8.66 + 128 * 6.42 + 16 * 0.84 + 128 * 0.066)
    # the packed bed's counts give the ~1030 bytes per particle-step quoted for it
    assert 1020 < bench.algorithmic_bytes(8.66, 6.42, 0.84, 0.066) < 1040
