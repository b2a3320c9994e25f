"""The benchmark's N-GPU path runs independent replicas (the solver does not
shard one volume): its only cross-rank step is the max-over-ranks of the
timed region.  Checked here with world_size 2 on the gloo backend (CPU)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.slowest_rank_ms(100.0 + 50.0 * rank, dist, torch.device("cpu"))
    q.put((rank, ms, bench.replica_steps_per_s(10, world, ms)))
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    import socket

    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        port = sck.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    assert [o[1] for o in out] == [150.0, 150.0]
    assert out[0][2] == pytest.approx(2 * 10 / 0.150)
