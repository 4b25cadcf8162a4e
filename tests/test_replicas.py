"""Replicas on several GPUs (bench.py under torchrun): each rank runs the same
workload on its own GPU, and the job's rate is all ranks' units over the
slowest rank's time.  The aggregation is checked here with two gloo ranks on
the CPU."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        assert bench.dist_env()[:2] == (rank, world)
        q.put((rank, bench.max_over_ranks(1.0 + rank, world), bench.replicas_rate(128, 2.0 + rank, world)))
    finally:
        dist.destroy_process_group()


def test_two_rank_aggregation():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # the slowest rank's time (3 ms) for both ranks' 2 x 128 units
    for rank, mx, rate in got:
        assert mx == 2.0
        assert rate == pytest.approx(2 * 128 / 3.0e-3)


def test_one_process_is_its_own_max():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(4.5, 1) == 4.5
    assert bench.replicas_rate(128, 2.0, 1) == pytest.approx(64000.0)
