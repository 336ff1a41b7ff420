"""The multi-GPU path is independent replicas; the only exchange is the
max-over-ranks of the timings, tested here with two gloo ranks on CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        vals = bench.reduce_max([1.0 + rank, 10.0 - rank, 5.0], world)
        q.put((rank, vals))
    finally:
        dist.destroy_process_group()


def test_reduce_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=5) for _ in range(2))
    assert got[0] == got[1] == [2.0, 10.0, 5.0]


def test_single_rank_is_identity():
    import bench

    assert bench.reduce_max([3.0, 4.0], 1) == [3.0, 4.0]
