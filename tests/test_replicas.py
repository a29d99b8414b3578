"""The N > 1 path of bench.py on CPU: world_size-2 gloo ranks (no GPU).

The path shards into independent replicas (no data-path collective); the
only exchange is the max-over-ranks of the step time, and the whole-job rate
is N replicas over the slowest rank's step.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 3.0 + rank  # rank 1 is the slower replica
        got = bench.max_over_ranks(ms, world)
        q.put((rank, got, bench.replica_rate(got, world)))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_agree_on_the_slowest_step():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(90)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [4.0, 4.0]
    assert all(abs(r[2] - 2 * 1e3 / 4.0) < 1e-9 for r in res)


def test_one_rank_is_its_own_maximum():
    import bench

    assert bench.max_over_ranks(2.5, 1) == 2.5
    assert bench.replica_rate(2.5, 1) == 400.0
