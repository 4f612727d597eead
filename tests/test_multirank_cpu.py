"""World-size-2 gloo test of bench.py's multi-rank host logic (replicas:
max-over-ranks step time, whole-job aggregate rate) -- on CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.reduce_max(1.0 + rank, dist, "cpu")
    rate = bench.aggregate_rate(world, 10, t)
    q.put((rank, t, rate))
    dist.destroy_process_group()


def test_bench_reduce_max_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get() for _ in range(2))
    assert all(t == 2.0 for _, t, _ in res)            # slowest rank's time on every rank
    assert all(abs(rate - 10.0) < 1e-12 for _, _, rate in res)
