"""Multi-rank host logic of bench.py on CPU (gloo, world size 2): replicas
report the slowest rank's time and the summed agent-steps."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms, steps = bench.reduce_over_ranks(10.0 + 5.0 * rank, 1000 * (rank + 1), world, "cpu")
    q.put((rank, ms, steps))
    dist.destroy_process_group()


def test_reduce_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    assert [o[1] for o in out] == [15.0, 15.0]
    assert [o[2] for o in out] == [3000.0, 3000.0]


def test_single_rank_passthrough():
    import bench

    assert bench.reduce_over_ranks(7.0, 11, 1, "cpu") == (7.0, 11.0)
