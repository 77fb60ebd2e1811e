"""Multi-GPU bench logic on CPU: two gloo ranks exchange their timings the
way bench.py does under torchrun (max over ranks, sum of replicas)."""
import os
import socket

import pytest


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, l = bench.dist_setup()
    assert (w, r, l) == (world, rank, rank)
    ms = [10.0, 12.5][rank]
    t = torch.tensor([ms], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    out.put((rank, float(t.item()), bench.replica_value(world, float(t.item()))))
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_max_time():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in res:
        assert ms == 12.5
        assert abs(value - 2 * 1e3 / 12.5) < 1e-9
