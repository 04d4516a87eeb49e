"""The replicas-only multi-GPU path of bench.py on CPU: two gloo ranks agree
on the max-over-ranks time and the whole-job throughput (no data-path
collective exists; each rank solves its own replica)."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = 1.0 + rank * 0.5                      # rank 1 is the slow one
    tmax = bench.max_over_ranks(t, dist)
    thr = bench.aggregate_throughput(world, 10.0, tmax)
    q.put((rank, tmax, thr))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_max_time():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, tmax, thr in res:
        assert tmax == pytest.approx(1.5)
        assert thr == pytest.approx(2 * 10.0 / 1.5)


def test_single_process_identity():
    import bench
    assert bench.max_over_ranks(3.0, None) == 3.0
