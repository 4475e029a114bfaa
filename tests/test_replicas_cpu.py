"""The multi-process path of bench.py on CPU: N replicas (one process per GPU
on a GPU machine) time the same build and report the whole-job rate over the
slowest rank's time.  Two gloo ranks here stand in for two GPUs."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        import bench
        t = bench.max_over_ranks(1.0 + rank, world, 'cpu')
        rate = bench.job_rate(1000, world, t / 4)
        dist.barrier()
        q.put((rank, t, rate))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_replicas_max_time_and_rate():
    world = 2
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=100) for _ in range(world))
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    # both ranks see the slowest rank's time; the rate counts both ranks' work
    assert [r[1] for r in res] == [2.0, 2.0]
    assert [r[2] for r in res] == [1000 * 2 / 0.5] * 2


def test_single_process_passthrough():
    import bench
    assert bench.max_over_ranks(3.5, 1, 'cpu') == 3.5
    assert bench.job_rate(10, 1, 2.) == 5.
