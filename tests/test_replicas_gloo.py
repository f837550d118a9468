"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

The hot path does not shard across GPUs (one system per GPU: replicas), so
the only cross-rank logic is the timing reduction: the job's step time is the
slowest rank's and the value is world x N / that time.
"""
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


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    my_ms = 10.0 + 5.0 * rank                   # rank 1 is the slow one
    value, ms = bench.job_throughput(1000, my_ms, world)
    bench.barrier(world)
    q.put((rank, value, ms))
    dist.destroy_process_group()


def test_job_throughput_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, ms in res:
        assert ms == pytest.approx(15.0)
        assert value == pytest.approx(2 * 1000 / 15e-3)


def test_single_rank_is_identity():
    import bench
    v, ms = bench.job_throughput(1000, 4.0, 1)
    assert ms == 4.0 and v == pytest.approx(1000 / 4e-3)
