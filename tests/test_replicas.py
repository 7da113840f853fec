"""Replica logic of the benchmark on several processes (gloo, CPU): every
rank gets the maximum of the ranks' times and the whole-job rate counts
every rank's units (rsvdt/replicas.py)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from rsvdt import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 10.0 + 5.0 * rank  # rank 1 is slower
    dist.barrier()
    m = replicas.max_over_ranks(ms, dist)
    out[rank] = (m, replicas.whole_job_rate(100.0, m, world), replicas.rank_seed(1234, rank))
    dist.destroy_process_group()


def test_single_process():
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.whole_job_rate(7.0, 2.0, 1) == 3500.0


@pytest.mark.parametrize("world", [2, 3])
def test_max_over_ranks_and_rate_with_gloo(world):
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    slowest = 10.0 + 5.0 * (world - 1)
    for r in range(world):
        m, rate, seed = res[r]
        assert m == slowest
        assert abs(rate - world * 100.0 / (slowest * 1e-3)) < 1e-9
        assert seed == 1234 + r
    assert len({res[r][2] for r in range(world)}) == world
