"""Multi-GPU runs are replicas only (independent solves per rank, no data-path
collective). The whole-job number is the summed work over the slowest rank's
time; check that reduction with two gloo ranks on CPU."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    ms, value = bench.replicas_value(100.0 * (rank + 1), 1.0e9)
    out[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_reduce_two_gloo_ranks():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    # slowest rank: 200 ms; total work 2e9 particle-steps -> 1e10 per second
    for r in range(world):
        assert res[r][0] == pytest.approx(200.0)
        assert res[r][1] == pytest.approx(2.0e9 / 0.2)


def test_replicas_single_process():
    import bench

    ms, value = bench.replicas_value(50.0, 1.0e8)
    assert ms == 50.0 and value == pytest.approx(2.0e9)
