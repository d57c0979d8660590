"""Multi-rank host logic of bench.py on CPU (gloo, world size 2): the step does
not shard, so N ranks run N replicas; the job time is the maximum over ranks
and the reference arm runs on rank 0 only."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(world, 1.0 + rank * 0.5, "cpu")
    bench.barrier(world)
    out[rank] = t
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1] == 1.5


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(1, 3.25, "cpu") == 3.25
