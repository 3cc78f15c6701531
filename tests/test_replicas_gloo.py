"""bench.py's replica mode on the CPU with two gloo ranks: every rank times its
own replica of the assembly and the whole-job time is the maximum over ranks
(max_over_ranks), and the reference arm runs on rank 0 only (the other ranks
return without work).  No GPU work."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    vals = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 0.5 * rank], "cpu")
    # the reference arm: ranks other than 0 leave at once
    class Args:
        steps, warmup, gpus = 1, 0, world
    ran = None
    if rank != 0:
        ran = bench.run_reference(Args()) is None
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, vals, ran))


def test_replica_times_are_the_maximum_over_two_gloo_ranks():
    world, port = 2, free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = dict((r, (v, ran)) for r, v, ran in (q.get(timeout=120) for _ in range(world)))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(world):
        assert out[r][0] == [2.0, 10.0, 0.5]
    assert out[1][1] is True
