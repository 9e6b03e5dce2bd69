"""Multi-process host logic of bench.py on CPU ranks (gloo, world size 2):
the barrier + max-over-ranks timing reduction and the whole-job aggregate.
The path is replicas only, so no data-path collective exists to test."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ws, r, local = bench.dist_env()
    assert (ws, r, local) == (world, rank, rank)
    bench.barrier(ws)
    t = bench.max_over_ranks(1.5 + rank, ws)   # rank 1 is the slow one
    q.put((rank, t))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(res) == [(0, 2.5), (1, 2.5)]


def test_reference_arm_other_ranks_exit_quietly(capsys):
    import bench

    class A:
        steps, warmup = 1, 0
    bench.run_reference(A, 2, 1)   # rank 1 of 2 prints nothing and does no work
    assert capsys.readouterr().out == ""
