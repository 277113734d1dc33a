"""The multi-GPU path of bench.py is replicas only (every rank runs the whole
workload on its own GPU); what ranks share is the timing reduction: max of
the per-rank times, sum of the per-rank work, a barrier.  Checked here with
two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, local = bench.dist_env()
        assert (ws, r, local) == (world, rank, rank)
        bench.barrier(ws)
        t = bench.max_over_ranks(ws, 10.0 + rank)      # the slowest rank's time
        u = bench.sum_over_ranks(ws, 1000.0 * (rank + 1))  # whole-job work
        out.put((rank, t, u))
    finally:
        dist.destroy_process_group()


def test_two_rank_timing_reduction():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=5) for _ in range(world))
    assert all(t == 11.0 for _, t, _ in res)
    assert all(u == 3000.0 for _, _, u in res)
