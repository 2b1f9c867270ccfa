"""Multi-GPU in this path is replicas only: every rank steps an independent
system and the bench reports the units of all ranks over the slowest rank's
time.  The host logic of that path (rendezvous, barrier, max over ranks,
per-rank seeds) runs here with two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    bench._has_cuda = lambda: False
    r, ws, _ = bench.dist_init()
    bench.barrier(ws)
    slowest = bench.max_over_ranks(float(10 * (r + 1)), ws)
    from pyrdsim_gb300 import workloads
    sd = workloads.active_wall_fluid(n=1024, seed=2 + r)
    import torch.distributed as dist
    dist.destroy_process_group()
    q.put((r, ws, slowest, float(sd.x[0, 0])))


def test_two_gloo_ranks_replicas():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 and o[2] == 20.0 for o in out)
    assert out[0][3] != out[1][3]  # different replicas (seeds)
