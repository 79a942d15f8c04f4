"""The bench's replica harness (one process per GPU, no exchange step): two gloo ranks on the
CPU each time their own small assembly with the oracle, meet at the barrier and agree on the
slowest rank's time, which is what the bench reports for N > 1."""
import os
import socket
import sys

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import time

        import bench
        import numpy as np
        from oracle import oracle as O

        v, f, a, n = bench._mesh_np(1)
        px, wx, py, wy = bench._rules_np(2)
        bench.replica_barrier(world)
        t0 = time.perf_counter()
        for _ in range(1 + rank):  # rank 1 does twice the work: it is the slowest replica
            z = O.mom_zmat_fe(v, f, a, n, px, wx, py, wy, 2.0, dtype=np.float64)
        mine = (time.perf_counter() - t0) * 1e3
        bench.replica_barrier(world)
        slowest = bench.replica_max(mine, world)
        out[rank] = (mine, slowest, float(np.abs(z).sum()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_report_the_slowest_time():
    world = 2
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    (m0, s0, z0), (m1, s1, z1) = out[0], out[1]
    assert s0 == s1 == max(m0, m1)
    assert z0 == z1  # identical replicas of the same work
    assert torch.distributed.is_available()
