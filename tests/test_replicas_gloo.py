"""Replica aggregation across ranks (CPU, gloo, world_size 2).

Each rank factors and solves its own seeded system with the oracle (the
GPU run does the same with the library, one GPU per rank); the host-side
aggregation the benchmark uses must give the slowest rank's time and the
total work, and every rank's result must be correct on its own.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import time

    import numpy as np
    import torch.distributed as dist

    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from dagger_gb300 import replicas
        from oracle import tiled as o
        n, nb = 256 + 64 * rank, 64
        A = o.spd_uniform(n, 100 + rank)
        B = o.rhs_normal(n, 3, rank)
        replicas.barrier()
        t0 = time.perf_counter()
        F, info = o.chol_tiled(A, nb, 'U')
        X = B.copy(order='F')
        o.ldiv_cholesky(F, 'U', X, nb)
        t = time.perf_counter() - t0 + 0.01 * rank   # ranks differ in time
        tmax = replicas.max_over_ranks(t)
        work = replicas.sum_over_ranks(n ** 3 / 3.0)
        ok = info == 0 and o.backward_error(A, X, B).max() < 1e-14
        out.put((rank, t, tmax, work, bool(ok)))
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    times = [r[1] for r in res]
    for _, t, tmax, work, ok in res:
        assert ok
        assert tmax == pytest.approx(max(times))
        assert work == pytest.approx(256 ** 3 / 3.0 + 320 ** 3 / 3.0)
