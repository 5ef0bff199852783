"""Multi-rank host logic on CPU (gloo, world size 2): row panels cover the rows exactly once,
each rank's panel product needs no exchange, the panels assemble into the full product, and
the timing reduction takes the slowest rank.  The per-rank compute is the oracle here (no
GPU in this test); on GPUs it is the library call."""
import os
import socket

import numpy as np
import pytest

from psmma_git_gb300.shard import local_panel, panels


def test_panels_partition():
    for n in [0, 1, 7, 100, 16384]:
        for w in [1, 2, 3, 8]:
            p = panels(n, w)
            assert len(p) == w and p[0][0] == 0 and p[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(p, p[1:]))
            sizes = [e - s for s, e in p]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, n, k, out_q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import psmma_oracle as O
        from psmma_git_gb300.shard import max_over_ranks, sharded_multiply
        A = O.cfg_matrix(n, k, seed=3)            # every rank can build the same inputs
        gen = O.cfg_cauchy_generators(k, seed=4)  # replicated O(k) generators
        lo, hi = local_panel(n, rank, world)

        def oracle_compute(rows, kk, alpha, Ap, g, beta, Qp):
            return O.dense_product("cauchy", alpha, Ap, g, beta, Qp, kk)

        Qp = sharded_multiply("cauchy", n, k, 1.0, A[lo:hi], gen, 0.0, np.zeros((hi - lo, k)), rank=rank,
                              world=world, compute=oracle_compute)
        slowest = max_over_ranks(float(rank + 1))
        out_q.put((rank, lo, hi, Qp, slowest))
    finally:
        dist.destroy_process_group()


def test_row_panels_assemble_the_full_product_gloo():
    import multiprocessing as mp
    from oracle import psmma_oracle as O
    n, k, world = 37, 29, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n, k, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    Q = np.zeros((n, k))
    for rank, lo, hi, Qp, slowest in got:
        Q[lo:hi] = Qp
        assert slowest == float(world)
    ref = O.dense_product("cauchy", 1.0, O.cfg_matrix(n, k, seed=3), O.cfg_cauchy_generators(k, seed=4), 0.0,
                          None, k)
    assert O.rel_fro(Q, ref) < 1e-14


def _strong_worker(rank, world, port, n, k, out_q):
    # the bench's --strong mode on CPU: one n x k problem, rank r holds rows local_panel(n, r, world)
    # of A only, multiplies them, and the slowest rank's time is the job's
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import psmma_oracle as O
        from psmma_git_gb300.shard import max_over_ranks, sharded_multiply
        lo, hi = local_panel(n, rank, world)
        A_rows = O.cfg_matrix(n, k, seed=5)[lo:hi]
        gen = O.cfg_vector(2 * k - 1, seed=6)

        def oracle_compute(rows, kk, alpha, Ap, g, beta, Qp):
            assert rows == Ap.shape[0] == hi - lo
            return O.dense_product("toeplitz", alpha, Ap, g, beta, Qp, kk)

        Qp = sharded_multiply("toeplitz", n, k, 0.5, A_rows, gen, 0.0, np.zeros((hi - lo, k)), rank=rank,
                              world=world, compute=oracle_compute)
        out_q.put((rank, lo, hi, Qp, max_over_ranks(float(hi - lo))))
    finally:
        dist.destroy_process_group()


def test_strong_scaling_row_panels_gloo():
    # world size 3 on n = 40 rows: uneven panels (14, 13, 13) that assemble the whole product
    import multiprocessing as mp
    from oracle import psmma_oracle as O
    n, k, world = 40, 23, 3
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_strong_worker, args=(r, world, port, n, k, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    Q = np.full((n, k), np.nan)
    for rank, lo, hi, Qp, slowest in got:
        Q[lo:hi] = Qp
        assert slowest == 14.0
    ref = O.dense_product("toeplitz", 0.5, O.cfg_matrix(n, k, seed=5), O.cfg_vector(2 * k - 1, seed=6), 0.0, None, k)
    assert O.rel_fro(Q, ref) < 1e-14
