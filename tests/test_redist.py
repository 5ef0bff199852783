"""Descriptor interop (REDIST / PDGEMR2D, psmma_cauchy.f90:113-162) and the 2.5D index helpers
(Auxil_2p5D.f90:315-419).

CPU tests check the library's plan (counts, maps, argument codes) by applying its maps with
numpy for every rank of a grid and comparing with the oracle's PDGEMR2D on the assembled
global matrices; gloo tests (world size 2 and 4) run the distributed multiply's host logic
and exchange with the oracle as the per-rank compute.  GPU tests run the pack / unpack
kernels and the distributed multiply with the ranks as threads of one process (each rank's
kernels finish before the emulated exchange reads their buffers: no kernel waits on
another)."""
import ctypes as C
import os
import socket
import threading

import numpy as np
import pytest

from oracle import psmma_oracle as O
from psmma_git_gb300 import _lib

# (m, n, desca, grid_a, ia, ja, descb-without-LLD, grid_b, ib, jb)
LAYOUTS = [
    # the reference's REDIST target: nb x nb block-cyclic -> blocked ceil(N/P) x ceil(K/Q)
    (37, 29, (37, 29, 4, 4, 0, 0), (2, 2, "R"), 1, 1, (37, 29, 19, 15, 0, 0), (2, 2, "R"), 1, 1),
    # to row panels over all ranks, column-major grid, nonzero source process
    (50, 23, (50, 23, 3, 5, 1, 1), (2, 3, "C"), 1, 1, (50, 23, 9, 23, 0, 0), (6, 1, "R"), 1, 1),
    # sub-matrices at offsets in both layouts
    (20, 17, (31, 40, 4, 3, 1, 0), (2, 2, "R"), 5, 9, (25, 19, 2, 7, 0, 1), (1, 4, "R"), 3, 2),
    # one process, blocks larger than the matrix
    (13, 9, (13, 9, 64, 64, 0, 0), (1, 1, "R"), 1, 1, (13, 9, 5, 2, 0, 0), (1, 1, "R"), 1, 1),
    # empty sub-matrix
    (0, 7, (10, 10, 3, 3, 0, 0), (2, 2, "R"), 1, 1, (10, 10, 2, 2, 1, 0), (4, 1, "R"), 1, 1),
]


def _grid(g):
    from psmma_git_gb300.redist import Grid
    return Grid(*g)


def _desc(d6, grid, rank):
    pr, _ = O.grid_coords(rank, *grid)
    lr = O.numroc(d6[0], d6[2], pr, d6[4], grid[0])
    return (1, 0) + tuple(d6) + (max(1, lr) + (rank % 2),)  # odd ranks get a padded LLD


def _local_arr(desc, grid, rank, G):
    pr, pc = O.grid_coords(rank, *grid)
    L = O.bc_local(G, desc, grid[0], grid[1], pr, pc)
    out = np.full((desc[8], max(L.shape[1], 1)), np.nan, dtype=G.dtype)
    out[:L.shape[0], :L.shape[1]] = L
    return out, L.shape


def _np_pack(plan, A):
    """The plan's maps applied with numpy (the kernels' contract, for the CPU tests)."""
    rp, rq = plan.maps(0)
    cp, cq = plan.maps(1)
    gb = plan.grid_b
    rcnt = np.bincount(rp[rp >= 0], minlength=gb.nprow)
    displ = np.concatenate([[0], np.cumsum(plan.send_counts)[:-1]]).astype(np.int64)
    buf = np.zeros(sum(plan.send_counts), dtype=A.dtype)
    for j in range(len(cp)):
        if cp[j] < 0:
            continue
        for i in range(len(rp)):
            if rp[i] < 0:
                continue
            peer = gb.rank_of(int(rp[i]), int(cp[j]))
            buf[displ[peer] + cq[j] * rcnt[rp[i]] + rq[i]] = A[i, j]
    return buf


def _np_unpack(plan, buf, B):
    rp, rq = plan.maps(2)
    cp, cq = plan.maps(3)
    ga = plan.grid_a
    rcnt = np.bincount(rp[rp >= 0], minlength=ga.nprow)
    displ = np.concatenate([[0], np.cumsum(plan.recv_counts)[:-1]]).astype(np.int64)
    for j in range(len(cp)):
        if cp[j] < 0:
            continue
        for i in range(len(rp)):
            if rp[i] < 0:
                continue
            peer = ga.rank_of(int(rp[i]), int(cp[j]))
            B[i, j] = buf[displ[peer] + cq[j] * rcnt[rp[i]] + rq[i]]


def _exchange_all(sends, plans):
    """All-to-all over in-process ranks: rank r's receive buffer gathers, in sender order, each
    sender's segment for r."""
    P = len(plans)
    out = []
    for r in range(P):
        parts = []
        for s in range(P):
            d = int(np.sum(plans[s].send_counts[:r]))
            parts.append(sends[s][d:d + plans[s].send_counts[r]])
        out.append(np.concatenate(parts) if parts else np.zeros(0))
    return out


def test_numroc_matches_oracle(lib):
    for n in [0, 1, 7, 64, 100, 1031]:
        for nb in [1, 3, 64]:
            for P in [1, 2, 3, 5]:
                for src in range(P):
                    for p in range(P):
                        assert lib.psmma_numroc(n, nb, p, src, P) == O.numroc(n, nb, p, src, P)


def test_plan_argument_codes(lib):
    from psmma_git_gb300.redist import RedistPlan
    from psmma_git_gb300 import PsmmaError
    g = _grid((2, 2, "R"))
    good = (1, 0, 10, 10, 2, 2, 0, 0, 6)
    cases = [
        (dict(desca=(2,) + good[1:]), -301),             # DTYPE_
        (dict(desca=good[:4] + (0,) + good[5:]), -305),  # MB_
        (dict(desca=good[:6] + (2,) + good[7:]), -307),  # RSRC_ outside the grid
        (dict(desca=good[:8] + (3,)), -309),             # LLD_ < local rows
        (dict(descb=good[:5] + (0,) + good[6:]), -706),  # NB_ of B
        (dict(ia=0), -4), (dict(ja=2), -5), (dict(ib=2), -8), (dict(jb=0), -9),
    ]
    for kw, code in cases:
        args = dict(m=10, n=10, desca=good, descb=good, ia=1, ja=1, ib=1, jb=1)
        args.update(kw)
        with pytest.raises(PsmmaError) as e:
            RedistPlan(args["m"], args["n"], args["desca"], g, args["descb"], g, 0, args["ia"], args["ja"],
                       args["ib"], args["jb"])
        assert e.value.status == code, (kw, e.value.status)
    with pytest.raises(PsmmaError) as e:
        RedistPlan(10, 10, good, g, good, _grid((3, 1, "R")), 0)       # different process counts
    assert e.value.status == -10
    with pytest.raises(PsmmaError) as e:
        RedistPlan(10, 10, good, g, good, g, 4)                         # rank outside the grid
    assert e.value.status == -6
    h = C.c_void_p()
    assert lib.psmma_redist_plan_create(-1, 3, None, 1, 1, g.c(), None, 1, 1, g.c(), 0, C.byref(h)) == -1


@pytest.mark.parametrize("case", range(len(LAYOUTS)))
def test_plan_counts_and_maps_match_oracle(case):
    from psmma_git_gb300.redist import RedistPlan
    m, n, da6, ga, ia, ja, db6, gb, ib, jb = LAYOUTS[case]
    P = ga[0] * ga[1]
    rng = np.random.default_rng(case)
    GA = rng.standard_normal((da6[0], da6[1]))
    GB = rng.standard_normal((db6[0], db6[1]))
    plans, sends, A_loc, B_loc, descs_b = [], [], {}, {}, {}
    for r in range(P):
        da, db = _desc(da6, ga, r), _desc(db6, gb, r)
        descs_b[r] = db
        A, ashape = _local_arr(da, ga, r, GA)
        B, bshape = _local_arr(db, gb, r, GB)
        p = RedistPlan(m, n, da, _grid(ga), db, _grid(gb), r, ia, ja, ib, jb)
        assert p.a_shape == ashape and p.b_shape == bshape
        plans.append(p)
        sends.append(_np_pack(p, A[:ashape[0], :ashape[1]]))
        A_loc[r], B_loc[r] = A[:ashape[0], :ashape[1]], B
    S = np.array([p.send_counts for p in plans])
    R = np.array([p.recv_counts for p in plans])
    assert (S == R.T).all() and S.sum() == m * n
    recvs = _exchange_all(sends, plans)
    got = {}
    for r in range(P):
        B = B_loc[r]
        _np_unpack(plans[r], recvs[r], B)
        got[r] = B[:plans[r].b_shape[0], :plans[r].b_shape[1]]
    want = O.pdgemr2d(m, n, A_loc, ia, ja, _desc(da6, ga, 0), ga,
                      {r: O.bc_local(GB, descs_b[r], gb[0], gb[1], *O.grid_coords(r, *gb)) for r in range(P)},
                      ib, jb, _desc(db6, gb, 0), gb)
    for r in range(P):
        assert np.array_equal(got[r], want[r]), r


def test_2p5d_index_helpers_match_oracle(lib):
    from psmma_git_gb300.redist import const_index1, redist2p5_index
    from psmma_git_gb300 import PsmmaError
    for k, nb, npzc, npcol in [(10, 2, 2, 4), (100, 7, 1, 3), (64, 8, 2, 2), (37, 5, 3, 6), (1, 4, 1, 1), (0, 3, 1, 2)]:
        got = redist2p5_index(k, nb, npzc, npcol)
        want = O.redist2p5a(k, nb, npzc, npcol)
        assert np.array_equal(got, want)
        assert sorted(got.tolist()) == list(range(1, k + 1))
        for mycol in range(npcol):
            ref = O.const_index1(k, nb, mycol, npcol, want)
            c1 = const_index1(k, nb, mycol, npcol, got)
            assert c1.tolist() == [x for x in ref if x is not None]
    with pytest.raises(PsmmaError) as e:
        redist2p5_index(10, 2, 3, 4)      # "NPZC must divide NPCOL"
    assert e.value.status == -3


# ---- gloo: the distributed multiply's host logic and exchange, oracle as compute --------
def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


class NumpyMover:
    """Applies the plan's maps on the CPU (test stand-in for the GPU kernels)."""

    @staticmethod
    def pack(plan, A_local, sendbuf):
        import torch
        sendbuf[:sum(plan.send_counts)] = torch.from_numpy(_np_pack(plan, A_local.numpy()))

    @staticmethod
    def unpack(plan, recvbuf, B_local):
        B = B_local.numpy()
        _np_unpack(plan, recvbuf[:sum(plan.recv_counts)].numpy(), B)


def _gloo_worker(rank, world, port, grid, kind, redist, beta, out_q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from psmma_git_gb300.redist import Grid, descinit, pstructured
        g = Grid(*grid)
        n, k, nb = 45, 38, 4
        GA = O.cfg_matrix(n, k, seed=3)
        GQ = O.cfg_matrix(n + 3, k + 2, seed=5)
        gen = O.cfg_cauchy_generators(k, seed=4) if kind == "cauchy" else O.cfg_vector(2 * k - 1, seed=4)
        pr, pc = g.coords(rank)
        da = descinit(n, k, nb, nb, 0, 0, g, rank)
        dq = descinit(n + 3, k + 2, 3, 5, 1 % grid[0], 0, g, rank) if redist else da
        A = torch.from_numpy(np.asfortranarray(O.bc_local(GA, da, grid[0], grid[1], pr, pc))).t().contiguous().t()
        Q0 = O.bc_local(GQ if redist else GQ[:n, :k], dq, grid[0], grid[1], pr, pc)
        Q = torch.from_numpy(np.asfortranarray(Q0)).t().contiguous().t()

        def oracle_compute(rows, kk, alpha, Ap, gg, beta_, Qp):
            Qp.copy_(torch.from_numpy(O.dense_product(kind, alpha, Ap.numpy(), gg, beta_, Qp.numpy(), kk)))
            return Qp

        iq, jq = (3, 2) if redist else (1, 1)
        pstructured(kind, n, k, 0.5, A, da, gen, beta, Q, dq, g, rank, iq=iq, jq=jq, redist=redist,
                    mover=NumpyMover, compute=oracle_compute)
        out_q.put((rank, Q.numpy().copy(), dq))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("grid,kind,redist,beta", [((2, 1, "R"), "cauchy", False, 0.0),
                                                   ((1, 2, "R"), "toeplitz", True, -1.5),
                                                   ((2, 2, "R"), "cauchy", True, 0.25),
                                                   ((2, 2, "C"), "hankel", False, 2.0)])
def test_distributed_multiply_gloo(grid, kind, redist, beta):
    import multiprocessing as mp
    world = grid[0] * grid[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_gloo_worker, args=(r, world, port, grid, kind, redist, beta, q))
             for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=180) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    n, k = 45, 38
    GA = O.cfg_matrix(n, k, seed=3)
    GQ = O.cfg_matrix(n + 3, k + 2, seed=5)
    gen = O.cfg_cauchy_generators(k, seed=4) if kind == "cauchy" else O.cfg_vector(2 * k - 1, seed=4)
    if redist:
        want = GQ.copy()
        want[2:2 + n, 1:1 + k] = O.dense_product(kind, 0.5, GA, gen, beta, GQ[2:2 + n, 1:1 + k], k)
    else:
        want = O.dense_product(kind, 0.5, GA, gen, beta, GQ[:n, :k], k)
    Q = O.bc_global({r: L for r, L, _ in got}, got[0][2], grid[0], grid[1], grid[2])
    assert O.rel_fro(Q, want) < 1e-14


# ---- GPU: pack / unpack kernels and the distributed multiply, ranks as threads ----------
def _dev_local(L, ld):
    import torch
    base = torch.full((max(L.shape[1], 1), ld), float("nan"), dtype=torch.from_numpy(L).dtype, device="cuda")
    t = base.t()[:L.shape[0], :L.shape[1]]
    t.copy_(torch.from_numpy(L))
    return t


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(len(LAYOUTS)))
@pytest.mark.parametrize("cplx", [False, True])
def test_pack_unpack_kernels_match_oracle(case, cplx):
    import torch
    from psmma_git_gb300.redist import RedistPlan
    m, n, da6, ga, ia, ja, db6, gb, ib, jb = LAYOUTS[case]
    P = ga[0] * ga[1]
    rng = np.random.default_rng(100 + case)
    GA = rng.standard_normal((da6[0], da6[1]))
    GB = rng.standard_normal((db6[0], db6[1]))
    if cplx:
        GA = GA + 1j * rng.standard_normal(GA.shape)
        GB = GB + 1j * rng.standard_normal(GB.shape)
    plans, sends, A_loc, B_dev, B_host = [], [], {}, {}, {}
    for r in range(P):
        da, db = _desc(da6, ga, r), _desc(db6, gb, r)
        pr, pc = O.grid_coords(r, *ga)
        A_loc[r] = O.bc_local(GA, da, ga[0], ga[1], pr, pc)
        qr, qc = O.grid_coords(r, *gb)
        B_host[r] = O.bc_local(GB, db, gb[0], gb[1], qr, qc)
        p = RedistPlan(m, n, da, _grid(ga), db, _grid(gb), r, ia, ja, ib, jb)
        plans.append(p)
        Ad = _dev_local(A_loc[r], da[8])
        send = torch.zeros(max(sum(p.send_counts), 1), dtype=Ad.dtype, device="cuda")
        if sum(p.send_counts):
            p.pack(Ad, send)
        torch.cuda.synchronize()
        s = send[:sum(p.send_counts)].cpu().numpy()
        assert np.array_equal(s, _np_pack(p, A_loc[r])), r
        sends.append(s)
        B_dev[r] = _dev_local(B_host[r], db[8])
    recvs = _exchange_all(sends, plans)
    want = O.pdgemr2d(m, n, A_loc, ia, ja, _desc(da6, ga, 0), ga, B_host, ib, jb, _desc(db6, gb, 0), gb)
    for r in range(P):
        if sum(plans[r].recv_counts):
            plans[r].unpack(torch.from_numpy(recvs[r]).cuda(), B_dev[r])
        torch.cuda.synchronize()
        assert np.array_equal(B_dev[r].cpu().numpy(), want[r]), r


class ThreadExchange:
    """All-to-all among threads of one process: each rank deposits its send buffer, waits for
    all, copies its segments, waits again before anyone reuses a buffer."""

    def __init__(self, world):
        self.world = world
        self.bar = threading.Barrier(world, timeout=120)
        self.box = {}

    def __call__(self, rank):
        def ex(send, send_counts, recv, recv_counts, group=None):
            import torch
            torch.cuda.synchronize()  # this rank's pack kernel is done
            self.box[rank] = (send, list(send_counts))
            self.bar.wait()
            off = 0
            for s in range(self.world):
                sb, sc = self.box[s]
                d = sum(sc[:rank])
                recv[off:off + sc[rank]].copy_(sb[d:d + sc[rank]])
                off += sc[rank]
            torch.cuda.synchronize()
            self.bar.wait()
        return ex


def _run_threads(world, fn):
    errs, res = [], {}

    def wrap(r):
        import torch
        try:
            # a stream per rank: the library's workspace pools are per stream
            with torch.cuda.stream(torch.cuda.Stream()):
                res[r] = fn(r)
        except BaseException as e:  # noqa: BLE001 - reported below
            errs.append((r, e))

    th = [threading.Thread(target=wrap, args=(r,)) for r in range(world)]
    for t in th:
        t.start()
    for t in th:
        t.join(timeout=300)
    assert not errs, errs
    return res


@pytest.mark.gpu
@pytest.mark.parametrize("grid,kind,redist,beta,prec", [((2, 2, "R"), "cauchy", True, 0.5, "split"),
                                                        ((2, 3, "C"), "toeplitz", False, 0.0, "fp64"),
                                                        ((3, 1, "R"), "hankel", True, -1.0, "split"),
                                                        ((2, 2, "R"), "cauchyeig", True, 0.0, "split")])
def test_distributed_multiply_gpu(grid, kind, redist, beta, prec):
    import torch
    from psmma_git_gb300.redist import Grid, descinit, pstructured
    g = Grid(*grid)
    world = g.nprocs
    n, k, nb = 300, 257, 32
    GA = O.cfg_matrix(n, k, seed=7)
    GQ = O.cfg_matrix(n + 5, k + 4, seed=8)
    if kind == "cauchyeig":
        F, U, V, dl, dr = O.eig_generators(k, seed=9, tiny=1)
        host_gen = (F, U, V, dl, dr)
        H = O.cauchy_like_eig(F, U, V, dl, dr)
        gen = tuple(torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in host_gen)
        ref = lambda A, Q0: 0.5 * A @ H + beta * Q0  # noqa: E731
    else:
        host_gen = O.cfg_cauchy_generators(k, seed=9) if kind == "cauchy" else O.cfg_vector(2 * k - 1, seed=9)
        gen = (torch.from_numpy(np.asfortranarray(host_gen)).cuda().t().contiguous().t() if kind == "cauchy"
               else torch.from_numpy(host_gen).cuda())
        ref = lambda A, Q0: O.dense_product(kind, 0.5, A, host_gen, beta, Q0, k)  # noqa: E731
    ex = ThreadExchange(world)
    iq, jq = (4, 3) if redist else (1, 1)

    def rank_fn(r):
        pr, pc = g.coords(r)
        da = descinit(n, k, nb, nb, 0, 0, g, r)
        dq = descinit(n + 5, k + 4, 16, 24, 1 % grid[0], 0, g, r, ) if redist else da
        A = _dev_local(O.bc_local(GA, da, grid[0], grid[1], pr, pc), da[8])
        Q = _dev_local(O.bc_local(GQ if redist else GQ[:n, :k], dq, grid[0], grid[1], pr, pc), dq[8])
        pstructured(kind, n, k, 0.5, A, da, gen, beta, Q, dq, g, r, iq=iq, jq=jq, redist=redist,
                    precision=prec, exchange=ex(r))
        torch.cuda.synchronize()
        return Q.cpu().numpy(), dq

    res = _run_threads(world, rank_fn)
    Qg = O.bc_global({r: res[r][0] for r in res}, res[0][1], grid[0], grid[1], grid[2])
    if redist:
        want = GQ.copy()
        want[iq - 1:iq - 1 + n, jq - 1:jq - 1 + k] = ref(GA, GQ[iq - 1:iq - 1 + n, jq - 1:jq - 1 + k])
        outside = np.ones_like(GQ, dtype=bool)
        outside[iq - 1:iq - 1 + n, jq - 1:jq - 1 + k] = False
        assert np.array_equal(Qg[outside], GQ[outside])
    else:
        want = ref(GA, GQ[:n, :k])
    tol = 1e-13 if prec == "fp64" else 1e-12
    assert O.rel_fro(Qg, want) < tol


@pytest.mark.gpu
@pytest.mark.parametrize("grid,beta", [((2, 2, "R"), 0.0), ((3, 2, "C"), -0.5), ((1, 3, "R"), 1.0)])
def test_distributed_dft_gpu(grid, beta):
    import torch
    from psmma_git_gb300.redist import Grid, pzmdftl_distributed
    g = Grid(*grid)
    n, k, nb, kb = 96, 70, 8, 6
    GB = O.cfg_matrix(n, k, seed=11, complex_=True)
    GC = O.cfg_matrix(n, k, seed=12, complex_=True)
    ex = ThreadExchange(g.nprocs)

    def rank_fn(r):
        pr, pc = g.coords(r)
        d = (1, 0, n, k, nb, kb, 1 % grid[0], 0, 0)
        lr = O.numroc(n, nb, pr, d[6], grid[0])
        d = d[:8] + (max(1, lr),)
        B = _dev_local(O.bc_local(GB, d, grid[0], grid[1], pr, pc), d[8])
        Cm = _dev_local(O.bc_local(GC, d, grid[0], grid[1], pr, pc), d[8])
        pzmdftl_distributed(n, k, nb, kb, 0.75, B, beta, Cm, d[6], 0, g, r, precision="split", exchange=ex(r))
        torch.cuda.synchronize()
        return Cm.cpu().numpy(), d

    res = _run_threads(g.nprocs, rank_fn)
    Cg = O.bc_global({r: res[r][0] for r in res}, res[0][1], grid[0], grid[1], grid[2])
    assert O.rel_fro(Cg, O.dft_product(0.75, GB, beta, GC)) < 1e-12


@pytest.mark.gpu
def test_redist2p5_permutes_generator_rows():
    import torch
    from psmma_git_gb300.redist import redist2p5
    k = 1000
    gen = O.cfg_cauchy_generators(k, seed=2)
    Bd = torch.from_numpy(np.asfortranarray(gen)).cuda().t().contiguous().t()
    TB = redist2p5(k, 16, 2, 4, Bd)
    torch.cuda.synchronize()
    perm = O.redist2p5a(k, 16, 2, 4) - 1
    assert np.array_equal(TB.cpu().numpy(), gen[perm])
