"""GPU tests of the serving loop: continuous batching under an HBM budget; every result is
the same alone and in the mix (split-path bound 1e-12, FP64 path bit-identical)."""
import time

import numpy as np
import pytest

from oracle import psmma_oracle as O

pytestmark = pytest.mark.gpu


def _col(x, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x).T)).to(cuda).t()


def _make(kind, n, seed, cuda):
    import torch
    import psmma_git_gb300 as P
    if kind == "dft":
        B = _col(O.cfg_matrix(n, n, seed=seed, complex_=True), cuda)
        return B, None, P.fortran_empty(n, n, torch.complex128, cuda)
    A = _col(O.cfg_matrix(n, n, seed=seed), cuda)
    if kind == "cauchy":
        gen = _col(O.cfg_cauchy_generators(n, seed=seed + 1), cuda)
    else:
        gen = torch.from_numpy(O.cfg_vector(2 * n - 1, seed=seed + 1)).to(cuda)
    return A, gen, P.fortran_empty(n, n, torch.float64, cuda)


def _alone(kind, n, A, gen, prec, cuda):
    import torch
    import psmma_git_gb300 as P
    if kind == "dft":
        C = P.fortran_empty(n, n, torch.complex128, cuda)
        P.pzmdftl(n, n, 1.0, A, 0.0, C, precision=prec)
        torch.cuda.synchronize()
        return C
    Q = P.fortran_empty(n, n, torch.float64, cuda)
    getattr(P, "psmma_" + kind)(n, n, 1.0, A, gen, 0.0, Q, precision=prec)
    torch.cuda.synchronize()
    return Q


def test_mixed_batch_same_alone_and_in_the_mix(cuda):
    import torch
    from psmma_git_gb300 import workspace_size
    from psmma_git_gb300.server import Server, KINDS
    rng = np.random.default_rng(7)
    kinds = ["cauchy", "toeplitz", "hankel", "dft"]
    reqs = []
    for i in range(16):
        kind = kinds[i % 4]
        n = int(np.exp(rng.uniform(np.log(200), np.log(1200))))
        prec = "split" if i % 8 != 7 else "fp64"
        reqs.append((kind, n, prec) + _make(kind, n, 100 + i, cuda))
    biggest = max(workspace_size(KINDS[k], n, n, p) for (k, n, p, *_r) in reqs)
    # a budget of ~2.5 of the largest workspaces forces admission to wait for memory
    budget = int(2.5 * biggest) + (1 << 20)
    with Server(budget, max_inflight=4) as srv:
        tickets = [srv.submit(k, n, n, 1.0, A, g, 0.0, Q, precision=p, tag=i)
                   for i, (k, n, p, A, g, Q) in enumerate(reqs)]
        seen_inflight = 0
        t_end = time.time() + 120
        while time.time() < t_end:
            q, f = srv.pending()
            seen_inflight = max(seen_inflight, f)
            assert f <= 4
            if q == 0 and f == 0:
                break
            time.sleep(0.0005)
        infos = [srv.wait(t) for t in tickets]
    assert all(i["status"] == 0 for i in infos)
    assert seen_inflight >= 2  # requests overlapped on the device
    for (k, n, p, A, g, Q), info in zip(reqs, infos):
        ref = _alone(k, n, A, g, p, cuda)
        err = (torch.linalg.norm(Q - ref) / torch.linalg.norm(ref)).item()
        if p == "fp64":
            assert torch.equal(Q, ref), (k, n)
        else:
            assert err < 1e-12, (k, n, err)
        assert info["latency_s"] >= info["queue_s"] >= 0.0


def test_request_larger_than_budget_is_rejected(cuda):
    from psmma_git_gb300 import PsmmaError
    from psmma_git_gb300.server import Server
    A, g, Q = _make("hankel", 512, 1, cuda)
    with Server(1 << 20, max_inflight=2) as srv:
        with pytest.raises(PsmmaError) as e:
            srv.submit("hankel", 512, 512, 1.0, A, g, 0.0, Q, precision="split")
        assert e.value.status == -110
        # an FP64 request needs no workspace and runs
        t = srv.submit("hankel", 512, 512, 1.0, A, g, 0.0, Q, precision="fp64")
        assert srv.wait(t)["status"] == 0


def test_server_results_match_oracle(cuda):
    from psmma_git_gb300.server import Server
    n = 300
    A, g, Q = _make("cauchy", n, 5, cuda)
    with Server(1 << 30, max_inflight=2) as srv:
        assert srv.wait(srv.submit("cauchy", n, n, 1.0, A, g, 0.0, Q, precision="split"))["status"] == 0
    An = A.t().contiguous().cpu().numpy().T
    gn = g.t().contiguous().cpu().numpy().T
    got = Q.t().contiguous().cpu().numpy().T
    assert O.rel_fro(got, O.dense_product("cauchy", 1.0, An, gn, 0.0, None, n)) < 1e-12


def test_server_cauchyeig_requests_match_oracle(cuda):
    import numpy as np
    import torch
    import psmma_git_gb300 as P
    from psmma_git_gb300.server import Server
    n = 257
    F, U, V, dl, dr = O.eig_generators(n, seed=8, tiny=3)
    gen = torch.from_numpy(np.ascontiguousarray(np.stack([F, U, V, dl, dr]))).cuda().t()  # n x 5
    A = O.cfg_matrix(n, n, seed=9)
    dA = P.fortran_empty(n, n)
    dA.copy_(torch.from_numpy(A))
    ref = A @ O.cauchy_like_eig(F, U, V, dl, dr)
    with Server(1 << 30, max_inflight=2) as srv:
        for prec, tol in [("fp64", 1e-13), ("split", 1e-12)]:
            Q = P.fortran_empty(n, n)
            assert srv.wait(srv.submit("cauchyeig", n, n, 1.0, dA, gen, 0.0, Q, precision=prec))["status"] == 0
            assert O.rel_fro(Q.cpu().numpy(), ref) < tol, prec


def test_large_request_between_small_ones(cuda):
    # small requests, two large ones (n = 8192, split DFT with its radix step, and a split
    # Cauchy multiply of n = 6144) in the middle, small ones after: every result is its multiply
    # alone within the split path's bound, all statuses are ok, and the small request admitted
    # first (highest-priority stream) is done before the large ones
    import torch
    from psmma_git_gb300.server import Server
    plan = [("hankel", 512), ("toeplitz", 700), ("dft", 8192), ("cauchy", 600), ("cauchy", 6144),
            ("hankel", 256), ("dft", 384), ("toeplitz", 1000)]
    reqs = [(k, n) + _make(k, n, 300 + i, cuda) for i, (k, n) in enumerate(plan)]
    torch.cuda.synchronize()
    with Server(64 << 30, max_inflight=4) as srv:
        tickets = [srv.submit(k, n, n, 1.0, A, g, 0.0, Q, precision="split", tag=i)
                   for i, (k, n, A, g, Q) in enumerate(reqs)]
        infos = [srv.wait(t) for t in tickets]
    assert all(i["status"] == 0 for i in infos)
    for (k, n, A, g, Q), info in zip(reqs, infos):
        ref = _alone(k, n, A, g, "split", cuda)
        assert (torch.linalg.norm(Q - ref) / torch.linalg.norm(ref)).item() < 1e-12, (k, n)
    large_end = max(infos[2]["end_s"], infos[4]["end_s"])
    assert infos[0]["end_s"] <= large_end
