"""GPU test of psmma_cauchy_split_noalloc, the entry point for callers that cannot let a
library allocate device memory (they own all of it through their own pool, or cannot take
cudaMalloc's device-wide synchronisation).  It must give the same result as the ordinary
split-path entry point, call after call, using only its fixed 96 MiB scratch array, and
refuse requests that do not fit.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from oracle import psmma_oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the split path's stated bound (relative Frobenius)
SCRATCH = 96 << 20  # the entry point's fixed scratch array


def _col(x, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x).T)).to(cuda).t()


def _noalloc(lib, n, k, alpha, dA, dg, beta, dQ, n_moduli=0, sync=True):
    import torch
    st = lib.psmma_cauchy_split_noalloc(n, k, alpha, C.c_void_p(dA.data_ptr()), dA.stride(1),
                                        C.c_void_p(dg.data_ptr()), dg.stride(1), beta,
                                        C.c_void_p(dQ.data_ptr()), dQ.stride(1), n_moduli,
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    if sync:
        torch.cuda.synchronize()
    return st


def _regular(lib, n, k, alpha, dA, dg, beta, dQ, n_moduli=0):
    import torch
    from psmma_git_gb300 import make_opts
    o = make_opts("split", n_moduli)
    st = lib.psmma_cauchy(n, k, alpha, C.c_void_p(dA.data_ptr()), dA.stride(1), C.c_void_p(dg.data_ptr()),
                          dg.stride(1), beta, C.c_void_p(dQ.data_ptr()), dQ.stride(1), C.byref(o),
                          C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st


def _largest_square(n_moduli):
    """The largest n (k = n) whose split workspace fits in the scratch array."""
    import psmma_git_gb300 as P
    lo, hi = 1, 4096
    while lo < hi:
        mid = (lo + hi + 1) // 2
        if P.workspace_size(P.KIND_CAUCHY, mid, mid, "split", n_moduli) <= SCRATCH:
            lo = mid
        else:
            hi = mid - 1
    return lo


def test_noalloc_matches_split_entry_point_twice(lib, cuda):
    import torch
    # two calls in a row with different inputs and shapes: the second must not see the
    # first call's leftovers in the shared scratch
    for (n, k, seed, beta) in [(1024, 1024, 1, 0.0), (700, 513, 2, -0.5)]:
        A = O.cfg_matrix(n, k, seed=seed, dist="normal")
        gen = O.cfg_cauchy_generators(k, seed=seed + 10, clustered=0.1)
        Q0 = O.cfg_matrix(n, k, seed=seed + 20)
        dA, dg = _col(A, cuda), _col(gen, cuda)
        dQ1, dQ2 = _col(Q0, cuda), _col(Q0, cuda)
        assert _noalloc(lib, n, k, 1.0, dA, dg, beta, dQ1) == 0
        assert _regular(lib, n, k, 1.0, dA, dg, beta, dQ2) == 0
        err = (torch.linalg.norm(dQ1 - dQ2) / torch.linalg.norm(dQ2)).item()
        assert err < TOL
        got = dQ1.t().contiguous().cpu().numpy().T
        assert O.rel_fro(got, O.dense_product("cauchy", 1.0, A, gen, beta, Q0, k)) < TOL


@pytest.mark.parametrize("n_moduli,alpha", [(8, 2.5), (16, 2.5), (16, 1.0)])
def test_noalloc_moduli_and_alpha(lib, cuda, n_moduli, alpha):
    # an explicit moduli count and alpha != 1, twice in a row, against the regular entry point
    # with the same moduli count (8 moduli carry fewer bits: compare the two paths, which
    # compute the same integers, and check the oracle error only at 16)
    import torch
    for n, k, seed in [(384, 320, 5), (257, 511, 6)]:
        A = O.cfg_matrix(n, k, seed=seed)
        gen = O.cfg_cauchy_generators(k, seed=seed + 1)
        Q0 = O.cfg_matrix(n, k, seed=seed + 2)
        dA, dg = _col(A, cuda), _col(gen, cuda)
        dQ1, dQ2 = _col(Q0, cuda), _col(Q0, cuda)
        assert _noalloc(lib, n, k, alpha, dA, dg, 0.5, dQ1, n_moduli) == 0
        assert _regular(lib, n, k, alpha, dA, dg, 0.5, dQ2, n_moduli) == 0
        assert torch.equal(dQ1, dQ2)
        if n_moduli == 16:
            ref = O.dense_product("cauchy", alpha, A, gen, 0.5, Q0, k)
            assert O.rel_fro(dQ1.t().contiguous().cpu().numpy().T, ref) < TOL


def test_noalloc_alpha_zero_scales_q_only(lib, cuda):
    # alpha = 0: Q := beta*Q without reading A or the generators (an Inf in A stays out)
    import torch
    n, k = 300, 200
    A = O.cfg_matrix(n, k, seed=7)
    A[3, 5] = np.inf
    gen = O.cfg_cauchy_generators(k, seed=8)
    Q0 = O.cfg_matrix(n, k, seed=9)
    dA, dg, dQ = _col(A, cuda), _col(gen, cuda), _col(Q0, cuda)
    assert _noalloc(lib, n, k, 0.0, dA, dg, -2.0, dQ) == 0
    assert torch.equal(dQ, _col(-2.0 * Q0, cuda))
    assert _noalloc(lib, n, k, 0.0, dA, dg, 0.0, dQ) == 0
    assert float(dQ.abs().max()) == 0.0
    # null operands are fine when alpha = 0 (as psmma_cauchy); a null Q is not
    st = lib.psmma_cauchy_split_noalloc(n, k, 0.0, None, n, None, k, 3.0, C.c_void_p(dQ.data_ptr()), n, 0,
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    from psmma_git_gb300 import _lib
    st = lib.psmma_cauchy_split_noalloc(n, k, 0.0, None, n, None, k, 3.0, None, n, 0,
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == _lib.PSMMA_ENULL


@pytest.mark.parametrize("n_moduli", [0, 16])
def test_noalloc_at_the_scratch_limit(lib, cuda, n_moduli):
    # the largest square request that fits runs (twice, the edge of the array in use); one
    # row and column more is refused before anything is written
    import torch
    import psmma_git_gb300 as P
    from psmma_git_gb300 import _lib
    n = _largest_square(n_moduli)
    assert P.workspace_size(P.KIND_CAUCHY, n, n, "split", n_moduli) <= SCRATCH
    assert P.workspace_size(P.KIND_CAUCHY, n + 1, n + 1, "split", n_moduli) > SCRATCH
    for seed in (11, 12):
        A = O.cfg_matrix(n, n, seed=seed)
        gen = O.cfg_cauchy_generators(n, seed=seed + 1)
        dA, dg = _col(A, cuda), _col(gen, cuda)
        dQ1 = P.fortran_empty(n, n, torch.float64, cuda)
        dQ2 = P.fortran_empty(n, n, torch.float64, cuda)
        assert _noalloc(lib, n, n, 1.0, dA, dg, 0.0, dQ1, n_moduli) == 0
        assert _regular(lib, n, n, 1.0, dA, dg, 0.0, dQ2, n_moduli) == 0
        assert torch.equal(dQ1, dQ2)
        ref = O.dense_product("cauchy", 1.0, A, gen, 0.0, None, n)
        assert O.rel_fro(dQ1.t().contiguous().cpu().numpy().T, ref) < TOL
    m = n + 1
    dA = _col(O.cfg_matrix(m, m, seed=13), cuda)
    dg = _col(O.cfg_cauchy_generators(m, seed=14), cuda)
    dQ = _col(np.zeros((m, m)), cuda)
    assert _noalloc(lib, m, m, 1.0, dA, dg, 0.0, dQ, n_moduli) == _lib.PSMMA_ESCRATCH
    assert float(dQ.abs().max()) == 0.0


def test_noalloc_returns_with_its_work_done(lib, cuda):
    # the call blocks until its work on the stream has finished: nothing is pending on the
    # stream when it returns, and Q holds the product without a further synchronisation
    import torch
    n, k = 512, 512
    A = O.cfg_matrix(n, k, seed=15)
    gen = O.cfg_cauchy_generators(k, seed=16)
    dA, dg = _col(A, cuda), _col(gen, cuda)
    s = torch.cuda.Stream()
    dQ = _col(np.zeros((n, k)), cuda)
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        assert _noalloc(lib, n, k, 1.0, dA, dg, 0.0, dQ, sync=False) == 0
        assert s.query()
    ref = O.dense_product("cauchy", 1.0, A, gen, 0.0, None, k)
    assert O.rel_fro(dQ.t().contiguous().cpu().numpy().T, ref) < TOL


def test_noalloc_rejects_requests_beyond_its_scratch(lib, cuda):
    from psmma_git_gb300 import _lib
    n = k = 2048  # split workspace ~330 MB > 96 MiB
    A = O.cfg_matrix(n, k, seed=3)
    gen = O.cfg_cauchy_generators(k, seed=4)
    dA, dg = _col(A, cuda), _col(gen, cuda)
    dQ = _col(np.zeros((n, k)), cuda)
    assert _noalloc(lib, n, k, 1.0, dA, dg, 0.0, dQ) == _lib.PSMMA_ESCRATCH
    assert float(dQ.abs().max()) == 0.0  # nothing was written
    assert "scratch" in _lib.status_string(_lib.PSMMA_ESCRATCH)
