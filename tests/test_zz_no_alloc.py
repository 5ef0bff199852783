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


def _col(x, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x).T)).to(cuda).t()


def _noalloc(lib, n, k, alpha, dA, dg, beta, dQ, n_moduli=0):
    import torch
    st = lib.psmma_cauchy_split_noalloc(n, k, alpha, C.c_void_p(dA.data_ptr()), dA.stride(1),
                                        C.c_void_p(dg.data_ptr()), dg.stride(1), beta,
                                        C.c_void_p(dQ.data_ptr()), dQ.stride(1), n_moduli,
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st


def _regular(lib, n, k, alpha, dA, dg, beta, dQ):
    import torch
    from psmma_git_gb300 import make_opts
    o = make_opts("split")
    st = lib.psmma_cauchy(n, k, alpha, C.c_void_p(dA.data_ptr()), dA.stride(1), C.c_void_p(dg.data_ptr()),
                          dg.stride(1), beta, C.c_void_p(dQ.data_ptr()), dQ.stride(1), C.byref(o),
                          C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st


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
