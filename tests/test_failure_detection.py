"""Failure detection without a GPU fault: a device-side wait that nothing releases must
expire after its limit and come back as PSMMA_ETIMEDOUT, leaving the context usable."""
import ctypes as C
import time

import numpy as np
import pytest

from oracle import psmma_oracle as O

pytestmark = pytest.mark.gpu


def test_bounded_wait_expires_and_context_survives(lib, cuda):
    import torch
    from psmma_git_gb300 import _lib
    import psmma_git_gb300 as P
    t0 = time.perf_counter()
    st = lib.psmma_selftest_wait_timeout(50_000_000)  # 50 ms
    dt = time.perf_counter() - t0
    assert st == _lib.PSMMA_ETIMEDOUT
    assert 0.04 < dt < 5.0
    # the context still works: a split multiply afterwards is correct
    n = k = 128
    A = O.cfg_matrix(n, k, seed=1)
    gen = O.cfg_cauchy_generators(k, seed=2)
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).to(cuda).t()
    dg = torch.from_numpy(np.ascontiguousarray(gen.T)).to(cuda).t()
    dQ = P.fortran_empty(n, k, torch.float64, cuda)
    P.psmma_cauchy(n, k, 1.0, dA, dg, 0.0, dQ, precision="split")
    torch.cuda.synchronize()
    got = dQ.t().contiguous().cpu().numpy().T
    assert O.rel_fro(got, O.dense_product("cauchy", 1.0, A, gen, 0.0, None, k)) < 1e-12


@pytest.mark.gpu
def test_fast_division_matches_ieee_within_one_ulp(lib, cuda):
    import ctypes as C
    mism, ulp = C.c_ulonglong(0), C.c_int(0)
    assert lib.psmma_selftest_division(1 << 26, 12345, C.byref(mism), C.byref(ulp)) == 0
    # correctly rounded in all but rare ties; never more than one ulp away
    assert ulp.value <= 1
    assert mism.value < (1 << 26) // 10000


@pytest.mark.gpu
def test_split_path_division_error_bound(lib, cuda):
    import ctypes as C
    mism, ulp = C.c_ulonglong(0), C.c_int(0)
    assert lib.psmma_selftest_division_split(1 << 26, 777, C.byref(mism), C.byref(ulp)) == 0
    # double-float entries on the FP32 pipe (an FP32-seeded FP64 Newton division for operands
    # outside their range): within 2^-44 relative
    assert ulp.value <= 256


@pytest.mark.gpu
def test_split_calls_report_device_status_per_stream(lib, cuda):
    # device-pointer split calls enqueue and return; their device status joins the stream's word,
    # which psmma_stream_status reads (clean after good calls) on that stream only
    import torch
    import psmma_git_gb300 as P
    n = k = 512
    A = O.cfg_matrix(n, k, seed=61)
    gen = O.cfg_cauchy_generators(k, seed=62)
    col = lambda x: torch.from_numpy(np.ascontiguousarray(np.asarray(x).T)).to(cuda).t()  # noqa: E731
    s = torch.cuda.Stream()
    dA, dg = col(A), col(gen)
    torch.cuda.synchronize()
    outs = []
    with torch.cuda.stream(s):
        for _ in range(3):
            dQ = P.fortran_empty(n, k, torch.float64, cuda)
            P.psmma_cauchy(n, k, 1.0, dA, dg, 0.0, dQ, precision="split", stream=s)
            outs.append(dQ)
    P.stream_status(s)  # waits; raises on a recorded timeout
    assert lib.psmma_stream_status(C.c_void_p(s.cuda_stream)) == 0
    ref = O.dense_product("cauchy", 1.0, A, gen, 0.0, None, k)
    for dQ in outs:
        assert O.rel_fro(dQ.cpu().numpy(), ref) < 1e-12
    # releasing the stream's record before the stream goes away; a later call makes a new one
    assert lib.psmma_stream_release(C.c_void_p(s.cuda_stream)) == 0
    assert lib.psmma_stream_release(C.c_void_p(s.cuda_stream)) == 0  # nothing left: waits only
    dQ = P.fortran_empty(n, k, torch.float64, cuda)
    with torch.cuda.stream(s):
        P.psmma_cauchy(n, k, 1.0, dA, dg, 0.0, dQ, precision="split", stream=s)
    P.stream_status(s)
    assert O.rel_fro(dQ.cpu().numpy(), ref) < 1e-12
    assert lib.psmma_stream_release(C.c_void_p(s.cuda_stream)) == 0
