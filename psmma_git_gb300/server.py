"""Python handle on the library's serving loop (psmma_server_* in include/psmma.h).

    with Server(hbm_budget_bytes=8 << 30, max_inflight=4) as srv:
        t = srv.submit("cauchy", n, k, 1.0, A, gen, 0.0, Q, precision="split")
        info = srv.wait(t)          # {'status', 'latency_s', 'queue_s', 'gpu_ms', ...}

Operands are column-major CUDA tensors (see fortran_empty); they must stay alive and Q must
not be touched until the request completes.  Kinds: cauchy, toeplitz, hankel, dft,
cauchyeig (PSMMA_CAUCHYEIG's matrix; gen is n x 5 [F|U|V|DIFL|DIFR]).
"""
from __future__ import annotations

import ctypes as C

from ._lib import (KIND_CAUCHY, KIND_CAUCHY_EIG, KIND_DFT, KIND_HANKEL, KIND_TOEPLITZ, PREC_FP64, PREC_SPLIT,
                   PsmmaCompletion, PsmmaError, PsmmaRequest, load)

KINDS = {"cauchy": KIND_CAUCHY, "toeplitz": KIND_TOEPLITZ, "hankel": KIND_HANKEL, "dft": KIND_DFT,
         "cauchyeig": KIND_CAUCHY_EIG}  # cauchyeig: gen is n x 5 [F|U|V|DIFL|DIFR]
PRECS = {"fp64": PREC_FP64, "split": PREC_SPLIT}


def _ptr_ld(t):
    if t is None:
        return 0, 1
    if t.dim() == 1:
        return t.data_ptr(), t.numel()
    return t.data_ptr(), (t.stride(1) if t.shape[1] > 1 else max(t.shape[0], 1))


class Server:
    def __init__(self, hbm_budget_bytes: int, max_inflight: int = 4):
        self.lib = load()
        h = C.c_void_p()
        st = self.lib.psmma_server_create(hbm_budget_bytes, max_inflight, C.byref(h))
        if st != 0:
            raise PsmmaError(st, "psmma_server_create")
        self.h = h
        self._keep = {}

    def submit(self, kind, n, k, alpha, A, gen, beta, Q, *, precision="split", n_moduli=0, tag=0) -> int:
        r = PsmmaRequest()
        r.kind = KINDS[kind]
        r.precision = PRECS[precision]
        r.n_moduli = n_moduli
        r.n, r.k = n, k
        r.alpha, r.beta = float(alpha), float(beta)
        r.A, r.lda = _ptr_ld(A)
        if gen is not None and kind == "cauchy" and gen.dim() == 1:
            r.gen, r.ldgen = gen.data_ptr(), gen.numel() // 4
        else:
            r.gen, r.ldgen = _ptr_ld(gen) if gen is not None else (0, 0)
        r.Q, r.ldq = _ptr_ld(Q)
        r.user_tag = tag
        t = C.c_ulonglong()
        st = self.lib.psmma_server_submit(self.h, C.byref(r), C.byref(t))
        if st != 0:
            raise PsmmaError(st, "psmma_server_submit")
        self._keep[t.value] = (A, gen, Q)
        return t.value

    def wait(self, ticket: int, timeout_s: float = 600.0) -> dict:
        c = PsmmaCompletion()
        st = self.lib.psmma_server_wait(self.h, ticket, timeout_s, C.byref(c))
        if st == -112 and c.ticket == 0:
            raise TimeoutError(f"ticket {ticket} not complete after {timeout_s} s")
        self._keep.pop(ticket, None)
        return {"ticket": c.ticket, "tag": c.user_tag, "status": c.status, "latency_s": c.end_s - c.submit_s,
                "queue_s": c.start_s - c.submit_s, "submit_s": c.submit_s, "end_s": c.end_s, "gpu_ms": c.gpu_ms}

    def pending(self):
        q, f = C.c_int(), C.c_int()
        self.lib.psmma_server_pending(self.h, C.byref(q), C.byref(f))
        return q.value, f.value

    def close(self):
        if self.h:
            self.lib.psmma_server_destroy(self.h)
            self.h = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
