"""ctypes binding of libpsmma_gb300.so (the C ABI declared in include/psmma.h).

The library is loaded from the package directory.  There is no fallback: if the shared
library is missing or lacks a symbol, loading raises, so no computation can silently run
anywhere but in the CUDA kernels.
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libpsmma_gb300.so"
HEADER = PKG.parent / "include" / "psmma.h"

PSMMA_OK = 0
PSMMA_EGEN = -108
PSMMA_ENULL = -109
PSMMA_ENOMEM = -110
PSMMA_EDEVICE = -111
PSMMA_ETIMEDOUT = -112
PSMMA_ESINGULAR = -113
PSMMA_EUNSUPPORTED = -114
PSMMA_EWORKSPACE = -115
PSMMA_ERANGE = -116
PSMMA_ESCRATCH = -117

PREC_FP64 = 0
PREC_SPLIT = 1

KIND_CAUCHY, KIND_TOEPLITZ, KIND_HANKEL, KIND_DFT = 0, 1, 2, 3
KIND_CAUCHY_EIG = 5

COMPRESS_RRQR = 0
COMPRESS_RRLU = 1


class PsmmaOpts(C.Structure):
    _fields_ = [
        ("precision", C.c_int),
        ("n_moduli", C.c_int),
        ("work", C.c_void_p),
        ("lwork", C.c_size_t),
        ("block_levels", C.c_int),
        ("reserved", C.c_int * 7),
    ]


class PsmmaGrid(C.Structure):
    _fields_ = [("nprow", C.c_int), ("npcol", C.c_int), ("order", C.c_int)]


class PsmmaRequest(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("precision", C.c_int), ("n_moduli", C.c_int), ("n", C.c_int), ("k", C.c_int),
        ("alpha", C.c_double), ("beta", C.c_double),
        ("A", C.c_void_p), ("lda", C.c_int), ("gen", C.c_void_p), ("ldgen", C.c_int),
        ("Q", C.c_void_p), ("ldq", C.c_int), ("user_tag", C.c_ulonglong),
    ]


class PsmmaCompletion(C.Structure):
    _fields_ = [
        ("ticket", C.c_ulonglong), ("user_tag", C.c_ulonglong), ("status", C.c_int),
        ("submit_s", C.c_double), ("start_s", C.c_double), ("end_s", C.c_double), ("gpu_ms", C.c_float),
    ]


class PsmmaBatchItem(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("A", C.c_void_p), ("lda", C.c_int), ("gen", C.c_void_p), ("ldgen", C.c_int),
        ("Q", C.c_void_p), ("ldq", C.c_int),
    ]


class PsmmaBatchStats(C.Structure):
    _fields_ = [
        ("effective_flops", C.c_double), ("executed_flops", C.c_double), ("compress_flops", C.c_double),
        ("n_blocks", C.c_int), ("max_rank", C.c_int), ("full_rank_blocks", C.c_int), ("graph_reused", C.c_int),
    ]


class PsmmaTuneResult(C.Structure):
    _fields_ = [
        ("narrow_max", C.c_int), ("mid_max", C.c_int), ("group_m", C.c_int), ("candidates", C.c_int),
        ("ms_best", C.c_float), ("ms_default", C.c_float),
    ]


_p = C.c_void_p
_i = C.c_int
_d = C.c_double
_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)
_op = C.POINTER(PsmmaOpts)

# name -> (restype, argtypes)
SIGNATURES = {
    "psmma_cauchy": (_i, [_i, _i, _d, _p, _i, _p, _i, _d, _p, _i, _op, _p]),
    "psmma_toeplitz": (_i, [_i, _i, _d, _p, _i, _p, _i, _d, _p, _i, _op, _p]),
    "psmma_hankel": (_i, [_i, _i, _d, _p, _i, _p, _i, _d, _p, _i, _op, _p]),
    "pzmdftl": (_i, [_i, _i, _d, _p, _i, _d, _p, _i, _op, _p]),
    "pzmdftl1": (_i, [_i, _i, _d, _p, _i, _d, _p, _i, _op, _p]),
    "psmma_cauchy_split_noalloc": (_i, [_i, _i, _d, _p, _i, _p, _i, _d, _p, _i, _i, _p]),
    "psmma_cauchy_host": (_i, [_i, _i, _d, _p, _i, _p, _i, _d, _p, _i, _op]),
    "psmma_toeplitz_host": (_i, [_i, _i, _d, _p, _i, _p, _i, _d, _p, _i, _op]),
    "psmma_hankel_host": (_i, [_i, _i, _d, _p, _i, _p, _i, _d, _p, _i, _op]),
    "pzmdftl_host": (_i, [_i, _i, _d, _p, _i, _d, _p, _i, _op]),
    "psmma_cauchyeig": (_i, [_i, _i, _d, _p, _i, _p, _p, _p, _p, _p, _p, _d, _p, _i, _op, _p]),
    "psmma_cauchyeig_host": (_i, [_i, _i, _d, _p, _i, _p, _p, _p, _p, _p, _p, _d, _p, _i, _op]),
    "psmma_cauchyeig_": (None, [_ip, _ip, _ip, _dp, _p, _ip, _ip, _ip, _p, _p, _p, _p, _p, _p, _dp, _p, _ip, _ip,
                                _ip, _p, _ip]),
    "psmma_cauchy_": (None, [_ip, _ip, _dp, _p, _ip, _ip, _ip, _p, _ip, _dp, _p, _ip, _ip, _ip, _p, _ip]),
    "psmma_toeplitz_": (None, [_ip, _ip, _dp, _p, _ip, _ip, _ip, _p, _ip, _dp, _p, _ip, _ip, _ip, _p, _ip]),
    "psmma_hankel_": (None, [_ip, _ip, _dp, _p, _ip, _ip, _ip, _p, _ip, _dp, _p, _ip, _ip, _ip, _p, _ip]),
    "pzmdftl_": (None, [_ip, _ip, _ip, _ip, _dp, _p, _ip, _dp, _p, _ip, _ip, _ip, _p, _p]),
    "pzmdftl1_": (None, [_ip, _ip, _ip, _ip, _dp, _p, _ip, _dp, _p, _ip, _ip, _ip, _p, _p]),
    "psmma_last_status": (_i, []),
    "psmma_workspace_size": (C.c_size_t, [_i, _i, _i, _op]),
    "psmma_release_workspace": (None, []),
    "psmma_stream_status": (_i, [_p]),
    "psmma_stream_release": (_i, [_p]),
    "psmma_split_dft_radix": (_i, [_i]),
    "psmma_split_block_levels": (_i, [_i, _i, _i]),
    "psmma_status_string": (C.c_char_p, [_i]),
    "psmma_set_profiling": (None, [_i]),
    "psmma_profile_read": (_i, [C.POINTER(C.c_float), C.POINTER(C.c_char_p), _i]),
    "psmma_profile_read_timeline": (_i, [C.POINTER(C.c_float), C.POINTER(C.c_char_p), _i]),
    "psmma_version": (C.c_char_p, []),
    "psmma_selftest_wait_timeout": (_i, [C.c_ulonglong]),
    "psmma_selftest_division": (_i, [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_ulonglong), C.POINTER(C.c_int)]),
    "psmma_selftest_division_split": (_i, [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_ulonglong),
                                           C.POINTER(C.c_int)]),
    "psmma_server_create": (_i, [C.c_size_t, _i, C.POINTER(C.c_void_p)]),
    "psmma_server_submit": (_i, [_p, C.POINTER(PsmmaRequest), C.POINTER(C.c_ulonglong)]),
    "psmma_server_wait": (_i, [_p, C.c_ulonglong, C.c_double, C.POINTER(PsmmaCompletion)]),
    "psmma_server_pending": (_i, [_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "psmma_server_destroy": (_i, [_p]),
    "psmma_cauchy_batch_lowrank": (_i, [_i, C.POINTER(PsmmaBatchItem), _d, _d, _i, _d, _op, _ip,
                                        C.POINTER(PsmmaBatchStats), _p]),
    "psmma_batch_workspace_size": (C.c_size_t, [_i, C.POINTER(PsmmaBatchItem), _i, _op]),
    "psmma_cauchyeig_batch_lowrank": (_i, [_i, C.POINTER(PsmmaBatchItem), _d, _d, _i, _d, _op, _ip,
                                           C.POINTER(PsmmaBatchStats), _p]),
    "psmma_cauchyeig_batch_workspace_size": (C.c_size_t, [_i, C.POINTER(PsmmaBatchItem), _i, _op]),
    "psmma_toeplitz_batch_lowrank": (_i, [_i, C.POINTER(PsmmaBatchItem), _d, _d, _d, _op, _ip,
                                          C.POINTER(PsmmaBatchStats), _p]),
    "psmma_toeplitz_batch_workspace_size": (C.c_size_t, [_i, C.POINTER(PsmmaBatchItem), _op]),
    "psmma_tune_batch": (_i, [_i, C.POINTER(PsmmaBatchItem), _d, _d, _i, _d, _op, C.POINTER(PsmmaTuneResult), _p]),
    "psmma_numroc": (_i, [_i, _i, _i, _i, _i]),
    "psmma_redist_plan_create": (_i, [_i, _i, _ip, _i, _i, PsmmaGrid, _ip, _i, _i, PsmmaGrid, _i,
                                      C.POINTER(C.c_void_p)]),
    "psmma_redist_counts": (_i, [_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "psmma_redist_local_shape": (_i, [_p, _ip, _ip, _ip, _ip]),
    "psmma_redist_maps": (_i, [_p, _i, _ip, _ip]),
    "psmma_redist_pack": (_i, [_p, _p, _p, _i, _p]),
    "psmma_redist_unpack": (_i, [_p, _p, _p, _i, _p]),
    "psmma_redist_plan_destroy": (_i, [_p]),
    "psmma_redist2p5_index": (_i, [_i, _i, _i, _i, _ip]),
    "psmma_redist2p5": (_i, [_i, _i, _i, _i, _p, _i, _i, _p, _i, _p]),
    "psmma_const_index1": (_i, [_i, _i, _i, _i, _ip, _ip]),
}


def header_symbols() -> list[str]:
    """Function names declared in include/psmma.h (used by the export test)."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if n.startswith(("psmma", "pzmdft"))))


_lib = None


def load() -> C.CDLL:
    """Loads the in-tree library and binds every C-ABI symbol; raises if anything is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -m psmma_git_gb300.build` "
            "(there is no CPU fallback)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)  # AttributeError if the symbol is not exported
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def status_string(st: int) -> str:
    return load().psmma_status_string(st).decode()


class PsmmaError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__(f"{where}: status {status} ({status_string(status)})")
