"""CPU tests of the C ABI: the library builds, loads, exports every declared symbol, and
its argument checks return the reference's INFO numbers (no GPU work is launched)."""
import ctypes as C

import numpy as np

from psmma_git_gb300 import _lib


def test_library_exports_every_header_symbol(lib):
    names = _lib.header_symbols()
    assert "psmma_cauchy" in names and "pzmdftl1_" in names and len(names) >= 19
    for name in names:
        assert hasattr(lib, name), f"libpsmma_gb300.so does not export {name}"
    assert set(names) <= set(_lib.SIGNATURES), "binding table out of date"
    assert lib.psmma_version().startswith(b"psmma-gb300")


def _call_real(lib, name, n, k, lda, ldgen, ldq, gen=True, alpha=1.0, beta=0.0):
    buf = np.zeros(16)
    p = C.c_void_p(buf.ctypes.data)
    return getattr(lib, name)(n, k, alpha, p, lda, p if gen else None, ldgen, beta, p, ldq, None, None)


def test_argument_checks_use_reference_info_numbers(lib):
    # PSCAUCHY_COMPUTE: N<0 -> 2, K<0 -> 3, LDA -> 9, LDC -> 14 (pscauchy_compute.f90:234-255)
    for name in ["psmma_cauchy", "psmma_toeplitz", "psmma_hankel"]:
        assert _call_real(lib, name, -1, 4, 4, 8, 4) == -2
        assert _call_real(lib, name, 4, -1, 4, 8, 4) == -3
        assert _call_real(lib, name, 4, 4, 3, 8, 4) == -9
        assert _call_real(lib, name, 4, 4, 4, 8, 3) == -14
        assert _call_real(lib, name, 4, 4, 4, 8, 4, gen=False) == _lib.PSMMA_EGEN
    assert _call_real(lib, "psmma_cauchy", 4, 4, 4, 3, 4) == _lib.PSMMA_EGEN     # ldgen < k
    assert _call_real(lib, "psmma_toeplitz", 4, 4, 4, 6, 4) == _lib.PSMMA_EGEN   # < 2k-1
    # quick returns touch nothing (N == 0; alpha == 0 and beta == 1)
    assert _call_real(lib, "psmma_cauchy", 0, 4, 1, 4, 1) == 0
    assert _call_real(lib, "psmma_cauchy", 4, 4, 4, 4, 4, alpha=0.0, beta=1.0) == 0
    # PZMDFTL: N<0 -> 1, K<0 -> 2, LDB -> 7, LDC -> 10 (pzmdftL.f90:182-205)
    buf = np.zeros(16)
    p = C.c_void_p(buf.ctypes.data)
    assert lib.pzmdftl(-1, 2, 1.0, p, 2, 0.0, p, 2, None, None) == -1
    assert lib.pzmdftl(2, -1, 1.0, p, 2, 0.0, p, 2, None, None) == -2
    assert lib.pzmdftl(4, 2, 1.0, p, 3, 0.0, p, 4, None, None) == -7
    assert lib.pzmdftl(4, 2, 1.0, p, 4, 0.0, p, 3, None, None) == -10
    assert lib.pzmdftl_host(0, 2, 1.0, p, 1, 0.0, p, 1, None) == 0


def test_options_are_validated(lib):
    buf = np.zeros(16)
    p = C.c_void_p(buf.ctypes.data)
    o = _lib.PsmmaOpts()
    o.precision = 7
    assert lib.psmma_cauchy(2, 2, 1.0, p, 2, p, 2, 0.0, p, 2, C.byref(o), None) == _lib.PSMMA_EUNSUPPORTED
    o.precision = _lib.PREC_SPLIT
    o.n_moduli = 30
    assert lib.pzmdftl(2, 2, 1.0, p, 2, 0.0, p, 2, C.byref(o), None) == _lib.PSMMA_EUNSUPPORTED
    o.n_moduli = 0
    o.precision = 0
    o.reserved[3] = 1
    assert lib.psmma_hankel(2, 2, 1.0, p, 2, p, 3, 0.0, p, 2, C.byref(o), None) == _lib.PSMMA_EUNSUPPORTED
    o.reserved[3] = 0
    for bad in (-2, 4):
        o.block_levels = bad
        assert lib.psmma_toeplitz(2, 2, 1.0, p, 2, p, 3, 0.0, p, 2, C.byref(o), None) == _lib.PSMMA_EUNSUPPORTED


def test_fortran_abi_argument_check(lib):
    # PSMMA_CAUCHY(N,K,ALPHA,A,IA,JA,DESCA,B,LDB,BETA,Q,IQ,JQ,DESCQ,WORK,REDIST) with N < 0
    i = lambda v: C.byref(C.c_int(v))
    d = lambda v: C.byref(C.c_double(v))
    desc = (C.c_int * 9)(1, 0, 4, 4, 4, 4, 0, 0, 4)
    buf = np.zeros(16)
    p = C.c_void_p(buf.ctypes.data)
    lib.psmma_cauchy_(i(-1), i(4), d(1.0), p, i(1), i(1), desc, p, i(4), d(0.0), p, i(1), i(1), desc, p, i(0))
    assert lib.psmma_last_status() == -2
    lib.pzmdftl_(i(4), i(4), i(2), i(2), d(1.0), p, i(3), d(0.0), p, i(4), i(0), i(0), p, p)
    assert lib.psmma_last_status() == -7


def test_status_strings(lib):
    for st in [0, -2, -3, -9, -14, _lib.PSMMA_EGEN, _lib.PSMMA_ETIMEDOUT, _lib.PSMMA_ESINGULAR]:
        assert _lib.status_string(st) != "unknown status"


def test_workspace_size_queries(lib):
    from psmma_git_gb300 import workspace_size
    # FP64 path: nothing once the output fills the SMs; small products may take split-K partials
    assert workspace_size(_lib.KIND_CAUCHY, 16384, 16384) == 0
    w = workspace_size(_lib.KIND_CAUCHY, 1024, 1024)
    assert w == 0 or w % (1024 * 1024 * 8) == 0
    assert workspace_size(_lib.KIND_DFT, 1000, 10) >= 1000 * 16


def test_split_block_levels_rule(lib):
    # the Toeplitz / Hankel block step chosen automatically: the L in {1, 2} with leaves of at
    # least 4096 columns (k padded to a multiple of 64 * 2^L) that minimises (k'/k)^2 (3/4)^L,
    # if at most 0.85; other kinds never take it (host logic only, no GPU work)
    ks = [1024, 2048, 4096, 6144, 8192, 8256, 12288, 16384, 24576, 32768, 0]
    for kind in (_lib.KIND_TOEPLITZ, _lib.KIND_HANKEL):
        assert [lib.psmma_split_block_levels(kind, 100, k) for k in ks] == [0, 0, 0, 0, 1, 1, 1, 2, 2, 2, 0]
        # padded: 8100 -> 8192 at L = 1; 16000 stays at L = 1 (padded to 16128, L = 2's leaves would
        # have 4032 columns); 16129 -> 16384 at L = 2 (0.58 of the work, below L = 1's 0.76)
        assert [lib.psmma_split_block_levels(kind, 100, k) for k in (8000, 8100, 16000, 16129)] == [0, 1, 1, 2]
    for kind in (_lib.KIND_CAUCHY, _lib.KIND_DFT):
        assert [lib.psmma_split_block_levels(kind, 100, k) for k in ks] == [0] * len(ks)
    # Cauchy (and CAUCHYEIG): Strassen's step only on request, never automatically
    assert [lib.psmma_split_block_levels(_lib.KIND_CAUCHY, k, k) for k in ks] == [0] * len(ks)
    assert lib.psmma_split_block_levels(5, 4096, 8192) == 0
    # the workspace covers the block step's operands and the single product's, for the
    # automatic choice and for levels asked for by opts->block_levels
    from psmma_git_gb300 import workspace_size
    for k, lv in ((8192, 0), (16384, 0), (2048, 2), (1536, 3), (4096, -1)):
        plain = workspace_size(_lib.KIND_TOEPLITZ, 4096, k, precision="split", block_levels=-1)
        assert workspace_size(_lib.KIND_TOEPLITZ, 4096, k, precision="split", block_levels=lv) >= plain
    assert workspace_size(_lib.KIND_HANKEL, 4096, 2048, precision="split", block_levels=2) > \
        workspace_size(_lib.KIND_HANKEL, 4096, 2048, precision="split", block_levels=-1)
    assert workspace_size(_lib.KIND_CAUCHY, 4096, 2048, precision="split", block_levels=1) > \
        workspace_size(_lib.KIND_CAUCHY, 4096, 2048, precision="split", block_levels=-1)


def test_fortran_module_binds_declared_and_exported_symbols(lib):
    # include/psmma_gb300.f90 (not compiled here: no Fortran compiler on either host) must name
    # only functions that psmma.h declares and the library exports, keep free-form lines within
    # 132 characters, close every interface body it opens, and give its bind(c) types the C
    # structs' fields in the same order
    import re
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    f90 = (root / "include" / "psmma_gb300.f90").read_text()
    header = (root / "include" / "psmma.h").read_text()
    code = "\n".join(line.split("!")[0] for line in f90.splitlines())
    assert all(len(line) <= 132 for line in f90.splitlines())
    names = re.findall(r'bind\(c,\s*name="([a-z0-9_]+)"\)', code)
    assert len(names) >= 29 and len(set(names)) == len(names)
    declared = set(_lib.header_symbols())
    for name in names:
        assert name in declared, f"{name} is not declared in psmma.h"
        assert hasattr(lib, name), f"{name} is not exported"
    opened = re.findall(r"^\s*(?:integer\(c_\w+\)\s+|type\(c_ptr\)\s+)?(function|subroutine)\s+(\w+)\s*\(", code,
                        flags=re.M)
    closed = re.findall(r"^\s*end\s+(function|subroutine)\s+(\w+)", code, flags=re.M)
    assert sorted(opened) == sorted(closed) and len(opened) == len(names)
    assert code.count("module psmma_gb300") == 2 and "end module psmma_gb300" in code
    for ctype in ["psmma_opts", "psmma_batch_item", "psmma_batch_stats", "psmma_tune_result", "psmma_grid"]:
        fbody = re.search(r"type, bind\(c\), public :: " + ctype + r"\n(.*?)end type " + ctype, code, flags=re.S)
        cbody = re.search(r"typedef struct " + ctype + r" \{(.*?)\} " + ctype + ";",
                          re.sub(r"/\*.*?\*/", "", header, flags=re.S), flags=re.S)
        assert fbody and cbody, ctype
        ffields = re.findall(r"([a-z_][a-z0-9_]*)(?:\(\d+\))?\s*(?:=\s*[^,\n]+)?(?=,|\n)",
                             "".join(ln.split("::")[1] + "\n" for ln in fbody.group(1).splitlines() if "::" in ln))
        cfields = re.findall(r"\b([a-z_][a-z0-9_]*)\s*(?:\[\d+\])?\s*[,;]", cbody.group(1))
        assert ffields == cfields, (ctype, ffields, cfields)
