"""Build recipe for libpsmma_gb300.so (sm_103a only).

Each CUDA translation unit under ``csrc/`` is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked into one shared
library in the package directory, so that the library that tests and benchmarks load is
the in-tree one.  ``python -m psmma_git_gb300.build`` runs it from the command line.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libpsmma_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["psmma_capi.cu", "fp64_structured.cu", "split_crt.cu", "split_noalloc.cu", "selftest.cu",
           "serving.cu", "lowrank.cu", "redist.cu"]
HEADERS = ["psmma_internal.h", "tcgen05_util.cuh"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpsmma_gb300")
    return cand


def _flags(extra: list[str] | None = None) -> list[str]:
    f = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                "--expt-relaxed-constexpr", "-I", str(PKG.parent / "include")]
    if os.environ.get("PSMMA_PTXAS_VERBOSE"):
        f += ["-Xptxas", "-v"]
    return f + (extra or [])


def _newest_dep() -> float:
    deps = [CSRC / h for h in HEADERS if (CSRC / h).exists()]
    deps.append(PKG.parent / "include" / "psmma.h")
    return max(p.stat().st_mtime for p in deps)


def _compile(src: str) -> tuple[Path, bool]:
    """(object file, whether nvcc ran): an object newer than its source and the shared
    headers is reused."""
    s = CSRC / src
    o = BUILD / (Path(src).stem + ".o")
    if o.exists() and o.stat().st_mtime >= max(s.stat().st_mtime, _newest_dep()):
        return o, False
    cmd = [nvcc(), "-c", str(s), "-o", str(o)] + _flags()
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and os.environ.get("PSMMA_PTXAS_VERBOSE"):
        sys.stderr.write(r.stderr)
    return o, True


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every CUDA source for sm_103a and link libpsmma_gb300.so; returns its path."""
    BUILD.mkdir(exist_ok=True)
    if force:
        for p in BUILD.glob("*.o"):
            p.unlink()
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        res = list(ex.map(_compile, SOURCES))
    objs = [o for o, _ in res]
    compiled = [src for src, (_, ran) in zip(SOURCES, res) if ran]
    linked = False
    if force or not LIB.exists() or LIB.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), "-shared", "-o", str(tmp)] + [str(o) for o in objs] + ARCH + ["-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
        linked = True
    if verbose:
        what = (f"compiled {len(compiled)} of {len(SOURCES)} sources ({', '.join(compiled)})" if compiled
                else "all objects up to date")
        print(f"{LIB}: {what}; {'linked' if linked else 'library up to date'}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
