"""Builds the oracle's C restatement into oracle/_build/liboracle.so, and,
where the reference's sources are present, three of the reference's own
files into oracle/_ref/libcosma_ref.so.

Test infrastructure: only tests/, the smoke check and bench.py's CPU
baseline use the results.  The reference as a whole is not built: its
one-rank path needs MPI, ScaLAPACK/BLACS and the COSTA / Tiled-MM sources,
none of which exist in this environment (the two libraries are fetched at
configure time by the reference's CMake).  What compiles on its own is its
CPU arithmetic: src/cosma/local_multiply.cpp (the naive local_multiply_cpu
loop and the CPU build's local_multiply -> cosma::gemm), src/cosma/blas.cpp
(cosma::gemm over CBLAS) and src/cosma/scalapack.cpp (numroc).  build_ref
compiles those files where they lie, with the stand-in headers of
oracle/ref_stubs/ for the missing dependencies and oracle/ref_shim.cpp for
C entry points and a CBLAS on top of scipy's OpenBLAS.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "oracle.c"
OUT = HERE / "_build" / "liboracle.so"
REF_ROOT = Path(os.environ.get("COSMA_REFERENCE_ROOT", "/root/reference"))
REF_FILES = ("src/cosma/local_multiply.cpp", "src/cosma/blas.cpp", "src/cosma/scalapack.cpp")
REF_OUT = HERE / "_ref" / "libcosma_ref.so"


def build(force: bool = False) -> Path:
    if not force and OUT.exists() and OUT.stat().st_mtime >= SRC.stat().st_mtime:
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler found for the oracle")
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [cc, "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11", str(SRC), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    tmp.replace(OUT)
    return OUT


def reference_available() -> bool:
    return all((REF_ROOT / f).exists() for f in REF_FILES)


def build_ref(force: bool = False) -> Path | None:
    """Compiles the reference's CPU files into oracle/_ref/libcosma_ref.so;
    None when the reference's sources are not present."""
    if not reference_available():
        return REF_OUT if REF_OUT.exists() else None
    deps = [REF_ROOT / f for f in REF_FILES] + [HERE / "ref_shim.cpp"] + list((HERE / "ref_stubs").rglob("*"))
    if not force and REF_OUT.exists() and all(REF_OUT.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return REF_OUT
    REF_OUT.parent.mkdir(exist_ok=True)
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("no C++ compiler found for the reference build")
    tmp = REF_OUT.with_suffix(".so.tmp")
    cmd = [cxx, "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17", "-DCOSMA_WITH_BLAS",
           f"-I{HERE / 'ref_stubs'}", f"-I{REF_ROOT / 'src'}",
           *[str(REF_ROOT / f) for f in REF_FILES], str(HERE / "ref_shim.cpp"), "-o", str(tmp), "-ldl"]
    subprocess.run(cmd, check=True)
    tmp.replace(REF_OUT)
    return REF_OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
