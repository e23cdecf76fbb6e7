"""Builds the oracle's C restatement into oracle/_build/liboracle.so.

Test infrastructure: only tests/, the smoke check and bench.py's CPU
baseline use the result.  The reference itself is not built: its one-rank
path needs MPI, ScaLAPACK/BLACS and the COSTA / Tiled-MM sources, none of
which exist in this environment (the two libraries are fetched at configure
time by the reference's CMake).
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "oracle.c"
OUT = HERE / "_build" / "liboracle.so"


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


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
