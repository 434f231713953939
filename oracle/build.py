"""Build recipe for the oracle shared library (test infrastructure).

Compiles ``oracle/gr_oracle.c`` -- the plain-C restatement of gratopy's
OpenCL kernels -- into ``oracle/_build/libgr_oracle.so`` with OpenMP and
``-ffp-contract=off`` (every product and sum rounds as written).

The reference itself (pure Python + OpenCL C templates that only compile
through an OpenCL runtime, absent here) has no C sources that build with a
C compiler, so there is no ``oracle/_ref`` build.
"""

from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "gr_oracle.c"
IMPL = HERE / "gr_oracle_impl.h"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "libgr_oracle.so"


def needs_build() -> bool:
    if not LIB.exists():
        return True
    mtime = LIB.stat().st_mtime
    return any(p.stat().st_mtime > mtime for p in (SRC, IMPL, Path(__file__)))


def build(force: bool = False) -> Path:
    if not force and not needs_build():
        return LIB
    OUT_DIR.mkdir(exist_ok=True)
    tmp = OUT_DIR / f"libgr_oracle.{os.getpid()}.so"
    cmd = [
        os.environ.get("CC", "gcc"),
        "-O2",
        "-fopenmp",
        "-ffp-contract=off",
        "-fPIC",
        "-shared",
        "-Wall",
        "-o",
        str(tmp),
        str(SRC),
        "-lm",
    ]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
