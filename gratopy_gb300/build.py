"""Build recipe for the CUDA extension ``libgratopy_gb300.so`` (sm_103a).

Compiles every ``csrc/*.cu`` translation unit in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and links
them into ``gratopy_gb300/_build/libgratopy_gb300.so`` (in-tree, git-ignored).
The library exports the C ABI declared in ``include/gratopy_gb300.h``.
"""

from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
OUT_DIR = PKG / "_build"
LIB = OUT_DIR / "libgratopy_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-fvisibility=hidden",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gratopy_gb300")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _deps() -> list[Path]:
    return sources() + sorted(CSRC.glob("*.cuh")) + [INCLUDE / "gratopy_gb300.h", Path(__file__)]


def source_hash() -> str:
    """Hex SHA-256 over the names and contents of every input of the build;
    compiled into the library (``gr_source_hash``) and compared at load."""
    h = hashlib.sha256()
    for p in _deps():
        h.update(p.name.encode() + b"\0" + p.read_bytes() + b"\0")
    return h.hexdigest()


def _built_hash() -> str | None:
    """``gr_source_hash`` of the library on disk, read in a subprocess so
    this process does not keep an outdated library mapped."""
    if not LIB.exists():
        return None
    code = ("import ctypes,sys; f=ctypes.CDLL(sys.argv[1]).gr_source_hash; "
            "f.restype=ctypes.c_char_p; print(f().decode())")
    res = subprocess.run([sys.executable, "-c", code, str(LIB)], capture_output=True, text=True)
    return res.stdout.strip() if res.returncode == 0 else None


def needs_build() -> bool:
    return _built_hash() != source_hash()


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    if not force and not needs_build():
        return LIB
    OUT_DIR.mkdir(exist_ok=True)
    cc = nvcc()
    flags = NVCC_FLAGS + [f'-DGR_SOURCE_HASH="{source_hash()}"'] + (extra_flags or [])

    def compile_one(src: Path) -> Path:
        obj = OUT_DIR / (src.stem + ".o")
        cmd = [cc, *ARCH, *flags, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
        if verbose and (res.stdout or res.stderr):
            print(res.stdout + res.stderr, flush=True)
        return obj

    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = OUT_DIR / f"libgratopy_gb300.{os.getpid()}.so"
    cmd = [cc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
