"""User-supplied projection kernels for the operators.

Counterpart of gratopy's ``OpenCLKernelSpec`` (gratopy/operator/opencl.py:54-155):
an operator can run a custom kernel bundle instead of the built-in
kernels.  Here a bundle is CUDA source compiled ahead of use with nvcc for
sm_103a into a shared library (cached under a content signature, so editing
a source file triggers a rebuild), or a prebuilt shared library.  The library
exports ``{base_name}_forward`` and ``{base_name}_backward`` with the
signature of ``gr_forward`` / ``gr_backward`` in ``include/gratopy_gb300.h``::

    int f(const gr_geometry* g, void* out, const void* in, int Nz,
          int out_order, int in_order, void* stream);

returning 0 on success; the geometry descriptor carries the per-angle tables
of the operator's settings.
"""

from __future__ import annotations

import ctypes
import hashlib
import os
import shutil
import subprocess
import tempfile
from dataclasses import dataclass
from pathlib import Path

_INCLUDE = Path(__file__).resolve().parents[2] / "include"
_ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
_LOADED: dict[str, ctypes.CDLL] = {}


def kernel_cache_dir() -> Path:
    """Where compiled bundles are kept: ``$GRATOPY_GB300_KERNEL_CACHE`` or
    ``~/.cache/gratopy_gb300/kernels``."""
    env = os.environ.get("GRATOPY_GB300_KERNEL_CACHE")
    return Path(env) if env else Path.home() / ".cache" / "gratopy_gb300" / "kernels"


@dataclass(frozen=True)
class CUDAKernelSpec:
    """A custom forward/backward kernel bundle (sources or one shared library)."""

    paths: tuple[str, ...]
    base_name: str
    build_options: tuple[str, ...] = ()

    def __post_init__(self) -> None:
        if not self.paths:
            raise ValueError("a kernel spec needs at least one source or library path")
        object.__setattr__(self, "paths",
                           tuple(str(Path(p).expanduser().resolve()) for p in self.paths))
        object.__setattr__(self, "build_options", tuple(self.build_options))

    @classmethod
    def from_path(cls, path, base_name: str, build_options=()) -> "CUDAKernelSpec":
        return cls(paths=(str(path),), base_name=base_name, build_options=tuple(build_options))

    @classmethod
    def from_paths(cls, paths, base_name: str, build_options=()) -> "CUDAKernelSpec":
        return cls(paths=tuple(str(p) for p in paths), base_name=base_name,
                   build_options=tuple(build_options))

    @property
    def prebuilt(self) -> bool:
        return len(self.paths) == 1 and self.paths[0].endswith(".so")

    def read_sources(self) -> tuple[bytes, ...]:
        return tuple(Path(p).read_bytes() for p in self.paths)

    @property
    def signature(self) -> str:
        """Content signature: base name, build options, paths and file contents."""
        h = hashlib.sha256()
        h.update(self.base_name.encode())
        for opt in self.build_options:
            h.update(b"\0" + opt.encode())
        for path, src in zip(self.paths, self.read_sources()):
            h.update(b"\0" + path.encode() + b"\0" + src)
        return h.hexdigest()

    def library_path(self) -> Path:
        """The shared library, compiled (once per signature) when given sources."""
        if self.prebuilt:
            return Path(self.paths[0])
        out = kernel_cache_dir() / f"{self.base_name}-{self.signature[:24]}.so"
        if out.exists():
            return out
        nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
        out.parent.mkdir(parents=True, exist_ok=True)
        fd, tmp = tempfile.mkstemp(dir=out.parent, suffix=".so")
        os.close(fd)
        cmd = [nvcc, *_ARCH, "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
               "-I", str(_INCLUDE), *self.build_options, *self.paths, "-o", tmp]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            os.unlink(tmp)
            raise RuntimeError(f"building kernel bundle {self.base_name!r} failed:\n{res.stderr}")
        os.replace(tmp, out)
        return out

    def functions(self):
        """(forward, backward) ctypes functions of the bundle."""
        path = str(self.library_path())
        lib = _LOADED.get(path)
        if lib is None:
            lib = ctypes.CDLL(path)
            _LOADED[path] = lib
        out = []
        for suffix in ("forward", "backward"):
            name = f"{self.base_name}_{suffix}"
            try:
                fn = getattr(lib, name)
            except AttributeError as e:
                raise RuntimeError(f"kernel bundle {path} does not export {name}") from e
            fn.restype = ctypes.c_int
            fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                           ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
            out.append(fn)
        return tuple(out)
