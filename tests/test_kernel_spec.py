"""Custom kernel bundles for the operators (gratopy's OpenCLKernelSpec,
operator/opencl.py:54-155): content signature, nvcc build and symbol lookup
on CPU; an operator running a bundle on the GPU."""

from __future__ import annotations

import numpy as np
import pytest

SOURCE = r"""
#include <cuda_runtime.h>
#include "gratopy_gb300.h"

// test bundle: the forward fills the output with 1 + Nz, the backward with -1
__global__ void fill(float* out, long long n, float v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) out[i] = v;
}

extern "C" int mybundle_forward(const gr_geometry* g, void* out, const void*, int Nz, int, int,
                                void* stream) {
  fill<<<64, 256, 0, (cudaStream_t)stream>>>((float*)out, (long long)g->Ns * g->Na * Nz,
                                             1.0f + (float)Nz);
  return cudaGetLastError() == cudaSuccess ? 0 : 3;
}

extern "C" int mybundle_backward(const gr_geometry* g, void* out, const void*, int Nz, int, int,
                                 void* stream) {
  fill<<<64, 256, 0, (cudaStream_t)stream>>>((float*)out, (long long)g->Nx * g->Ny * Nz, -1.0f);
  return cudaGetLastError() == cudaSuccess ? 0 : 3;
}
"""


@pytest.fixture
def bundle(tmp_path, monkeypatch):
    monkeypatch.setenv("GRATOPY_GB300_KERNEL_CACHE", str(tmp_path / "cache"))
    src = tmp_path / "mybundle.cu"
    src.write_text(SOURCE)
    return src


def test_signature_follows_content_and_options(bundle):
    from gratopy_gb300.operator import CUDAKernelSpec

    a = CUDAKernelSpec.from_path(bundle, "mybundle")
    b = CUDAKernelSpec.from_path(bundle, "mybundle", build_options=("-DX=1",))
    assert a.signature != b.signature
    sig = a.signature
    bundle.write_text(SOURCE + "\n// edited\n")
    assert CUDAKernelSpec.from_path(bundle, "mybundle").signature != sig
    with pytest.raises(ValueError):
        CUDAKernelSpec(paths=(), base_name="x")


def test_bundle_builds_and_exports_both_entry_points(bundle):
    from gratopy_gb300.operator import CUDAKernelSpec

    spec = CUDAKernelSpec.from_path(bundle, "mybundle")
    path = spec.library_path()
    assert path.exists() and path.suffix == ".so"
    assert spec.library_path() == path  # cached by signature
    fwd, bwd = spec.functions()
    assert fwd is not None and bwd is not None
    prebuilt = CUDAKernelSpec.from_path(path, "mybundle")
    assert prebuilt.prebuilt and prebuilt.library_path() == path
    with pytest.raises(RuntimeError, match="does not export"):
        CUDAKernelSpec.from_path(path, "other").functions()


def test_operator_rejects_other_spec_types():
    from gratopy_gb300.operator import Radon

    with pytest.raises(TypeError):
        Radon(16, 10, kernel_spec="radon.cl")


@pytest.mark.gpu
def test_operator_runs_the_bundle(cuda_device, bundle):
    import torch

    from gratopy_gb300.operator import CUDAKernelSpec, Radon

    spec = CUDAKernelSpec.from_path(bundle, "mybundle")
    R = Radon(image_domain=24, angles=12, detectors=30, kernel_spec=spec)
    x = torch.rand(24, 24, device=cuda_device)
    y = R.apply_to(x)
    assert tuple(y.shape) == (30, 12) and bool((y == 2.0).all())
    y3 = R.apply_to(torch.rand(24, 24, 3, device=cuda_device))
    assert bool((y3 == 4.0).all())
    z = R.T.apply_to(y)
    assert tuple(z.shape) == (24, 24) and bool((z == -1.0).all())
    assert bool(((2.0 * R).apply_to(x) == 4.0).all())
