"""Sparse matrix of the forward projection (tests/test_radon.py:715-796 and
tests/test_fanbeam.py:1489-1580 of gratopy): matrix-vector products with a
phantom reproduce the reference's control numbers, and equal the projection
kernels."""

from __future__ import annotations

import numpy as np
import pytest

from tests.golden import configs
from tests.helpers import assert_control, device_settings, rel_l2

pytestmark = pytest.mark.gpu

GOLDEN = {"radon_sparse": (6.5315, 1.03955), "fan_sparse": (233.96, 2690.00)}


@pytest.mark.parametrize("name", sorted(GOLDEN))
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_sparse_matrix_control_numbers(cuda_device, name, dtype):
    import gratopy_gb300 as gg

    ps = device_settings(configs.configs()[name], cuda_device)
    Nx, Ny = ps.img_shape
    Ns, Na = ps.sinogram_shape
    M = ps.create_sparse_matrix(dtype=dtype, order="F")
    assert M.shape == (Ns * Na, Nx * Ny)
    assert M.nnz <= 2 * Nx * Ny * Na and (M.data > 0).all()
    img = gg.phantom(cuda_device, Nx, dtype=np.dtype(dtype)).cpu().numpy()
    flat = img.reshape(Nx * Ny, order="F")
    sino = (M @ flat).reshape(Ns, Na, order="F")
    back = (M.T @ sino.reshape(Ns * Na, order="F")).reshape(Nx, Ny, order="F")
    dims = (Nx, Ny, Ns, Na, 1)
    assert_control(img, dims, 7.1182, "img", "original image")
    assert_control(sino, dims, GOLDEN[name][0], "sino", "sinogram")
    assert_control(back, dims, GOLDEN[name][1], "img", "backprojected image")


@pytest.mark.parametrize("name", sorted(GOLDEN))
@pytest.mark.parametrize("dtype,tol", [(np.float32, 1e-5), (np.float64, 1e-12)])
@pytest.mark.parametrize("order", ["F", "C"])
def test_sparse_matrix_equals_projection(cuda_device, name, dtype, tol, order):
    import torch

    import gratopy_gb300 as gg

    ps = device_settings(configs.configs()[name], cuda_device)
    Nx, Ny = ps.img_shape
    Ns, Na = ps.sinogram_shape
    M = ps.create_sparse_matrix(dtype=dtype, order=order)
    img = np.random.default_rng(3).random((Nx, Ny)).astype(dtype)
    img_d = gg.core.empty((Nx, Ny), torch.float32 if dtype == np.float32 else torch.float64,
                          order, cuda_device)
    img_d.copy_(torch.from_numpy(img))
    want = gg.forwardprojection(img_d, ps).cpu().numpy()
    got = (M @ img.reshape(-1, order=order)).reshape(Ns, Na, order=order)
    assert rel_l2(got, want) < tol
