"""Device ellipse rasteriser against the host rasteriser (bit for bit)."""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order", ["F", "C"])
@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_device_volume_equals_host_slices(cuda_device, order, dtype):
    from gratopy_gb300.phantom import random_ellipse_image, random_ellipse_volume

    Nx, Ny, nz = 67, 45, 3
    vol = random_ellipse_volume(cuda_device, (Nx, Ny), nz, seed=11, count=7, dtype=dtype,
                                order=order)
    assert tuple(vol.shape) == (Nx, Ny, nz)
    got = vol.cpu().numpy()
    for k in range(nz):
        want = random_ellipse_image(11 + k, (Ny, Nx), count=7, dtype=dtype).T
        assert np.array_equal(got[:, :, k], want)


def test_device_single_slice_and_degenerate_grid(cuda_device):
    from gratopy_gb300.phantom import random_ellipse_image, random_ellipse_volume

    img = random_ellipse_volume(cuda_device, 128, 1, seed=3)
    assert np.array_equal(img.cpu().numpy(), random_ellipse_image(3, 128).T)
    one = random_ellipse_volume(cuda_device, (1, 5), 1, seed=4, count=3)
    assert np.array_equal(one.cpu().numpy(), random_ellipse_image(4, (5, 1), count=3).T)
