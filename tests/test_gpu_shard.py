"""Sharded solvers' GPU backends on one rank equal the per-call solvers bit for bit."""

from __future__ import annotations

import numpy as np
import pytest

from tests.helpers import device_settings

pytestmark = pytest.mark.gpu

CFG = dict(geometry="fanbeam", img_shape=(40, 40), angles=36, n_detectors=64, detector_width=40.0,
           R=70.0, RE=30.0)


def _stack(device, ps, nz):
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300.phantom import random_ellipse_volume

    vol = random_ellipse_volume(device, ps.img_shape, nz, seed=5)
    sino = gg.forwardprojection(vol, ps)
    gen = torch.Generator(device=device).manual_seed(1)
    return sino + 0.01 * torch.rand(sino.shape, generator=gen, device=device)


@pytest.mark.parametrize("nz", [1, 6])
def test_kernel_cg_one_rank_equals_conjugate_gradients(cuda_device, nz):
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import shard

    ps = device_settings(CFG, cuda_device)
    sino = _stack(cuda_device, ps, nz)
    a = shard.conjugate_gradients_sharded(sino, ps, 12)
    b = gg.conjugate_gradients(sino, ps, 12)
    assert torch.equal(a, b)
    c = shard.conjugate_gradients_sharded(sino, ps, 40, epsilon=0.05)
    d = gg.conjugate_gradients(sino, ps, 40, epsilon=0.05)
    assert torch.equal(c, d)


def test_kernel_tv_one_rank_equals_total_variation(cuda_device):
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import shard

    ps = device_settings(CFG, cuda_device)
    sino = _stack(cuda_device, ps, 6)
    nrm = gg.normest(ps, 20, x0=np.ones(ps.img_shape))
    a = shard.total_variation_sharded(sino, ps, 10.0, 15, slice_thickness=1.0, norm_estimate=nrm)
    b = gg.total_variation(sino, ps, 10.0, 15, slice_thickness=1.0, norm_estimate=nrm)
    assert torch.equal(a, b)


def test_batch_sharded_one_rank_solves_everything(cuda_device):
    import torch

    from gratopy_gb300 import batch as gb
    from gratopy_gb300 import shard

    def problems():
        return gb.heterogeneous_problems(5, seed=4, device=cuda_device, landweber_iterations=4,
                                         cg_iterations=3, tv_iterations=4, sizes=(32, 48),
                                         angle_range=(20, 40))

    a = shard.batch_sharded(problems(), cuda_device, normest_iterations=5)
    b = gb.BatchedReconstruction(problems(), cuda_device, normest_iterations=5).run()
    assert sorted(a) == list(range(5))
    for k in range(5):
        assert torch.equal(a[k], b[k])
