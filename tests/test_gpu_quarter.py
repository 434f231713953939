"""Quarter-turn shared forward projection (float32 fan beam, single slices)
against the oracle, the per-angle kernel, and through the fused solver
epilogues."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import device_settings, host_settings, rel_l2

pytestmark = pytest.mark.gpu

CFGS = {
    "plain": dict(geometry="fanbeam", img_shape=(40, 40), angles=36, n_detectors=64,
                  detector_width=40.0, R=70.0, RE=30.0),
    "odd_side_reversed": dict(geometry="fanbeam", img_shape=(37, 37), angles=20, n_detectors=50,
                              detector_width=40.0, R=70.0, RE=30.0, reverse_detector=True),
    "shifted_detector": dict(geometry="fanbeam", img_shape=(64, 64), angles=48, n_detectors=90,
                             detector_width=60.0, R=150.0, RE=60.0, detector_shift=4.0),
    "one_pixel": dict(geometry="fanbeam", img_shape=(1, 1), angles=4, n_detectors=3,
                      detector_width=4.0, R=10.0, RE=5.0),
    "bench_like": dict(geometry="fanbeam", img_shape=(128, 128), angles=360, n_detectors=192,
                       detector_width=400.0, R=400.0, RE=200.0),
}


def _forward(ps, img_np, order, sym, cuda_device):
    import torch

    import gratopy_gb300 as gg

    g = ps.gr_geometry(np.float32)
    saved = g.sym
    g.sym = sym
    try:
        x = gg.core.empty(ps.img_shape, torch.float32, order, cuda_device)
        x.copy_(torch.from_numpy(img_np.astype(np.float32)))
        return gg.forwardprojection(x, ps).double().cpu().numpy()
    finally:
        g.sym = saved


@pytest.mark.parametrize("name", sorted(CFGS))
@pytest.mark.parametrize("order", ["F", "C"])
def test_quarter_forward(cuda_device, name, order):
    ps = device_settings(CFGS[name], cuda_device)
    assert ps.quarter_maps() is not None and ps.gr_geometry(np.float32).sym == 4
    img = np.random.default_rng(1).random(ps.img_shape)
    ref = O.forward(np.asfortranarray(img), host_settings(CFGS[name]))
    shared = _forward(ps, img, order, 4, cuda_device)
    direct = _forward(ps, img, order, 0, cuda_device)
    assert rel_l2(shared, ref) < 1e-5
    # float32 sums of a few hundred terms in another order (the turned
    # image's rows are walked along the base angle's axis)
    assert rel_l2(shared, direct) < 4e-6


@pytest.mark.parametrize("name", ["plain", "shifted_detector"])
def test_quarter_forward_in_solver_steps(cuda_device, name):
    """Landweber and TV agree with the per-angle kernel to float32 rounding;
    CG amplifies rounding, so it must be as close to the float64 oracle as
    the per-angle kernel is."""
    import torch

    import gratopy_gb300 as gg

    ps = device_settings(CFGS[name], cuda_device)
    hps = host_settings(CFGS[name])
    f_np = np.asfortranarray(np.random.default_rng(2).random(ps.sinogram_shape))
    f = gg.core.empty(ps.sinogram_shape, torch.float32, "F", cuda_device)
    f.copy_(torch.from_numpy(f_np.astype(np.float32)))
    g = ps.gr_geometry(np.float32)
    res = {}
    for sym in (4, 0):
        g.sym = sym
        res[sym] = (gg.conjugate_gradients(f, ps, 5).double().cpu().numpy(),
                    gg.landweber(f, ps, 5, norm_estimate=5.0).double().cpu().numpy(),
                    gg.total_variation(f, ps, 10.0, 5, norm_estimate=5.0).double().cpu().numpy())
    g.sym = 4
    cg_ref = O.conjugate_gradients(np.asfortranarray(f_np.astype(np.float32).astype(np.float64)),
                                   hps, 5)
    assert rel_l2(res[4][0], cg_ref) <= 2 * rel_l2(res[0][0], cg_ref) + 1e-6
    for a, b in zip(res[4][1:], res[0][1:]):
        assert rel_l2(a, b) < 1e-5


def test_asymmetric_geometry_keeps_the_per_angle_kernel(cuda_device):
    ps = device_settings(dict(CFGS["plain"], img_shape=(40, 36)), cuda_device)
    assert ps.quarter_maps() is None and ps.gr_geometry(np.float32).sym == 0
