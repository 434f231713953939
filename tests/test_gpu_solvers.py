"""GPU parity of the reconstruction loops against the oracle and gratopy's goldens.

The GPU solvers run the same iteration as the oracle's restatement of
gratopy.py:2329-2762 (same float32 scalar casts, float64 reductions), with
the operator-norm estimate injected so both sides use one value.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import configs  # noqa: E402

from oracle import oracle as O  # noqa: E402
from tests.helpers import (  # noqa: E402
    assert_control,
    device_settings,
    host_settings,
    rel_l2,
    walnut_sinogram,
)

pytestmark = pytest.mark.gpu

CFG = {
    "radon": dict(geometry="radon", img_shape=(48, 48), angles=40, n_detectors=70),
    "fan": dict(geometry="fanbeam", img_shape=(48, 40), angles=36, n_detectors=72,
                detector_width=40.0, R=70.0, RE=30.0),
}
# Relative L2 error bounds against the float64 oracle.  Iterative solvers
# amplify rounding differences by the problem's sensitivity, measured here as
# the distance between the float32 and float64 runs of the oracle (``base``):
# * float64: within max(1e-11, 1e-7 * base) -- float64 rounding is 5e8 times
#   finer than float32, so 1e-7 * base leaves a margin of 50;
# * float32: within 1e-5, or -- when the float32 restatement of the
#   reference's own arithmetic is already further off -- 3 * base (two
#   float32 runs with different rounding drift from float64 by comparable,
#   not equal, amounts).
TOL = {np.float32: 1e-5, np.float64: 1e-11}


def _check(out, ref64, ref32, dtype, what):
    err = rel_l2(out, ref64)
    base = rel_l2(ref32, ref64)
    if dtype == np.float64:
        bound = max(TOL[np.float64], 1e-7 * base)
        assert err <= bound, f"{what} float64 rel err {err:.3e} (float32 oracle: {base:.3e})"
        return
    bound = max(TOL[np.float32], 3.0 * base)
    assert err <= bound, f"{what} float32 rel err {err:.3e} (float32 oracle: {base:.3e})"


def _to_torch(a, device):
    import torch

    if a.flags.c_contiguous:
        return torch.from_numpy(a).to(device)
    return torch.from_numpy(np.ascontiguousarray(a.T)).to(device).permute(*reversed(range(a.ndim)))


def _data(hps, nz, order, dtype, seed=0):
    from gratopy_gb300.phantom import random_ellipse_image

    imgs = [random_ellipse_image(seed + k, hps.img_shape[::-1]).T for k in range(nz)]
    img = np.stack(imgs, axis=-1) if nz > 1 else imgs[0]
    img = np.require(img, np.float64, order)
    sino = O.forward(img, hps)
    return np.require(sino, dtype, order)


@pytest.mark.parametrize("geom", ["radon", "fan"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("order", ["F", "C"])
@pytest.mark.parametrize("nz", [1, 3])
def test_landweber_parity(cuda_device, geom, dtype, order, nz):
    import gratopy_gb300 as gg

    hps = host_settings(CFG[geom])
    ps = device_settings(CFG[geom], cuda_device)
    sino = _data(hps, nz, order, dtype)
    nrm = 3.0
    ref = O.landweber(np.require(sino, np.float64, order), hps, 25, w=1.0, norm_estimate=nrm)
    ref32 = O.landweber(np.require(sino, np.float32, order), hps, 25, w=1.0, norm_estimate=nrm)
    out = gg.landweber(_to_torch(sino, cuda_device), ps, 25, w=1.0, norm_estimate=nrm)
    assert gg.core.order_of(out) == order
    _check(out.cpu().numpy(), ref, ref32, dtype, "Landweber")


@pytest.mark.parametrize("geom", ["radon", "fan"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("order", ["F", "C"])
@pytest.mark.parametrize("nz", [1, 3])
def test_cg_parity(cuda_device, geom, dtype, order, nz):
    import gratopy_gb300 as gg

    hps = host_settings(CFG[geom])
    ps = device_settings(CFG[geom], cuda_device)
    sino = _data(hps, nz, order, dtype, seed=5)
    ref = O.conjugate_gradients(np.require(sino, np.float64, order), hps, 8)
    ref32 = O.conjugate_gradients(np.require(sino, np.float32, order), hps, 8)
    out = gg.conjugate_gradients(_to_torch(sino, cuda_device), ps, 8)
    _check(out.cpu().numpy(), ref, ref32, dtype, "CG")


@pytest.mark.parametrize("geom", ["radon", "fan"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("order", ["F", "C"])
@pytest.mark.parametrize("nz", [1, 3])
def test_tv_parity(cuda_device, geom, dtype, order, nz):
    import gratopy_gb300 as gg

    hps = host_settings(CFG[geom])
    ps = device_settings(CFG[geom], cuda_device)
    sino = _data(hps, nz, order, dtype, seed=11)
    nrm = 2.5
    ref = O.total_variation(np.require(sino, np.float64, order), hps, 20.0, 30,
                            slice_thickness=1.0, norm_estimate=nrm)
    ref32 = O.total_variation(np.require(sino, np.float32, order), hps, 20.0, 30,
                              slice_thickness=1.0, norm_estimate=nrm)
    out = gg.total_variation(_to_torch(sino, cuda_device), ps, 20.0, 30, slice_thickness=1.0,
                             norm_estimate=nrm)
    _check(out.cpu().numpy(), ref, ref32, dtype, "TV")


@pytest.mark.parametrize("geom", ["radon", "fan"])
def test_normest_parity(cuda_device, geom):
    import gratopy_gb300 as gg

    hps = host_settings(CFG[geom])
    ps = device_settings(CFG[geom], cuda_device)
    x0 = np.random.default_rng(2).standard_normal(hps.img_shape)
    ref = O.normest(hps, 20, dtype="float64", x0=x0)
    out = gg.normest(ps, 20, dtype="float64", x0=x0)
    assert abs(out - ref) / ref < 1e-12
    out32 = gg.normest(ps, 20, x0=x0)
    assert abs(out32 - ref) / ref < 1e-5


def test_cg_early_stop_matches_oracle(cuda_device):
    import gratopy_gb300 as gg

    hps = host_settings(CFG["radon"])
    ps = device_settings(CFG["radon"], cuda_device)
    sino = _data(hps, 1, "F", np.float64, seed=9)
    ref_full = O.conjugate_gradients(sino, hps, 40)
    # pick an epsilon that stops after a few iterations
    eps = 0.02
    ref = O.conjugate_gradients(sino, hps, 40, epsilon=eps)
    assert rel_l2(ref, ref_full) > 1e-6
    out = gg.conjugate_gradients(_to_torch(sino, cuda_device), ps, 40, epsilon=eps)
    assert rel_l2(out.cpu().numpy(), ref) < 1e-11


def _walnut_stack(ps_host, dtype=np.float32):
    """Walnut sinogram + a phantom sinogram as second slice (test_fanbeam.py:1112-1140)."""
    from gratopy_gb300.phantom import shepp_logan_host

    walnut = walnut_sinogram("float32")
    walnut = walnut / np.mean(walnut)
    ph = np.ascontiguousarray(shepp_logan_host((600, 600), dtype="float32"))
    phs = O.forward(ph, ps_host)
    sino = np.zeros(ps_host.sinogram_shape + (2,))
    sino[:, :, 0] = walnut / np.max(walnut)
    sino[:, :, 1] = phs / np.max(phs)
    return np.require(sino, dtype, "F")


def test_landweber_walnut_golden(cuda_device):
    """gratopy tests/test_fanbeam.py:1094-1164: control number 0.971266."""
    import gratopy_gb300 as gg

    cfg = configs.configs()["fan_walnut600"]
    sino = _walnut_stack(host_settings(cfg))
    ps = device_settings(cfg, cuda_device)
    U = gg.landweber(_to_torch(sino, cuda_device), ps, 100)
    assert_control(U.cpu().numpy(), (600, 600, 328, 120, 2), 0.971266, "img", "Landweber")


def test_cg_walnut_golden(cuda_device):
    """gratopy tests/test_fanbeam.py:1167-1246: control number 0.75674."""
    import gratopy_gb300 as gg

    cfg = configs.configs()["fan_walnut600"]
    sino = _walnut_stack(host_settings(cfg))
    ps = device_settings(cfg, cuda_device)
    U = gg.conjugate_gradients(_to_torch(sino, cuda_device), ps, number_iterations=50)
    assert_control(U.cpu().numpy(), (600, 600, 328, 120, 2), 0.75674, "img", "CG")


@pytest.mark.parametrize("noisy,mu,golden", [(False, 1e8, 0.251590), (True, 20.0, 0.038413)])
def test_tv_walnut_golden(cuda_device, noisy, mu, golden):
    """gratopy tests/test_fanbeam.py:1249-1382 (2000 iterations, 400^2)."""
    import gratopy_gb300 as gg

    cfg = configs.configs()["fan_walnut400"]
    ps = device_settings(cfg, cuda_device)
    walnut = walnut_sinogram("float32")
    walnut = walnut / np.mean(walnut)
    if noisy:
        rng = np.random.default_rng(1)
        walnut = walnut + rng.normal(0, 1, walnut.shape) * 0.2
    sino = _to_torch(np.require(walnut, np.float32, "F"), cuda_device)
    U = gg.total_variation(sino, ps, mu=mu, number_iterations=2000, slice_thickness=0,
                           stepsize_weighting=10)
    assert_control(U.cpu().numpy(), (400, 400, 328, 120, 1), golden, "img", "TV")
