"""GPU parity of the projection kernels against the CPU oracle.

Tolerances (relative L2 error against the float64 oracle on the same
inputs): 1e-5 for the float32 kernels, 1e-12 for the float64 kernels.
Adjointness <A x, W y> ds = <x, A^T y> dx^2 to 1e-6 relative.
"""

from __future__ import annotations

import sys
import zlib
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import configs  # noqa: E402

from oracle import oracle as O  # noqa: E402
from tests.helpers import (  # noqa: E402
    assert_control,
    create_phantoms,
    device_settings,
    host_settings,
    rel_l2,
)

pytestmark = pytest.mark.gpu

TOL = {np.float32: 1e-5, np.float64: 1e-12}

SMALL = {
    "radon_sq": dict(geometry="radon", img_shape=(67, 67), angles=45, n_detectors=81),
    "radon_rect": dict(geometry="radon", img_shape=(70, 41), angles=[(23, 0, 2.0), (17, 2.5, 3.1)],
                       n_detectors=57, detector_width=2.4, midpoint_shift=[0.1, -0.2],
                       detector_shift=0.05),
    "fan_sq": dict(geometry="fanbeam", img_shape=(64, 64), angles=50, n_detectors=90,
                   detector_width=40.0, R=60.0, RE=25.0),
    "fan_rect": dict(geometry="fanbeam", img_shape=(45, 70), angles=33, n_detectors=77,
                     detector_width=55.0, R=90.0, RE=40.0, detector_shift=2.0,
                     midpoint_shift=[1.0, -0.5], reverse_detector=True),
}


def _to_torch(a: np.ndarray, device):
    import torch

    if a.flags.c_contiguous:
        return torch.from_numpy(a).to(device)
    return torch.from_numpy(np.ascontiguousarray(a.T)).to(device).permute(*reversed(range(a.ndim)))


def _np(t) -> np.ndarray:
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("name", sorted(SMALL))
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("io", ["F", "C"])
@pytest.mark.parametrize("so", ["F", "C"])
@pytest.mark.parametrize("nz", [1, 2, 5])
def test_projection_parity(cuda_device, name, dtype, io, so, nz):
    import gratopy_gb300 as gg
    import torch

    cfg = SMALL[name]
    hps = host_settings(cfg)
    ps = device_settings(cfg, cuda_device)
    rng = np.random.default_rng(zlib.crc32(f"{name}{io}{so}{nz}".encode()))
    shape_img = hps.img_shape + ((nz,) if nz > 1 else ())
    shape_sino = hps.sinogram_shape + ((nz,) if nz > 1 else ())
    img = np.require(rng.random(shape_img), dtype, io)
    sino_in = np.require(rng.random(shape_sino), dtype, so)

    # oracle in float64 on the same (rounded) inputs
    ref_fwd = O.forward(np.require(img, np.float64, io), hps, order=so)
    ref_bwd = O.backward(np.require(sino_in, np.float64, so), hps, order=io)

    img_d = _to_torch(img, cuda_device)
    sino_d = gg.core.empty(shape_sino, img_d.dtype, so, cuda_device)
    gg.forwardprojection(img_d, ps, sino=sino_d)
    back_d = gg.core.empty(shape_img, img_d.dtype, io, cuda_device)
    gg.backprojection(_to_torch(sino_in, cuda_device), ps, img=back_d)
    torch.cuda.synchronize()
    assert gg.core.order_of(sino_d) == so and gg.core.order_of(back_d) == io
    e_fwd = rel_l2(_np(sino_d), ref_fwd)
    e_bwd = rel_l2(_np(back_d), ref_bwd)
    assert e_fwd <= TOL[dtype], f"forward rel err {e_fwd:.3e} vs float64 oracle"
    assert e_bwd <= TOL[dtype], f"backward rel err {e_bwd:.3e} vs float64 oracle"


@pytest.mark.parametrize("name", ["radon_sq", "fan_sq"])
def test_matches_float32_oracle_closely(cuda_device, name):
    """float32 kernels against the float32 oracle (same arithmetic): ~1e-6."""
    import gratopy_gb300 as gg

    cfg = SMALL[name]
    hps = host_settings(cfg)
    ps = device_settings(cfg, cuda_device)
    img = np.require(np.random.default_rng(3).random(hps.img_shape), np.float32, "F")
    ref = O.forward(img, hps)
    out = _np(gg.forwardprojection(_to_torch(img, cuda_device), ps))
    assert rel_l2(out, ref) < 2e-6
    back_ref = O.backward(ref, hps)
    back = _np(gg.backprojection(_to_torch(ref, cuda_device), ps))
    assert rel_l2(back, back_ref) < 2e-6


@pytest.mark.parametrize("name", ["radon_adjoint", "fan_adjoint"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_adjointness(cuda_device, name, dtype):
    """<A x, W y> ds == <x, A^T y> dx^2 (gratopy tests/test_radon.py:340-424)."""
    import gratopy_gb300 as gg
    import torch

    cfg = configs.configs()[name]
    ps = device_settings(cfg, cuda_device)
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    gen = torch.Generator(device=cuda_device).manual_seed(7)
    worst = 0.0
    for _ in range(10):
        x = gg.core.empty(ps.img_shape, tdt, "F", cuda_device)
        x.copy_(torch.rand(ps.img_shape, generator=gen, device=cuda_device, dtype=tdt))
        y = gg.core.empty(ps.sinogram_shape, tdt, "F", cuda_device)
        y.copy_(torch.rand(ps.sinogram_shape, generator=gen, device=cuda_device, dtype=tdt))
        Ax = gg.forwardprojection(x, ps)
        ATy = gg.backprojection(y, ps)
        wy = gg.weight_sinogram(y, ps)
        lhs = float((Ax.double() * wy.double()).sum()) * ps.delta_s
        rhs = float((x.double() * ATy.double()).sum()) * ps.delta_x**2
        worst = max(worst, abs(lhs - rhs) / min(abs(lhs), abs(rhs)))
    assert worst < 1e-6, f"adjointness error {worst:.3e}"


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("order1", ["F", "C"])
@pytest.mark.parametrize("order2", ["F", "C"])
@pytest.mark.parametrize("geometry,golden", [("radon_types", (6.69419, 20.2049)),
                                             ("fan_types", (416.107, 7851.41))])
def test_types_contiguity_golden(cuda_device, dtype, order1, order2, geometry, golden):
    """gratopy tests/test_radon.py:164-270 and tests/test_fanbeam.py:166-277 on the GPU."""
    import gratopy_gb300 as gg
    from gratopy_gb300.phantom import shepp_logan_host

    ps = device_settings(configs.configs()[geometry], cuda_device)
    img = _to_torch(np.require(shepp_logan_host(600, dtype=dtype), dtype, order1), cuda_device)
    sino = gg.core.zeros(ps.sinogram_shape, img.dtype, order2, cuda_device)
    back = gg.core.zeros(ps.img_shape, img.dtype, order1, cuda_device)
    gg.forwardprojection(img, ps, sino=sino)
    gg.backprojection(sino, ps, img=back)
    dims = (600, 600, 300, 180, 1)
    assert_control(_np(sino), dims, golden[0], "sino", "sinogram")
    assert_control(_np(back), dims, golden[1], "img", "backprojection")


@pytest.mark.parametrize("name,golden", [
    ("radon_projection", (4737.367, 7427.70)),
    ("fan_projection", (94031.43, 1482240.72)),
])
def test_projection_golden_stack(cuda_device, name, golden):
    """gratopy tests/test_radon.py:35-148 and tests/test_fanbeam.py:43-150 (two slices)."""
    import gratopy_gb300 as gg

    ps = device_settings(configs.configs()[name], cuda_device)
    img = _to_torch(create_phantoms(1200, "float32", "F"), cuda_device)
    sino = gg.forwardprojection(img, ps)
    back = gg.backprojection(sino, ps)
    dims = (1200, 1200, ps.sinogram_shape[0], ps.sinogram_shape[1], 2)
    assert_control(_np(sino), dims, golden[0], "sino", "sinogram")
    assert_control(_np(back), dims, golden[1], "img", "backprojection")


def test_outputs_follow_input_order(cuda_device):
    import gratopy_gb300 as gg

    ps = device_settings(SMALL["radon_sq"], cuda_device)
    for order in ("F", "C"):
        img = gg.core.zeros((67, 67, 3), __import__("torch").float32, order, cuda_device)
        sino = gg.forwardprojection(img, ps)
        assert gg.core.order_of(sino) == order and tuple(sino.shape) == (81, 45, 3)
        back = gg.backprojection(sino, ps)
        assert gg.core.order_of(back) == order and tuple(back.shape) == (67, 67, 3)


def test_bitwise_deterministic(cuda_device):
    import gratopy_gb300 as gg
    import torch

    ps = device_settings(SMALL["fan_sq"], cuda_device)
    img = torch.rand((64, 64, 4), device=cuda_device).permute(2, 1, 0).contiguous().permute(2, 1, 0)
    a = gg.forwardprojection(img, ps)
    b = gg.forwardprojection(img, ps)
    assert torch.equal(a, b)
    ba = gg.backprojection(a, ps)
    bb = gg.backprojection(a, ps)
    assert torch.equal(ba, bb)


def test_shape_errors_raise(cuda_device):
    import gratopy_gb300 as gg
    import torch

    ps = device_settings(SMALL["radon_sq"], cuda_device)
    with pytest.raises(AssertionError):
        gg.forwardprojection(torch.zeros((66, 67), device=cuda_device), ps)
    with pytest.raises(AssertionError):
        gg.forwardprojection(torch.zeros((67, 67), device=cuda_device, dtype=torch.float64), ps,
                             sino=torch.zeros((81, 45), device=cuda_device))
    with pytest.raises(TypeError):
        gg.forwardprojection(torch.zeros((67, 67)), ps)
