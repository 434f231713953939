"""The operator API on the GPU with its built-in kernels.

* gratopy's device tests of ``operator.Radon`` (tests/test_operator.py:114-250)
  in this build's terms -- a ``torch.device`` or a CUDA tensor where the
  reference takes an OpenCL queue or a ``clarray.Array``: NumPy coercion, the
  remembered device, the missing-device error, composites forwarding the
  device, a preallocated output, a product writing its final result into
  ``output``, a sum accumulating into ``output``.
* Parity of ``Radon``, ``Radon.T``, ``R.T * R`` and ``2 * R - R``, and of
  ``Fanbeam`` / ``Fanbeam.T``, with the float64 oracle on the same inputs, in
  both memory orders and with a trailing slice dimension: relative L2 within
  1e-5 (float32) and 1e-12 (float64).
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import HostSettings, rel_l2

pytestmark = pytest.mark.gpu

TOL = {np.float32: 1e-5, np.float64: 1e-12}


def _radon_host(R):
    return HostSettings("radon", R.image_domain.size, np.asarray(R.angles.angles),
                        n_detectors=R.detectors.number,
                        angle_weights=np.asarray(R.angles.weights),
                        detector_width=float(R.detectors.extent),
                        image_width=float(R.image_domain.extent),
                        detector_shift=R.detectors.center,
                        midpoint_shift=tuple(R.image_domain.center))


def _fan_host(F):
    return HostSettings("fanbeam", F.image_domain.size, np.asarray(F.angles.angles),
                        n_detectors=F.detectors.number,
                        angle_weights=np.asarray(F.angles.weights),
                        detector_width=float(F.detectors.extent),
                        image_width=float(F.image_domain.extent),
                        R=F.state["R"], RE=F.state["RE"], detector_shift=F.detectors.center,
                        midpoint_shift=tuple(F.image_domain.center),
                        reverse_detector=bool(F.detectors.reversed))


def _device_array(a: np.ndarray, device):
    import torch

    import gratopy_gb300 as gg

    order = "C" if a.flags.c_contiguous else "F"
    t = gg.core.empty(a.shape, torch.float64 if a.dtype == np.float64 else torch.float32, order,
                      device)
    t.copy_(torch.from_numpy(np.ascontiguousarray(a)))
    return t


# ------------------------------------------- gratopy tests/test_operator.py:114-250


def test_radon_numpy_coercion(cuda_device):
    """A NumPy image with an explicit device gives a CUDA sinogram (test_operator.py:114-130)."""
    import torch

    from gratopy_gb300.operator import Radon

    R = Radon(image_domain=16, angles=10)
    sino = R.apply_to(np.zeros((16, 16), dtype=np.float32), queue=cuda_device)
    assert isinstance(sino, torch.Tensor) and sino.is_cuda
    assert tuple(sino.shape) == (R.detectors.number, 10)
    assert not bool(sino.any())


def test_radon_device_input_without_queue(cuda_device):
    """A CUDA tensor input needs no queue (test_operator.py:133-147)."""
    import torch

    from gratopy_gb300.operator import Radon

    R = Radon(image_domain=16, angles=10)
    img = torch.zeros((16, 16), dtype=torch.float32, device=cuda_device)
    sino = R.apply_to(img)
    assert isinstance(sino, torch.Tensor) and sino.device == img.device
    assert tuple(sino.shape) == (R.detectors.number, 10)


def test_radon_reuses_device(cuda_device):
    """The device of the last call is remembered (test_operator.py:150-168)."""
    import torch

    from gratopy_gb300.operator import Radon

    R = Radon(image_domain=16, angles=10)
    img = np.zeros((16, 16), dtype=np.float32)
    R.apply_to(img, queue=cuda_device)
    assert R.projection_settings is not None
    again = R.apply_to(img)
    assert isinstance(again, torch.Tensor) and again.is_cuda


def test_radon_no_device_error():
    """NumPy input and nothing to infer a device from (test_operator.py:171-179)."""
    from gratopy_gb300.operator import Radon

    R = Radon(image_domain=16, angles=10)
    with pytest.raises(ValueError, match="No CUDA device available"):
        R.apply_to(np.zeros((16, 16), dtype=np.float32))


def test_composite_forwards_queue(cuda_device):
    """``R.T * R`` passes the device to both factors (test_operator.py:182-196)."""
    import torch

    from gratopy_gb300.operator import Radon

    R = Radon(image_domain=16, angles=10)
    out = (R.T * R).apply_to(np.zeros((16, 16), dtype=np.float32), queue=cuda_device)
    assert isinstance(out, torch.Tensor) and out.is_cuda and tuple(out.shape) == (16, 16)


def test_radon_uses_preallocated_output(cuda_device):
    """The result is written into ``output`` (test_operator.py:199-215)."""
    import torch

    from gratopy_gb300.operator import Radon

    R = Radon(image_domain=16, angles=10)
    img = torch.zeros((16, 16), dtype=torch.float32, device=cuda_device)
    output = torch.full(R.output_shape, 42.0, dtype=torch.float32, device=cuda_device)
    result = R.apply_to(img, output=output)
    assert result.data_ptr() == output.data_ptr()
    assert not bool(output.any())


def test_composite_uses_output_for_final_result(cuda_device):
    """A product writes its last factor's result into ``output`` (test_operator.py:218-234)."""
    import torch

    from gratopy_gb300.operator import Radon

    R = Radon(image_domain=16, angles=10)
    img = torch.zeros((16, 16), dtype=torch.float32, device=cuda_device)
    output = torch.full((16, 16), 42.0, dtype=torch.float32, device=cuda_device)
    result = (R.T * R).apply_to(img, output=output)
    assert result.data_ptr() == output.data_ptr()
    assert not bool(output.any())


def test_sum_accumulates_into_output(cuda_device):
    """``R + R`` writes its first term into ``output`` and adds the second (test_operator.py:237-254)."""
    import torch

    from gratopy_gb300.operator import Radon

    R = Radon(image_domain=16, angles=10)
    img = torch.ones((16, 16), dtype=torch.float32, device=cuda_device)
    expected = (R + R).apply_to(img).cpu().numpy()
    output = torch.full(R.output_shape, 42.0, dtype=torch.float32, device=cuda_device)
    result = (R + R).apply_to(img, output=output)
    assert result.data_ptr() == output.data_ptr()
    np.testing.assert_allclose(output.cpu().numpy(), expected, rtol=1e-5, atol=1e-5)


# ------------------------------------------------------------ oracle parity


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("order", ["F", "C"])
@pytest.mark.parametrize("nz", [1, 3])
def test_radon_operator_parity(cuda_device, dtype, order, nz):
    from gratopy_gb300.operator import Radon
    from gratopy_gb300.utilities import Angles, Detectors, ImageDomain

    R = Radon(image_domain=ImageDomain(size=(40, 33), extent=2.0, center=(0.1, -0.05)),
              angles=Angles.uniform_interval(0.2, 2.9, 27, half_circle=True),
              detectors=Detectors(number=48, extent=2.4, center=0.03))
    hps = _radon_host(R)
    rng = np.random.default_rng(nz + (order == "C"))
    tail = (nz,) if nz > 1 else ()
    x = np.require(rng.random(R.input_shape + tail), dtype, order)
    y = np.require(rng.random(R.output_shape + tail), dtype, order)
    x64 = np.require(x, np.float64, order)
    y64 = np.require(y, np.float64, order)
    Ax = O.forward(x64, hps)
    ATy = O.backward(y64, hps)
    ATAx = O.backward(Ax, hps)
    xd, yd = _device_array(x, cuda_device), _device_array(y, cuda_device)
    tol = TOL[dtype]
    cases = [("R", R, xd, Ax), ("R.T", R.T, yd, ATy), ("R.T*R", R.T * R, xd, ATAx),
             ("2*R - R", 2 * R - R, xd, Ax)]
    for name, op, arg, ref in cases:
        out = op.apply_to(arg)
        assert tuple(out.shape) == ref.shape, name
        assert out.dtype == arg.dtype, name
        err = rel_l2(out.cpu().numpy(), ref)
        assert err <= tol, f"{name} {dtype.__name__} {order} nz={nz}: rel err {err:.3e}"
    # the operators applied to NumPy input give the same values
    out = R.apply_to(x, queue=cuda_device)
    assert rel_l2(out.cpu().numpy(), Ax) <= tol


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("order", ["F", "C"])
@pytest.mark.parametrize("nz", [1, 3])
@pytest.mark.parametrize("symmetric", [False, True])
def test_fanbeam_operator_parity(cuda_device, dtype, order, nz, symmetric):
    """``Fanbeam``; the symmetric case (square centred image, 40 equispaced
    full-circle angles) runs the quarter-turn orbit kernels in float32."""
    from gratopy_gb300.operator import Fanbeam
    from gratopy_gb300.utilities import Angles, Detectors, ImageDomain

    if symmetric:
        F = Fanbeam((90.0, 40.0), ImageDomain(size=(36, 36), extent=30.0), 40,
                    detectors=Detectors(number=60))
    else:
        F = Fanbeam((90.0, 40.0), ImageDomain(size=(36, 29), extent=30.0, center=(1.0, -0.5)),
                    Angles.uniform_interval(0.3, 5.9, 31),
                    detectors=Detectors(number=-55, extent=70.0, center=1.5))
    hps = _fan_host(F)
    rng = np.random.default_rng(3 * nz + (order == "C") + 7 * symmetric)
    tail = (nz,) if nz > 1 else ()
    x = np.require(rng.random(F.input_shape + tail), dtype, order)
    y = np.require(rng.random(F.output_shape + tail), dtype, order)
    Ax = O.forward(np.require(x, np.float64, order), hps)
    ATy = O.backward(np.require(y, np.float64, order), hps)
    tol = TOL[dtype]
    for name, op, arg, ref in (("F", F, _device_array(x, cuda_device), Ax),
                               ("F.T", F.T, _device_array(y, cuda_device), ATy)):
        out = op.apply_to(arg)
        err = rel_l2(out.cpu().numpy(), ref)
        assert err <= tol, f"{name} {dtype.__name__} {order} nz={nz}: rel err {err:.3e}"
    if symmetric and dtype == np.float32:
        assert F.projection_settings.gr_geometry(np.float32).sym == 4


def test_operator_adjointness(cuda_device):
    """<R x, W y> ds = <x, R.T y> dx^2 (float64): R.T is gratopy's
    backprojection, the adjoint of R in the angle-weighted sinogram inner
    product.  It holds to 1e-6, not to float64 rounding: the Radon forward
    scales by dx and ds rounded to float32 (radon.cl:82-83) in both
    precisions, an offset of ~1e-8 relative."""
    import torch

    from gratopy_gb300.operator import Radon

    R = Radon(image_domain=32, angles=24)
    gen = torch.Generator(device=cuda_device).manual_seed(4)
    x = torch.rand(R.input_shape, generator=gen, device=cuda_device, dtype=torch.float64)
    y = torch.rand(R.output_shape, generator=gen, device=cuda_device, dtype=torch.float64)
    Rx = R.apply_to(x)
    ps = R.projection_settings
    w = torch.as_tensor(np.asarray(ps.angle_weights), device=cuda_device, dtype=torch.float64)
    lhs = float((Rx * y * w[None, :]).sum()) * ps.delta_s
    rhs = float((x * R.T.apply_to(y)).sum()) * ps.delta_x ** 2
    assert abs(lhs - rhs) <= 1e-6 * abs(rhs)
