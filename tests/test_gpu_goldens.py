"""gratopy's projection control numbers on the GPU kernels, and the public
utility functions against the oracle.

Each golden is a control number hard-coded in gratopy's test-suite
(file:line per test), pinned at gratopy's rtol 1e-3; the same outputs are
also compared with the float64 oracle on the same inputs.  The float32
bound is 1e-5 relative L2, or 1.25 x the error of the reference's own
float32 arithmetic (the float32 oracle) where that is larger: on the
strongly magnifying midpoint-shifted fan geometry (R = 5, RE = 3) the
float32 oracle itself is 1.09e-5 from float64.  The oracle side of these
cases is pinned to the same numbers on the CPU by tests/test_oracle_pins.py.
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
    create_phantoms,
    device_settings,
    host_settings,
    rel_l2,
)

pytestmark = pytest.mark.gpu

CFG = configs.configs()


def _dev(a: np.ndarray, device):
    import torch

    import gratopy_gb300 as gg

    order = "C" if a.flags.c_contiguous else "F"
    t = gg.core.empty(a.shape, torch.float64 if a.dtype == np.float64 else torch.float32, order,
                      device)
    t.copy_(torch.from_numpy(np.ascontiguousarray(a)))
    return t


def _np(t):
    return t.detach().cpu().numpy()


def _fwd_parity(gpu_sino, img, hps):
    """Forward projection within max(1e-5, 1.25 x the float32 oracle's error)."""
    ref = O.forward(np.asfortranarray(img, np.float64), hps)
    err = rel_l2(gpu_sino, ref)
    if err <= 1e-5:
        return
    own = rel_l2(O.forward(np.asfortranarray(img, np.float32), hps), ref)
    assert err <= 1.25 * own, f"forward rel err {err:.3e} (float32 oracle {own:.3e})"


def _bwd_parity(gpu_back, sino, hps):
    """Backprojection of ``sino`` within max(1e-5, 1.25 x the float32 oracle's error)."""
    ref = O.backward(np.asfortranarray(sino, np.float64), hps)
    err = rel_l2(gpu_back, ref)
    if err <= 1e-5:
        return
    own = rel_l2(O.backward(np.asfortranarray(sino, np.float32), hps), ref)
    assert err <= 1.25 * own, f"backprojection rel err {err:.3e} (float32 oracle {own:.3e})"


@pytest.fixture(scope="module")
def phantoms1200():
    return create_phantoms(1200, "float32", "F")


def _fwd(name, img, device, **extra):
    import gratopy_gb300 as gg

    cfg = dict(CFG[name], **extra)
    ps = device_settings(cfg, device)
    return ps, gg.forwardprojection(_dev(img, device), ps)


def test_radon_limited_angles(cuda_device, phantoms1200):
    """tests/test_radon.py:427-623."""
    import gratopy_gb300 as gg

    img = phantoms1200
    dims = (1200, 1200, 360, 3, 2)  # the reference passes len(angles_correct) == 3
    correct, s_c = _fwd("radon_limited_correct", img, cuda_device)
    correct2, s_c2 = _fwd("radon_limited_correct2", img, cuda_device)
    incorrect, s_i = _fwd("radon_limited_incorrect", img, cuda_device)
    for s in (s_c, s_c2, s_i):
        assert_control(_np(s), dims, 340.93, "sino", "limited-angle sinogram")
    assert_control(_np(gg.backprojection(s_c, correct)), dims, 3385.137, "img", "back correct")
    assert_control(_np(gg.backprojection(s_c2, correct2)), dims, 3385.137, "img", "back correct2")
    back_i = gg.backprojection(s_c, incorrect)
    assert_control(_np(back_i), dims, 3453.203, "img", "back incorrect")
    # repair by copying the correct weights (set_angle_weights)
    incorrect.set_angle_weights(correct.angle_weights)
    assert_control(_np(gg.backprojection(s_c, incorrect)), dims, 3385.137, "img", "back repaired")
    # the oracle on the same inputs
    _fwd_parity(_np(s_c), img, host_settings(CFG["radon_limited_correct"]))
    _bwd_parity(_np(back_i), _np(s_c), host_settings(CFG["radon_limited_incorrect"]))


def test_fan_limited_angles(cuda_device, phantoms1200):
    """tests/test_fanbeam.py:452-675."""
    import gratopy_gb300 as gg

    img = phantoms1200
    dims = (1200, 1200, 360, 2, 2)  # the reference passes len(angles_correct) == 2
    correct, s_c = _fwd("fan_limited_correct", img, cuda_device)
    incorrect, s_i = _fwd("fan_limited_incorrect", img, cuda_device)
    correct2, s_c2 = _fwd("fan_limited_incorrect", img, cuda_device,
                          angle_weights=correct.angle_weights)
    for s in (s_c, s_i, s_c2):
        assert_control(_np(s), dims, -131.00, "sino", "limited-angle sinogram")
    assert_control(_np(gg.backprojection(s_c, correct)), dims, 19495.96, "img", "back correct")
    assert_control(_np(gg.backprojection(s_c2, correct2)), dims, 19495.96, "img", "back correct2")
    back_i = gg.backprojection(s_c, incorrect)
    assert_control(_np(back_i), dims, 23043.191, "img", "back incorrect")
    _fwd_parity(_np(s_c), img, host_settings(CFG["fan_limited_correct"]))
    _bwd_parity(_np(back_i), _np(s_c), host_settings(CFG["fan_limited_incorrect"]))


@pytest.mark.parametrize("name,golden", [
    ("radon_nonquadratic", (999.4965, 2401.26, 3310.3464)),   # tests/test_radon.py:626-699
    ("fan_nonquadratic", (999.4965, 530.45, 16101.3542)),     # tests/test_fanbeam.py:1385-1475
])
def test_nonquadratic(cuda_device, phantoms1200, name, golden):
    import gratopy_gb300 as gg

    img = np.asfortranarray(phantoms1200[:, 0:800, :])
    ps, sino = _fwd(name, img, cuda_device)
    back = gg.backprojection(sino, ps)
    dims = (1200, 800, 600, 360, 2)
    assert_control(img, dims, golden[0], "img", "image")
    assert_control(_np(sino), dims, golden[1], "sino", "sinogram")
    assert_control(_np(back), dims, golden[2], "img", "backprojection")
    hps = host_settings(CFG[name])
    _fwd_parity(_np(sino), img, hps)
    _bwd_parity(_np(back), _np(sino), hps)


@pytest.mark.parametrize("name,golden", [
    ("radon_midpoint", (2083.80, 6269.703)),   # tests/test_radon.py:799-884
    ("fan_midpoint", (297.880, 12217.92)),     # tests/test_fanbeam.py:678-766
])
def test_midpoint_shift(cuda_device, phantoms1200, name, golden):
    import gratopy_gb300 as gg

    ps, sino = _fwd(name, phantoms1200, cuda_device)
    back = gg.backprojection(sino, ps)
    dims = (1200, 1200, 600, 360, 2)
    assert_control(_np(sino), dims, golden[0], "sino", "sinogram")
    assert_control(_np(back), dims, golden[1], "img", "backprojection")
    hps = host_settings(CFG[name])
    _fwd_parity(_np(sino), phantoms1200, hps)
    _bwd_parity(_np(back), _np(sino), hps)


ORIENTATION = [  # tests/test_fanbeam.py:769-943
    (-22.6691, 1760.90, 131.301, 1157.280),
    (51.959, -61.3725, 85.7716, 1058.5918),
    (-703.53, 881.399, 542.11, 1050.41),
    (390.100, 173.108, 110.7186, 1202.997),
    (935.812, 1775.13, 578.73, 951.169),
    (51.3383, 1225.368, -322.945, 579.33),
]


@pytest.mark.parametrize("j", range(6))
def test_geometric_orientation(cuda_device, j):
    """tests/test_fanbeam.py:769-943 (C-ordered float32 test images)."""
    import gratopy_gb300 as gg

    Nx = 600
    img1 = np.zeros([Nx, Nx], dtype=np.float32)
    img1[0:int(Nx * 0.3)][:, 0:int(Nx * 0.3)] = 1
    img2 = img1.copy()
    img2[0:int(Nx * 0.3)][:, 0:int(Nx)] = 1
    dims = (Nx, Nx, 300, 360, 1)
    golden = ORIENTATION[j]
    for k, geom in enumerate((f"orient_par_{j}", f"orient_fan_{j}")):
        ps = device_settings(CFG[geom], cuda_device)
        hps = host_settings(CFG[geom])
        for m, img in enumerate((img1, img2)):
            sino = _np(gg.forwardprojection(_dev(img, cuda_device), ps))
            assert_control(sino, dims, golden[2 * k + m], "sino", f"{geom} image {m + 1}")
            _fwd_parity(sino, img, hps)


# ------------------------------------------------------- utility functions


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("order", ["F", "C"])
@pytest.mark.parametrize("divide", [False, True])
@pytest.mark.parametrize("geom", ["radon_limited_correct", "fan_types"])
def test_weight_sinogram(cuda_device, dtype, order, divide, geom):
    """gratopy.py:2188-2266 (utilities.cl:38-67): multiply or divide every
    angle's column by its weight; into a new array, into ``sino_out`` and in place."""
    import gratopy_gb300 as gg

    cfg = dict(CFG[geom], img_shape=(64, 64))
    hps = host_settings(cfg)
    ps = device_settings(cfg, cuda_device)
    y = np.require(np.random.default_rng(int(divide)).random(hps.sinogram_shape + (3,)),
                   dtype, order)
    ref = O.weight_sinogram(np.require(y, np.float64, order), hps, divide=divide)
    yd = _dev(y, cuda_device)
    out = gg.weight_sinogram(yd, ps, divide=divide)
    tol = 2e-7 if dtype == np.float32 else 1e-15
    assert gg.core.order_of(out) == order
    assert rel_l2(_np(out), ref) <= tol
    into = gg.core.zeros(yd.shape, yd.dtype, order, cuda_device)
    res = gg.weight_sinogram(yd, ps, sino_out=into, divide=divide)
    assert res.data_ptr() == into.data_ptr() and rel_l2(_np(into), ref) <= tol
    gg.weight_sinogram(yd, ps, sino_out=yd, divide=divide)
    assert rel_l2(_np(yd), ref) <= tol


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("order", ["F", "C"])
def test_equ_mul_add_and_mul_add_add(cuda_device, dtype, order):
    """gratopy.py:2269-2326 (utilities.cl:69-80): rhs += a x and rhs = a x + y."""
    import gratopy_gb300 as gg

    rng = np.random.default_rng(2)
    rhs = np.require(rng.random((37, 21, 2)), dtype, order)
    x = np.require(rng.random((37, 21, 2)), dtype, order)
    y = np.require(rng.random((37, 21, 2)), dtype, order)
    a = -0.625
    tol = 2e-7 if dtype == np.float32 else 1e-15
    want = np.require(rhs, np.float64) + a * np.require(x, np.float64)
    r = _dev(rhs, cuda_device)
    out = gg.equ_mul_add(r, a, _dev(x, cuda_device))
    assert out.data_ptr() == r.data_ptr() and rel_l2(_np(r), want) <= tol
    want = a * np.require(x, np.float64) + np.require(y, np.float64)
    r = _dev(rhs, cuda_device)
    out = gg.mul_add_add(r, a, _dev(x, cuda_device), _dev(y, cuda_device))
    assert out.data_ptr() == r.data_ptr() and rel_l2(_np(r), want) <= tol
