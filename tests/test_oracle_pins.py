"""Pin the CPU oracle to gratopy's golden values (CPU only).

Every expected number below is a control number hard-coded in gratopy's own
test-suite (file:line given per test), computed by the reference's OpenCL
kernels; the oracle must reproduce each at gratopy's tolerance (rtol 1e-3).
The 2000-iteration TV pins are run by ``python -m oracle.pin_solvers``
(minutes on a CPU); their recorded outcome is checked here.
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
import configs  # noqa: E402

from gratopy_gb300.phantom import shepp_logan_host  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.helpers import (  # noqa: E402
    assert_control,
    create_phantoms,
    host_settings,
    walnut_sinogram,
)

CFG = configs.configs()


@pytest.fixture(scope="module")
def phantoms1200():
    return create_phantoms(1200, "float32", "F")


def test_radon_projection(phantoms1200):
    """tests/test_radon.py:35-148."""
    ps = host_settings(CFG["radon_projection"])
    img = phantoms1200
    sino = O.forward(img, ps)
    back = O.backward(sino, ps)
    dims = (1200, 1200, 600, 360, 2)
    assert_control(img, dims, 2949.3738, "img", "image")
    assert_control(sino, dims, 4737.367, "sino", "sinogram")
    assert_control(back, dims, 7427.70, "img", "backprojection")


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("geometry,golden", [("radon_types", (7.89220, 6.69419, 20.2049)),
                                             ("fan_types", (7.8922043, 416.107, 7851.41))])
def test_types_contiguity(dtype, geometry, golden):
    """tests/test_radon.py:164-270, tests/test_fanbeam.py:166-277 (all four order pairs)."""
    ps = host_settings(CFG[geometry])
    phantom = shepp_logan_host(600, dtype=dtype)
    dims = (600, 600, 300, 180, 1)
    for o1 in ("F", "C"):
        for o2 in ("F", "C"):
            img = np.require(phantom, dtype, o1)
            sino = O.forward(img, ps, order=o2)
            back = O.backward(sino, ps, order=o1)
            assert_control(img, dims, golden[0], "img", "image")
            assert_control(sino, dims, golden[1], "sino", f"sinogram {dtype.__name__} {o1}{o2}")
            assert_control(back, dims, golden[2], "img", f"backprojection {dtype.__name__} {o1}{o2}")


def test_radon_limited_angles(phantoms1200):
    """tests/test_radon.py:427-623."""
    correct = host_settings(CFG["radon_limited_correct"])
    incorrect = host_settings(CFG["radon_limited_incorrect"])
    correct2 = host_settings(CFG["radon_limited_correct2"])
    img = phantoms1200
    dims = (1200, 1200, 360, 3, 2)  # the reference passes len(angles_correct) == 3
    s_c = O.forward(img, correct)
    s_c2 = O.forward(img, correct2)
    s_i = O.forward(img, incorrect)
    for s in (s_c, s_c2, s_i):
        assert_control(s, dims, 340.93, "sino", "limited-angle sinogram")
    assert_control(O.backward(s_c, correct), dims, 3385.137, "img", "back correct")
    assert_control(O.backward(s_c2, correct2), dims, 3385.137, "img", "back correct2")
    assert_control(O.backward(s_c, incorrect), dims, 3453.203, "img", "back incorrect")
    # repair by copying the correct weights (set_angle_weights)
    fixed = host_settings(dict(CFG["radon_limited_incorrect"], angle_weights=correct.angle_weights))
    assert_control(O.backward(s_c, fixed), dims, 3385.137, "img", "back repaired")


def test_radon_nonquadratic(phantoms1200):
    """tests/test_radon.py:626-699."""
    img = np.ascontiguousarray(phantoms1200[:, 0:800, :])
    ps = host_settings(CFG["radon_nonquadratic"])
    sino = O.forward(img, ps)
    back = O.backward(sino, ps)
    dims = (1200, 800, 600, 360, 2)
    assert_control(img, dims, 999.4965, "img", "image")
    assert_control(sino, dims, 2401.26, "sino", "sinogram")
    assert_control(back, dims, 3310.3464, "img", "backprojection")


def test_radon_midpoint_shift(phantoms1200):
    """tests/test_radon.py:799-884."""
    ps = host_settings(CFG["radon_midpoint"])
    sino = O.forward(phantoms1200, ps)
    back = O.backward(sino, ps)
    dims = (1200, 1200, 600, 360, 2)
    assert_control(sino, dims, 2083.80, "sino", "sinogram")
    assert_control(back, dims, 6269.703, "img", "backprojection")


def test_radon_mass_preservation():
    """tests/test_radon.py:273-337: projections preserve mass to 1e-3."""
    ps = host_settings(CFG["radon_weighting"])
    N = 900
    img = np.zeros((N, N))
    img[int(N / 3.0):int(2 * N / 3.0)][:, int(N / 3.0):int(2 * N / 3.0)] = 1
    img = np.require(img, np.float32, "F")
    sino = O.forward(img, ps)
    mass_img = np.sum(img) * ps.delta_x**2
    for a in range(ps.n_angles):
        mass_sino = np.sum(sino[:, a]) * ps.delta_s
        assert abs(1 - mass_img / mass_sino) < 0.001


def test_fan_projection(phantoms1200):
    """tests/test_fanbeam.py:43-150."""
    ps = host_settings(CFG["fan_projection"])
    sino = O.forward(phantoms1200, ps)
    back = O.backward(sino, ps)
    dims = (1200, 1200, 600, 360, 2)
    assert_control(sino, dims, 94031.43, "sino", "sinogram")
    assert_control(back, dims, 1482240.72, "img", "backprojection")


def test_fan_limited_angles(phantoms1200):
    """tests/test_fanbeam.py:452-675."""
    correct = host_settings(CFG["fan_limited_correct"])
    incorrect = host_settings(CFG["fan_limited_incorrect"])
    correct2 = host_settings(dict(CFG["fan_limited_incorrect"], angle_weights=correct.angle_weights))
    img = phantoms1200
    dims = (1200, 1200, 360, 2, 2)  # the reference passes len(angles_correct) == 2
    s_c = O.forward(img, correct)
    s_i = O.forward(img, incorrect)
    s_c2 = O.forward(img, correct2)
    for s in (s_c, s_i, s_c2):
        assert_control(s, dims, -131.00, "sino", "limited-angle sinogram")
    assert_control(O.backward(s_c, correct), dims, 19495.96, "img", "back correct")
    assert_control(O.backward(s_c2, correct2), dims, 19495.96, "img", "back correct2")
    assert_control(O.backward(s_c, incorrect), dims, 23043.191, "img", "back incorrect")


def test_fan_midpoint_shift(phantoms1200):
    """tests/test_fanbeam.py:678-766."""
    ps = host_settings(CFG["fan_midpoint"])
    sino = O.forward(phantoms1200, ps)
    back = O.backward(sino, ps)
    dims = (1200, 1200, 600, 360, 2)
    assert_control(sino, dims, 297.880, "sino", "sinogram")
    assert_control(back, dims, 12217.92, "img", "backprojection")


def test_fan_nonquadratic(phantoms1200):
    """tests/test_fanbeam.py:1385-1475."""
    img = np.ascontiguousarray(phantoms1200[:, 0:800, :])
    ps = host_settings(CFG["fan_nonquadratic"])
    sino = O.forward(img, ps)
    back = O.backward(sino, ps)
    dims = (1200, 800, 600, 360, 2)
    assert_control(sino, dims, 530.45, "sino", "sinogram")
    assert_control(back, dims, 16101.3542, "img", "backprojection")


ORIENTATION = [
    (-22.6691, 1760.90, 131.301, 1157.280),
    (51.959, -61.3725, 85.7716, 1058.5918),
    (-703.53, 881.399, 542.11, 1050.41),
    (390.100, 173.108, 110.7186, 1202.997),
    (935.812, 1775.13, 578.73, 951.169),
    (51.3383, 1225.368, -322.945, 579.33),
]


@pytest.mark.parametrize("j", range(6))
def test_geometric_orientation(j):
    """tests/test_fanbeam.py:769-943 (C-ordered float32 test images)."""
    Nx = 600
    img1 = np.zeros([Nx, Nx], dtype=np.float32)
    img1[0:int(Nx * 0.3)][:, 0:int(Nx * 0.3)] = 1
    img2 = img1.copy()
    img2[0:int(Nx * 0.3)][:, 0:int(Nx)] = 1
    par = host_settings(CFG[f"orient_par_{j}"])
    fan = host_settings(CFG[f"orient_fan_{j}"])
    dims = (Nx, Nx, 300, 360, 1)
    golden = ORIENTATION[j]
    assert_control(O.forward(img1, par), dims, golden[0], "sino", "radon 1")
    assert_control(O.forward(img2, par), dims, golden[1], "sino", "radon 2")
    assert_control(O.forward(img1, fan), dims, golden[2], "sino", "fan 1")
    assert_control(O.forward(img2, fan), dims, golden[3], "sino", "fan 2")


@pytest.mark.parametrize("geometry,golden", [("radon_sparse", 6.5315), ("fan_sparse", 233.96)])
def test_sparse_case_sinograms(geometry, golden):
    """Forward projection of the sparse-matrix cases (tests/test_radon.py:715-796,
    tests/test_fanbeam.py:1491-1584): the matrix-vector product equals the projection."""
    ps = host_settings(CFG[geometry])
    img = np.require(shepp_logan_host(150, dtype=np.float64), np.float64, "F")
    sino = O.forward(img, ps)
    if geometry == "fan_sparse":
        sino = np.where(sino > 0, sino, 0)
    assert_control(sino, (150, 150, 100, 30, 1), golden, "sino", "sparse-case sinogram")


def test_fan_mass_ratio():
    """tests/test_fanbeam.py:280-355: fan mass ~ R/RE times the image mass (10%)."""
    for nd in (50, 200, 800):
        r = 1 / 40.0 * np.sqrt(2)
        ps = host_settings(dict(geometry="fanbeam", img_shape=(400, 400), angles=720,
                                detector_width=400.0 * r, R=1200.0 * r, RE=200.0 * r,
                                n_detectors=nd, image_width=40.0 * r))
        img = np.ones((400, 400), dtype=np.float32, order="F")
        sino = O.forward(img, ps)
        ratio = np.sum(sino) * ps.delta_s / 720 / (np.sum(img) * ps.delta_x**2)
        assert abs(ratio / (1200.0 / 200.0) - 1) < 0.1


@pytest.mark.parametrize("name", ["radon_adjoint", "fan_adjoint"])
def test_adjointness_oracle(name):
    """tests/test_radon.py:340-424 / tests/test_fanbeam.py:358-449 (eps 1e-5)."""
    ps = host_settings(CFG[name])
    rng = np.random.default_rng(0)
    fails = 0
    for _ in range(10):
        x = np.require(rng.random(ps.img_shape), np.float32, "F")
        y = np.require(rng.random(ps.sinogram_shape), np.float32, "F")
        Ax = O.forward(x, ps)
        ATy = O.backward(y, ps)
        lhs = O.dot(O.weight_sinogram(y, ps), Ax) * ps.delta_s
        rhs = O.dot(x, ATy) * ps.delta_x**2
        fails += abs(lhs - rhs) / min(abs(lhs), abs(rhs)) > 1e-5
    assert fails == 0


def _walnut_stack(ps):
    walnut = walnut_sinogram("float32")
    walnut = walnut / np.mean(walnut)
    ph = np.ascontiguousarray(shepp_logan_host((600, 600), dtype="float32"))
    phs = O.forward(ph, ps)
    sino = np.zeros(ps.sinogram_shape + (2,))
    sino[:, :, 0] = walnut / np.max(walnut)
    sino[:, :, 1] = phs / np.max(phs)
    return np.require(sino, np.float32, "F")


def test_landweber_walnut():
    """tests/test_fanbeam.py:1094-1164: 0.971266."""
    ps = host_settings(CFG["fan_walnut600"])
    U = O.landweber(_walnut_stack(ps), ps, 100)
    assert_control(U, (600, 600, 328, 120, 2), 0.971266, "img", "Landweber")


def test_cg_walnut():
    """tests/test_fanbeam.py:1167-1246: 0.75674."""
    ps = host_settings(CFG["fan_walnut600"])
    U = O.conjugate_gradients(_walnut_stack(ps), ps, number_iterations=50)
    assert_control(U, (600, 600, 328, 120, 2), 0.75674, "img", "CG")


def test_tv_pins_recorded():
    """The recorded outcome of ``python -m oracle.pin_solvers`` (tests/test_fanbeam.py:1249-1382)."""
    rec = json.loads((GOLDEN / "oracle_solver_pins.json").read_text())
    for key, golden in (("exact_mu1e8", 0.251590), ("noisy_mu20", 0.038413)):
        assert rec[key]["golden"] == golden
        assert abs(rec[key]["control_number"] - golden) < 1e-3 * abs(golden)
