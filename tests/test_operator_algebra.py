"""Operator algebra, shapes and geometry descriptions (CPU only).

Mirrors gratopy's tests/test_operator.py:11-92, tests/test_shaped_operators.py,
tests/test_radon_shapes.py and tests/test_operator.py:252-270.
"""

from __future__ import annotations

import numpy as np
import pytest

from gratopy_gb300.operator import IDENTITY, ZERO, Fanbeam, Operator, Radon
from gratopy_gb300.operator.base import OperatorArithmeticOperation
from gratopy_gb300.utilities import Angles, Detectors, ExtentPlaceholder, ImageDomain


def test_identity_and_zero():
    assert repr(IDENTITY) == "[Id]" and repr(ZERO) == "[0]"
    assert IDENTITY.apply_to([1, 2, 3]) == [1, 2, 3]
    assert IDENTITY * [1, 2, 3] == [1, 2, 3]
    data = np.array([1, 2, 3])
    np.testing.assert_equal(ZERO.apply_to(data), np.zeros_like(data))
    np.testing.assert_equal(ZERO * data, np.zeros_like(data))
    assert ZERO + ZERO == ZERO and ZERO - ZERO == ZERO
    assert ZERO + IDENTITY == IDENTITY and IDENTITY + ZERO == IDENTITY
    assert IDENTITY - ZERO == IDENTITY
    assert 0 * ZERO == ZERO and 42 * ZERO == ZERO
    assert ZERO * ZERO == ZERO and ZERO * IDENTITY == ZERO and IDENTITY * ZERO == ZERO
    A = Operator(name="A")
    assert IDENTITY * A == A and A * IDENTITY == A


def test_representation():
    A, B, C = Operator(name="A"), Operator(name="B"), Operator(name="C")
    assert repr(A * B) == "A*B"
    assert repr(A + B) == "A + B"
    assert repr(5 * (A + IDENTITY) - B) == "5*A + 5*[Id] + (-1)*B"
    assert repr(5 * (A + IDENTITY) * C - B) == "(5*A + 5*[Id])*C + (-1)*B"
    assert repr(A * B * A * B * A * B) == "A*B*A*B*A*B"
    assert repr(5 * A * B * A * B * A * B) == "5*A*B*A*B*A*B"
    assert repr(5 * (A * B * B * A)) == "5*A*B*B*A"


def test_composition_structure():
    A, B = Operator(name="A"), Operator(name="B")
    op = 5 * (A + IDENTITY) - B
    assert op.is_composite()
    assert op._arithmetic_operation == OperatorArithmeticOperation.ADDITION
    assert len(op._operands) == 3
    assert 5 * (A + B + A) == 5 * A + 5 * B + 5 * A
    assert 5 * (A * B * B * A) == 5 * A * B * B * A


def test_shape_propagation():
    A = Operator(name="A", input_shape=(20,), output_shape=(30,))
    B = Operator(name="B", input_shape=(10,), output_shape=(20,))
    C = A * B
    assert C.input_shape == (10,) and C.output_shape == (30,)
    with pytest.raises(ValueError, match="Shape mismatch"):
        _ = A * Operator(name="D", input_shape=(10,), output_shape=(25,))
    with pytest.raises(ValueError, match="Input shape mismatch"):
        _ = A + Operator(name="E", input_shape=(21,), output_shape=(30,))
    with pytest.raises(ValueError, match="Output shape mismatch"):
        _ = A + Operator(name="F", input_shape=(20,), output_shape=(31,))
    P = A + Operator(name="G")
    assert P.input_shape == (20,) and P.output_shape == (30,)


def test_radon_shapes_and_transpose():
    R = Radon(image_domain=128, angles=180, detectors=200)
    assert R.input_shape == (128, 128) and R.output_shape == (200, 180)
    assert R.T.input_shape == (200, 180) and R.T.output_shape == (128, 128)
    assert (R.T * R).input_shape == (128, 128) and (R.T * R).output_shape == (128, 128)
    assert (R * R.T).input_shape == (200, 180)
    assert repr(R.T * R) == "Radon.T*Radon"
    with pytest.raises(ValueError, match="Input shape mismatch"):
        _ = Radon(image_domain=128, angles=180) + Radon(image_domain=129, angles=180)
    with pytest.raises(ValueError, match="Shape mismatch"):
        _ = Radon(image_domain=128, angles=180).T * Radon(image_domain=128, angles=100)


def test_radon_defaults():
    R = Radon(image_domain=16, angles=10)
    assert R.angles.half_circle is True
    np.testing.assert_allclose(R.angles.angles, np.linspace(0, np.pi, 10, endpoint=False))
    np.testing.assert_allclose(R.angles.weights, np.full(10, np.pi / 10))
    assert R.detectors.number == int(np.ceil(np.hypot(16, 16)))
    angles = Angles.uniform(10)
    R2 = Radon(image_domain=16, angles=angles)
    assert R2.angles is angles and R2.angles.half_circle is False


def test_radon_placeholders_resolve():
    r = Radon(ImageDomain(size=16, extent=2.0), 10, Detectors(number=20, extent=ExtentPlaceholder.FULL))
    assert isinstance(r.detectors.extent, float) and r.detectors.extent > 0
    r = Radon(ImageDomain(size=16, extent=ExtentPlaceholder.FULL), 10, Detectors(number=20, extent=2.0))
    assert isinstance(r.image_domain.extent, float) and r.image_domain.extent > 0
    with pytest.raises(NotImplementedError):
        Radon(ImageDomain(size=16, extent=ExtentPlaceholder.FULL), 10,
              Detectors(number=20, extent=ExtentPlaceholder.VALID))


def test_radon_without_device_raises_value_error():
    R = Radon(image_domain=16, angles=10)
    with pytest.raises(ValueError, match="No CUDA device available"):
        R.apply_to(np.zeros((16, 16), dtype=np.float32))


def test_angles_constructors():
    a = Angles.uniform_interval(0.0, 1.0, 4)
    np.testing.assert_allclose(a.angles, [0.125, 0.375, 0.625, 0.875])
    np.testing.assert_allclose(a.weights, 0.25)
    b = Angles.intervals([2, 2], [0.0, 2.0], [1.0, 3.0])
    assert len(b) == 4
    with pytest.raises(ValueError):
        Angles.intervals([1], [0.0, 1.0], [1.0])
    c = Angles.from_list([0.0, np.pi / 2, np.pi, 3 * np.pi / 2])
    np.testing.assert_allclose(c.weights, np.pi / 2)
    with pytest.raises(ValueError):
        Angles([0.0, 1.0], [1.0])
    d = Detectors(-10)
    assert d.number == 10 and d.reversed is True


def test_fanbeam_operator_shapes():
    F = Fanbeam((4.0, 2.0), 16, 12)
    assert F.input_shape == (16, 16) and F.output_shape == (23, 12)
    assert F.angles.half_circle is False
    assert repr(F.T) == "Fanbeam.T"
    assert F.state["RE"] == 2.0
    G = Fanbeam(6.0, 16, 12)
    assert G.state["RE"] == 3.0
    with pytest.raises(ValueError):
        Fanbeam((4.0, 0.5), 16, 12)
