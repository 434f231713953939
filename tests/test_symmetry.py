"""Quarter-turn symmetry detection (CPU): the index maps returned for a
symmetric fan-beam geometry turn the image so that the float64 oracle's
projection at angle a equals its projection at angle a + m*Na/4 of the
original image; asymmetric geometries are rejected."""

from __future__ import annotations

import numpy as np
import pytest

from gratopy_gb300.symmetry import fan_quarter_maps
from oracle import oracle as O
from tests.helpers import host_settings

BASE = dict(geometry="fanbeam", img_shape=(40, 40), angles=36, n_detectors=64,
            detector_width=40.0, R=70.0, RE=30.0)
SYMMETRIC = {
    "plain": {},
    "reversed_detector": dict(reverse_detector=True),
    "shifted_detector": dict(detector_shift=3.0),
    "odd_side": dict(img_shape=(37, 37), angles=20),
    "large": dict(img_shape=(96, 96), angles=64, n_detectors=140),
}
ASYMMETRIC = {
    "not_square": dict(img_shape=(40, 36)),
    "angles_not_multiple_of_4": dict(angles=34),
    "shifted_image": dict(midpoint_shift=(1.0, 0.0)),
    "half_circle": dict(angles=[(36, 0.0, np.pi)]),
}


@pytest.mark.parametrize("name", sorted(SYMMETRIC))
def test_maps_turn_the_image_between_quarter_angles(name):
    ps = host_settings(dict(BASE, **SYMMETRIC[name]))
    maps = fan_quarter_maps(ps.struct, ps.img_shape)
    assert maps is not None and len(maps) == 3
    N = ps.img_shape[0]
    Q = ps.n_angles // 4
    img = np.asfortranarray(np.random.default_rng(0).random((N, N)))
    sino = O.forward(img, ps)
    x, y = np.meshgrid(np.arange(N), np.arange(N), indexing="ij")
    for m, (axx, axy, ayx, ayy, cx, cy) in enumerate(maps, 1):
        mx, my = cx + axx * x + axy * y, cy + ayx * x + ayy * y
        assert mx.min() == 0 and mx.max() == N - 1 and my.min() == 0 and my.max() == N - 1
        turned = O.forward(np.asfortranarray(img[mx, my]), ps)
        err = np.abs(turned[:, :Q] - sino[:, m * Q:(m + 1) * Q]).max()
        assert err <= 1e-12 * np.abs(sino).max()


@pytest.mark.parametrize("name", sorted(ASYMMETRIC))
def test_asymmetric_geometries_are_rejected(name):
    ps = host_settings(dict(BASE, **ASYMMETRIC[name]))
    assert fan_quarter_maps(ps.struct, ps.img_shape) is None
