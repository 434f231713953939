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


# parallel beam: the half-circle orbits (quarter turn and detector mirror)
RADON_BASE = dict(geometry="radon", img_shape=(40, 40), angles=30, n_detectors=57)
RADON_SYMMETRIC = {
    "plain": {},
    "odd_side_odd_detectors": dict(img_shape=(37, 37), angles=18, n_detectors=53),
    "even_detectors": dict(n_detectors=60),
    "wide_detector": dict(detector_width=3.0, image_width=2.0),
    "bench_256": dict(img_shape=(256, 256), angles=180, n_detectors=363,
                      detector_width=2.0 * np.sqrt(2.0)),
}
RADON_ASYMMETRIC = {
    "not_square": dict(img_shape=(40, 36)),
    "odd_angle_count": dict(angles=31),
    "shifted_detector": dict(detector_shift=0.01),
    "shifted_image": dict(midpoint_shift=(0.02, 0.0)),
    "limited_range": dict(angles=[(30, 0.0, 2.0)]),
}


@pytest.mark.parametrize("name", sorted(RADON_SYMMETRIC))
def test_radon_maps_give_the_four_outputs(name):
    """The oracle's projection of the image looked up through map m, at the
    base angles k < Na/2, equals the outputs (s, k + Na/2), (Ns-1-s, k),
    (Ns-1-s, k + Na/2) of the original image (float64, 1e-12)."""
    from gratopy_gb300.symmetry import radon_half_maps

    ps = host_settings(dict(RADON_BASE, **RADON_SYMMETRIC[name]))
    maps = radon_half_maps(ps.struct, ps.img_shape)
    assert maps is not None
    N = ps.img_shape[0]
    Ns, Na = ps.sinogram_shape
    Q = Na // 2
    img = np.asfortranarray(np.random.default_rng(4).random((N, N)))
    ref = O.forward(img, ps)
    x, y = np.meshgrid(np.arange(N), np.arange(N), indexing="ij")
    want = {1: ref[:, Q:], 2: ref[::-1, :Q], 3: ref[::-1, Q:]}
    for m, (axx, axy, ayx, ayy, cx, cy) in enumerate(maps, start=1):
        turned = np.asfortranarray(img[cx + axx * x + axy * y, cy + ayx * x + ayy * y])
        got = O.forward(turned, ps)[:, :Q]
        assert np.abs(got - want[m]).max() <= 1e-12 * np.abs(want[m]).max(), m


@pytest.mark.parametrize("name", sorted(RADON_ASYMMETRIC))
def test_radon_asymmetric_geometries_are_rejected(name):
    from gratopy_gb300.symmetry import radon_half_maps

    ps = host_settings(dict(RADON_BASE, **RADON_ASYMMETRIC[name]))
    assert radon_half_maps(ps.struct, ps.img_shape) is None


# fan beam: the mirror (reflection through the axis, detector reversed)
MIRROR_SYMMETRIC = {
    "plain": {},
    "reversed_detector": dict(reverse_detector=True),
    "odd_side": dict(img_shape=(37, 37), angles=20),
    "odd_detectors": dict(n_detectors=63),
    "half_circle": dict(angles=[(36, 0.0, np.pi)]),
    "bench": dict(img_shape=(64, 64), angles=360, n_detectors=96, detector_width=400.0,
                  R=400.0, RE=200.0),
}
MIRROR_ASYMMETRIC = {
    "shifted_detector": dict(detector_shift=3.0),
    "shifted_image": dict(midpoint_shift=(1.0, 0.0)),
    "not_square": dict(img_shape=(40, 36)),
    "uneven_angles": dict(angles=[0.0, 0.3, 1.1, 2.0, 4.0]),
}


@pytest.mark.parametrize("name", sorted(MIRROR_SYMMETRIC))
def test_fan_mirror_maps_reversed_views(name):
    """For the mirror (M, c0): the oracle's projection of the image looked up
    through M, at angle b and bin s, equals the original image's projection
    at angle (c0 - b) mod Na and bin Ns - 1 - s (float64, 1e-12)."""
    from gratopy_gb300.symmetry import fan_mirror_map

    ps = host_settings(dict(BASE, **MIRROR_SYMMETRIC[name]))
    found = fan_mirror_map(ps.struct, ps.img_shape)
    assert found is not None
    (axx, axy, ayx, ayy, cx, cy), c0 = found
    assert axx * ayy - axy * ayx == -1  # a reflection
    N = ps.img_shape[0]
    Ns, Na = ps.sinogram_shape
    img = np.asfortranarray(np.random.default_rng(2).random((N, N)))
    sino = O.forward(img, ps)
    x, y = np.meshgrid(np.arange(N), np.arange(N), indexing="ij")
    mx, my = cx + axx * x + axy * y, cy + ayx * x + ayy * y
    assert mx.min() == 0 and mx.max() == N - 1 and my.min() == 0 and my.max() == N - 1
    mirrored = O.forward(np.asfortranarray(img[mx, my]), ps)
    b = np.arange(Na)
    err = np.abs(mirrored[:, b] - sino[::-1, (c0 - b) % Na]).max()
    assert err <= 1e-12 * np.abs(sino).max()


@pytest.mark.parametrize("name", sorted(MIRROR_ASYMMETRIC))
def test_fan_mirror_rejected(name):
    from gratopy_gb300.symmetry import fan_mirror_map

    ps = host_settings(dict(BASE, **MIRROR_ASYMMETRIC[name]))
    assert fan_mirror_map(ps.struct, ps.img_shape) is None
