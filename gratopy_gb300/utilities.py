"""Geometry descriptions for the operator API (gratopy/utilities.py:15-580).

:class:`GeometryType`, :class:`Angles`, :class:`Detectors`,
:class:`ImageDomain`, :class:`ExtentPlaceholder` and the half-circle extent
formulas that resolve a FULL/VALID placeholder from the other extent.  Pure
host Python with the reference's semantics and error types.
"""

from __future__ import annotations

from dataclasses import dataclass
from enum import Enum
from typing import Union

import numpy as np

Numeric = Union[float, int, np.integer, np.floating]


class ExtentPlaceholder(Enum):
    """Symbolic image/detector extents (utilities.py:15-41).

    FULL: detector -- smallest extent such that every ray through the image
    hits the detector; image -- largest extent with the same property.
    VALID: detector -- largest extent such that every ray hitting the
    detector passes through the image; image -- smallest such extent.
    """

    FULL = "full"
    VALID = "valid"


class GeometryType(Enum):
    """Projection geometry (utilities.py:44-50)."""

    RADON = "radon"
    FANBEAM = "fanbeam"


def _natural_weights(angles: np.ndarray, period: float) -> np.ndarray:
    """Half the distance between circular neighbours; equal share for repeats."""
    order = np.argsort(angles % period)
    srt = angles[order] % period
    ext = np.array(np.hstack([-period + srt[-1], srt, srt[0] + period]))
    na = len(srt)
    w = 0.5 * (abs(ext[2 : na + 2] - ext[0:na]))
    tol = 0.000001
    i = 0
    while i < na - 1:
        count = 1
        total = w[i]
        while abs(srt[i] - srt[i + count]) < tol:
            total += w[i + count]
            count += 1
            if i + count > na - 1:
                break
        for j in range(i, i + count):
            w[j] = total / count
        i += count
    w[order] = w
    return w


class Angles:
    """Projection angles (radians) with their weights (utilities.py:53-250)."""

    def __init__(self, angles, weights, half_circle: bool = False):
        angles = np.asarray(angles)
        weights = np.asarray(weights)
        if len(angles) != len(weights):
            raise ValueError("Angles and weights must have the same length.")
        self.angles = angles
        self.weights = weights
        self.half_circle = half_circle

    def __repr__(self):
        return f"Angles({self.angles}, weights={self.weights})"

    def __len__(self):
        return len(self.angles)

    @staticmethod
    def sparse(number: int, half_circle: bool = False) -> "Angles":
        """Equispaced angles on [0, pi) or [0, 2pi), all weights 1."""
        top = np.pi if half_circle else 2 * np.pi
        angles = np.linspace(0, top, number, endpoint=False)
        return Angles(angles=angles, weights=np.ones_like(angles), half_circle=half_circle)

    @staticmethod
    def uniform(number: int, half_circle: bool = False) -> "Angles":
        """Equispaced angles with the uniform weight period/number."""
        top = np.pi if half_circle else 2 * np.pi
        out = Angles.sparse(number, half_circle=half_circle)
        out.weights = out.weights * (top / number)
        return out

    @staticmethod
    def uniform_interval(start: float, end: float, number: int,
                         half_circle: bool = False) -> "Angles":
        """Midpoints of ``number`` equal cells of [start, end]."""
        half = abs(end - start) / (2 * number)
        angles = np.linspace(start + half, end - half, number)
        return Angles(angles=angles, weights=2 * half * np.ones_like(angles), half_circle=half_circle)

    @staticmethod
    def intervals(number_list, start_list, end_list, half_circle: bool = False) -> "Angles":
        """Concatenation of :meth:`uniform_interval` samplings."""
        if not len(number_list) == len(start_list) == len(end_list):
            raise ValueError("All input lists must have the same length.")
        angles, weights = [], []
        for n, start, end in zip(number_list, start_list, end_list):
            part = Angles.uniform_interval(start, end, n, half_circle=half_circle)
            angles.extend(part.angles)
            weights.extend(part.weights)
        return Angles(angles=np.array(angles), weights=np.array(weights), half_circle=half_circle)

    @staticmethod
    def from_list(angles, half_circle: bool = False) -> "Angles":
        """Explicit angles with natural (neighbour-distance) weights."""
        angles = np.asarray(angles)
        period = np.pi if half_circle else 2 * np.pi
        return Angles(angles=angles, weights=_natural_weights(angles, period), half_circle=half_circle)


@dataclass
class Detectors:
    """Detector line: pixel count, extent, centre shift, orientation."""

    number: int
    extent: Union[float, ExtentPlaceholder] = ExtentPlaceholder.FULL
    center: float = 0.0
    reversed: bool = False

    def __init__(self, number: int, extent=ExtentPlaceholder.FULL, center: float = 0.0,
                 reversed: bool | None = None):
        self.number = abs(number)
        self.extent = extent
        self.center = center
        self.reversed = (number < 0) if reversed is None else reversed


@dataclass
class ImageDomain:
    """Image grid size, physical extent (longer side) and centre shift."""

    size: tuple
    extent: Union[float, ExtentPlaceholder] = 2.0
    center: tuple = (0.0, 0.0)

    def __init__(self, size, extent=2.0, center=(0.0, 0.0)):
        if isinstance(size, (int, np.integer)):
            size = (int(size), int(size))
        self.size = tuple(size)
        self.extent = extent
        self.center = center


# ---------------------------------------------------------------------------
# Half-circle extent formulas (phi in [0, pi]); utilities.py:353-580.
# The sinogram coordinate of a point (x, y) is s(phi) = x sin(phi) - y cos(phi).
# ---------------------------------------------------------------------------


def _solve_quadratic(a: float, b: float, d: float) -> tuple[float, float]:
    """Roots x1 <= x2 of a x^2 + b x + d (NaNs if complex)."""
    disc = b**2 - 4 * a * d
    if disc < 0:
        return (float("nan"), float("nan"))
    r = np.sqrt(disc)
    return ((-b - r) / (2 * a), (-b + r) / (2 * a))


def _select_extent_from_linear_case(lower_root, upper_root, linear_bound):
    if upper_root <= linear_bound:
        return upper_root
    if lower_root <= linear_bound:
        return linear_bound
    return None


def _point_image_fits_detector_halfcircle(M, Dd) -> bool:
    """Whether the degenerate image (its centre only) projects inside the detector."""
    (Md, Mx, My) = M
    r = np.sqrt(Mx**2 + My**2)
    sgn = 1.0 if Mx >= 0 else -1.0
    return r <= sgn * Md + Dd / 2 and abs(My) <= Dd / 2 - sgn * Md


def _select_extent_from_case_a(x1, x2, y1, y2):
    if (y2 <= x2) and (x1 <= y2):
        return y2
    if (x2 <= y2) and (y1 <= x2):
        return x2
    return None


def full_detector_given_image_halfcircle(M, D) -> float:
    """Smallest detector width such that every ray through the image hits it."""
    (Md, Mx, My) = M
    (Dx, Dy) = D
    # rotate so that the extrema formulas for a cos + b sin apply
    (Mx, My) = (-My, Mx)
    (Dx, Dy) = (Dy, Dx)
    if My >= -Dy / 2:
        hi = np.sqrt((abs(Mx) + Dx / 2) ** 2 + (My + Dy / 2) ** 2)
    else:
        hi = abs(Mx) + Dx / 2
    if My <= Dy / 2:
        lo = -np.sqrt((abs(Mx) + Dx / 2) ** 2 + (My - Dy / 2) ** 2)
    else:
        lo = -abs(Mx) - Dx / 2
    return 2 * max(Md - lo, hi - Md)


def full_image_given_detector_halfcircle(M, Dd, c: float = 1.0):
    """Largest image (Dx, Dy=Dx/c) whose every ray hits the detector, or None."""
    (Md, Mx, My) = M
    if not _point_image_fits_detector_halfcircle(M, Dd):
        return None
    a1 = (1 + c**2) / (4 * c**2)
    b1 = abs(My) / c + Mx
    d1 = -((Md + Dd / 2) ** 2) + Mx**2 + My**2
    (x1, x2) = _solve_quadratic(a1, b1, d1)
    a2 = (1 + c**2) / (4 * c**2)
    b2 = abs(My) / c - Mx
    d2 = -((Md - Dd / 2) ** 2) + Mx**2 + My**2
    (y1, y2) = _solve_quadratic(a2, b2, d2)
    Dx = _select_extent_from_case_a(x1, x2, y1, y2)
    if Dx is not None and Dx >= 2 * abs(Mx):
        return (Dx, Dx / c)
    if Mx < 0:
        z = (Md + Dd / 2 - abs(My)) * 2 * c
        Dx = _select_extent_from_linear_case(y1, y2, z)
    elif Mx > 0:
        z = (Dd / 2 - Md - abs(My)) * 2 * c
        Dx = _select_extent_from_linear_case(x1, x2, z)
    else:
        return None
    if Dx is None or Dx < 0:
        return None
    return (Dx, Dx / c)


def valid_image_given_detector_halfcircle(M, Dd, c: float = 1.0):
    """Smallest image (Dx, Dy) such that every detector ray passes through it."""
    (Md, Mx, My) = M
    Dx = 2 * max(Mx - Md + Dd / 2, -Mx + Md + Dd / 2)
    Dy = 2 * max(abs(Md) + Dd / 2 - My, abs(Md) + Dd / 2 + My)
    Dx = max(Dx, c * Dy)
    return (Dx, Dx / c)


def valid_detector_given_image_halfcircle(M, D):
    """Largest detector width such that every ray hitting it crosses the image."""
    (Md, Mx, My) = M
    (Dx, Dy) = D
    Dd = 2 * min(-Mx + Dx / 2 + Md, Mx - Md + Dx / 2, My - abs(Md) + Dy / 2,
                 -My - abs(Md) + Dy / 2)
    if Dd <= 0:
        return None
    return Dd
