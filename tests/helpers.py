"""Test helpers: gratopy's control-number check, phantoms, settings factories.

The control-number mechanism restates gratopy's tests/helpers.py:38-110: a
fixed list of 1000 (index, factor) pairs -- drawn from
``numpy.random.default_rng(1)`` exactly as gratopy's tests/rng.txt was
(helpers.py:13-35; the regenerated list is pinned against that file's
SHA-256) -- gives the number sum_i factor_i * data[idx_i], compared with
the reference's hard-coded value at rtol 1e-3.
"""

from __future__ import annotations

import hashlib
import json
from functools import lru_cache
from pathlib import Path

import numpy as np

from gratopy_gb300.geometry import fanbeam_struct, radon_struct, read_angles
from gratopy_gb300.phantom import shepp_logan_host
from gratopy_gb300.utilities import GeometryType

GOLDEN = Path(__file__).resolve().parent / "golden"


@lru_cache(maxsize=1)
def control_lists():
    m, M = 1000, 2000
    rng = np.random.default_rng(1)
    lists = [rng.integers(0, M, m), rng.integers(0, M, m), rng.integers(0, M, m),
             rng.normal(0, 1, m), rng.integers(0, M, m), rng.integers(0, M, m)]
    return lists


def control_text() -> str:
    lists = control_lists()
    return "".join(str(lists[j][i]) + "\n" for j in range(6) for i in range(1000))


def control_sha256() -> str:
    return hashlib.sha256(control_text().encode()).hexdigest()


def pinned_control_sha256() -> str:
    return json.loads((GOLDEN / "control_rng.json").read_text())["rng_txt_sha256"]


def control_number(data: np.ndarray, dims, classified: str) -> float:
    """sum_i factor_i * data[idx_i] with gratopy's index lists (helpers.py:63-99)."""
    Nx, Ny, Ns, Na, Nz = dims
    s, phi, z, factors, x, y = control_lists()
    factors = [float(f) for f in factors]
    if classified == "img":
        v1 = [int(a) % Nx for a in x]
        v2 = [int(a) % Ny for a in y]
    else:
        v1 = [int(a) % Ns for a in s]
        v2 = [int(a) % Na for a in phi]
    v3 = [int(a) % Nz for a in z]
    data = np.asarray(data)
    if Nz == 1:
        data = data.reshape(data.shape[0], data.shape[1], 1)
    total = 0
    for i in range(1000):
        total += factors[i] * data[v1[i], v2[i], v3[i]]
    return total


def assert_control(data, dims, expected, classified, name, rtol=1e-3):
    expected = np.asarray(data).dtype.type(expected)
    got = control_number(data, dims, classified)
    assert abs(got - expected) < abs(expected) * rtol, (
        f"control number of {name}: expected {expected}, got {got}"
    )


def create_phantoms(N: int, dtype="float32", order="F") -> np.ndarray:
    """Shepp-Logan scaled to max 255 stacked with a two-bar image (helpers.py:114-134)."""
    dtype = np.dtype(dtype)
    A = shepp_logan_host(N, dtype=dtype)
    A = A * (dtype.type(255) / A.max())
    B = np.empty(A.shape, dtype=dtype)
    B[:] = 255 - 120
    B[int(N / 3):int(2 * N / 3)] = 0
    B[0:int(N / 4)] = 0
    B[int(N - N / 4):N] = 0
    return np.require(np.stack([A, B], axis=-1), dtype, order)


class HostSettings:
    """Host-only geometry bundle with the attributes the oracle reads.

    Built by the same table functions as ``gratopy_gb300.ProjectionSettings``
    (no device needed), so the CPU suite runs without CUDA.
    """

    def __init__(self, geometry, img_shape, angles, n_detectors=None, angle_weights=None,
                 detector_width=2.0, image_width=None, R=None, RE=None, detector_shift=0.0,
                 midpoint_shift=(0.0, 0.0), reverse_detector=False):
        self.geometry = GeometryType(geometry)
        self.img_shape = tuple(img_shape[:2])
        angles, weights = read_angles(angles, angle_weights, self)
        self.angles, self.n_angles = angles, len(angles)
        self.n_detectors = (int(np.ceil(np.hypot(*self.img_shape))) if n_detectors is None
                            else n_detectors)
        self.sinogram_shape = (self.n_detectors, self.n_angles)
        if self.is_fan:
            self.struct = fanbeam_struct(None, self.img_shape, angles, detector_width, R, RE, weights,
                                         self.n_detectors, detector_shift, image_width,
                                         midpoint_shift, reverse_detector)
            self.image_width = self.struct["image_width"]
            self.delta_x = float(self.image_width) / max(self.img_shape)
            self.delta_s = float(detector_width) / self.n_detectors
        else:
            self.image_width = 2.0 if image_width is None else float(image_width)
            self.struct = radon_struct(None, self.img_shape, angles, weights, self.n_detectors,
                                       detector_width, self.image_width, midpoint_shift,
                                       detector_shift)
            self.delta_x = self.image_width / max(self.img_shape)
            self.delta_s = detector_width / self.n_detectors
        self.delta_ratio = self.delta_s / self.delta_x
        self.angle_weights = np.asarray(self.struct["angle_diff_dict"][np.dtype("float64")]).copy()

    @property
    def is_fan(self):
        return self.geometry == GeometryType.FANBEAM

    @property
    def is_parallel(self):
        return self.geometry == GeometryType.RADON


def host_settings(cfg: dict) -> HostSettings:
    cfg = dict(cfg)
    geometry = cfg.pop("geometry")
    img_shape = cfg.pop("img_shape")
    angles = cfg.pop("angles")
    return HostSettings(geometry, img_shape, angles, **cfg)


def device_settings(cfg: dict, device):
    import gratopy_gb300 as gg

    cfg = dict(cfg)
    geometry = gg.RADON if cfg.pop("geometry") == "radon" else gg.FANBEAM
    img_shape = cfg.pop("img_shape")
    angles = cfg.pop("angles")
    return gg.ProjectionSettings(device, geometry, img_shape, angles, **cfg)


def walnut_sinogram(dtype="float32") -> np.ndarray:
    """gratopy's walnut sinogram as matplotlib reads it: raw / 65535, shape (328, 120)."""
    raw = np.load(GOLDEN / "walnut_sinogram.npz")["raw"]
    return (raw.astype(np.float32) / np.float32(65535.0)).astype(dtype)


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
