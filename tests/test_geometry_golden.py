"""Host geometry against fixtures generated from the reference (CPU only).

tests/golden/make_golden.py produced the fixtures by running gratopy's own
radon_struct / fanbeam_struct / read_angles / ct_shepp_logan / operator.Radon.
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

from gratopy_gb300.geometry import read_angles  # noqa: E402
from gratopy_gb300.phantom import shepp_logan_host  # noqa: E402
from gratopy_gb300.utilities import GeometryType  # noqa: E402
from tests.helpers import (  # noqa: E402
    control_sha256,
    host_settings,
    pinned_control_sha256,
)

TABLES = np.load(GOLDEN / "tables.npz")
ANGLES = np.load(GOLDEN / "angles.npz")


@pytest.mark.parametrize("name", sorted(configs.configs()))
def test_tables_bit_identical(name):
    cfg = configs.configs()[name]
    ps = host_settings(cfg)
    f64, f32 = np.dtype("float64"), np.dtype("float32")
    ref_ofs = TABLES[f"{name}/ofs"]
    np.testing.assert_array_equal(np.asarray(ps.struct["ofs_dict"][f64]), ref_ofs)
    np.testing.assert_array_equal(np.asarray(ps.struct["ofs_dict"][f32]), ref_ofs.astype(f32))
    np.testing.assert_array_equal(np.asarray(ps.struct["geo_dict"][f64]), TABLES[f"{name}/geo"])
    np.testing.assert_array_equal(np.asarray(ps.angles, dtype=f64), TABLES[f"{name}/angles"])
    np.testing.assert_array_equal(ps.angle_weights, TABLES[f"{name}/weights"])
    assert float(ps.image_width) == float(TABLES[f"{name}/image_width"])
    np.testing.assert_array_equal([ps.delta_x, ps.delta_s, ps.delta_ratio], TABLES[f"{name}/delta"])
    if ps.is_fan:
        np.testing.assert_array_equal(np.asarray(ps.struct["sdpd_dict"][f64]).reshape(-1),
                                      TABLES[f"{name}/sdpd"])


@pytest.mark.parametrize("j", range(len(configs.angle_variants())))
@pytest.mark.parametrize("geom", ["radon", "fanbeam"])
@pytest.mark.parametrize("wname,w", [("auto", None), ("scalar", 1.0)])
def test_read_angles_matches_reference(j, geom, wname, w):
    spec = configs.angle_variants()[j]
    fake = type("PS", (), {"is_fan": geom == "fanbeam", "is_parallel": geom == "radon"})()
    a, wts = read_angles(spec, w, fake)
    np.testing.assert_array_equal(np.atleast_1d(np.asarray(a, dtype=np.float64)),
                                  ANGLES[f"{j}/{geom}/{wname}/angles"])
    np.testing.assert_array_equal(np.atleast_1d(np.asarray(wts, dtype=np.float64)),
                                  ANGLES[f"{j}/{geom}/{wname}/weights"])


def test_angle_variants_expected_values():
    """Spot values stated in gratopy tests/test_radon.py:904-1077."""
    fake = type("PS", (), {"is_fan": False, "is_parallel": True})()
    a, w = read_angles(100, None, fake)
    np.testing.assert_allclose(a, np.linspace(0, np.pi, 101)[:-1])
    np.testing.assert_allclose(w, np.pi / 100)
    a, w = read_angles([(1, 0, np.pi)], None, fake)
    np.testing.assert_allclose(a, [np.pi / 2])
    np.testing.assert_allclose(w, [np.pi])
    a, w = read_angles([0, 0, np.pi / 2, np.pi / 2, np.pi / 2, np.pi * 2 / 3, 0], None, fake)
    np.testing.assert_allclose(w[0], (np.pi / 4 + np.pi / 6) / 3)
    np.testing.assert_allclose(w[5], np.pi / 6 + np.pi / 12)
    with pytest.raises(AssertionError):
        read_angles(10, np.ones(9), fake)


@pytest.mark.parametrize("key", ["64x64", "40x56", "150x150"])
def test_phantom_matches_reference(key):
    M, N = (int(v) for v in key.split("x"))
    ph = np.load(GOLDEN / "phantom.npz")
    np.testing.assert_array_equal(shepp_logan_host((M, N)), ph[key])
    np.testing.assert_array_equal(shepp_logan_host((M, N), modified=False), ph[key + "_orig"])


def test_control_numbers_regenerate_reference_rng():
    assert control_sha256() == pinned_control_sha256()


def test_placeholders_match_reference():
    from gratopy_gb300.operator import Radon
    from gratopy_gb300.utilities import Detectors, ExtentPlaceholder, ImageDomain

    cases = json.loads((GOLDEN / "placeholders.json").read_text())
    assert len(cases) == 240
    for c in cases:
        ph = ExtentPlaceholder(c["placeholder"])
        Ny = int(c["side_ratio"] * 400)
        ic = tuple(c["image_center"])
        dc = c["detector_center"]

        def make():
            if c["side"] == "detector":
                return Radon(ImageDomain(size=(400, Ny), center=ic, extent=2.0), 180,
                             Detectors(number=100, center=dc, extent=ph))
            return Radon(ImageDomain(size=(400, Ny), center=ic, extent=ph), 180,
                         Detectors(number=100, center=dc, extent=2.0))

        if c["extent"] is None:
            with pytest.raises(ValueError):
                make()
        else:
            r = make()
            got = r.detectors.extent if c["side"] == "detector" else r.image_domain.extent
            assert float(got) == pytest.approx(c["extent"], rel=1e-12, abs=1e-12), c


def test_projection_settings_attributes_without_device():
    """ProjectionSettings builds its tables on the host; the device is touched lazily."""
    import gratopy_gb300 as gg

    ps = gg.ProjectionSettings(None, gg.FANBEAM, (600, 600, 2), 180, n_detectors=300,
                               detector_width=400.0, R=752.0, RE=200.0)
    assert ps.img_shape == (600, 600) and ps.sinogram_shape == (300, 180)
    assert ps.is_fan and not ps.is_parallel and ps.geometry == GeometryType.FANBEAM
    ref = TABLES["fan_types/delta"]
    assert [ps.delta_x, ps.delta_s, ps.delta_ratio] == list(ref)
    with pytest.raises(AssertionError):
        gg.ProjectionSettings(None, gg.FANBEAM, (64, 64), 10, R=None, RE=3.0)
    with pytest.raises(AssertionError):
        gg.ProjectionSettings(None, gg.FANBEAM, (64, 64), 10, R=3.0, RE=4.0)
