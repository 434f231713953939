"""Geometry configurations shared by the fixture generator and the tests.

Each entry mirrors a ``ProjectionSettings`` call of gratopy's test-suite
(file:line in gratopy's ``tests/``) or a benchmark workload.  ``geometry`` is
"radon" or "fanbeam"; the remaining keys are ``ProjectionSettings``
keyword arguments.
"""

from __future__ import annotations

import numpy as np


def _radon_limited():
    # tests/test_radon.py:443-470
    na = 180
    delta = np.pi * 3 / 4 / (na - 1)
    incorrect = np.linspace(0, np.pi * 3 / 4.0, na) + np.pi / 8
    correct = (np.linspace(0, np.pi * 3 / 4.0, na) + np.pi / 8, np.pi / 8 - delta / 2,
               np.pi * 7 / 8 + delta / 2)
    return correct, incorrect, delta


def _fan_limited():
    # tests/test_fanbeam.py:476-503
    n1 = 180
    a1, b1 = np.pi / 8.0, np.pi / 8 + np.pi * 3 / 4.0
    angles1 = np.linspace(a1, b1, n1)
    d1 = (b1 - a1) / (n1 - 1) * 0.5
    n2 = 90
    a2, b2 = 5.0 / 4 * np.pi, 2 * np.pi
    d2 = (b2 - a2) / (n2 - 1) * 0.5
    angles2 = np.linspace(a2, b2, n2)[:-1]
    incorrect = list(angles1) + list(angles2)
    correct = [(angles1, a1 - d1, b1 + d1), (angles2, a2 - d2, b2 - d2)]
    return correct, incorrect


WALNUT_ANGLES = -np.linspace(0, 2 * np.pi, 121)[:-1]


def configs() -> dict:
    rl_correct, rl_incorrect, rl_delta = _radon_limited()
    fl_correct, fl_incorrect = _fan_limited()
    c = {
        # tests/test_radon.py:63-72
        "radon_projection": dict(geometry="radon", img_shape=(1200, 1200), angles=360,
                                 n_detectors=600, image_width=4.0, detector_width=4.0,
                                 detector_shift=0),
        # tests/test_radon.py:182-188
        "radon_types": dict(geometry="radon", img_shape=(600, 600), angles=180, n_detectors=300),
        # tests/test_radon.py:286-295
        "radon_weighting": dict(geometry="radon", img_shape=(900, 900), angles=30,
                                n_detectors=500, detector_width=4.0, image_width=4.0),
        # tests/test_radon.py:365-367
        "radon_adjoint": dict(geometry="radon", img_shape=(400, 400), angles=180, n_detectors=230),
        # tests/test_radon.py:472-500
        "radon_limited_correct": dict(geometry="radon", img_shape=(1200, 1200), angles=rl_correct,
                                      n_detectors=360, detector_width=2.0, detector_shift=0.0),
        "radon_limited_incorrect": dict(geometry="radon", img_shape=(1200, 1200),
                                        angles=rl_incorrect, n_detectors=360,
                                        detector_width=2.0, detector_shift=0.0),
        "radon_limited_correct2": dict(geometry="radon", img_shape=(1200, 1200),
                                       angles=rl_incorrect, n_detectors=360, detector_width=2.0,
                                       detector_shift=0.0, angle_weights=rl_delta),
        # tests/test_radon.py:641-642
        "radon_nonquadratic": dict(geometry="radon", img_shape=(1200, 800), angles=360,
                                   n_detectors=600),
        # tests/test_radon.py:824-836
        "radon_midpoint": dict(geometry="radon", img_shape=(1200, 1200), angles=360,
                               n_detectors=600, image_width=3.0, detector_width=2.0,
                               midpoint_shift=[0.0, 0.4]),
        # tests/test_fanbeam.py:64-74
        "fan_projection": dict(geometry="fanbeam", img_shape=(1200, 1200), angles=360,
                               detector_width=400.0, RE=200.0, R=752.0, n_detectors=600),
        # tests/test_fanbeam.py:183-192
        "fan_types": dict(geometry="fanbeam", img_shape=(600, 600), angles=180,
                          detector_width=400.0, RE=200.0, R=752.0, n_detectors=300),
        # tests/test_fanbeam.py:380-392
        "fan_adjoint": dict(geometry="fanbeam", img_shape=(400, 400), angles=360, n_detectors=230,
                            detector_width=83.0, detector_shift=0.0, midpoint_shift=[0.0, 0.0],
                            R=900.0, RE=300.0, image_width=None),
        # tests/test_fanbeam.py:505-540
        "fan_limited_correct": dict(geometry="fanbeam", img_shape=(1200, 1200), angles=fl_correct,
                                    n_detectors=360, image_width=2.0, R=5.0, RE=2.0,
                                    detector_width=6.0, detector_shift=0),
        "fan_limited_incorrect": dict(geometry="fanbeam", img_shape=(1200, 1200),
                                      angles=fl_incorrect, n_detectors=360, image_width=2.0,
                                      R=5.0, RE=2.0, detector_width=6.0, detector_shift=0),
        # tests/test_fanbeam.py:696-708
        "fan_midpoint": dict(geometry="fanbeam", img_shape=(1200, 1200), angles=360,
                             n_detectors=600, image_width=2.0, R=5.0, RE=3.0, detector_width=6.0,
                             detector_shift=0.0, midpoint_shift=[0, 0.5]),
        # tests/test_fanbeam.py:1401-1414 (non-square fan)
        "fan_nonquadratic": dict(geometry="fanbeam", img_shape=(1200, 800), angles=360,
                                 n_detectors=600, image_width=None, R=5.0, RE=3.0,
                                 detector_width=5.0, detector_shift=0.0, midpoint_shift=[0, 0.0]),
        # tests/test_radon.py:730-732 and tests/test_fanbeam.py:1508-1516 (sparse-matrix cases)
        "radon_sparse": dict(geometry="radon", img_shape=(150, 150), angles=30, n_detectors=100),
        "fan_sparse": dict(geometry="fanbeam", img_shape=(150, 150), angles=30,
                           detector_width=400.0, R=752.0, RE=200.0, n_detectors=100),
        # tests/test_fanbeam.py:1120-1131 (walnut, 600^2) and :1281-1292 (400^2)
        "fan_walnut600": dict(geometry="fanbeam", img_shape=(600, 600), angles=WALNUT_ANGLES,
                              detector_width=114.8, R=300.0, RE=110.0, n_detectors=328,
                              detector_shift=0.27, reverse_detector=True),
        "fan_walnut400": dict(geometry="fanbeam", img_shape=(400, 400), angles=WALNUT_ANGLES,
                              detector_width=114.8, R=300.0, RE=110.0, n_detectors=328,
                              detector_shift=0.27, reverse_detector=True),
        # benchmark workloads: Radon 256^2 / 180 / 363 and fan 512^2 / 360 / 768
        "bench_radon256": dict(geometry="radon", img_shape=(256, 256), angles=180,
                               n_detectors=363, detector_width=2.0 * np.sqrt(2.0), image_width=2.0),
        "bench_fan512": dict(geometry="fanbeam", img_shape=(512, 512), angles=360,
                             n_detectors=768, detector_width=400.0, RE=200.0, R=400.0,
                             image_width=0.9 * (2 * 0.5 * 200.0 / np.sqrt(1 + 0.25))),
    }
    # tests/test_fanbeam.py:787-856: six shifted geometries, Radon and fan
    orient = [(0, 0, 0), (50, 0, 0), (0, 20, 0), (0, -20, 0), (0, 0, 30), (0, 0, -30)]
    for j, (dshift, mx, my) in enumerate(orient):
        c[f"orient_fan_{j}"] = dict(geometry="fanbeam", img_shape=(600, 600), angles=360,
                                    detector_width=170.0, RE=200.0, R=350, n_detectors=300,
                                    detector_shift=dshift, image_width=94.39,
                                    midpoint_shift=[mx, my])
        c[f"orient_par_{j}"] = dict(geometry="radon", img_shape=(600, 600), angles=360,
                                    image_width=94.39, detector_width=94.39, n_detectors=300,
                                    detector_shift=dshift, midpoint_shift=[mx, my])
    return c


def angle_variants() -> list:
    """Angle specifications of tests/test_radon.py:904-1077 (inputs only)."""
    v = []
    v.append(100)
    v.append(np.linspace(0, np.pi, 101)[:-1])
    three = (list(np.linspace(0, np.pi / 3, 101)[:-1])
             + list(np.linspace(np.pi / 3, np.pi * 2.0 / 3, 51)[:-1])
             + list(np.linspace(np.pi * 2 / 3, np.pi, 101)[:-1]))
    v.append(three)
    v.append(np.array(three))
    v.append([
        (list(np.linspace(0, np.pi / 2, 101)[:-1] + np.pi / 4 / 100), 0, np.pi / 2),
        (50, np.pi / 2, np.pi * 3 / 4),
        (np.linspace(np.pi * 3 / 4, np.pi, 51)[:-1] + np.pi / 4 / 100, np.pi * 3 / 4, np.pi),
    ])
    v.append([(50, 0, np.pi / 3), (50, np.pi * 2 / 3, np.pi)])
    v.append([(1, 0, np.pi)])
    v.append(np.linspace(0, 2 * np.pi, 101)[:-1])
    v.append([(np.linspace(0, 2 * np.pi, 101)[:-1] + np.pi / 100, 0, 2 * np.pi)])
    v.append(-np.linspace(0, np.pi, 101)[:-1])
    v.append((-100, 0, np.pi))
    v.append(-100)
    v.append(([0, 0, np.pi / 2, np.pi / 2, np.pi / 2, np.pi * 2 / 3, 0], 0, np.pi))
    v.append([0, 0, np.pi / 2, np.pi / 2, np.pi / 2, np.pi * 2 / 3, 0])
    return v
