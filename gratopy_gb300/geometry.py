"""Host-side projection geometry: per-angle tables and angle parsing.

Restates the table builders of gratopy (``gratopy/gratopy.py``):

* :func:`radon_struct`   -- gratopy.py:380-578
* :func:`fanbeam_struct` -- gratopy.py:706-1003
* :func:`read_angles`    -- gratopy.py:1109-1296

The tables are computed in float64 with the same sequence of numpy operations
as the reference, so the float32/float64 casts are bit-identical to the
reference tables (pinned by tests against fixtures generated from the
reference).  Layout of the per-angle ``ofs`` table: shape ``(8, Na)`` in
Fortran order, i.e. each angle's 8 reals are contiguous in memory -- the
layout the CUDA kernels read as one 32-byte (fp32) record per angle.
"""

from __future__ import annotations

import numpy as np

DTYPES = (np.dtype("float64"), np.dtype("float32"))


def radon_struct(
    queue,
    img_shape,
    angles,
    angle_weights,
    n_detectors=None,
    detector_width=2.0,
    image_width=2.0,
    midpoint_shift=(0.0, 0.0),
    detector_shift=0.0,
):
    """Parallel-beam geometry tables (gratopy.py:380-578).

    ofs rows: 0 X = cos(phi - pi/2)/(ds/dx), 1 Y = sin(phi - pi/2)/(ds/dx),
    2 detector offset, 3 1/X (or 1/Y when the axes are flipped),
    4 angle weight, 5 flip flag, 6-7 unused.
    geo = [delta_x, delta_s, Nx, Ny, Ns, Na].  ``queue`` is accepted for
    signature compatibility and ignored.
    """
    if n_detectors is None:
        nd = int(np.ceil(np.hypot(img_shape[0], img_shape[1])))
    else:
        nd = n_detectors
    # detector pixel width relative to the image pixel width (delta_s/delta_x)
    ratio = detector_width / float(image_width) * max(img_shape) / nd

    delta_x = image_width / float(max(img_shape))
    delta_s = float(detector_width) / nd

    midpoint_domain = (
        np.array([img_shape[0] - 1, img_shape[1] - 1]) / 2.0
        - np.array(midpoint_shift) / delta_x
    )
    midpoint_detectors = (nd - 1.0) / 2.0

    angles = np.asarray(angles)
    X = np.cos(angles - np.pi * 0.5) / ratio
    Y = np.sin(angles - np.pi * 0.5) / ratio
    Xinv = 1.0 / X
    flipped = np.where(abs(X) < abs(Y))
    Xinv[flipped] = 1.0 / Y[flipped]
    flip = np.zeros(Xinv.shape)
    flip[flipped] = 1.0
    offset = (
        midpoint_detectors
        - X * midpoint_domain[0]
        - Y * midpoint_domain[1]
        - detector_shift / delta_s
    )

    n_angles = len(angles)
    sinogram_shape = (nd, n_angles)
    ofs_dict, geo_dict, weights_dict = {}, {}, {}
    for dtype in DTYPES:
        ofs = np.zeros((8, n_angles), dtype=dtype, order="F")
        ofs[0, :] = X
        ofs[1, :] = Y
        ofs[2, :] = offset
        ofs[3, :] = Xinv
        ofs[4, :] = angle_weights
        ofs[5, :] = flip
        ofs_dict[dtype] = ofs
        weights_dict[dtype] = np.array(angle_weights, dtype=dtype)
        geo_dict[dtype] = np.array(
            [delta_x, delta_s, img_shape[0], img_shape[1], nd, n_angles],
            dtype=dtype,
            order="F",
        )
    return {
        "ofs_dict": ofs_dict,
        "img_shape": img_shape,
        "sinogram_shape": sinogram_shape,
        "geo_dict": geo_dict,
        "angle_diff_dict": weights_dict,
    }


def fanbeam_struct(
    queue,
    img_shape,
    angles,
    detector_width,
    source_detector_dist,
    source_origin_dist,
    angle_weights,
    n_detectors=None,
    detector_shift=0.0,
    image_width=None,
    midpoint_shift=(0.0, 0.0),
    reverse_detector=False,
):
    """Fan-beam geometry tables (gratopy.py:706-1003).

    ofs rows: 0-1 detector direction (length delta_s), 2-3 source position
    (length RE), 4-5 foot of the origin on the detector line, 6 angle weight.
    sdpd[s] = sqrt(xi_s^2 + R^2) in pixel units.
    geo = [R, RE, ds/dx, x_mid, y_mid, s_mid, Nx, Ny, Ns, Na, delta_x] with
    distances in image-pixel units.
    """
    detector_width = float(detector_width)
    source_detector_dist = float(source_detector_dist)
    source_origin_dist = float(source_origin_dist)
    midpointshift = np.array(midpoint_shift)
    image_pixels = max(img_shape[0], img_shape[1])

    if n_detectors is None:
        nd = int(np.ceil(np.hypot(img_shape[0], img_shape[1])))
    else:
        nd = n_detectors
    assert isinstance(nd, int), "Number of detectors must be integer"

    midpoint_detectors = (nd - 1.0) / 2.0
    midpoint_detectors = midpoint_detectors - detector_shift * nd / detector_width

    assert source_detector_dist > source_origin_dist, (
        "The origin is not between detector and source"
    )

    if image_width is None:
        # widest square image that stays inside the fan from every direction
        slope = (0.5 * detector_width - abs(detector_shift)) / source_detector_dist
        image_width = 2 * slope * source_origin_dist / np.sqrt(1 + slope**2)
        assert image_width > 0, (
            "The automatism for choosing the image_width"
            + " failed as the image can never"
            + " be fully contained in the fans from all directions "
            + "(most likely due to detector_shift being "
            + "larger than half the detector_width)! "
            + "Please set the image_width parameter by hand!"
        )

    assert (
        image_width * 0.5 * np.sqrt(1 + (min(img_shape) / max(img_shape)) ** 2)
        + np.linalg.norm(midpointshift)
        < source_origin_dist
    ), "The source is not outside the image domain"

    midpoint_x = (img_shape[0] - 1) * 0.5 - (
        midpointshift[0] * image_pixels / float(image_width)
    )
    midpoint_y = (img_shape[1] - 1) * 0.5 - (
        midpointshift[1] * image_pixels / float(image_width)
    )

    # lengths in units of one image pixel
    source_detector_dist *= image_pixels / float(image_width)
    source_origin_dist *= image_pixels / float(image_width)
    detector_width *= image_pixels / float(image_width)

    angles = np.asarray(angles)
    thetaX = np.cos(angles)
    thetaY = np.sin(angles)
    orientation = -1 if reverse_detector else 1
    XD = thetaY * detector_width / nd * orientation
    YD = -thetaX * detector_width / nd * orientation
    Qx = -thetaX * source_origin_dist
    Qy = -thetaY * source_origin_dist
    Dx0 = thetaX * (source_detector_dist - source_origin_dist)
    Dy0 = thetaY * (source_detector_dist - source_origin_dist)

    sinogram_shape = (nd, len(angles))
    ofs_dict, sdpd_dict, geo_dict, weights_dict = {}, {}, {}, {}
    for dtype in DTYPES:
        ofs = np.zeros((8, len(angles)), dtype=dtype, order="F")
        ofs[0, :] = XD
        ofs[1, :] = YD
        ofs[2, :] = Qx
        ofs[3, :] = Qy
        ofs[4, :] = Dx0
        ofs[5] = Dy0
        ofs[6] = angle_weights
        ofs_dict[dtype] = ofs

        xi = (np.arange(0, nd) - midpoint_detectors) * detector_width / nd
        dist = np.sqrt((xi) ** 2 + source_detector_dist**2)
        dist = np.array(dist, dtype=dtype, order="F")
        sdpd = np.zeros((1, len(dist)), dtype=dtype, order="F")
        sdpd[0, :] = dist[:]
        sdpd_dict[dtype] = sdpd

        geo_dict[dtype] = np.array(
            [
                source_detector_dist,
                source_origin_dist,
                detector_width / nd,
                midpoint_x,
                midpoint_y,
                midpoint_detectors,
                img_shape[0],
                img_shape[1],
                sinogram_shape[0],
                sinogram_shape[1],
                image_width / float(max(img_shape)),
            ],
            dtype=dtype,
            order="F",
        )
        weights_dict[dtype] = np.array(angle_weights, dtype=dtype)

    return {
        "img_shape": img_shape,
        "sinogram_shape": sinogram_shape,
        "ofs_dict": ofs_dict,
        "sdpd_dict": sdpd_dict,
        "image_width": image_width,
        "geo_dict": geo_dict,
        "angle_diff_dict": weights_dict,
    }


def _even_out_duplicates(sorted_angles, weights):
    """Share the weight of (numerically) repeated angles equally among them.

    Restates the duplicate-angle pass of gratopy.py:1163-1178: runs of angles
    closer than 1e-6 to the first of the run get the mean weight of the run.
    """
    tol = 0.000001
    na = len(sorted_angles)
    i = 0
    while i < na - 1:
        count = 1
        total = weights[i]
        while abs(sorted_angles[i] - sorted_angles[i + count]) < tol:
            total += weights[i + count]
            count += 1
            if i + count > na - 1:
                break
        mean = total / count
        for j in range(i, i + count):
            weights[j] = mean
        i += count
    return weights


def read_angles(angles, angle_weights, projectionsetting):
    """Parse an angle specification into (angles, angle_weights).

    Restates gratopy.py:1109-1296.  Accepted forms: an int (uniform angles on
    the half circle for parallel beam, full circle for fan beam; negative for
    reversed order), a list/array of angles (full-angle setting, weights from
    neighbour distances on the circle), or limited-angle sections
    ``(n | angles, lower, upper)`` / a list of such tuples.
    """
    is_fan = projectionsetting.is_fan
    is_parallel = projectionsetting.is_parallel
    if np.isscalar(angles):
        na = abs(angles)
        reverse = angles < 0
        if is_fan:
            angles = np.linspace(0, 2 * np.pi, abs(angles) + 1)[:-1]
            if angle_weights is None:
                angles_diff = np.ones(len(angles)) * (2 * np.pi / len(angles))
        if is_parallel:
            angles = np.linspace(0, np.pi, abs(angles) + 1)[:-1]
            if angle_weights is None:
                angles_diff = np.ones(len(angles)) * (np.pi / len(angles))
        if reverse:
            angles = np.flip(angles)
            if angle_weights is None:
                angles_diff = np.flip(angles_diff)
    elif isinstance(angles, (list, np.ndarray)) and np.isscalar(angles[0]):
        na = len(angles)
        angles = np.array(angles)
        period = 2 * np.pi if is_fan else np.pi
        order = np.argsort(angles % period)
        angles_sorted = angles[order] % period
        extended = np.array(
            np.hstack([-period + angles_sorted[-1], angles_sorted, angles_sorted[0] + period])
        )
        angles_diff = 0.5 * (abs(extended[2 : na + 2] - extended[0:na]))
        angles_diff = _even_out_duplicates(angles_sorted, angles_diff)
        unsorted = np.zeros(angles_diff.shape)
        unsorted[order] = angles_diff
        angles_diff = unsorted
    elif isinstance(angles[0], tuple) or isinstance(angles, tuple):
        if isinstance(angles, tuple):
            angles = [angles]
        na = len(angles)
        for section in angles:
            assert isinstance(section, tuple), (
                "When giving angles via tuples for limited angle setting "
                + " all subsets must be given in tuple form!"
            )
            assert len(section) == 3, (
                "When tuples are given for the limited angle setting,"
                + " also angular bounds need to be given, i.e., "
                + "tuple consists of number of angles or angles themselves "
                + "as first entry and lower bound of  angular range as "
                + "second, upper bound as third entry!"
            )
        angles_new = []
        angles_diff = []
        for section in angles:
            if isinstance(section[0], int):
                n = abs(section[0])
                lower, upper = section[1], section[2]
                half_step = (upper - lower) / (n) * 0.5
                current = np.linspace(lower + half_step, upper - half_step, n)
                if section[0] < 0:
                    current = np.flip(current)
            if isinstance(section[0], (list, np.ndarray)):
                current = np.array(section[0])
                lower, upper = section[1], section[2]
            angles_new += list(current)
            if angle_weights is None:
                cur_sorted = np.sort(current)
                order = np.argsort(current)
                extended = np.array(
                    np.hstack([2 * lower - cur_sorted[0], cur_sorted, 2 * upper - cur_sorted[-1]])
                )
                diff = 0.5 * (abs(extended[2 : len(extended)] - extended[0 : len(extended) - 2]))
                diff = _even_out_duplicates(cur_sorted, diff)
                unsorted = np.zeros(diff.shape)
                unsorted[order] = diff
                angles_diff += list(unsorted)
        angles = np.array(angles_new)
        na = len(angles)

    if angle_weights is None:
        angle_weights = np.array(angles_diff)
    elif np.isscalar(angle_weights):
        angle_weights = np.ones(na) * angle_weights
    elif isinstance(angle_weights, (list, np.ndarray)):
        assert na == len(angle_weights), (
            "The angle_weights given by the user do not have the same "
            + "length as the number of angles considered"
        )
        angle_weights = np.array(angle_weights)
    return angles, angle_weights
