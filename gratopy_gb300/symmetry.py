"""Quarter-turn symmetry of fan-beam angle sets.

With a square image centred on the rotation axis and angles equispaced over
the full circle in a multiple of 4, the angle a + m*Na/4 sees the pixel grid
exactly as angle a sees it after a quarter turn (m = 1), a half turn (2) or a
three-quarter turn (3).  Then, for every detector bin s,

    sino[s, a + m Na/4] = sum_P img(S_m^-1 P) K(a, P; s),

so the forward projection can evaluate the interpolation weights K of a
candidate pixel once for angle a and apply them to four pixels, one per
angle of the quarter-turn orbit.  This module finds the index maps S_m^-1 by
evaluating the geometry (detector coordinate and distance weight of the
fan-beam kernels, fanbeam.cl:290-391) in float64 for every base angle on
sample pixels, and returns None when any check fails.
"""

from __future__ import annotations

import numpy as np

# the 8 signed permutations of the plane, as (S00, S01, S10, S11)
_MAPS = [(1, 0, 0, 1), (-1, 0, 0, -1), (0, -1, 1, 0), (0, 1, -1, 0),
         (-1, 0, 0, 1), (1, 0, 0, -1), (0, 1, 1, 0), (0, -1, -1, 0)]


def _sample_pixels(N: int, rng_seed: int = 0) -> tuple[np.ndarray, np.ndarray]:
    if N <= 48:
        x, y = np.meshgrid(np.arange(N), np.arange(N), indexing="ij")
        return x.ravel().astype(np.float64), y.ravel().astype(np.float64)
    rng = np.random.default_rng(rng_seed)
    x = np.concatenate([[0, 0, N - 1, N - 1, N // 2], rng.integers(0, N, 251)])
    y = np.concatenate([[0, N - 1, 0, N - 1, N // 3], rng.integers(0, N, 251)])
    return x.astype(np.float64), y.astype(np.float64)


def fan_quarter_maps(struct, img_shape, atol_bins: float = 1e-6, rtol_t: float = 1e-9):
    """Index maps of the quarter-turn orbit of a fan-beam geometry, or None.

    Returns a list of three tuples ``(Axx, Axy, Ayx, Ayy, Cx, Cy)``, one per
    m = 1, 2, 3: the pixel of array indices ``(x, y)`` seen by base angle a
    corresponds, for angle a + m*Na/4, to the pixel
    ``(Cx + Axx*x + Axy*y, Cy + Ayx*x + Ayy*y)``.
    """
    Nx, Ny = (int(v) for v in img_shape)
    ofs = np.asarray(struct["ofs_dict"][np.dtype("float64")], dtype=np.float64)
    geo = np.asarray(struct["geo_dict"][np.dtype("float64")], dtype=np.float64)
    Na = ofs.shape[1]
    if Nx != Ny or Na < 4 or Na % 4 != 0:
        return None
    c = (Nx - 1) * 0.5
    if geo[3] != c or geo[4] != c:  # image not centred on the rotation axis
        return None
    R, RE, dxi, mid_det = geo[0], geo[1], geo[2], geo[5]
    Q = Na // 4
    px, py = _sample_pixels(Nx)
    px, py = px - c, py - c

    def u_t(a, X, Y):
        XD, YD, Qx, Qy, Dx0, Dy0 = (ofs[k, a][:, None] for k in range(6))
        t = ((Dx0 - Qx) * X + (Dy0 - Qy) * Y) / (R * R) + RE / R
        ss = (XD * X + YD * Y) / (dxi * dxi)
        return ss / t + mid_det, t

    base = np.arange(Q)
    maps = []
    for m in (1, 2, 3):
        u1, t1 = u_t(base + m * Q, px[None, :], py[None, :])
        found = None
        for S in _MAPS:
            X = S[0] * px + S[1] * py
            Y = S[2] * px + S[3] * py
            u0, t0 = u_t(base, X[None, :], Y[None, :])
            if (np.all(np.abs(u1 - u0) <= atol_bins)
                    and np.all(np.abs(t1 - t0) <= rtol_t * np.abs(t1))):
                found = S
                break
        if found is None:
            return None
        # the load for angle a + m Q at base candidate P is img(S^-1 P), S^-1 = S^T
        Axx, Axy, Ayx, Ayy = found[0], found[2], found[1], found[3]
        Cx = int(round(c * (1 - Axx - Axy)))
        Cy = int(round(c * (1 - Ayx - Ayy)))
        maps.append((Axx, Axy, Ayx, Ayy, Cx, Cy))
    return maps


def fan_mirror_map(struct, img_shape, atol_bins: float = 1e-6, rtol_t: float = 1e-9):
    """Mirror symmetry of a fan-beam geometry, or None.

    With a square image centred on the rotation axis and a detector centred
    on the central ray, a reflection M of the grid through the rotation axis
    maps the view of angle b to the view of angle c0 - b with the detector
    reversed: u(c0 - b, M P) = Ns - 1 - u(b, P) with the same distance
    weight, for every angle b (angles equispaced over the full circle pair
    up this way about the mirror axis).  Then

        sino[Ns-1-s, c0 - b] = sum_P img(M P) K(b, P; s),

    so a forward projection that has the weights K of angle b can fill the
    mirrored bin of angle c0 - b as well.  Returns ``((Axx, Axy, Ayx, Ayy,
    Cx, Cy), c0)``, the lookup M in the format of :func:`fan_quarter_maps`
    and the angle index c0 (the pairing is b <-> (c0 - b) mod Na), checked
    in float64 on sample pixels for every angle; None when no reflection
    and pairing pass.
    """
    Nx, Ny = (int(v) for v in img_shape)
    ofs = np.asarray(struct["ofs_dict"][np.dtype("float64")], dtype=np.float64)
    geo = np.asarray(struct["geo_dict"][np.dtype("float64")], dtype=np.float64)
    Na = ofs.shape[1]
    if Nx != Ny or Na < 2:
        return None
    c = (Nx - 1) * 0.5
    if geo[3] != c or geo[4] != c:
        return None
    R, RE, dxi, mid_det = geo[0], geo[1], geo[2], geo[5]
    Ns = int(round(geo[8]))
    px, py = _sample_pixels(Nx)
    px, py = px - c, py - c

    def u_t(a, X, Y):
        XD, YD, Qx, Qy, Dx0, Dy0 = (ofs[k, a][:, None] for k in range(6))
        t = ((Dx0 - Qx) * X + (Dy0 - Qy) * Y) / (R * R) + RE / R
        ss = (XD * X + YD * Y) / (dxi * dxi)
        return ss / t + mid_det, t

    total = 2.0 * mid_det  # u + u' = Ns - 1 when the detector is centred
    if abs(total - (Ns - 1)) > atol_bins:
        return None
    allb = np.arange(Na)
    u_b, t_b = u_t(allb, px[None, :], py[None, :])
    for S in _MAPS[4:8]:  # the four reflections
        X = S[0] * px + S[1] * py
        Y = S[2] * px + S[3] * py
        # the angle paired with angle 0, then every angle
        u_m, t_m = u_t(allb, X[None, :], Y[None, :])
        cand = np.nonzero(np.all(np.abs(u_m + u_b[0][None, :] - total) <= atol_bins, axis=1)
                          & np.all(np.abs(t_m - t_b[0][None, :])
                                   <= rtol_t * np.abs(t_b[0][None, :]), axis=1))[0]
        for c0 in cand:
            pair = (int(c0) - allb) % Na
            if (np.all(np.abs(u_m[pair] + u_b - total) <= atol_bins)
                    and np.all(np.abs(t_m[pair] - t_b) <= rtol_t * np.abs(t_b))):
                # a reflection is its own inverse: the lookup is M itself
                Axx, Axy, Ayx, Ayy = S
                Cx = int(round(c * (1 - Axx - Axy)))
                Cy = int(round(c * (1 - Ayx - Ayy)))
                return (Axx, Axy, Ayx, Ayy, Cx, Cy), int(c0)
    return None


def radon_half_maps(struct, img_shape, atol_bins: float = 1e-6):
    """Index maps of the quarter-turn-and-mirror orbit of a parallel-beam
    geometry, or None.

    With a square image centred on the rotation axis, a detector centred on
    the central ray and Na angles equispaced over [0, pi) (Na even), angle
    k + Na/2 sees the grid as angle k sees it after a quarter turn S, and
    angle k sees the grid turned by a half as its own detector reversed
    (bin s <-> Ns - 1 - s; p(-s, phi) = p(s, phi + pi)).  For a base angle
    k < Na/2 and a bin s the four outputs

        (s, k), (s, k + Na/2), (Ns-1-s, k), (Ns-1-s, k + Na/2)

    are then sums of the weights of angle k applied to img(P), img(S^-1 P),
    img(-P) and img(-S^-1 P).  Returned in the format of
    :func:`fan_quarter_maps`: three tuples ``(Axx, Axy, Ayx, Ayy, Cx, Cy)``
    for those three lookups, or None when a check fails (the detector
    coordinate xi = X x + Y y + offset of radon.cl:183-241 is evaluated in
    float64 on sample pixels for every base angle).
    """
    Nx, Ny = (int(v) for v in img_shape)
    ofs = np.asarray(struct["ofs_dict"][np.dtype("float64")], dtype=np.float64)
    geo = np.asarray(struct["geo_dict"][np.dtype("float64")], dtype=np.float64)
    Na = ofs.shape[1]
    if Nx != Ny or Na < 2 or Na % 2 != 0:
        return None
    Ns = int(round(geo[4]))
    c = (Nx - 1) * 0.5
    mid = (Ns - 1) * 0.5
    X, Y, off = ofs[0], ofs[1], ofs[2]
    # the image centre projects onto the detector centre at every angle
    if not np.all(np.abs(X * c + Y * c + off - mid) <= atol_bins):
        return None
    Q = Na // 2
    px, py = _sample_pixels(Nx)
    px, py = px - c, py - c

    def xi(a, Xr, Yr):
        return X[a][:, None] * Xr + Y[a][:, None] * Yr + mid

    base = np.arange(Q)
    x1 = xi(base + Q, px[None, :], py[None, :])
    found = None
    for S in _MAPS[2:4]:  # the two quarter turns
        Xr = S[0] * px + S[1] * py
        Yr = S[2] * px + S[3] * py
        if np.all(np.abs(x1 - xi(base, Xr[None, :], Yr[None, :])) <= atol_bins):
            found = S
            break
    if found is None:
        return None
    # lookups: S^-1 = S^T, then -I, then -S^-1
    inv = (found[0], found[2], found[1], found[3])
    maps = []
    for A in (inv, (-1, 0, 0, -1), tuple(-v for v in inv)):
        Cx = int(round(c * (1 - A[0] - A[1])))
        Cy = int(round(c * (1 - A[2] - A[3])))
        maps.append((A[0], A[1], A[2], A[3], Cx, Cy))
    return maps
