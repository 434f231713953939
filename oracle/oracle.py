"""Oracle: CPU restatement of gratopy's projection kernels and solvers.

TEST INFRASTRUCTURE ONLY.  Used by ``tests/`` as the checker, by
``bench.py`` as the timed CPU baseline, and by ``__graft_entry__.smoke()``.
The product (``gratopy_gb300``) never imports this module.

Kernels come from ``oracle/gr_oracle.c`` (loaded through ctypes; see that
file for the kernel-by-kernel citations).  The solvers restate the host
loops of ``gratopy/gratopy.py``:

* :func:`normest`             -- gratopy.py:2329-2377
* :func:`landweber`           -- gratopy.py:2380-2446
* :func:`conjugate_gradients` -- gratopy.py:2449-2551
* :func:`total_variation`     -- gratopy.py:2554-2762

Deliberate differences from the reference, shared with the GPU product so
that the two agree: reductions (sum, dot products) accumulate in float64
instead of the array dtype, ``normest`` takes an explicit start vector or
seeded generator instead of the unseeded global ``np.random``, and the 3-D
total-variation path uses ``img_shape + (Nz,)`` (the reference raises a
TypeError there, gratopy.py:2626-2628).

Arrays are numpy arrays of shape ``(Nx, Ny[, Nz])`` / ``(Ns, Na[, Nz])``,
either Fortran- or C-contiguous; outputs follow the input's order unless
given.
"""

from __future__ import annotations

import ctypes
import os
from typing import Any

import numpy as np

from . import build as _build

_LIB = None


def threads() -> int:
    env = os.environ.get("GR_ORACLE_THREADS")
    if env:
        return max(1, int(env))
    return os.cpu_count() or 1


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build()
        _LIB = ctypes.CDLL(str(path))
        _declare(_LIB)
    return _LIB


_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_D = ctypes.c_double
_Z = ctypes.c_size_t


def _declare(L):
    for sfx, real in (("f32", _F), ("f64", _D)):
        getattr(L, f"or_radon_fwd_{sfx}").argtypes = [_P, _P, _P, _P, _I, _I, _I, _I, _I, _I]
        getattr(L, f"or_radon_bwd_{sfx}").argtypes = [_P, _P, _P, _P, _I, _I, _I, _I, _I, _I]
        getattr(L, f"or_fan_fwd_{sfx}").argtypes = [_P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I]
        getattr(L, f"or_fan_bwd_{sfx}").argtypes = [_P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I]
        getattr(L, f"or_tv_update_v_{sfx}").argtypes = [_P, _P, _F, _F, _I, _I, _I, _I, _I]
        getattr(L, f"or_tv_normv_{sfx}").argtypes = [_P, _Z, _I]
        getattr(L, f"or_tv_update_lambda_{sfx}").argtypes = [_P, _P, _P, _F, _F, _Z, _I]
        getattr(L, f"or_tv_update_u_{sfx}").argtypes = [_P, _P, _P, _P, _F, _F, _F, _I, _I, _I, _I, _I]
        getattr(L, f"or_tv_extra_{sfx}").argtypes = [_P, _P, _Z, _I]
        getattr(L, f"or_weight_sino_{sfx}").argtypes = [_P, _P, _P, _I, _I, _I, _I, _I, _I]
        getattr(L, f"or_equ_mul_add_{sfx}").argtypes = [_P, real, _P, _Z, _I]
        getattr(L, f"or_mul_add_add_{sfx}").argtypes = [_P, real, _P, _P, _Z, _I]
        f = getattr(L, f"or_dot_f64_{sfx}")
        f.argtypes = [_P, _P, _Z, _I]
        f.restype = _D


def _sfx(dtype) -> str:
    dtype = np.dtype(dtype)
    if dtype == np.float32:
        return "f32"
    if dtype == np.float64:
        return "f64"
    raise TypeError(f"oracle supports float32/float64, got {dtype}")


def order_of(a: np.ndarray) -> str:
    if a.flags.c_contiguous:
        return "C"
    if a.flags.f_contiguous:
        return "F"
    raise ValueError("array must be C- or F-contiguous")


def _oflag(order: str) -> int:
    return 1 if order.upper() == "C" else 0


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _nz(a: np.ndarray) -> int:
    return a.shape[2] if a.ndim > 2 else 1


def _tables(ps, dtype):
    dtype = np.dtype(dtype)
    s = ps.struct
    ofs = np.require(s["ofs_dict"][dtype], dtype, "F")
    geo = np.require(s["geo_dict"][dtype], dtype)
    sdpd = np.require(s["sdpd_dict"][dtype], dtype) if ps.is_fan else None
    return ofs, geo, sdpd


# ---------------------------------------------------------------- projections


def forward(img: np.ndarray, ps, sino: np.ndarray | None = None, order: str | None = None,
            nthreads: int | None = None) -> np.ndarray:
    """Forward projection sino = A img (radon.cl:66-161 / fanbeam.cl:72-256)."""
    nthreads = nthreads or threads()
    Nz = _nz(img)
    if sino is None:
        shape = tuple(ps.sinogram_shape) + ((img.shape[2],) if img.ndim > 2 else ())
        sino = np.zeros(shape, dtype=img.dtype, order=order or order_of(img))
    assert sino.dtype == img.dtype
    ofs, geo, sdpd = _tables(ps, img.dtype)
    Ns, Na = ps.sinogram_shape
    L = lib()
    sfx = _sfx(img.dtype)
    if ps.is_fan:
        getattr(L, f"or_fan_fwd_{sfx}")(_ptr(sino), _ptr(img), _ptr(ofs), _ptr(sdpd), _ptr(geo),
                                        Ns, Na, Nz, _oflag(order_of(sino)), _oflag(order_of(img)), nthreads)
    else:
        getattr(L, f"or_radon_fwd_{sfx}")(_ptr(sino), _ptr(img), _ptr(ofs), _ptr(geo),
                                          Ns, Na, Nz, _oflag(order_of(sino)), _oflag(order_of(img)), nthreads)
    return sino


def backward(sino: np.ndarray, ps, img: np.ndarray | None = None, order: str | None = None,
             nthreads: int | None = None) -> np.ndarray:
    """Backprojection img = A^T sino (radon.cl:183-241 / fanbeam.cl:290-391)."""
    nthreads = nthreads or threads()
    Nz = _nz(sino)
    if img is None:
        shape = tuple(ps.img_shape) + ((sino.shape[2],) if sino.ndim > 2 else ())
        img = np.zeros(shape, dtype=sino.dtype, order=order or order_of(sino))
    assert sino.dtype == img.dtype
    ofs, geo, sdpd = _tables(ps, sino.dtype)
    Nx, Ny = ps.img_shape
    L = lib()
    sfx = _sfx(sino.dtype)
    if ps.is_fan:
        getattr(L, f"or_fan_bwd_{sfx}")(_ptr(img), _ptr(sino), _ptr(ofs), _ptr(sdpd), _ptr(geo),
                                        Nx, Ny, Nz, _oflag(order_of(img)), _oflag(order_of(sino)), nthreads)
    else:
        getattr(L, f"or_radon_bwd_{sfx}")(_ptr(img), _ptr(sino), _ptr(ofs), _ptr(geo),
                                          Nx, Ny, Nz, _oflag(order_of(img)), _oflag(order_of(sino)), nthreads)
    return img


def weight_sinogram(sino: np.ndarray, ps, sino_out: np.ndarray | None = None,
                    divide: bool = False) -> np.ndarray:
    """Angle weighting (utilities.cl:38-67, gratopy.py:2188-2266)."""
    if sino_out is None:
        sino_out = np.zeros(sino.shape, dtype=sino.dtype, order=order_of(sino))
    w = np.require(ps.struct["angle_diff_dict"][np.dtype(sino.dtype)], sino.dtype)
    Ns, Na = sino.shape[:2]
    getattr(lib(), f"or_weight_sino_{_sfx(sino.dtype)}")(
        _ptr(sino_out), _ptr(sino), _ptr(w), Ns, Na, _nz(sino), _oflag(order_of(sino)),
        int(divide), threads())
    return sino_out


def dot(a: np.ndarray, b: np.ndarray) -> float:
    """float64-accumulated dot product over the memory of two same-order arrays."""
    assert a.dtype == b.dtype and a.shape == b.shape and order_of(a) == order_of(b)
    return float(getattr(lib(), f"or_dot_f64_{_sfx(a.dtype)}")(_ptr(a), _ptr(b), a.size, threads()))


def _equ_mul_add(rhs, a, x):
    getattr(lib(), f"or_equ_mul_add_{_sfx(rhs.dtype)}")(_ptr(rhs), float(a), _ptr(x), rhs.size, threads())


def _mul_add_add(rhs, a, x, y):
    getattr(lib(), f"or_mul_add_add_{_sfx(rhs.dtype)}")(_ptr(rhs), float(a), _ptr(x), _ptr(y), rhs.size, threads())


# -------------------------------------------------------------------- solvers


def normest(ps, number_iterations: int = 50, dtype: Any = "float32", x0: np.ndarray | None = None,
            rng: np.random.Generator | None = None) -> float:
    """Power iteration on A^T A normalised by the plain sum (gratopy.py:2329-2377)."""
    dtype = np.dtype(dtype)
    if x0 is None:
        rng = rng if rng is not None else np.random.default_rng(0)
        x0 = rng.standard_normal(ps.img_shape)
    img = np.require(np.array(x0, dtype=dtype), dtype, "F").copy(order="F")
    sino = forward(img, ps)
    normsqr = 1.0
    for _ in range(number_iterations):
        normsqr = float(np.sum(img, dtype=np.float64))
        img /= dtype.type(normsqr)
        forward(img, ps, sino=sino)
        backward(sino, ps, img=img)
    return float(np.sqrt(normsqr))


def landweber(sino: np.ndarray, ps, number_iterations: int = 100, w: float = 1.0,
              norm_estimate: float | None = None) -> np.ndarray:
    """Landweber / SIRT: U <- U - (w/|A|^2) A^T (A U - f) (gratopy.py:2380-2446)."""
    order = order_of(sino)
    if norm_estimate is None:
        norm_estimate = normest(ps)
    w = sino.dtype.type(w / norm_estimate**2)
    sinonew = sino.copy(order=order)
    shape = tuple(ps.img_shape) + ((sino.shape[2],) if sino.ndim > 2 else ())
    U = np.zeros(shape, dtype=sino.dtype, order=order)
    Unew = np.zeros(shape, dtype=sino.dtype, order=order)
    for _ in range(number_iterations):
        forward(Unew, ps, sino=sinonew)
        sinonew -= sino
        backward(sinonew, ps, img=U)
        _equ_mul_add(Unew, -w, U)
    return Unew


def conjugate_gradients(sino: np.ndarray, ps, number_iterations: int = 20, epsilon: float = 0.0,
                        x0: np.ndarray | None = None) -> np.ndarray:
    """CG on the normal equations in the weighted inner products (gratopy.py:2449-2551)."""
    order = order_of(sino)
    dims = tuple(ps.img_shape) + ((sino.shape[2],) if sino.ndim > 2 else ())
    dtype = sino.dtype
    if x0 is None:
        x0 = np.zeros(dims, dtype=dtype, order=order)
    assert order_of(x0) == order, "The data sino and initial guess x0 must have the same contiguity!"
    x = x0.copy(order=order)
    d = sino - forward(x, ps)
    d = np.require(d, dtype, order)
    p = backward(d, ps)
    q = np.zeros_like(d, order=order)
    q_rescaled = np.zeros_like(d, order=order)
    snew = backward(d, ps)
    sold = snew.copy(order=order)
    sino_sq = dot(sino, sino)
    for _ in range(number_iterations):
        forward(p, ps, sino=q)
        weight_sinogram(q, ps, q_rescaled)
        alpha = dtype.type(ps.delta_x**2 / ps.delta_s * (dot(sold, sold) / dot(q_rescaled, q)))
        _equ_mul_add(x, alpha, p)
        _equ_mul_add(d, -alpha, q)
        backward(d, ps, img=snew)
        beta = dot(snew, snew) / dot(sold, sold)
        sold, snew = snew, sold
        _mul_add_add(p, dtype.type(beta), p, sold)
        residue = np.sqrt(dot(d, d) / sino_sq)
        if residue < epsilon:
            break
    return x


def total_variation(sino: np.ndarray, ps, mu: float, number_iterations: int = 1000,
                    slice_thickness: float = 1.0, stepsize_weighting: float = 10.0,
                    norm_estimate: float | None = None) -> np.ndarray:
    """L2-TV Chambolle-Pock primal-dual reconstruction (gratopy.py:2554-2762)."""
    dtype = sino.dtype
    order = order_of(sino)
    sfx = _sfx(dtype)
    L = lib()
    nt = threads()
    img_shape = tuple(ps.img_shape)
    if sino.ndim == 2:
        slice_thickness = 0
        Nz = 1
    else:
        Nz = sino.shape[2]
        img_shape = img_shape + (Nz,)
    Nx, Ny = ps.img_shape
    n_img = Nx * Ny * Nz
    U = np.zeros(img_shape, dtype=dtype, order=order)
    U_ = np.zeros(img_shape, dtype=dtype, order=order)
    V = np.zeros(4 * n_img, dtype=dtype)
    Lamb = np.zeros(sino.shape, dtype=dtype, order=order)
    KU = np.zeros(sino.shape, dtype=dtype, order=order)
    KST = np.zeros(img_shape, dtype=dtype, order=order)
    if norm_estimate is None:
        norm_estimate = normest(ps)
    Lsqr = 13
    sigma = 1.0 / np.sqrt(Lsqr) * stepsize_weighting
    tau = 1.0 / np.sqrt(Lsqr) / stepsize_weighting
    assert mu > 0, "Regularization parameter mu must be positive"
    mu = mu * norm_estimate**2 * ps.delta_x
    mu = mu / (sigma + mu)
    of = _oflag(order)
    for _ in range(number_iterations):
        getattr(L, f"or_tv_update_v_{sfx}")(_ptr(V), _ptr(U_), float(np.float32(sigma)),
                                           float(np.float32(slice_thickness)), Nx, Ny, Nz, of, nt)
        getattr(L, f"or_tv_normv_{sfx}")(_ptr(V), n_img, nt)
        forward(U_, ps, sino=KU)
        getattr(L, f"or_tv_update_lambda_{sfx}")(_ptr(Lamb), _ptr(KU), _ptr(sino),
                                                float(np.float32(sigma / norm_estimate)),
                                                float(np.float32(mu)), Lamb.size, nt)
        backward(Lamb, ps, img=KST)
        getattr(L, f"or_tv_update_u_{sfx}")(_ptr(U_), _ptr(U), _ptr(V), _ptr(KST),
                                           float(np.float32(tau)), float(np.float32(1.0 / norm_estimate)),
                                           float(np.float32(slice_thickness)), Nx, Ny, Nz, of, nt)
        getattr(L, f"or_tv_extra_{sfx}")(_ptr(U_), _ptr(U), n_img, nt)
        U, U_ = U_, U
    return U
