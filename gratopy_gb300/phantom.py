"""Test images: the (modified) Shepp-Logan phantom and seeded random ellipses.

``phantom``/``ct_shepp_logan`` and ``easy_phantom`` keep the signatures of
gratopy's ``gratopy/phantom.py:33-151`` (queue first), returning a torch
tensor on the device the queue names.  The rasteriser is the usual
inside-ellipse test on the grid ``x = linspace(-1, 1, N)``,
``y = -linspace(-1, 1, M)`` summed over ellipses (phantom.py:159-177).

The ellipse table is the one published by Shepp and Logan (1974); the
"modified" grey values are the higher-contrast set of Toft (1996), Table B.1.
"""

from __future__ import annotations

import numpy as np


def ct_shepp_logan_params_2d() -> np.ndarray:
    """Original Shepp-Logan ellipses: columns grey, a, b, xc, yc, theta."""
    E = np.zeros((10, 6))
    E[:, 0] = [2.0, -0.98, -0.02, -0.02, 0.01, 0.01, 0.01, 0.01, 0.01, 0.01]
    E[:, 1] = [0.69, 0.6624, 0.11, 0.16, 0.21, 0.046, 0.046, 0.046, 0.023, 0.023]
    E[:, 2] = [0.92, 0.874, 0.31, 0.41, 0.25, 0.046, 0.046, 0.023, 0.023, 0.046]
    E[:, 3] = [0.0, 0.0, 0.22, -0.22, 0.0, 0.0, 0.0, -0.08, 0.0, 0.06]
    E[:, 4] = [0.0, -0.0184, 0.0, 0.0, 0.35, 0.1, -0.1, -0.605, -0.605, -0.605]
    E[:, 5] = np.deg2rad([0.0, 0.0, -18.0, 18.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0])
    return E


def ct_modified_shepp_logan_params_2d() -> np.ndarray:
    """Modified (higher contrast) Shepp-Logan ellipses."""
    E = ct_shepp_logan_params_2d()
    E[:, 0] = [1.0, -0.8, -0.2, -0.2, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1]
    return E


def rasterize_ellipses(M: int, N: int, E: np.ndarray) -> np.ndarray:
    """Sum of filled ellipses on an (M, N) grid covering [-1, 1]^2 (float64).

    Row index runs along -y, column index along x, as in phantom.py:159-177.
    """
    X, Y = np.meshgrid(np.linspace(-1, 1, N), -np.linspace(-1, 1, M))
    ph = np.zeros((M, N))
    ct = np.cos(E[:, 5])
    st = np.sin(E[:, 5])
    for k in range(E.shape[0]):
        xc, yc = E[k, 3], E[k, 4]
        a, b = E[k, 1], E[k, 2]
        inside = ((X - xc) * ct[k] + (Y - yc) * st[k]) ** 2 / a**2 + (
            (X - xc) * st[k] - (Y - yc) * ct[k]
        ) ** 2 / b**2 <= 1
        ph[inside] += E[k, 0]
    return ph


def shepp_logan_host(N, modified: bool = True, E=None, dtype="float64") -> np.ndarray:
    """Shepp-Logan phantom as a C-ordered numpy array of shape (M, N)."""
    if np.isscalar(N):
        M, N = N, N
    elif len(N) == 2:
        M, N = N[:]
    else:
        raise ValueError("Dimension must be scalar or 2D!")
    if E is None:
        E = ct_modified_shepp_logan_params_2d() if modified else ct_shepp_logan_params_2d()
    return rasterize_ellipses(M, N, np.asarray(E, dtype=np.float64)).astype(dtype)


def _device_of(queue):
    import torch

    if queue is None:
        return torch.device("cuda", torch.cuda.current_device())
    if isinstance(queue, torch.device):
        return queue
    if isinstance(queue, str):
        return torch.device(queue)
    dev = getattr(queue, "device", None)
    if dev is not None:
        return torch.device(dev)
    raise TypeError(f"cannot derive a device from {queue!r}")


def ct_shepp_logan(queue, N, modified: bool = True, E=None, ret_E: bool = False,
                   dtype="double", allocator=None):
    """Shepp-Logan phantom on the device (gratopy phantom.py:58-151).

    ``queue`` is a ``torch.device`` (or ``None`` for the current CUDA device);
    ``allocator`` is accepted and ignored.
    """
    import torch

    if E is None:
        E = ct_modified_shepp_logan_params_2d() if modified else ct_shepp_logan_params_2d()
    host = shepp_logan_host(N, modified, E, dtype=np.dtype(dtype))
    ph = torch.from_numpy(np.ascontiguousarray(host)).to(_device_of(queue))
    if ret_E:
        return ph, E
    return ph


def easy_phantom(N, queue=None, modified: bool = True, E=None, ret_E: bool = False,
                 dtype=None, allocator=None):
    """Convenience wrapper (phantom.py:33-55); float64 unless told otherwise."""
    if dtype is None:
        dtype = "float64"
    return ct_shepp_logan(queue, N, modified=modified, E=E, ret_E=ret_E, dtype=dtype)


phantom = ct_shepp_logan


def random_ellipses(rng: np.random.Generator, count: int = 10) -> np.ndarray:
    """Seeded random ellipse table (grey, a, b, xc, yc, theta).

    Centres U[-0.8, 0.8]^2, semi-axes U[0.05, 0.5], angle U[0, pi),
    intensity U[0, 1] -- the synthetic input of the benchmark workloads.
    """
    E = np.zeros((count, 6))
    E[:, 0] = rng.uniform(0.0, 1.0, count)
    E[:, 1] = rng.uniform(0.05, 0.5, count)
    E[:, 2] = rng.uniform(0.05, 0.5, count)
    E[:, 3] = rng.uniform(-0.8, 0.8, count)
    E[:, 4] = rng.uniform(-0.8, 0.8, count)
    E[:, 5] = rng.uniform(0.0, np.pi, count)
    return E


def random_ellipse_image(seed: int, N, count: int = 10, dtype="float32") -> np.ndarray:
    """(M, N) C-ordered image of ``count`` seeded random ellipses."""
    if np.isscalar(N):
        M, N = N, N
    else:
        M, N = N
    rng = np.random.default_rng(seed)
    return rasterize_ellipses(M, N, random_ellipses(rng, count)).astype(dtype)


def ellipse_records(E: np.ndarray) -> np.ndarray:
    """Per-ellipse records (grey, a^2, b^2, xc, yc, cos theta, sin theta) as the
    device rasteriser reads them, with the host rasteriser's rounding."""
    E = np.asarray(E, dtype=np.float64)
    return np.stack([E[:, 0], E[:, 1] ** 2, E[:, 2] ** 2, E[:, 3], E[:, 4], np.cos(E[:, 5]),
                     np.sin(E[:, 5])], axis=1)


def random_ellipse_volume(device, img_shape, nz: int = 1, seed: int = 0, count: int = 10,
                          dtype="float32", order: str = "F"):
    """(Nx, Ny[, nz]) stack rasterised on the device; slice k equals
    ``random_ellipse_image(seed + k, (Ny, Nx), count, dtype).T``."""
    import ctypes

    import torch

    from . import _lib, core

    Nx, Ny = (int(img_shape), int(img_shape)) if np.isscalar(img_shape) else map(int, img_shape)
    recs = np.concatenate([ellipse_records(random_ellipses(np.random.default_rng(seed + k), count))
                           for k in range(nz)])
    dev = _device_of(device)
    tdt = torch.float32 if np.dtype(dtype) == np.float32 else torch.float64
    shape = (Nx, Ny) + ((nz,) if nz > 1 else ())
    out = core.empty(shape, tdt, order, dev)
    e = torch.from_numpy(np.ascontiguousarray(recs.reshape(-1))).to(dev)
    with torch.cuda.device(dev):
        _lib.call("gr_ellipses", ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(e.data_ptr()),
                  count, Nx, Ny, nz, _lib.GR_F32 if tdt == torch.float32 else _lib.GR_F64,
                  _lib.GR_ORDER_F if order == "F" else _lib.GR_ORDER_C, core._stream_ptr(dev))
    return out
