"""Launch-shape autotuner for the projection kernels.

The projection kernels have one free launch parameter per direction:

* forward: lanes that share a group of detector bins (``fwd_split`` in 1, 2,
  4, 8 -- the rows of the image are split over that many lanes and reduced
  with warp shuffles);
* backprojection: thread rows that split the angles of a pixel tile
  (``bwd_split`` in 1, 2, 4, 8).

The best choice depends on the geometry (image size, detector count, angle
count, slices) and the precision.  :func:`tune` times every candidate with
CUDA events on the actual geometry, stores the winner in the geometry
descriptor of the :class:`~gratopy_gb300.ProjectionSettings` (every later
projection and solver call of that settings object uses it) and caches it in
a JSON file keyed by device and geometry, so a geometry is timed once per
machine.  Splits change only the order of float additions, never which terms
are added.
"""

from __future__ import annotations

import ctypes
import json
import os
import tempfile
from pathlib import Path

import numpy as np
import torch

from . import _lib
from . import core

SPLITS = (1, 2, 4, 8)
SPLITS_F64 = (1, 4)  # float64 kernels are instantiated for these only


def cache_path() -> Path:
    """Tuning cache: ``$GRATOPY_GB300_TUNE_CACHE`` or ``~/.cache/gratopy_gb300/tune.json``."""
    env = os.environ.get("GRATOPY_GB300_TUNE_CACHE")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "gratopy_gb300" / "tune.json"


def geometry_key(device_name: str, kind: str, dtype, img_shape, sino_shape, nz: int) -> str:
    """Cache key: device, geometry kind, precision, sizes and whether slices are stacked."""
    dt = np.dtype(dtype).name
    Nx, Ny = img_shape
    Ns, Na = sino_shape
    zcls = "z1" if nz == 1 else "zN"
    return f"{device_name}|{kind}|{dt}|{Nx}x{Ny}|{Ns}x{Na}|{zcls}"


def load_cache(path: Path | None = None) -> dict:
    path = cache_path() if path is None else Path(path)
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def store_cache(entries: dict, path: Path | None = None) -> None:
    """Merge ``entries`` into the cache file (atomic replace)."""
    path = cache_path() if path is None else Path(path)
    data = load_cache(path)
    data.update(entries)
    path.parent.mkdir(parents=True, exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=path.parent, prefix=".tune", suffix=".json")
    with os.fdopen(fd, "w") as fh:
        json.dump(data, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def select(timings: dict) -> int:
    """Fastest candidate; ties go to the smaller split (fewer shuffles)."""
    if not timings:
        raise ValueError("no timings")
    return min(sorted(timings), key=lambda k: timings[k])


def _time_launch(launch, repeats: int) -> float:
    """Median device time in ms of ``launch()`` over ``repeats`` runs (after one warm-up)."""
    launch()
    times = []
    for _ in range(repeats):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        launch()
        b.record()
        b.synchronize()
        times.append(a.elapsed_time(b))
    return float(np.median(times))


def measure(ps, dtype=np.float32, nz: int = 1, repeats: int = 10, candidates=None) -> dict:
    """Time every split candidate on the geometry of ``ps``; returns
    ``{"fwd": {split: ms}, "bwd": {split: ms}}``."""
    ndt = np.dtype(dtype)
    tdt = core._torch_dtype(ndt)
    if candidates is None:
        candidates = SPLITS if ndt == np.float32 else SPLITS_F64
    dev = ps.device
    g = ps.gr_geometry(ndt)
    z = (nz,) if nz > 1 else ()
    gen = torch.Generator(device=dev).manual_seed(0)
    img = core.empty(tuple(ps.img_shape) + z, tdt, "F", dev)
    img.copy_(torch.rand(img.shape, generator=gen, device=dev, dtype=tdt))
    sino = core.empty(tuple(ps.sinogram_shape) + z, tdt, "F", dev)
    sino.copy_(torch.rand(sino.shape, generator=gen, device=dev, dtype=tdt))
    old = (g.fwd_split, g.bwd_split)
    out = {"fwd": {}, "bwd": {}}
    try:
        with torch.cuda.device(dev):
            for sp in candidates:
                g.fwd_split = sp

                def fwd():
                    _lib.call("gr_forward", ctypes.byref(g), core._ptr(sino), core._ptr(img), nz,
                              _lib.GR_ORDER_F, _lib.GR_ORDER_F, core._stream_ptr(dev))

                out["fwd"][sp] = _time_launch(fwd, repeats)
            g.fwd_split = old[0]
            for sp in candidates:
                g.bwd_split = sp

                def bwd():
                    _lib.call("gr_backward", ctypes.byref(g), core._ptr(img), core._ptr(sino), nz,
                              _lib.GR_ORDER_F, _lib.GR_ORDER_F, core._stream_ptr(dev))

                out["bwd"][sp] = _time_launch(bwd, repeats)
    finally:
        g.fwd_split, g.bwd_split = old
    return out


def tune(ps, dtype=np.float32, nz: int = 1, repeats: int = 10, use_cache: bool = True,
         cache_file=None, candidates=None) -> dict:
    """Pick and apply the fastest splits for ``ps`` in precision ``dtype``.

    Returns ``{"fwd_split": f, "bwd_split": b, "timings": {...} | None,
    "cached": bool}``.  The splits are written into ``ps``'s geometry
    descriptor for ``dtype``, so all later calls with ``ps`` use them.
    """
    ndt = np.dtype(dtype)
    dev = ps.device
    name = torch.cuda.get_device_name(dev)
    kind = "fanbeam" if ps.is_fan else "radon"
    key = geometry_key(name, kind, ndt, ps.img_shape, ps.sinogram_shape, nz)
    cache = load_cache(cache_file) if use_cache else {}
    timings = None
    cached = key in cache
    if cached:
        fwd_split, bwd_split = int(cache[key]["fwd_split"]), int(cache[key]["bwd_split"])
    else:
        timings = measure(ps, ndt, nz, repeats, candidates)
        fwd_split, bwd_split = select(timings["fwd"]), select(timings["bwd"])
        if use_cache:
            store_cache({key: {"fwd_split": fwd_split, "bwd_split": bwd_split,
                               "fwd_ms": timings["fwd"], "bwd_ms": timings["bwd"]}}, cache_file)
    for g in (ps.gr_geometry(ndt), ps.gr_geometry_adjoint(ndt)):
        g.fwd_split, g.bwd_split = fwd_split, bwd_split
    return {"fwd_split": fwd_split, "bwd_split": bwd_split, "timings": timings, "cached": cached}
