"""The reference-style C entries (``gr_radon_fwd``, ``gr_radon_bwd``,
``gr_fan_fwd``, ``gr_fan_bwd``: gratopy's kernel argument lists, the
per-angle table and the geometry vector instead of a descriptor) against the
float64 oracle, and against the descriptor path of the Python API with the
same (automatic) launch shapes and no quarter-turn sharing, bit for bit."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import device_settings, host_settings, rel_l2

pytestmark = pytest.mark.gpu

CFGS = {
    "radon": dict(geometry="radon", img_shape=(24, 20), angles=18, n_detectors=32),
    "fan": dict(geometry="fanbeam", img_shape=(24, 24), angles=20, n_detectors=36,
                detector_width=40.0, R=70.0, RE=30.0),
}


def _device(arr, order, dtype, device):
    import torch

    import gratopy_gb300 as gg

    t = gg.core.empty(arr.shape, dtype, order, device)
    t.copy_(torch.from_numpy(np.ascontiguousarray(arr)))
    return t


def _entry(ps, fwd, out, inp, out_order, in_order):
    from gratopy_gb300 import _lib, core

    dtype = np.dtype("float32") if out.dtype == core._torch_dtype(np.float32) else np.dtype("float64")
    t = ps.device_tables(dtype)
    geo_v = np.asarray(ps.struct["geo_dict"][dtype], dtype=np.float64)
    geo = (ctypes.c_double * len(geo_v))(*geo_v)
    fan = ps.is_fan
    shape = ps.sinogram_shape if fwd else ps.img_shape
    name = ("gr_fan_" if fan else "gr_radon_") + ("fwd" if fwd else "bwd")
    tables = [core._ptr(t["ofs"])] + ([core._ptr(t["sdpd"])] if fan else [])
    with core.torch.cuda.device(out.device):
        _lib.call(name, core._ptr(out), core._ptr(inp), *tables, geo, core._dt(out), shape[0],
                  shape[1], core._nz(out), core._oflag(out_order), core._oflag(in_order),
                  core._stream_ptr(out.device))


@pytest.mark.parametrize("name", sorted(CFGS))
@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("order", ["F", "C"])
@pytest.mark.parametrize("nz", [1, 3])
def test_reference_entries(cuda_device, name, dtype, order, nz):
    import torch

    import gratopy_gb300 as gg

    cfg = CFGS[name]
    ps = device_settings(cfg, cuda_device)
    hps = host_settings(cfg)
    tdt = torch.float32 if dtype == "float32" else torch.float64
    z = (nz,) if nz > 1 else ()
    rng = np.random.default_rng(11)
    img_np = rng.random(tuple(ps.img_shape) + z)
    sino_np = rng.random(tuple(ps.sinogram_shape) + z)
    img = _device(img_np, order, tdt, cuda_device)
    sino_in = _device(sino_np, order, tdt, cuda_device)
    sino = gg.core.empty(tuple(ps.sinogram_shape) + z, tdt, order, cuda_device)
    back = gg.core.empty(tuple(ps.img_shape) + z, tdt, order, cuda_device)
    _entry(ps, True, sino, img, order, order)
    _entry(ps, False, back, sino_in, order, order)
    tol = 1e-5 if dtype == "float32" else 1e-12
    want_s = O.forward(np.asfortranarray(img_np), hps)
    want_b = O.backward(np.asfortranarray(sino_np), hps)
    assert rel_l2(sino.double().cpu().numpy(), want_s) < tol
    assert rel_l2(back.double().cpu().numpy(), want_b) < tol
    # the descriptor path with automatic launch shapes and every angle's own
    # geometry runs the same kernels
    g = ps.gr_geometry(np.dtype(dtype))
    saved = (g.sym, g.fwd_split, g.bwd_split)
    g.sym, g.fwd_split, g.bwd_split = 0, 0, 0
    try:
        s2 = gg.forwardprojection(img, ps, sino=torch.empty_like(sino))
        b2 = gg.backprojection(sino_in, ps, img=torch.empty_like(back))
    finally:
        g.sym, g.fwd_split, g.bwd_split = saved
    assert torch.equal(s2, sino) and torch.equal(b2, back)
