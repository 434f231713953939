"""Fan-beam forward projection over quarter turns and the mirror (float32).

A centred square image, a centred detector and angles equispaced over the
full circle in a multiple of 4 give, besides the quarter-turn orbits, a
mirror: angle c0 - b sees the reflected grid as angle b sees it, with the
detector reversed.  The forward projection that reads the orbit copy then
walks only the bins s < ceil(Ns/2) and writes each bin's mirrored outputs
from the same weights.  Checked against the float64 oracle (1e-5) and
against the same geometry with the mirror switched off (4e-6), in every
memory-order pair, for every launch shape, odd detector counts, a reversed
detector, stacks, and through the fused solver epilogues.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import device_settings, host_settings, rel_l2

pytestmark = pytest.mark.gpu

# at least 16 * 2^20 pixel-angles per slice: the forward reads the orbit copy
BENCH = dict(geometry="fanbeam", img_shape=(512, 512), angles=360, n_detectors=768,
             detector_width=400.0, R=400.0, RE=200.0)
CFGS = {
    "bench": BENCH,
    "odd_detectors": dict(BENCH, n_detectors=767),
    "reversed": dict(BENCH, reverse_detector=True),
    "wide_fan": dict(BENCH, img_shape=(384, 384), angles=400, n_detectors=601, R=300.0,
                     RE=150.0, detector_width=500.0),
    "odd_side": dict(BENCH, img_shape=(389, 389), angles=360, n_detectors=583),
}


def _dev(a, order, device):
    import torch

    import gratopy_gb300 as gg

    t = gg.core.empty(a.shape, torch.float32, order, device)
    t.copy_(torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)))
    return t


def _forward(ps, img, io, so, device, mirror=True, split=None):
    import torch

    import gratopy_gb300 as gg

    g = ps.gr_geometry(np.float32)
    saved = (g.mirror, g.fwd_split)
    try:
        if not mirror:
            g.mirror = 0
        if split is not None:
            g.fwd_split = split
        out = gg.core.empty(tuple(ps.sinogram_shape) + tuple(img.shape[2:]), torch.float32, so,
                            device)
        gg.forwardprojection(_dev(img, io, device), ps, sino=out)
        torch.cuda.synchronize()
        return out.double().cpu().numpy()
    finally:
        g.mirror, g.fwd_split = saved


@pytest.mark.parametrize("name", sorted(CFGS))
@pytest.mark.parametrize("io", ["F", "C"])
@pytest.mark.parametrize("so", ["F", "C"])
def test_fan_mirror_forward(cuda_device, name, io, so):
    from gratopy_gb300 import _lib

    cfg = CFGS[name]
    ps = device_settings(cfg, cuda_device)
    g = ps.gr_geometry(np.float32)
    assert g.sym == 4 and g.mirror == 1
    assert ps.mirror_map() is not None
    # the mirrored forward is the one that runs: half the bins, twice the lanes
    assert int(_lib.raw("gr_work_bytes")(ctypes.byref(g), 1)) > 0 and g.work
    rng = np.random.default_rng(len(name) + 3 * (io == "C") + 5 * (so == "C"))
    img = rng.random(ps.img_shape)
    got = _forward(ps, img, io, so, cuda_device)
    plain = _forward(ps, img, io, so, cuda_device, mirror=False)
    ref = O.forward(np.asfortranarray(img), host_settings(cfg))
    err = rel_l2(got, ref)
    assert err <= 1e-5, f"{name} {io}{so}: rel err {err:.3e} vs float64 oracle"
    # the mirrored bins' sums from the base angle's weights, in another order
    assert rel_l2(got, plain) <= 4e-6
    Ns = ps.sinogram_shape[0]
    H = (Ns + 1) // 2
    assert rel_l2(got[H:], ref[H:]) <= 1e-5  # the mirrored half on its own


@pytest.mark.parametrize("split", [1, 2, 4, 8])
def test_fan_mirror_launch_shapes(cuda_device, split):
    cfg = CFGS["odd_detectors"]
    ps = device_settings(cfg, cuda_device)
    img = np.random.default_rng(split).random(ps.img_shape)
    got = _forward(ps, img, "F", "F", cuda_device, split=split)
    ref = O.forward(np.asfortranarray(img), host_settings(cfg))
    assert rel_l2(got, ref) <= 1e-5


def test_fan_mirror_stack_and_partials(cuda_device):
    """A 3-slice stack of 1024^2 x 720 (the orbit kernels slice by slice):
    each slice against the mirror switched off, and the block partials of
    CG's fused forward reduction written once each."""
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import _lib

    cfg = dict(BENCH, img_shape=(1024, 1024), angles=720, n_detectors=1536)
    ps = device_settings(cfg, cuda_device)
    g = ps.gr_geometry(np.float32)
    assert g.mirror == 1
    img = np.random.default_rng(4).random(tuple(ps.img_shape) + (3,))
    got = _forward(ps, img, "F", "F", cuda_device)
    plain = _forward(ps, img, "F", "F", cuda_device, mirror=False)
    for z in range(3):
        assert rel_l2(got[..., z], plain[..., z]) <= 4e-6, f"slice {z}"
    g = ps.gr_geometry(np.float32)
    n = int(_lib.raw("gr_forward_partials")(ctypes.byref(g), 3))
    part = torch.full((n + 64,), float("nan"), dtype=torch.float64, device=cuda_device)
    x = _dev(img, "F", cuda_device)
    q = gg.core.empty(tuple(ps.sinogram_shape) + (3,), torch.float32, "F", cuda_device)
    w = ps.device_tables(np.float32)["w"]
    _lib.call("gr_forward_wsq", ctypes.byref(g), gg.core._ptr(q), gg.core._ptr(x),
              gg.core._ptr(w), gg.core._ptr(part), None, 3, _lib.GR_ORDER_F,
              gg.core._stream_ptr(cuda_device))
    torch.cuda.synchronize()
    p = part.cpu().numpy()
    assert np.isfinite(p[:n]).all() and np.isnan(p[n:]).all()
    qh = q.double().cpu().numpy()
    want = float((qh * qh * w.double().cpu().numpy()[None, :, None]).sum())
    assert abs(p[:n].sum() - want) <= 1e-6 * want
    assert rel_l2(qh, got) <= 1e-7


def test_fan_mirror_in_solvers(cuda_device):
    """Landweber, TV and CG through the mirrored forward's fused epilogues
    against the same solvers with the mirror switched off."""
    import gratopy_gb300 as gg

    ps = device_settings(BENCH, cuda_device)
    img = np.random.default_rng(9).random(ps.img_shape)
    sino = _dev(_forward(ps, img, "F", "F", cuda_device, mirror=False), "F", cuda_device)
    g = ps.gr_geometry(np.float32)
    runs = {}
    for mirror in (1, 0):
        g.mirror = mirror
        runs[mirror] = [gg.landweber(sino, ps, 5, norm_estimate=200.0).double().cpu().numpy(),
                        gg.total_variation(sino, ps, 20.0, 5, norm_estimate=200.0)
                        .double().cpu().numpy(),
                        gg.conjugate_gradients(sino, ps, 4).double().cpu().numpy()]
    g.mirror = 1
    for a, b, what in zip(runs[1], runs[0], ("landweber", "tv", "cg")):
        err = rel_l2(a, b)
        assert err <= (1e-4 if what == "cg" else 1e-5), f"{what}: {err:.3e}"
