"""Parallel-beam projections over half-circle orbits (float32).

For angles equispaced over [0, pi) with Na even, a centred square image and
a centred detector, the forward projection shares each candidate pixel's
weights over the four outputs (s, k), (s, k + Na/2), (Ns-1-s, k),
(Ns-1-s, k + Na/2), and the backprojection shares two detector positions
over the eight pixel-angles of a pixel orbit.  Checked against the float64
oracle (1e-5), against the per-angle kernels (the same geometry with the
symmetry switched off), with the scratch that holds the copies and without
it, in every memory-order pair and for every launch shape.  The forward of a
single slice reads the orbit copy from 4 * 2^20 pixel-angles (the bench
geometry here) and gathers the four orbit members from the image below that
or without scratch (the other geometries here); the backprojection reads
the row copy likewise from 4 * 2^20 pixel-angles when the scratch holds it
and gathers from the sinogram otherwise; copies and gathers give the same
sums.
Stacks of slices from 32 * 2^20 pixel-angles take the orbit forward slice by
slice when the scratch holds a slice's copy, and the per-angle
backprojection.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import device_settings, host_settings, rel_l2

pytestmark = pytest.mark.gpu

CFGS = {
    "even": dict(geometry="radon", img_shape=(64, 64), angles=40, n_detectors=91),
    "even_detectors": dict(geometry="radon", img_shape=(48, 48), angles=36, n_detectors=70),
    "odd_side": dict(geometry="radon", img_shape=(37, 37), angles=18, n_detectors=53),
    "wide_detector": dict(geometry="radon", img_shape=(40, 40), angles=30, n_detectors=57,
                          detector_width=3.0),
    "two_pixels": dict(geometry="radon", img_shape=(2, 2), angles=4, n_detectors=3),
    "bench": dict(geometry="radon", img_shape=(256, 256), angles=180, n_detectors=363,
                  detector_width=2.0 * np.sqrt(2.0), image_width=2.0),
}


def _dev(a, order, device):
    import torch

    import gratopy_gb300 as gg

    t = gg.core.empty(a.shape, torch.float32, order, device)
    t.copy_(torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)))
    return t


def _project(ps, fwd, data, io, so, device, sym=None, work=True):
    """Forward (fwd) or backprojection of data with the orbit symmetry as
    detected (sym None), switched off (sym 0), with or without scratch."""
    import torch

    import gratopy_gb300 as gg

    g = ps.gr_geometry(np.float32)
    dt = np.dtype("float32")
    saved = (g.sym, g.work, g.work_bytes, ps._work_bytes[dt])
    try:
        if sym is not None:
            g.sym = sym
        if not work:
            # the settings object rebinds its scratch on every call unless it
            # holds none for this precision
            ps._work_bytes[dt] = 0
            g.work, g.work_bytes = None, 0
        tail = tuple(data.shape[2:])  # slices of a stack
        if fwd:
            out = gg.core.empty(tuple(ps.sinogram_shape) + tail, torch.float32, so, device)
            gg.forwardprojection(_dev(data, io, device), ps, sino=out)
        else:
            out = gg.core.empty(tuple(ps.img_shape) + tail, torch.float32, io, device)
            gg.backprojection(_dev(data, so, device), ps, img=out)
        torch.cuda.synchronize()
        return out.double().cpu().numpy()
    finally:
        g.sym, g.work, g.work_bytes, ps._work_bytes[dt] = saved


@pytest.mark.parametrize("name", sorted(CFGS))
@pytest.mark.parametrize("io", ["F", "C"])
@pytest.mark.parametrize("so", ["F", "C"])
def test_radon_orbit_parity(cuda_device, name, io, so):
    cfg = CFGS[name]
    ps = device_settings(cfg, cuda_device)
    hps = host_settings(cfg)
    assert ps.quarter_maps() is not None and ps.gr_geometry(np.float32).sym == 2
    g = ps.gr_geometry(np.float32)
    # scratch for the copies from 4 * 2^20 pixel-angles (the bench geometry)
    assert bool(g.work) == (name == "bench") and g.work_bytes == ps._work_bytes[np.dtype("f4")]
    rng = np.random.default_rng(len(name) + 7 * (io == "C") + 13 * (so == "C"))
    img = rng.random(ps.img_shape)
    sino = rng.random(ps.sinogram_shape)
    ref_f = O.forward(np.asfortranarray(img), hps)
    ref_b = O.backward(np.asfortranarray(sino), hps)
    orbit_f = _project(ps, True, img, io, so, cuda_device)
    orbit_b = _project(ps, False, sino, io, so, cuda_device)
    angle_f = _project(ps, True, img, io, so, cuda_device, sym=0)
    angle_b = _project(ps, False, sino, io, so, cuda_device, sym=0)
    bare_f = _project(ps, True, img, io, so, cuda_device, work=False)
    bare_b = _project(ps, False, sino, io, so, cuda_device, work=False)
    for got, ref, what in ((orbit_f, ref_f, "forward"), (orbit_b, ref_b, "backprojection")):
        err = rel_l2(got, ref)
        assert err <= 1e-5, f"{name} {io}{so} {what}: rel err {err:.3e} vs float64 oracle"
    # the same sums in another order as the per-angle kernels
    assert rel_l2(orbit_f, angle_f) <= 4e-6
    assert rel_l2(orbit_b, angle_b) <= 4e-6
    # without scratch the orbit kernels gather the orbit members from the
    # image and the sinogram: the same sums as from the copies, bit for bit
    if name == "bench":
        assert ps.gr_geometry(np.float32).work_bytes >= 256 * 256 * 16
    assert np.array_equal(bare_f, orbit_f)
    assert np.array_equal(bare_b, orbit_b)


@pytest.mark.parametrize("fwd_split", [1, 2, 4, 8])
@pytest.mark.parametrize("bwd_split", [1, 2, 4, 8])
def test_radon_orbit_launch_shapes(cuda_device, fwd_split, bwd_split):
    cfg = CFGS["even"]
    ps = device_settings(cfg, cuda_device)
    hps = host_settings(cfg)
    g = ps.gr_geometry(np.float32)
    g.fwd_split, g.bwd_split = fwd_split, bwd_split
    rng = np.random.default_rng(fwd_split * 10 + bwd_split)
    img = rng.random(ps.img_shape)
    sino = rng.random(ps.sinogram_shape)
    assert rel_l2(_project(ps, True, img, "F", "F", cuda_device),
                  O.forward(np.asfortranarray(img), hps)) <= 1e-5
    assert rel_l2(_project(ps, False, sino, "F", "F", cuda_device),
                  O.backward(np.asfortranarray(sino), hps)) <= 1e-5


def test_radon_orbit_deterministic_and_weighted(cuda_device):
    """Bitwise repeatable; random angle weights are applied per row (the
    rows k and k + Na/2 of a base angle carry their own weights)."""
    import torch

    import gratopy_gb300 as gg

    rng = np.random.default_rng(3)
    cfg = dict(CFGS["even"], angle_weights=rng.uniform(0.5, 1.5, 40))
    ps = device_settings(cfg, cuda_device)
    hps = host_settings(cfg)
    assert ps.gr_geometry(np.float32).sym == 2
    sino = rng.random(ps.sinogram_shape)
    a = _project(ps, False, sino, "F", "F", cuda_device)
    b = _project(ps, False, sino, "F", "F", cuda_device)
    assert np.array_equal(a, b)
    assert rel_l2(a, O.backward(np.asfortranarray(sino), hps)) <= 1e-5
    img = torch.rand(ps.img_shape, device=cuda_device)
    assert torch.equal(gg.forwardprojection(img, ps), gg.forwardprojection(img, ps))


def test_radon_orbit_solvers(cuda_device):
    """Landweber and TV through the orbit kernels' fused epilogues match the
    same solvers through the per-angle kernels (1e-5); CG, which amplifies
    the rounding of every operation, is held to the float64 oracle within
    10 x the float32 oracle's own distance from it (the bound of the batched
    solves in tests/test_gpu_batch.py)."""
    import gratopy_gb300 as gg

    cfg = CFGS["even"]
    ps = device_settings(cfg, cuda_device)
    hps = host_settings(cfg)
    img = np.random.default_rng(8).random(ps.img_shape)
    f64 = O.forward(np.asfortranarray(img), hps)
    sino = _dev(f64, "F", cuda_device)
    g = ps.gr_geometry(np.float32)
    runs = {}
    for sym in (2, 0):
        g.sym = sym
        runs[sym] = (gg.landweber(sino, ps, 12, norm_estimate=3.0).double().cpu().numpy(),
                     gg.total_variation(sino, ps, 20.0, 10, norm_estimate=3.0)
                     .double().cpu().numpy())
    g.sym = 2
    for a, b, what in zip(runs[2], runs[0], ("landweber", "tv")):
        assert rel_l2(a, b) <= 1e-5, what
    f32 = np.asfortranarray(f64.astype(np.float32))
    ref64 = O.conjugate_gradients(np.asfortranarray(f32, np.float64), hps, 6)
    base = rel_l2(O.conjugate_gradients(f32, hps, 6), ref64)
    err = rel_l2(gg.conjugate_gradients(sino, ps, 6).double().cpu().numpy(), ref64)
    assert err <= max(1e-5, 10.0 * base), f"CG rel err {err:.3e} (float32 oracle {base:.3e})"


@pytest.mark.parametrize("io", ["F", "C"])
@pytest.mark.parametrize("so", ["F", "C"])
@pytest.mark.parametrize("copies", [0, 1, 2, 8])
def test_radon_orbit_stack(cuda_device, io, so, copies):
    """A 5-slice stack of 256^2 x 512 (2^25 pixel-angles per slice, the
    smallest that takes the orbit forward): scratch for 1 slice (one copy and
    one single-slice forward per slice), 2 (slices in pairs, the last one
    alone) or 8 (one copy of the 5 slices), against the per-angle kernels
    and, for the Fortran pair, the float64 oracle; without scratch the stack
    keeps the per-angle kernels.  The
    fused reduction of CG's forward (block partials of <W q, q>, one slice's
    after another's) covers every partial exactly once."""
    import ctypes

    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import _lib

    cfg = dict(geometry="radon", img_shape=(256, 256), angles=512, n_detectors=363)
    ps = device_settings(cfg, cuda_device)
    dt = np.dtype("float32")
    assert ps.gr_geometry(dt).sym == 2
    # the settings bind two slices' forward copies (the stack's pairs); one
    # slice's is smaller than the single slice's backprojection rows
    per_slice, rows = 256 * 256 * 16, 256 * (363 + 3) * 16
    one = ps._work_bytes[dt]
    assert one == 2 * per_slice
    rng = np.random.default_rng(31 + copies + 2 * (io == "C") + 4 * (so == "C"))
    img = rng.random(tuple(ps.img_shape) + (5,))
    saved = dict(ps._work)
    nbytes = max(rows, per_slice * copies) if copies else 0
    assert nbytes // per_slice == copies
    try:
        ps._work_bytes[dt] = nbytes
        ps._work = {}
        orbit = _project(ps, True, img, io, so, cuda_device, work=copies > 0)
        if copies:
            assert ps.gr_geometry(dt).work_bytes == nbytes
    finally:
        ps._work_bytes[dt] = one
        ps._work = saved
    angle = _project(ps, True, img, io, so, cuda_device, sym=0)
    if copies == 0:
        assert np.array_equal(orbit, angle)
        return
    assert rel_l2(orbit, angle) <= 4e-6
    for z in range(5):  # every slice, not only the stack's norm
        assert rel_l2(orbit[..., z], angle[..., z]) <= 4e-6, f"slice {z}"
    if io == "F" and so == "F":
        ref = O.forward(np.asfortranarray(img), host_settings(cfg))
        assert rel_l2(orbit, ref) <= 1e-5
    if io != so:
        return
    order = _lib.GR_ORDER_F if io == "F" else _lib.GR_ORDER_C
    g = ps.gr_geometry(dt)
    n = int(_lib.raw("gr_forward_partials")(ctypes.byref(g), 5))
    assert n == 5 * int(_lib.raw("gr_forward_partials")(ctypes.byref(g), 1))
    part = torch.full((n + 64,), float("nan"), dtype=torch.float64, device=cuda_device)
    x = _dev(img, io, cuda_device)
    q = gg.core.empty(tuple(ps.sinogram_shape) + (5,), torch.float32, so, cuda_device)
    w = ps.device_tables(dt)["w"]
    _lib.call("gr_forward_wsq", ctypes.byref(g), gg.core._ptr(q), gg.core._ptr(x),
              gg.core._ptr(w), gg.core._ptr(part), None, 5, order,
              gg.core._stream_ptr(cuda_device))
    torch.cuda.synchronize()
    got = part[:n].cpu().numpy()
    assert np.isfinite(got).all(), "a block partial was not written"
    assert np.isnan(part[n:].cpu().numpy()).all(), "a partial past the count was written"
    qh = q.double().cpu().numpy()
    want = float((qh * qh * w.double().cpu().numpy()[None, :, None]).sum())
    assert abs(got.sum() - want) <= 1e-6 * want
