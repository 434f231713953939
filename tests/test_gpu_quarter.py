"""Quarter-turn shared projections (float32 fan beam, single slices): the
forward projection sharing a pixel's weights over the four angles of an
orbit and the backprojection over pixel orbits, against the oracle, the
per-angle kernels, and through the fused solver epilogues."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import device_settings, host_settings, rel_l2

pytestmark = pytest.mark.gpu

CFGS = {
    "plain": dict(geometry="fanbeam", img_shape=(40, 40), angles=36, n_detectors=64,
                  detector_width=40.0, R=70.0, RE=30.0),
    "odd_side_reversed": dict(geometry="fanbeam", img_shape=(37, 37), angles=20, n_detectors=50,
                              detector_width=40.0, R=70.0, RE=30.0, reverse_detector=True),
    "shifted_detector": dict(geometry="fanbeam", img_shape=(64, 64), angles=48, n_detectors=90,
                             detector_width=60.0, R=150.0, RE=60.0, detector_shift=4.0),
    "one_pixel": dict(geometry="fanbeam", img_shape=(1, 1), angles=4, n_detectors=3,
                      detector_width=4.0, R=10.0, RE=5.0),
    "bench_like": dict(geometry="fanbeam", img_shape=(128, 128), angles=360, n_detectors=192,
                       detector_width=400.0, R=400.0, RE=200.0),
    "two_pixels": dict(geometry="fanbeam", img_shape=(2, 2), angles=8, n_detectors=5,
                       detector_width=6.0, R=10.0, RE=5.0),
    "narrow_detector": dict(geometry="fanbeam", img_shape=(70, 70), angles=12, n_detectors=30,
                            detector_width=30.0, R=200.0, RE=90.0),
}


def _forward(ps, img_np, order, sym, cuda_device):
    import torch

    import gratopy_gb300 as gg

    g = ps.gr_geometry(np.float32)
    saved = g.sym
    g.sym = sym
    try:
        x = gg.core.empty(ps.img_shape, torch.float32, order, cuda_device)
        x.copy_(torch.from_numpy(img_np.astype(np.float32)))
        return gg.forwardprojection(x, ps).double().cpu().numpy()
    finally:
        g.sym = saved


@pytest.mark.parametrize("name", sorted(CFGS))
@pytest.mark.parametrize("order", ["F", "C"])
def test_quarter_forward(cuda_device, name, order):
    ps = device_settings(CFGS[name], cuda_device)
    assert ps.quarter_maps() is not None and ps.gr_geometry(np.float32).sym == 4
    img = np.random.default_rng(1).random(ps.img_shape)
    ref = O.forward(np.asfortranarray(img), host_settings(CFGS[name]))
    shared = _forward(ps, img, order, 4, cuda_device)
    direct = _forward(ps, img, order, 0, cuda_device)
    assert rel_l2(shared, ref) < 1e-5
    # float32 sums of a few hundred terms in another order (the turned
    # image's rows are walked along the base angle's axis)
    assert rel_l2(shared, direct) < 4e-6


def _backward(ps, sino_np, order, sym, split, cuda_device):
    import torch

    import gratopy_gb300 as gg

    g = ps.gr_geometry(np.float32)
    saved = (g.sym, g.bwd_split)
    g.sym, g.bwd_split = sym, split
    try:
        s = gg.core.empty(ps.sinogram_shape, torch.float32, order, cuda_device)
        s.copy_(torch.from_numpy(sino_np.astype(np.float32)))
        return gg.backprojection(s, ps).double().cpu().numpy()
    finally:
        g.sym, g.bwd_split = saved


@pytest.mark.parametrize("name", sorted(CFGS))
@pytest.mark.parametrize("order", ["F", "C"])
@pytest.mark.parametrize("split", [1, 2, 4, 8])
def test_quarter_backprojection(cuda_device, name, order, split):
    """Even sides run on pixel orbits with ``split`` angle groups, odd sides
    keep the per-angle kernel; bins off the detector contribute nothing."""
    ps = device_settings(CFGS[name], cuda_device)
    sino = np.random.default_rng(3).random(ps.sinogram_shape)
    ref = O.backward(np.asfortranarray(sino), host_settings(CFGS[name]))
    shared = _backward(ps, sino, order, 4, split, cuda_device)
    direct = _backward(ps, sino, order, 0, split, cuda_device)
    assert rel_l2(shared, ref) < 1e-5
    assert rel_l2(shared, direct) < 4e-6


def _raw(ps, fwd, data_np, work, work_bytes, cuda_device, mirror=True):
    """One projection through gr_forward / gr_backward with the given scratch
    (and the geometry's mirror switched off with ``mirror=False``)."""
    import ctypes

    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import _lib, core

    g = _lib.GrGeometry.from_buffer_copy(ps.gr_geometry(np.float32))
    g.work, g.work_bytes = work, work_bytes
    if not mirror:
        g.mirror = 0
    in_shape, out_shape = ((ps.img_shape, ps.sinogram_shape) if fwd
                           else (ps.sinogram_shape, ps.img_shape))
    x = gg.core.empty(in_shape, torch.float32, "F", cuda_device)
    x.copy_(torch.from_numpy(data_np.astype(np.float32)))
    out = gg.core.empty(out_shape, torch.float32, "F", cuda_device)
    _lib.call("gr_forward" if fwd else "gr_backward", ctypes.byref(g), core._ptr(out),
              core._ptr(x), 1, 0, 0, core._stream_ptr(cuda_device))
    return out.double().cpu().numpy()


# sizes at which the orbit kernels work from interleaved scratch copies
# (16 * 2^20 pixel-angles for the forward, 12 * 2^20 for the backprojection)
COPY_CFGS = {
    "copy_even": dict(geometry="fanbeam", img_shape=(360, 360), angles=480, n_detectors=540,
                      detector_width=400.0, R=400.0, RE=200.0),
    "copy_odd": dict(geometry="fanbeam", img_shape=(361, 361), angles=480, n_detectors=530,
                     detector_width=400.0, R=400.0, RE=200.0, detector_shift=3.0),
}


def test_small_problems_bind_no_scratch(cuda_device):
    for name in ("plain", "bench_like", "two_pixels"):
        ps = device_settings(CFGS[name], cuda_device)
        g = ps.gr_geometry(np.float32)
        assert g.sym == 4 and not g.work and g.work_bytes == 0


@pytest.mark.parametrize("name", sorted(COPY_CFGS))
@pytest.mark.parametrize("fwd", [True, False])
def test_orbit_scratch_and_direct_gather_agree(cuda_device, name, fwd):
    """With the interleaved scratch copy, without scratch, and with scratch
    one float4 too small (the kernels then read their input directly).  The
    copy and the direct gathers sum in the same order within 1e-6 with the
    mirror switched off; the forward from the copy with the mirror (the bins
    beyond the middle from the mirrored weights) within 4e-6."""
    import ctypes

    from gratopy_gb300 import _lib

    cfg = COPY_CFGS[name]
    ps = device_settings(cfg, cuda_device)
    hps = host_settings(cfg)
    g = ps.gr_geometry(np.float32)
    Nx, Ny = ps.img_shape
    Ns, Na = ps.sinogram_shape
    fwd_need = Nx * Ny * 16
    # row copy: Ns + 3 entries (one zero before the detector, two after) and
    # a 4-float4 geometry record per base angle
    bwd_need = (Na // 4) * (Ns + 3 + 4) * 16 if Nx % 2 == 0 else 0
    need = int(_lib.raw("gr_work_bytes")(ctypes.byref(g), 1))
    assert need == max(fwd_need, bwd_need)
    assert g.sym == 4 and g.work and g.work_bytes == need
    rng = np.random.default_rng(6)
    if fwd:
        data = rng.random(ps.img_shape)
        ref = O.forward(np.asfortranarray(data), hps)
        own = fwd_need
    else:
        data = rng.random(ps.sinogram_shape)
        ref = O.backward(np.asfortranarray(data), hps)
        own = bwd_need
    with_copy = _raw(ps, fwd, data, g.work, need, cuda_device, mirror=False)
    direct = _raw(ps, fwd, data, None, 0, cuda_device)
    assert rel_l2(with_copy, ref) < 1e-5 and rel_l2(direct, ref) < 1e-5
    assert rel_l2(with_copy, direct) < 1e-6
    mirrored = _raw(ps, fwd, data, g.work, need, cuda_device)
    assert rel_l2(mirrored, ref) < 1e-5 and rel_l2(mirrored, direct) < 4e-6
    if own:
        small = _raw(ps, fwd, data, g.work, own - 16, cuda_device)
        assert (small == direct).all()


# a stack whose slices take the orbit kernels (from 256 * 2^20 pixel-angles
# per slice); one slice of copy per launch pair unless the scratch holds more
STACK_CFG = dict(geometry="fanbeam", img_shape=(768, 768), angles=480, n_detectors=1100,
                 detector_width=400.0, R=400.0, RE=200.0)


def _stack_call(ps, fwd, x, nz, order, work, work_bytes, cuda_device, sym=4, mirror=True):
    import ctypes

    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import _lib, core

    g = _lib.GrGeometry.from_buffer_copy(ps.gr_geometry(np.float32))
    g.sym, g.work, g.work_bytes = sym, work, work_bytes
    if not mirror:
        g.mirror = 0
    shape = (ps.sinogram_shape if fwd else ps.img_shape) + (nz,)
    out = gg.core.empty(shape, torch.float32, order, cuda_device)
    of = core._oflag(order)
    _lib.call("gr_forward" if fwd else "gr_backward", ctypes.byref(g), core._ptr(out),
              core._ptr(x), nz, of, of, core._stream_ptr(cuda_device))
    return out


@pytest.mark.parametrize("order", ["F", "C"])
@pytest.mark.parametrize("fwd", [True, False])
def test_orbit_kernels_on_stacks(cuda_device, order, fwd):
    """Slices of a stack in chunks of 1, 2 and 3 slices of scratch and without
    scratch agree with each other, with the per-angle 4-slice kernels, and
    (first and last slice) with the oracle."""
    import ctypes

    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import _lib

    nz = 3
    ps = device_settings(STACK_CFG, cuda_device)
    hps = host_settings(STACK_CFG)
    g = ps.gr_geometry(np.float32)
    per_slice = int(_lib.raw("gr_work_bytes")(ctypes.byref(g), 1))
    assert per_slice > 0 and int(_lib.raw("gr_work_bytes")(ctypes.byref(g), nz)) == nz * per_slice
    buf = torch.empty(nz * per_slice, dtype=torch.uint8, device=cuda_device)
    in_shape = (ps.img_shape if fwd else ps.sinogram_shape) + (nz,)
    data = np.random.default_rng(8).random(in_shape)
    x = gg.core.empty(in_shape, torch.float32, order, cuda_device)
    x.copy_(torch.from_numpy(data.astype(np.float32)))
    runs = {k: _stack_call(ps, fwd, x, nz, order, buf.data_ptr(), k * per_slice, cuda_device)
            for k in (1, 2, 3)}
    direct = _stack_call(ps, fwd, x, nz, order, None, 0, cuda_device)
    per_angle = _stack_call(ps, fwd, x, nz, order, None, 0, cuda_device, sym=0)
    unmirrored = _stack_call(ps, fwd, x, nz, order, buf.data_ptr(), per_slice, cuda_device,
                             mirror=False)
    assert torch.equal(runs[1], runs[2]) and torch.equal(runs[1], runs[3])
    d = direct.double().cpu().numpy()
    r = runs[1].double().cpu().numpy()
    # the copy against the direct gathers with the mirror off (the same
    # order of sums), and with the mirror (another order for half the bins)
    assert rel_l2(unmirrored.double().cpu().numpy(), d) < 1e-6
    assert rel_l2(r, d) < (4e-6 if fwd else 1e-6)
    assert rel_l2(r, per_angle.double().cpu().numpy()) < 4e-6
    for k in (0, nz - 1):
        sl = np.asfortranarray(data[:, :, k])
        ref = O.forward(sl, hps) if fwd else O.backward(sl, hps)
        assert rel_l2(r[:, :, k], ref) < 1e-5


def test_orbit_stack_solver_partials(cuda_device):
    """CG's fused reductions on a stack run in per-slice chunks: the block
    partials of every chunk land after the previous chunk's."""
    import torch

    import gratopy_gb300 as gg

    nz = 2
    ps = device_settings(STACK_CFG, cuda_device)
    rng = np.random.default_rng(9)
    img = gg.core.empty(ps.img_shape + (nz,), torch.float32, "F", cuda_device)
    img.copy_(torch.from_numpy(rng.random(ps.img_shape + (nz,)).astype(np.float32)))
    sino = gg.forwardprojection(img, ps)
    g = ps.gr_geometry(np.float32)
    res = {}
    for sym in (4, 0):
        g.sym = sym
        res[sym] = gg.conjugate_gradients(sino, ps, 4).double().cpu().numpy()
    g.sym = 4
    assert rel_l2(res[4], res[0]) < 1e-5


def test_orbit_scratch_per_stream(cuda_device):
    import torch

    import gratopy_gb300 as gg

    ps = device_settings(COPY_CFGS["copy_even"], cuda_device)
    sino = torch.rand(ps.sinogram_shape, device=cuda_device).T.contiguous().T
    a = gg.backprojection(sino, ps)
    side = torch.cuda.Stream(cuda_device)
    side.wait_stream(torch.cuda.current_stream(cuda_device))
    with torch.cuda.stream(side):
        b = gg.backprojection(sino, ps)
    torch.cuda.current_stream(cuda_device).wait_stream(side)
    keys = [k for k in ps._work if k[0] == np.dtype(np.float32)]
    assert len(keys) == 2 and keys[0][1] != keys[1][1]
    assert torch.equal(a, b)


@pytest.mark.parametrize("size", ["small", "copy"])
def test_orbit_kernels_apply_each_angles_own_weight(cuda_device, size):
    """Random angle weights (equispaced angles otherwise weigh alike): every
    row a + j Na/4 of the orbit backprojection carries its own angle's
    weight, with and without the row copy, in the solver epilogues too."""
    base = CFGS["shifted_detector"] if size == "small" else COPY_CFGS["copy_even"]
    na = base["angles"]
    cfg = dict(base, angle_weights=np.random.default_rng(12).uniform(0.5, 1.5, na))
    ps = device_settings(cfg, cuda_device)
    hps = host_settings(cfg)
    g = ps.gr_geometry(np.float32)
    assert g.sym == 4 and (bool(g.work) == (size == "copy"))
    sino = np.random.default_rng(13).random(ps.sinogram_shape)
    ref = O.backward(np.asfortranarray(sino), hps)
    shared = _backward(ps, sino, "F", 4, 0, cuda_device)
    direct = _backward(ps, sino, "F", 0, 0, cuda_device)
    assert rel_l2(shared, ref) < 1e-5
    assert rel_l2(shared, direct) < 4e-6


def test_quarter_backprojection_is_deterministic(cuda_device):
    ps = device_settings(CFGS["bench_like"], cuda_device)
    sino = np.random.default_rng(4).random(ps.sinogram_shape)
    a = _backward(ps, sino, "F", 4, 4, cuda_device)
    b = _backward(ps, sino, "F", 4, 4, cuda_device)
    assert (a == b).all()


@pytest.mark.parametrize("name", ["plain", "shifted_detector", "bench_like", "copy_even"])
def test_quarter_projections_in_solver_steps(cuda_device, name):
    """Landweber and TV agree with the per-angle kernels to float32 rounding;
    CG amplifies rounding, so it is held to the float32 solver bound of the
    parity tests: within max(1e-5, 3 x the float32 oracle's own distance
    from the float64 oracle)."""
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300.phantom import random_ellipse_image

    cfg = {**CFGS, **COPY_CFGS}[name]
    ps = device_settings(cfg, cuda_device)
    hps = host_settings(cfg)
    # a phantom's projection with 1% noise (a well-posed problem, as in the
    # solver parity tests)
    img = np.asfortranarray(random_ellipse_image(2, hps.img_shape[::-1]).T.astype(np.float64))
    f_np = O.forward(img, hps)
    f_np = np.asfortranarray(
        f_np + 0.01 * np.abs(f_np).max() * np.random.default_rng(2).standard_normal(f_np.shape))
    f = gg.core.empty(ps.sinogram_shape, torch.float32, "F", cuda_device)
    f.copy_(torch.from_numpy(f_np.astype(np.float32)))
    g = ps.gr_geometry(np.float32)
    res = {}
    for sym in (4, 0):
        g.sym = sym
        res[sym] = (gg.conjugate_gradients(f, ps, 5).double().cpu().numpy(),
                    gg.landweber(f, ps, 5, norm_estimate=5.0).double().cpu().numpy(),
                    gg.total_variation(f, ps, 10.0, 5, norm_estimate=5.0).double().cpu().numpy())
    g.sym = 4
    f32 = np.asfortranarray(f_np.astype(np.float32))
    cg_ref = O.conjugate_gradients(f32.astype(np.float64), hps, 5)
    base = rel_l2(O.conjugate_gradients(f32, hps, 5), cg_ref)
    for sym in (4, 0):
        err = rel_l2(res[sym][0], cg_ref)
        assert err <= max(1e-5, 3 * base), f"sym {sym}: CG rel err {err:.3e}, float32 oracle {base:.3e}"
    for a, b in zip(res[4][1:], res[0][1:]):
        assert rel_l2(a, b) < 1e-5


def test_asymmetric_geometry_keeps_the_per_angle_kernel(cuda_device):
    ps = device_settings(dict(CFGS["plain"], img_shape=(40, 36)), cuda_device)
    assert ps.quarter_maps() is None and ps.gr_geometry(np.float32).sym == 0
