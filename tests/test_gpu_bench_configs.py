"""GPU parity of the benchmarked workloads, built exactly as ``bench.py`` builds them.

* Fan beam 512 x 512, 360 angles over [0, 2 pi), 768 detectors, RE 200,
  R 400, detector width 400, image width 0.9 x automatic (``bench.WORKLOAD``
  and ``bench.make_image``): the angle set is quarter-turn symmetric, so the
  forward runs ``orbit_pixels``/``orbit_pixels_tiled`` + ``fan_fwd_quarter``
  and the backprojection ``orbit_rows`` + ``fan_bwd_orbit``; every launch
  shape the autotuner can pick is checked, in all four memory-order pairs.
* Radon 256 x 256, 180 angles, 363 detectors, float32 and float64.
* 50 CG iterations on the fan-beam workload with 1% Gaussian noise.

Tolerances (relative L2 against the float64 oracle on the same inputs):
projections 1e-5 (float32) and 1e-12 (float64); CG in float32 within
max(1e-5, 3 x the float32 oracle's own drift from float64), the solver bound
of tests/test_gpu_solvers.py.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "tests" / "golden"))
import configs  # noqa: E402

import bench  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.helpers import device_settings, host_settings, rel_l2  # noqa: E402

pytestmark = pytest.mark.gpu

SPLITS = (1, 2, 4, 8)


def _to_device(a: np.ndarray, order: str, device):
    import torch

    import gratopy_gb300 as gg

    t = gg.core.empty(a.shape, torch.float64 if a.dtype == np.float64 else torch.float32, order,
                      device)
    t.copy_(torch.from_numpy(np.ascontiguousarray(a)))
    return t


@pytest.fixture(scope="module")
def fan512(cuda_device):
    cfg = dict(bench.WORKLOAD)
    hps = host_settings(cfg)
    ps = device_settings(cfg, cuda_device)
    img = bench.make_image()  # (Nx, Ny) float32, Fortran order, as the bench uploads it
    sino_in = np.asfortranarray(
        np.random.default_rng(11).random(hps.sinogram_shape).astype(np.float32))
    ref_fwd = O.forward(np.asfortranarray(img, dtype=np.float64), hps)
    ref_bwd = O.backward(np.asfortranarray(sino_in, dtype=np.float64), hps)
    return dict(hps=hps, ps=ps, img=img, sino_in=sino_in, ref_fwd=ref_fwd, ref_bwd=ref_bwd)


def test_bench_fan512_uses_orbit_kernels_and_copies(cuda_device, fan512):
    """The benchmark geometry takes the quarter-turn kernels with scratch bound."""
    import ctypes

    from gratopy_gb300 import _lib

    ps = fan512["ps"]
    g = ps.gr_geometry(np.float32)
    assert g.sym == 4, "the benchmark angle set must be detected as quarter-turn symmetric"
    need = int(_lib.raw("gr_work_bytes")(ctypes.byref(g), 1))
    assert need > 0 and g.work and g.work_bytes >= need, "orbit-copy scratch not bound"


@pytest.mark.parametrize("io", ["F", "C"])
@pytest.mark.parametrize("so", ["F", "C"])
@pytest.mark.parametrize("fwd_split", SPLITS)
def test_bench_fan512_forward(cuda_device, fan512, io, so, fwd_split):
    import torch

    import gratopy_gb300 as gg

    ps = fan512["ps"]
    g = ps.gr_geometry(np.float32)
    saved = g.fwd_split
    g.fwd_split = fwd_split
    try:
        img = _to_device(fan512["img"], io, cuda_device)
        sino = gg.core.empty(ps.sinogram_shape, torch.float32, so, cuda_device)
        gg.forwardprojection(img, ps, sino=sino)
        torch.cuda.synchronize()
    finally:
        g.fwd_split = saved
    err = rel_l2(sino.double().cpu().numpy(), fan512["ref_fwd"])
    assert err <= 1e-5, f"forward rel err {err:.3e} vs float64 oracle ({io}{so}, split {fwd_split})"


@pytest.mark.parametrize("io", ["F", "C"])
@pytest.mark.parametrize("so", ["F", "C"])
@pytest.mark.parametrize("bwd_split", SPLITS)
def test_bench_fan512_backward(cuda_device, fan512, io, so, bwd_split):
    import torch

    import gratopy_gb300 as gg

    ps = fan512["ps"]
    g = ps.gr_geometry(np.float32)
    saved = g.bwd_split
    g.bwd_split = bwd_split
    try:
        sino = _to_device(fan512["sino_in"], so, cuda_device)
        back = gg.core.empty(ps.img_shape, torch.float32, io, cuda_device)
        gg.backprojection(sino, ps, img=back)
        torch.cuda.synchronize()
    finally:
        g.bwd_split = saved
    err = rel_l2(back.double().cpu().numpy(), fan512["ref_bwd"])
    assert err <= 1e-5, f"backward rel err {err:.3e} vs float64 oracle ({io}{so}, split {bwd_split})"


def test_bench_fan512_step_as_timed(cuda_device, fan512):
    """forward then backprojection of the bench image, with the bench's default
    pinned shapes (8, 8), compared end to end with the oracle's A* A x."""
    import torch

    import gratopy_gb300 as gg

    ps = fan512["ps"]
    g = ps.gr_geometry(np.float32)
    saved = (g.fwd_split, g.bwd_split)
    g.fwd_split, g.bwd_split = 8, 8
    try:
        img = _to_device(fan512["img"], "F", cuda_device)
        sino = gg.core.empty(ps.sinogram_shape, torch.float32, "F", cuda_device)
        back = gg.core.empty(ps.img_shape, torch.float32, "F", cuda_device)
        for _ in range(3):  # repeated steps reuse the scratch copies
            gg.forwardprojection(img, ps, sino=sino)
            gg.backprojection(sino, ps, img=back)
        torch.cuda.synchronize()
    finally:
        g.fwd_split, g.bwd_split = saved
    ref_back = O.backward(fan512["ref_fwd"], fan512["hps"])
    assert rel_l2(sino.double().cpu().numpy(), fan512["ref_fwd"]) <= 1e-5
    err = rel_l2(back.double().cpu().numpy(), ref_back)
    assert err <= 1e-5, f"A*A x rel err {err:.3e} vs float64 oracle"


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("io", ["F", "C"])
@pytest.mark.parametrize("so", ["F", "C"])
def test_bench_radon256(cuda_device, dtype, io, so):
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300.phantom import random_ellipse_image

    cfg = dict(bench.RADON_WORKLOAD)
    hps = host_settings(cfg)
    ps = device_settings(cfg, cuda_device)
    host = random_ellipse_image(bench.SEED, (256, 256), count=10, dtype="float64").T
    img_np = np.require(host, dtype, io)
    sino_in = np.require(np.random.default_rng(5).random(hps.sinogram_shape), dtype, so)
    ref_fwd = O.forward(np.require(img_np, np.float64, io), hps, order=so)
    ref_bwd = O.backward(np.require(sino_in, np.float64, so), hps, order=io)
    img = _to_device(img_np, io, cuda_device)
    sino = gg.core.empty(ps.sinogram_shape, img.dtype, so, cuda_device)
    gg.forwardprojection(img, ps, sino=sino)
    back = gg.core.empty(ps.img_shape, img.dtype, io, cuda_device)
    gg.backprojection(_to_device(sino_in, so, cuda_device), ps, img=back)
    torch.cuda.synchronize()
    tol = 1e-5 if dtype == np.float32 else 1e-12
    e_f = rel_l2(sino.cpu().numpy(), ref_fwd)
    e_b = rel_l2(back.cpu().numpy(), ref_bwd)
    assert e_f <= tol, f"forward rel err {e_f:.3e}"
    assert e_b <= tol, f"backward rel err {e_b:.3e}"


@pytest.mark.parametrize("fwd_split", SPLITS)
@pytest.mark.parametrize("bwd_split", SPLITS)
def test_bench_radon256_launch_shapes(cuda_device, fwd_split, bwd_split):
    """Every launch shape the autotuner can pick for the Radon workload (float32)."""
    import torch

    import gratopy_gb300 as gg

    cfg = dict(bench.RADON_WORKLOAD)
    hps = host_settings(cfg)
    ps = device_settings(cfg, cuda_device)
    img_np = np.asfortranarray(np.random.default_rng(9).random(hps.img_shape), np.float32)
    g = ps.gr_geometry(np.float32)
    g.fwd_split, g.bwd_split = fwd_split, bwd_split
    sino = gg.forwardprojection(_to_device(img_np, "F", cuda_device), ps)
    back = gg.backprojection(sino, ps)
    torch.cuda.synchronize()
    ref_fwd = O.forward(np.asfortranarray(img_np, np.float64), hps)
    ref_bwd = O.backward(np.asfortranarray(sino.double().cpu().numpy()), hps)
    assert rel_l2(sino.cpu().numpy(), ref_fwd) <= 1e-5
    assert rel_l2(back.cpu().numpy(), ref_bwd) <= 1e-5


def test_cg50_bench_fan512(cuda_device, fan512):
    """50 CG iterations on the benchmark geometry with 1% Gaussian noise."""
    import torch

    import gratopy_gb300 as gg

    hps, ps = fan512["hps"], fan512["ps"]
    clean = fan512["ref_fwd"]
    noise = np.random.default_rng(bench.SEED).standard_normal(clean.shape)
    sino32 = np.asfortranarray((clean + 0.01 * np.abs(clean).max() * noise).astype(np.float32))
    ref64 = O.conjugate_gradients(np.asfortranarray(sino32, np.float64), hps, 50)
    ref32 = O.conjugate_gradients(sino32, hps, 50)
    out = gg.conjugate_gradients(_to_device(sino32, "F", cuda_device), ps, 50)
    torch.cuda.synchronize()
    err = rel_l2(out.double().cpu().numpy(), ref64)
    base = rel_l2(ref32, ref64)
    print(f"CG-50 fan 512^2: GPU float32 vs float64 oracle {err:.3e}; "
          f"float32 oracle vs float64 oracle {base:.3e}")
    assert err <= max(1e-5, 3.0 * base), f"CG-50 rel err {err:.3e} (float32 oracle {base:.3e})"
