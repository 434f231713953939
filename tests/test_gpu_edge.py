"""Degenerate sizes (single pixel rows/columns, one angle, one or two
detector bins) through every projection kernel, against the oracle."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import device_settings, host_settings

pytestmark = pytest.mark.gpu

FAN = dict(detector_width=4.0, R=10.0, RE=5.0)
CASES = {
    "radon_1x1": dict(geometry="radon", img_shape=(1, 1), angles=3, n_detectors=2),
    "radon_1x7": dict(geometry="radon", img_shape=(1, 7), angles=5, n_detectors=9),
    "radon_7x1_one_ray": dict(geometry="radon", img_shape=(7, 1), angles=1, n_detectors=1),
    "radon_33x17_one_angle": dict(geometry="radon", img_shape=(33, 17), angles=1, n_detectors=40),
    "fan_1x1": dict(geometry="fanbeam", img_shape=(1, 1), angles=3, n_detectors=2, **FAN),
    "fan_1x7": dict(geometry="fanbeam", img_shape=(1, 7), angles=5, n_detectors=9, **FAN),
    "fan_7x1_one_ray": dict(geometry="fanbeam", img_shape=(7, 1), angles=1, n_detectors=1, **FAN),
    "fan_33x17_two_angles": dict(geometry="fanbeam", img_shape=(33, 17), angles=2, n_detectors=40,
                                 detector_width=40.0, R=70.0, RE=30.0),
}


def _rel(got, ref):
    scale = max(np.linalg.norm(ref), 1e-30)
    return np.linalg.norm(got - ref) / scale


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-12), (np.float32, 1e-5)])
@pytest.mark.parametrize("order", ["F", "C"])
@pytest.mark.parametrize("nz", [1, 3])
def test_degenerate_sizes(cuda_device, name, dtype, tol, order, nz):
    import torch

    import gratopy_gb300 as gg

    ps = device_settings(CASES[name], cuda_device)
    hps = host_settings(CASES[name])
    shape = tuple(ps.img_shape) + ((nz,) if nz > 1 else ())
    img = np.require(np.random.default_rng(1).random(shape), np.float64, order)
    ref_sino = O.forward(img, hps)
    ref_back = O.backward(np.require(ref_sino, np.float64, order), hps)
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    img_d = gg.core.empty(shape, tdt, order, cuda_device)
    img_d.copy_(torch.from_numpy(img.astype(dtype)))
    sino = gg.forwardprojection(img_d, ps)
    back = gg.backprojection(sino, ps)
    assert tuple(sino.shape) == ref_sino.shape
    assert _rel(sino.double().cpu().numpy(), ref_sino) < tol
    assert _rel(back.double().cpu().numpy(), ref_back) < tol


@pytest.mark.parametrize("name", sorted(CASES))
def test_degenerate_sparse_matrix_equals_projection(cuda_device, name):
    import torch

    import gratopy_gb300 as gg

    ps = device_settings(CASES[name], cuda_device)
    Nx, Ny = ps.img_shape
    Ns, Na = ps.sinogram_shape
    M = ps.create_sparse_matrix(dtype=np.float64, order="F")
    img = np.random.default_rng(2).random((Nx, Ny))
    x = gg.core.empty((Nx, Ny), torch.float64, "F", cuda_device)
    x.copy_(torch.from_numpy(img))
    want = gg.forwardprojection(x, ps).cpu().numpy()
    got = (M @ img.reshape(-1, order="F")).reshape(Ns, Na, order="F")
    assert _rel(got, want) < 1e-12


def test_degenerate_problems_in_a_batch(cuda_device):
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import batch as gb

    problems = []
    for k, name in enumerate(sorted(CASES)):
        ps = device_settings(CASES[name], cuda_device)
        img = gg.core.empty(ps.img_shape, torch.float32, "F", cuda_device)
        img.copy_(torch.from_numpy(np.random.default_rng(k).random(ps.img_shape)))
        sino = gg.forwardprojection(img, ps)
        # CG only where 4 iterations cannot exhaust the rank (0/0 step sizes
        # after exact convergence, as in the reference)
        rank = min(ps.img_shape[0] * ps.img_shape[1], ps.sinogram_shape[0] * ps.sinogram_shape[1])
        solver = "cg" if rank > 8 else ("landweber", "tv")[k % 2]
        nrm = gg.normest(ps, 20, x0=np.ones(ps.img_shape))
        problems.append(gb.Problem(ps, sino, solver, 4, mu=10.0, norm_estimate=nrm))
    out = gb.BatchedReconstruction(problems, cuda_device).run()
    for pr, got in zip(problems, out):
        ps = pr.settings
        ps.gr_geometry(np.float32).bwd_split = 1  # the batched launch shapes
        ps.gr_geometry(np.float32).sym = 0
        if pr.solver == "landweber":
            want = gg.landweber(pr.sino, ps, 4, norm_estimate=pr.norm_estimate)
        elif pr.solver == "cg":
            want = gg.conjugate_gradients(pr.sino, ps, 4)
        else:
            want = gg.total_variation(pr.sino, ps, 10.0, 4, norm_estimate=pr.norm_estimate)
        assert torch.isfinite(got).all()
        assert _rel(got.double().cpu().numpy(), want.double().cpu().numpy()) < 1e-5
