"""Gradients through the projections and the unrolled TV reconstruction (GPU).

* the transposes are exact: <A x, y> = <x, A^T y> and <A* y, x> = <y, A*^T x>
  in float64 to 1e-12;
* the gradient of ||A x - y||^2 equals gratopy's analytic form
  2 (dx^2/ds) A*(W^-1 (A x - y)) (A* = gratopy's backprojection, W = angle
  weights), computed here with the float64 oracle;
* the hand-written adjoint of the unrolled TV primal-dual method (20
  iterations, checkpoint every 5) equals torch autograd through a restatement
  of the same iteration in torch operations (built on the differentiable
  projections), to 1e-12 in float64, and matches float64 central finite
  differences along 32 random directions to 1e-4 relative.

The unrolled TV map is only piecewise smooth (positivity max(0, .) and the
pointwise unit-ball projection).  With eps = 1e-3 the +-eps perturbations of
20 iterations cross those kinks for a sizeable share of pixels: measured on
these problems, the finite-difference error is ~1e-3 (2-D) up to 7e-2 (3-D
Radon, eps = 1e-4 .. 1e-5) in the directions that cross one, and ~1e-8 in
every direction at eps = 1e-6.  The TV check therefore uses eps = 1e-6 and,
like gratopy's own adjointness test, tolerates a kink crossing in at most 2
of the 32 directions.  The smooth data term is checked at eps = 1e-3.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import device_settings, host_settings, rel_l2

pytestmark = pytest.mark.gpu

CFG = {
    "radon": dict(geometry="radon", img_shape=(40, 36), angles=30, n_detectors=56),
    "fan": dict(geometry="fanbeam", img_shape=(40, 40), angles=36, n_detectors=64,
                detector_width=40.0, R=70.0, RE=30.0),
}


def _rand(shape, dtype, device, seed, order="F"):
    import torch

    import gratopy_gb300 as gg

    gen = torch.Generator(device=device).manual_seed(seed)
    t = gg.core.empty(shape, dtype, order, device)
    t.copy_(torch.rand(shape, generator=gen, device=device, dtype=dtype) - 0.5)
    return t


@pytest.mark.parametrize("geom", ["radon", "fan"])
@pytest.mark.parametrize("nz", [1, 3])
def test_transposes_exact(cuda_device, geom, nz):
    import torch

    from gratopy_gb300 import autograd as ga
    import gratopy_gb300 as gg

    ps = device_settings(CFG[geom], cuda_device)
    z = (nz,) if nz > 1 else ()
    x = _rand(ps.img_shape + z, torch.float64, cuda_device, 1)
    y = _rand(ps.sinogram_shape + z, torch.float64, cuda_device, 2)
    lhs = float((gg.forwardprojection(x, ps) * y).sum())
    rhs = float((x * ga.transpose_forward(y, ps)).sum())
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    lhs = float((gg.backprojection(y, ps) * x).sum())
    rhs = float((y * ga.transpose_back(x, ps)).sum())
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


@pytest.mark.parametrize("geom", ["radon", "fan"])
@pytest.mark.parametrize("dtype_name", ["float64", "float32"])
def test_data_term_gradient_matches_analytic(cuda_device, geom, dtype_name):
    import torch

    from gratopy_gb300 import autograd as ga

    ps = device_settings(CFG[geom], cuda_device)
    hps = host_settings(CFG[geom])
    tdt = getattr(torch, dtype_name)
    x = _rand(ps.img_shape, tdt, cuda_device, 3).requires_grad_(True)
    y = _rand(ps.sinogram_shape, tdt, cuda_device, 4)
    loss = ((ga.forward_project(x, ps) - y) ** 2).sum()
    loss.backward()
    # analytic gradient with gratopy's operators, float64 oracle
    xh = np.asfortranarray(x.detach().cpu().numpy().astype(np.float64))
    yh = np.asfortranarray(y.cpu().numpy().astype(np.float64))
    r = O.forward(xh, hps) - yh
    r = O.weight_sinogram(np.asfortranarray(r), hps, divide=True)
    # dx^2/ds as the forward kernel applies it (float32-rounded factors for
    # Radon, radon.cl:82-83)
    grad = 2 * ps.forward_scale(np.float64) * O.backward(r, hps)
    tol = 1e-10 if dtype_name == "float64" else 1e-5
    assert rel_l2(x.grad.cpu().numpy(), grad) < tol


@pytest.mark.parametrize("geom", ["radon", "fan"])
def test_backprojection_gradient(cuda_device, geom):
    import torch

    from gratopy_gb300 import autograd as ga

    ps = device_settings(CFG[geom], cuda_device)
    y = _rand(ps.sinogram_shape, torch.float64, cuda_device, 5).requires_grad_(True)
    c = _rand(ps.img_shape, torch.float64, cuda_device, 6)
    (ga.back_project(y, ps) * c).sum().backward()
    v = _rand(ps.sinogram_shape, torch.float64, cuda_device, 7)
    eps = 1e-3  # linear map: no kinks
    with torch.no_grad():
        fp = (ga.back_project(y + eps * v, ps) * c).sum()
        fm = (ga.back_project(y - eps * v, ps) * c).sum()
    fd = float((fp - fm) / (2 * eps))
    an = float((y.grad * v).sum())
    assert abs(fd - an) <= 1e-9 * abs(an)


@pytest.mark.parametrize("geom", ["radon", "fan"])
@pytest.mark.parametrize("nz,slice_thickness", [(1, 0.0), (2, 1.0)])
def test_unrolled_tv_matches_finite_differences(cuda_device, geom, nz, slice_thickness):
    import torch

    from gratopy_gb300 import autograd as ga
    import gratopy_gb300 as gg
    from gratopy_gb300.phantom import random_ellipse_image

    ps = device_settings(CFG[geom], cuda_device)
    Nx, Ny = ps.img_shape
    imgs = [random_ellipse_image(20 + k, (Ny, Nx), dtype="float64").T for k in range(nz)]
    img = np.stack(imgs, -1) if nz > 1 else imgs[0]
    img_d = torch.from_numpy(np.ascontiguousarray(img.T)).to(cuda_device).permute(
        *reversed(range(img.ndim)))
    f = gg.forwardprojection(img_d, ps)
    f = (f + 0.01 * _rand(tuple(f.shape), torch.float64, cuda_device, 8)).detach()
    nrm = gg.normest(ps, 30, dtype="float64", x0=np.ones(ps.img_shape))
    kw = dict(mu=20.0, number_iterations=20, checkpoint_every=5, slice_thickness=slice_thickness,
              norm_estimate=nrm)
    c = _rand(ps.img_shape + ((nz,) if nz > 1 else ()), torch.float64, cuda_device, 9)

    fr = f.clone().requires_grad_(True)
    (ga.tv_unrolled(fr, ps, **kw) * c).sum().backward()
    grad = fr.grad.detach()

    eps, worst, fails, errs = 1e-6, 0.0, 0, []
    for d in range(32):
        v = _rand(tuple(f.shape), torch.float64, cuda_device, 100 + d)
        with torch.no_grad():
            lp = float((ga.tv_unrolled(f + eps * v, ps, **kw) * c).sum())
            lm = float((ga.tv_unrolled(f - eps * v, ps, **kw) * c).sum())
        fd = (lp - lm) / (2 * eps)
        an = float((grad * v).sum())
        err = abs(fd - an) / max(abs(fd), 1e-12)
        errs.append(err)
        worst = max(worst, err)
        fails += err > 1e-4
    assert fails <= 2, f"{fails}/32 directions off by more than 1e-4 (worst {worst:.2e})"
    assert np.median(errs) < 1e-6

    # the float32 gradient agrees with the float64 one
    f32 = f.float().clone().requires_grad_(True)
    (ga.tv_unrolled(f32, ps, **kw) * c.float()).sum().backward()
    assert rel_l2(f32.grad.double().cpu().numpy(), grad.cpu().numpy()) < 1e-4


def _tv_torch(f, ps, mu, iterations, slice_thickness, norm_estimate, stepsize_weighting=10.0,
              detach_at=None):
    """gratopy's TV primal-dual iteration (total_variation.cl:54-167,
    gratopy.py:2686-2717) in torch operations, differentiated by torch; the
    state entering iteration ``detach_at`` is cut from the graph."""
    import torch
    import torch.nn.functional as Fn

    from gratopy_gb300 import autograd as ga

    p = ga._TVProblem(f.detach(), ps, mu, slice_thickness, stepsize_weighting, norm_estimate)
    three = f.dim() > 2 and p.z > 0

    def forward_diff(u, dim):  # u[k+1] - u[k], 0 on the last index
        pad = [0, 0] * u.dim()
        pad[2 * (u.dim() - 1 - dim) + 1] = 1
        return Fn.pad(torch.diff(u, dim=dim), pad)

    def backward_diff(v, dim):  # v[k] (0 on the last index) - v[k-1]
        n = v.shape[dim]
        zero = torch.zeros_like(v.narrow(dim, 0, 1))
        head = v.narrow(dim, 0, n - 1)
        return torch.cat([head, zero], dim) - torch.cat([zero, head], dim)

    U = torch.zeros(p.img_shape, dtype=f.dtype, device=f.device)
    Ubar, L = U, torch.zeros_like(f)
    V = [U, U, U]
    for i in range(iterations):
        if i == detach_at:
            U, Ubar, L, V = U.detach(), Ubar.detach(), L.detach(), [v.detach() for v in V]
        g = [forward_diff(Ubar, 0), forward_diff(Ubar, 1),
             forward_diff(Ubar, 2) / p.z if three else torch.zeros_like(Ubar)]
        W = [V[i] + p.sigma * g[i] for i in range(3)]
        n = torch.clamp(torch.sqrt(W[0] ** 2 + W[1] ** 2 + W[2] ** 2), min=1.0)
        V = [w / n for w in W]
        L = (L + p.sigma_l * (ga.forward_project(Ubar, ps) - f)) * p.mu2
        div = backward_diff(V[0], 0) + backward_diff(V[1], 1)
        if three:
            div = div + backward_diff(V[2], 2) / p.z
        Un = torch.clamp(U + p.tau * (div - p.norming * ga.back_project(L, ps)), min=0.0)
        Ubar, U = 2 * Un - U, Un
    return U


@pytest.mark.parametrize("geom", ["radon", "fan"])
@pytest.mark.parametrize("nz,slice_thickness", [(1, 0.0), (2, 1.0)])
def test_unrolled_tv_adjoint_equals_autograd_of_restatement(cuda_device, geom, nz,
                                                             slice_thickness):
    import torch

    from gratopy_gb300 import autograd as ga
    import gratopy_gb300 as gg

    ps = device_settings(CFG[geom], cuda_device)
    z = (nz,) if nz > 1 else ()
    x = _rand(ps.img_shape + z, torch.float64, cuda_device, 12) + 0.5
    f = (gg.forwardprojection(x, ps) + 0.01 * _rand(ps.sinogram_shape + z, torch.float64,
                                                      cuda_device, 13)).detach()
    nrm = gg.normest(ps, 30, dtype="float64", x0=np.ones(ps.img_shape))
    c = _rand(ps.img_shape + z, torch.float64, cuda_device, 14)
    fa = f.clone().requires_grad_(True)
    ua = ga.tv_unrolled(fa, ps, 20.0, number_iterations=20, checkpoint_every=5,
                        slice_thickness=slice_thickness, norm_estimate=nrm)
    (ua * c).sum().backward()
    fb = f.clone().requires_grad_(True)
    ub = _tv_torch(fb, ps, 20.0, 20, slice_thickness, nrm)
    (ub * c).sum().backward()
    assert rel_l2(ua.detach().cpu().numpy(), ub.detach().cpu().numpy()) < 1e-12
    assert rel_l2(fa.grad.cpu().numpy(), fb.grad.cpu().numpy()) < 1e-12


@pytest.mark.parametrize("geom", ["radon", "fan"])
def test_unrolled_tv_truncated_backward(cuda_device, geom):
    """Differentiation through the last 7 of 17 iterations (checkpoints every
    3 from iteration 10) equals torch autograd of the restatement with its
    state cut from the graph at iteration 10; the forward value is the full
    17-iteration one."""
    import torch

    from gratopy_gb300 import autograd as ga
    import gratopy_gb300 as gg

    ps = device_settings(CFG[geom], cuda_device)
    x = _rand(ps.img_shape, torch.float64, cuda_device, 21) + 0.5
    f = (gg.forwardprojection(x, ps) + 0.01 * _rand(ps.sinogram_shape, torch.float64,
                                                      cuda_device, 22)).detach()
    nrm = gg.normest(ps, 30, dtype="float64", x0=np.ones(ps.img_shape))
    c = _rand(ps.img_shape, torch.float64, cuda_device, 23)
    fa = f.clone().requires_grad_(True)
    ua = ga.tv_unrolled(fa, ps, 20.0, number_iterations=17, checkpoint_every=3,
                        slice_thickness=0.0, norm_estimate=nrm, backward_iterations=7)
    (ua * c).sum().backward()
    fb = f.clone().requires_grad_(True)
    ub = _tv_torch(fb, ps, 20.0, 17, 0.0, nrm, detach_at=10)
    (ub * c).sum().backward()
    assert rel_l2(ua.detach().cpu().numpy(), ub.detach().cpu().numpy()) < 1e-12
    assert rel_l2(fa.grad.cpu().numpy(), fb.grad.cpu().numpy()) < 1e-12
    full = ga.tv_unrolled(f, ps, 20.0, number_iterations=17, norm_estimate=nrm)
    assert torch.equal(ua.detach(), full)


def test_tv_unrolled_forward_equals_total_variation(cuda_device):
    import torch

    from gratopy_gb300 import autograd as ga
    import gratopy_gb300 as gg

    ps = device_settings(CFG["radon"], cuda_device)
    f = _rand(ps.sinogram_shape, torch.float32, cuda_device, 10)
    a = ga.tv_unrolled(f, ps, 20.0, number_iterations=17, checkpoint_every=5, norm_estimate=2.0)
    b = gg.total_variation(f, ps, 20.0, number_iterations=17, norm_estimate=2.0)
    assert torch.equal(a, b)


@pytest.mark.parametrize("solver", ["landweber", "cg", "tv"])
def test_graph_and_direct_launches_agree(cuda_device, solver):
    """Loops replayed from CUDA graphs give the same bits as direct launches."""
    import torch

    import gratopy_gb300 as gg

    ps = device_settings(CFG["fan"], cuda_device)
    f = _rand(ps.sinogram_shape, torch.float32, cuda_device, 11)
    nrm = gg.normest(ps, 40, x0=np.ones(ps.img_shape))
    if solver == "landweber":
        run = lambda g: gg.landweber(f, ps, 60, norm_estimate=nrm, use_graph=g)  # noqa: E731
    elif solver == "cg":
        run = lambda g: gg.conjugate_gradients(f, ps, 60, use_graph=g)  # noqa: E731
    else:
        run = lambda g: gg.total_variation(f, ps, 10.0, 60, norm_estimate=nrm, use_graph=g)  # noqa: E731
    a, b = run(True), run(False)
    assert torch.isfinite(a).all()
    assert torch.equal(a, b)
    x0 = np.random.default_rng(0).standard_normal(ps.img_shape)
    assert gg.normest(ps, 40, x0=x0, use_graph=True) == gg.normest(ps, 40, x0=x0, use_graph=False)
