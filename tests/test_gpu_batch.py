"""Batched persistent reconstruction against the per-call solvers (GPU).

A heterogeneous batch (Radon and fan beam, different image sizes, angle
counts and solvers) runs through :class:`gratopy_gb300.batch.BatchedReconstruction`;
every problem must reproduce what the per-call API gives for it alone:

* the batched ``normest`` equals :func:`gratopy_gb300.normest` with the same
  start vector (same partial-sum layout and order, so to the last bit);
* Landweber and TV iterates equal the per-call iterates for the same norm
  estimate (same tile functions and epilogue arithmetic);
* CG differs from the per-call form only in how the first <p, p> is reduced,
  so it is held to a float32 tolerance.
"""

from __future__ import annotations

import numpy as np
import pytest

from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu


def _problems(device):
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import batch as gb
    from gratopy_gb300.phantom import random_ellipse_image

    specs = [
        ("radon", (40, 36), 30, "landweber", 7),
        ("fan", (48, 48), 44, "landweber", 5),
        ("radon", (64, 64), 50, "cg", 6),
        ("fan", (40, 40), 36, "cg", 9),
        ("radon", (33, 47), 25, "tv", 8),
        ("fan", (56, 56), 60, "tv", 4),
        ("radon", (24, 24), [(20, 0.0, 2.0)], "tv", 11),
    ]
    rng = np.random.default_rng(5)
    out = []
    for k, (geom, shape, angles, solver, iters) in enumerate(specs):
        if geom == "radon":
            ps = gg.ProjectionSettings(device, gg.RADON, shape, angles)
        else:
            ps = gg.ProjectionSettings(device, gg.FANBEAM, shape, angles,
                                       n_detectors=int(1.5 * shape[0]), detector_width=40.0,
                                       R=70.0, RE=30.0)
        img = random_ellipse_image(30 + k, shape[::-1], dtype="float32").T
        img_d = gg.core.empty(shape, torch.float32, "F", device)
        img_d.copy_(torch.from_numpy(np.ascontiguousarray(img.T)).T)
        sino = gg.forwardprojection(img_d, ps)
        sino += 0.5 * torch.rand(sino.shape, generator=torch.Generator(device).manual_seed(k),
                                 device=device)
        pr = gb.Problem(ps, sino, solver, iters, mu=15.0 + k)
        pr.normest_x0 = rng.standard_normal(shape).astype(np.float32)
        out.append(pr)
    return out


# problems of _problems whose angle sets have an orbit symmetry (square
# centred images; fan beam Na a multiple of 4, parallel beam Na even over
# [0, pi)): with the size floor lifted the batch runs them on orbit tiles,
# forward and backprojection
ORBIT_PROBLEMS = {1: 3, 2: 3, 3: 3, 5: 3}


def test_batched_matches_per_call(cuda_device):
    import ctypes

    import gratopy_gb300 as gg
    from gratopy_gb300 import _lib
    from gratopy_gb300 import batch as gb

    problems = _problems(cuda_device)
    default = gb.BatchedReconstruction(problems, cuda_device)
    assert not any(default.desc[k].orbit for k in range(len(problems)))  # all below 4 Mi
    assert default.launches_per_iteration() == 6
    runner = gb.BatchedReconstruction(problems, cuda_device, normest_iterations=20,
                                      orbit_min_pixel_angles=0)
    assert {k: runner.desc[k].orbit for k in range(len(problems))
            if runner.desc[k].orbit} == ORBIT_PROBLEMS
    assert runner.launches_per_iteration() == 4 + 3 + 3
    results = runner.run()
    for k, (pr, got) in enumerate(zip(problems, results)):
        ps = pr.settings
        # the per-call form with the batched launch shapes, so both add in the
        # same order: per-angle problems with one thread row per angle set in
        # the backprojection, every angle's own forward, and for Radon the
        # batch's lanes per bin group (a per-call single Radon slice runs
        # twice fwd_split lanes); orbit problems with 8 angle groups in the
        # backprojection (their orbit forwards derive the lanes from
        # fwd_split alike)
        g = ps.gr_geometry(np.float32)
        orbit = int(_lib.raw("gr_orbit_kinds")(ctypes.byref(g), 1))
        assert orbit == ORBIT_PROBLEMS.get(k, 0)
        g.bwd_split = 8 if orbit & 2 else 1
        g.fwd_split = pr.fwd_split // 2 if ps.is_parallel and not orbit & 1 else pr.fwd_split
        if pr.solver in ("landweber", "tv"):
            want_n = gg.normest(ps, 20, x0=pr.normest_x0)
            assert abs(pr.norm_estimate - want_n) <= 1e-12 * want_n
        if pr.solver == "landweber":
            want = gg.landweber(pr.sino, ps, pr.iterations, w=pr.w, norm_estimate=pr.norm_estimate)
        elif pr.solver == "cg":
            want = gg.conjugate_gradients(pr.sino, ps, pr.iterations)
        else:
            want = gg.total_variation(pr.sino, ps, pr.mu, pr.iterations,
                                      stepsize_weighting=pr.stepsize_weighting,
                                      norm_estimate=pr.norm_estimate)
        err = rel_l2(got.cpu().numpy(), want.cpu().numpy())
        tol = 1e-5 if pr.solver == "cg" else 1e-6
        assert err <= tol, f"{pr.solver} {ps.geometry} {ps.img_shape}: rel err {err:.3e}"


def test_batched_graph_and_direct_agree(cuda_device):
    from gratopy_gb300 import batch as gb

    a = gb.BatchedReconstruction(_problems(cuda_device), cuda_device, normest_iterations=10,
                                 use_graph=True, orbit_min_pixel_angles=0).run()
    b = gb.BatchedReconstruction(_problems(cuda_device), cuda_device, normest_iterations=10,
                                 use_graph=False, orbit_min_pixel_angles=0).run()
    for x, y in zip(a, b):
        assert (x == y).all()


def test_heterogeneous_generator_runs(cuda_device):
    import torch

    from gratopy_gb300 import batch as gb

    problems = gb.heterogeneous_problems(6, seed=3, device=cuda_device, landweber_iterations=4,
                                         cg_iterations=3, tv_iterations=5, sizes=(32, 48),
                                         angle_range=(20, 40))
    out = gb.BatchedReconstruction(problems, cuda_device, normest_iterations=5).run()
    assert len(out) == 6
    for x, pr in zip(out, problems):
        assert tuple(x.shape) == tuple(pr.settings.img_shape)
        assert torch.isfinite(x).all()


def test_batched_against_fp64_oracle(cuda_device):
    """Every problem of a heterogeneous batch against the float64 oracle's
    solver on the same sinogram and norm estimate (gratopy.py:2380-2762).

    Bound: max(1e-5, k x the float32 envelope), the envelope being the
    largest distance from the float64 result among float32 runs of the
    reference's arithmetic (the float32 oracle on the sinogram and on three
    copies perturbed by one unit in the last place).  Landweber and TV keep
    float32 runs within ~1e-6 of float64 and k = 3.  CG amplifies the
    rounding of every operation inside its iteration (its iterates lose
    orthogonality), more than a perturbation of its input alone: the GPU,
    whose operations round differently (fused multiply-adds, other
    summation orders), measured 5.7 x the envelope on the 64^2 Radon problem
    below and 1.0 x on 50 iterations at 512^2, so k = 10 for CG.  The CG
    algorithm itself is pinned by the float64 parity of the per-call solver
    (tests/test_gpu_solvers.py) and the bitwise equality of batched and
    per-call CG (test_batched_matches_per_call).
    """
    from gratopy_gb300 import batch as gb
    from oracle import oracle as O
    from tests.helpers import HostSettings

    problems = _problems(cuda_device)
    results = gb.BatchedReconstruction(problems, cuda_device, normest_iterations=20,
                                       orbit_min_pixel_angles=0).run()
    for pr, got in zip(problems, results):
        ps = pr.settings
        hps = HostSettings(ps.geometry, ps.img_shape, np.asarray(ps.angles),
                           n_detectors=ps.n_detectors, angle_weights=np.asarray(ps.angle_weights),
                           detector_width=ps.detector_width, image_width=ps.image_width,
                           R=ps.R, RE=ps.RE, detector_shift=ps.detector_shift,
                           midpoint_shift=ps.midpoint_shift,
                           reverse_detector=ps.reverse_detector)
        f32 = np.asfortranarray(pr.sino.cpu().numpy())
        rng = np.random.default_rng(0)
        perturbed = []
        for _ in range(3):  # every value moved by one unit in the last place, either way
            up = rng.random(f32.shape) < 0.5
            moved = np.where(up, np.nextafter(f32, np.float32(np.inf)),
                             np.nextafter(f32, np.float32(-np.inf)))
            perturbed.append(np.asfortranarray(moved.astype(np.float32)))
        outs = []
        for f in [np.asfortranarray(f32, np.float64), f32] + perturbed:
            if pr.solver == "landweber":
                outs.append(O.landweber(f, hps, pr.iterations, w=pr.w,
                                        norm_estimate=pr.norm_estimate))
            elif pr.solver == "cg":
                outs.append(O.conjugate_gradients(f, hps, pr.iterations))
            else:
                outs.append(O.total_variation(f, hps, pr.mu, pr.iterations,
                                              stepsize_weighting=pr.stepsize_weighting,
                                              norm_estimate=pr.norm_estimate))
        ref64 = outs[0]
        err = rel_l2(got.cpu().numpy(), ref64)
        envelope = max(rel_l2(o, ref64) for o in outs[1:])
        k = 10.0 if pr.solver == "cg" else 3.0
        assert err <= max(1e-5, k * envelope), (
            f"{pr.solver} {ps.geometry} {ps.img_shape}: rel err vs float64 {err:.3e} "
            f"(float32 envelope {envelope:.3e})")
