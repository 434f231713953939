"""Benchmark: fan-beam forward + backprojection throughput on one GB300.

Workload (the fan-beam configuration the headline metric is quoted on):
512 x 512 float32 image of 10 seeded random ellipses, fan beam, 360 angles
over [0, 2 pi), 768 detectors, RE = 200, R = 400, detector width 400,
image width 0.9 x the automatic width (the image fills 90% of the fan).
A step is one forward projection plus one backprojection; the metric is
pixel-angle pairs processed per second (Nx Ny Na for each projection).

Timing: device time with CUDA events on the launching stream; the L2 cache
(129 MB) is flushed by writing a 256 MB buffer before every timed step,
outside the events.  ``e2e`` repeats the step through the public API with
the image copied in from pinned host memory and the backprojection copied
back, copies inside the timed region; its steps alternate between two
streams, so one step's copies overlap the other step's projections, and
their inputs rotate through buffers larger than twice the L2 (the one-stream
form with an L2 flush before every step is reported beside it).

``--impl reference`` times the CPU restatement of gratopy's kernels (the
reference's OpenCL kernels need an OpenCL runtime that this machine lacks)
on all host cores for the same workload and metric.

Multi-GPU (``torchrun``): every rank runs the same single-GPU workload
(independent replicas, no collective on the data path); the value is the
sum over ranks divided by the slowest rank's time.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

MEASURED_PEAKS = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0
METRIC = "fwd+back Gpixel-angle/s"
UNIT = "Gpixel-angle/s"

WORKLOAD = dict(geometry="fanbeam", img_shape=(512, 512), angles=360, n_detectors=768,
                detector_width=400.0, RE=200.0, R=400.0,
                image_width=0.9 * (2 * 0.5 * 200.0 / np.sqrt(1 + 0.25)))
# Radon 256 x 256, 180 angles over [0, pi), 363 detectors of width
# 2 sqrt(2) / 363 (the detector spans the image diagonal), image width 2
RADON_WORKLOAD = dict(geometry="radon", img_shape=(256, 256), angles=180, n_detectors=363,
                      detector_width=2.0 * np.sqrt(2.0), image_width=2.0)
SEED = 1234


def peaks():
    try:
        d = json.loads(MEASURED_PEAKS.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def make_image(seed=SEED):
    from gratopy_gb300.phantom import random_ellipse_image

    img = random_ellipse_image(seed, (512, 512), count=10, dtype="float32")
    return np.asfortranarray(img.T)  # (Nx, Ny), Fortran order


def pixel_angles():
    Nx, Ny = WORKLOAD["img_shape"]
    return Nx * Ny * WORKLOAD["angles"]


def config_block():
    return {"workload": "fanbeam 512x512 float32, 360 angles [0,2pi), 768 detectors, RE=200, "
                        "R=400, image width 0.9x automatic; step = forward + backprojection",
            "image": [512, 512], "angles": 360, "detectors": 768, "RE": 200.0, "R": 400.0,
            "l2": "flushed before every timed step (256 MB write)", "seed": SEED}


# ------------------------------------------------------------------ clocks


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._proc = None
        self._thread = None

    def start(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self._proc = None
            return self

        def reader():
            for line in self._proc.stdout:
                self.rows.append([c.strip() for c in line.split(",")])

        self._thread = threading.Thread(target=reader, daemon=True)
        self._thread.start()
        t0 = time.time()
        while not self.rows and time.time() - t0 < 3.0 and self._proc.poll() is None:
            time.sleep(0.01)
        return self

    def stop(self):
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
        if self._thread is not None:
            self._thread.join(timeout=5)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for name, val in zip(names, r[5:9]):
                if val.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------- GPU arm


def run_gpu(args, rank, world, device):
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import _lib

    _lib.load()
    cfg = dict(WORKLOAD)
    cfg.pop("geometry")
    img_shape = cfg.pop("img_shape")
    angles = cfg.pop("angles")
    ps = gg.ProjectionSettings(device, gg.FANBEAM, img_shape, angles, **cfg)
    host = make_image()
    img = gg.core.empty(img_shape, torch.float32, "F", device)
    img.copy_(torch.from_numpy(np.ascontiguousarray(host.T)).T)
    sino = gg.core.empty(ps.sinogram_shape, torch.float32, "F", device)
    back = gg.core.empty(img_shape, torch.float32, "F", device)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)
    stream = torch.cuda.current_stream(device)

    from gratopy_gb300 import autotune

    if args.splits:
        # pinned launch shapes (profiling: under ncu the tuner's own timings
        # are perturbed and it may pick another shape than in a plain run)
        fs, bs = (int(v) for v in args.splits.split(","))
        g = ps.gr_geometry(np.float32)
        g.fwd_split, g.bwd_split = fs, bs
        tuned = {"fwd_split": fs, "bwd_split": bs, "pinned": True}
    else:
        t = autotune.tune(ps, np.float32, use_cache=False)
        tuned = {"fwd_split": t["fwd_split"], "bwd_split": t["bwd_split"]}

    def step(ev=None):
        if ev is not None:
            ev[0].record(stream)
        gg.forwardprojection(img, ps, sino=sino)
        if ev is not None:
            ev[1].record(stream)
        gg.backprojection(sino, ps, img=back)
        if ev is not None:
            ev[2].record(stream)

    for _ in range(args.warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize(device)

    events = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    sampler = ClockSampler(device.index).start() if rank == 0 else None
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(device)
    for k in range(args.steps):
        flush.zero_()
        step(events[k])
    torch.cuda.synchronize(device)
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop() if sampler is not None else None
    t_fwd = [events[k][0].elapsed_time(events[k][1]) * 1e-3 for k in range(args.steps)]
    t_bwd = [events[k][1].elapsed_time(events[k][2]) * 1e-3 for k in range(args.steps)]
    total = sum(t_fwd) + sum(t_bwd)
    if world > 1:
        t = torch.tensor([total], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total = float(t.item())

    # end to end through the public API with host buffers
    h_img = torch.from_numpy(np.ascontiguousarray(host.T)).pin_memory()
    h_back = torch.empty((img_shape[1], img_shape[0]), dtype=torch.float32).pin_memory()
    d_img = gg.core.empty(img_shape, torch.float32, "F", device)
    e_events = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(args.steps)]

    def e2e_step(ev=None):
        if ev is not None:
            ev[0].record(stream)
        d_img.T.copy_(h_img, non_blocking=True)
        s = gg.forwardprojection(d_img, ps)
        b = gg.backprojection(s, ps)
        h_back.copy_(b.T, non_blocking=True)
        if ev is not None:
            ev[1].record(stream)

    for _ in range(args.warmup):
        flush.zero_()
        e2e_step()
    torch.cuda.synchronize(device)
    for k in range(args.steps):
        flush.zero_()
        e2e_step(e_events[k])
    torch.cuda.synchronize(device)
    e2e_serial = sum(e[0].elapsed_time(e[1]) * 1e-3 for e in e_events)
    want = back.cpu().numpy()
    tol = 1e-6 * float(back.abs().max())
    if not np.allclose(h_back.numpy().T, want, rtol=1e-6, atol=tol):
        raise RuntimeError("end-to-end result differs from the device-resident run")

    # The same steps on two streams: step k's copies and projections run on
    # stream k % 2, so one step's copies overlap the other step's
    # projections (each stream has its own orbit-copy scratch).  Every step
    # still uploads its image from pinned host memory and reads its
    # backprojection back.  Inputs and outputs rotate through buffers
    # totalling more than twice the L2, so no step finds its data cached
    # (no flush inside this loop).
    l2 = int(getattr(torch.cuda.get_device_properties(device), "L2_cache_size", 0)) or (128 << 20)
    nbuf = max(4, -(-2 * l2 // (h_img.numel() * 4)))
    nbuf += nbuf % 2
    h_imgs = torch.empty((nbuf,) + tuple(h_img.shape), dtype=torch.float32).pin_memory()
    h_imgs.copy_(h_img.expand_as(h_imgs))
    h_backs = torch.empty_like(h_imgs).pin_memory()
    d_imgs = gg.core.empty(tuple(img_shape) + (nbuf,), torch.float32, "F", device)
    sinos = gg.core.empty(tuple(ps.sinogram_shape) + (nbuf,), torch.float32, "F", device)
    backs = gg.core.empty(tuple(img_shape) + (nbuf,), torch.float32, "F", device)
    streams = [torch.cuda.Stream(device), torch.cuda.Stream(device)]

    def piped_step(k):
        j = k % nbuf
        with torch.cuda.stream(streams[k % 2]):
            d_imgs[:, :, j].T.copy_(h_imgs[j], non_blocking=True)
            gg.forwardprojection(d_imgs[:, :, j], ps, sino=sinos[:, :, j])
            gg.backprojection(sinos[:, :, j], ps, img=backs[:, :, j])
            h_backs[j].copy_(backs[:, :, j].T, non_blocking=True)

    cur = torch.cuda.current_stream(device)
    for st in streams:
        st.wait_stream(cur)
    for k in range(2 * args.warmup):
        piped_step(k)
    torch.cuda.synchronize(device)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(cur)
    for st in streams:
        st.wait_event(t0)
    for k in range(args.steps):
        piped_step(k)
    for st in streams:
        cur.wait_stream(st)
    t1.record(cur)
    torch.cuda.synchronize(device)
    e2e_piped = t0.elapsed_time(t1) * 1e-3
    last = (args.steps - 1) % nbuf
    if not np.allclose(h_backs[last].numpy().T, want, rtol=1e-6, atol=tol):
        raise RuntimeError("pipelined end-to-end result differs from the device-resident run")
    del h_imgs, h_backs, d_imgs, sinos, backs

    return dict(total=total, t_fwd=t_fwd, t_bwd=t_bwd, clocks=clocks, e2e_piped=e2e_piped,
                e2e_serial=e2e_serial, e2e_buffers=nbuf,
                h2d=h_img.numel() * 4, d2h=h_back.numel() * 4, ps=ps, tuned=tuned, flush=flush,
                img=img, sino=sino, back=back)


def l1_load_peak(device, reps=5):
    """Measured L1 load bandwidth (GB/s, whole GPU): the denominator of the
    gather roofline.  float4 loads over a 16 KB buffer resident in every SM's
    L1, one wave of 8 blocks of 256 threads per SM; best of ``reps``."""
    import ctypes

    import torch

    from gratopy_gb300 import _lib, core

    sms = torch.cuda.get_device_properties(device).multi_processor_count
    n_vec, iters, blocks = 1024, 4096, sms * 8
    buf = torch.zeros(4 * n_vec, dtype=torch.float32, device=device)
    out = torch.zeros(blocks * 256, dtype=torch.float32, device=device)

    def run():
        _lib.call("gr_probe_l1_bandwidth", ctypes.c_void_p(out.data_ptr()),
                  ctypes.c_void_p(buf.data_ptr()), n_vec, iters, blocks, core._stream_ptr(device))

    run()
    t = min(_event_times(run, reps))
    return blocks * 256 * iters * 16 / t / 1e9


def _event_times(fn, reps, flush=None):
    """Device seconds of ``fn()`` per repetition (CUDA events on the current stream)."""
    import torch

    out = []
    for _ in range(reps):
        if flush is not None:
            flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        out.append(a.elapsed_time(b) * 1e-3)
    return out


def extra_radon256(device, flush):
    """Plain Radon forward + backprojection, 256 x 256, 180 angles, 363 detectors."""
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300.phantom import random_ellipse_image

    res = {}
    host = random_ellipse_image(SEED, (256, 256), count=10, dtype="float64").T
    cfg = dict(RADON_WORKLOAD)
    cfg.pop("geometry")
    shape, angles = cfg.pop("img_shape"), cfg.pop("angles")
    for name, tdt in (("float32", torch.float32), ("float64", torch.float64)):
        ps = gg.ProjectionSettings(device, gg.RADON, shape, angles, **cfg)
        img = gg.core.empty((256, 256), tdt, "F", device)
        img.copy_(torch.from_numpy(np.ascontiguousarray(host.T)).T)
        sino = gg.core.empty(ps.sinogram_shape, tdt, "F", device)
        back = gg.core.empty((256, 256), tdt, "F", device)

        def step():
            gg.forwardprojection(img, ps, sino=sino)
            gg.backprojection(sino, ps, img=back)

        _event_times(step, 3, flush)
        t = _event_times(step, 50, flush)
        res[name] = 2 * 256 * 256 * 180 / statistics.median(t) / 1e9
    return {"workload": "radon 256x256, 180 angles [0,pi), 363 detectors (width 2 sqrt 2), "
                        "image width 2, fwd+back, L2 flushed",
            "unit": UNIT, **res}


def extra_cg50(device, ps, img):
    """50-iteration CG reconstruction of the headline fan-beam workload (1% noise)."""
    import torch

    import gratopy_gb300 as gg

    sino = gg.forwardprojection(img, ps)
    gen = torch.Generator(device=device).manual_seed(SEED)
    noise = torch.randn(sino.shape, generator=gen, device=device)
    sino += 0.01 * float(sino.abs().max()) * noise
    run = lambda: gg.conjugate_gradients(sino, ps, 50)  # noqa: E731
    _event_times(run, 2)
    t = _event_times(run, 5)
    # error against a float64 solve of the same data: the float64 kernels
    # (reference operation order, pinned to the float64 oracle at 1e-12)
    out = run().double()
    ref = gg.conjugate_gradients(sino.double(), ps, 50)
    err = float(torch.linalg.norm(out - ref) / torch.linalg.norm(ref))
    return {"workload": "fanbeam 512x512, 360 angles, 768 detectors, 50 CG iterations, "
                        "1% Gaussian noise", "recon_per_s": 1.0 / statistics.median(t),
            "ms_per_recon": statistics.median(t) * 1e3, "rel_err_vs_fp64": err,
            "fp64_reference": "float64 CG on the same sinogram through the float64 kernels"}


def extra_batched(device, small=False, fp64_every=4):
    """Heterogeneous batch of 64 problems: batched persistent launches against per-call."""
    import torch

    from gratopy_gb300 import batch as gb

    kw = dict(sizes=(32, 48, 64, 96, 128), angle_range=(30, 180)) if small else {}
    probs = gb.heterogeneous_problems(64, seed=0, device=device, **kw)

    def fresh():
        return [gb.Problem(p.settings, p.sino, p.solver, p.iterations, mu=p.mu) for p in probs]

    def wall(fn):
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize(device)
        return time.perf_counter() - t0, out

    gb.BatchedReconstruction(fresh()[:6], device, normest_iterations=3, autotune=True).run()
    gb.solve_plain(fresh()[:6])
    t_b, _ = wall(lambda: gb.BatchedReconstruction(fresh(), device, autotune=True).run())
    solved = fresh()
    t_b2, out_b = wall(lambda: gb.BatchedReconstruction(solved, device, autotune=True).run())
    t_b = min(t_b, t_b2)
    t_pg, _ = wall(lambda: gb.solve_plain(fresh(), use_graph=True))
    t_pd, _ = wall(lambda: gb.solve_plain(fresh(), use_graph=False))
    # accuracy: the per-call solvers with the batch's norm estimates and launch
    # shapes (batched backprojection tiles use one thread row per angle set)
    for p in solved:
        p.settings.gr_geometry(np.float32).bwd_split = 1
        p.settings.gr_geometry(np.float32).sym = 0
    same = [gb.Problem(p.settings, p.sino, p.solver, p.iterations, mu=p.mu,
                       norm_estimate=p.norm_estimate) for p in solved]
    ref = gb.solve_plain(same)
    err = {}
    for p, a, b in zip(solved, out_b, ref):
        e = float(torch.linalg.norm((a - b).double()) / torch.linalg.norm(b.double()))
        err[p.solver] = max(err.get(p.solver, 0.0), e)
    # error against float64 solves of the same data (float64 kernels, the
    # batch's norm estimates) for every fp64_every-th problem: float64
    # projections run ~30x slower than float32 ones
    err64, t64 = {}, time.perf_counter()
    for k in range(0, len(solved), fp64_every):
        p = solved[k]
        q = gb.Problem(p.settings, p.sino.double(), p.solver, p.iterations, mu=p.mu,
                       norm_estimate=p.norm_estimate)
        b = gb.solve_plain([q])[0]
        e = float(torch.linalg.norm(out_b[k].double() - b) / torch.linalg.norm(b))
        err64[p.solver] = max(err64.get(p.solver, 0.0), e)
    t64 = time.perf_counter() - t64
    # pixel-angles the solves project: normest (50 iterations of A then A^T
    # for Landweber and TV), the CG start (A x0, A^T d), two per iteration
    pa = 0
    for p in probs:
        Nx, Ny = p.settings.img_shape
        per = Nx * Ny * p.settings.n_angles
        n = 2 * p.iterations + (2 if p.solver == "cg" else 2 * 50)
        pa += n * per
    name = ("64 problems, side U{32..128}, angles U[30,180]" if small else
            "64 problems, side U{128,192,256,384,512}, angles U[60,720]")
    return {"workload": name + ", half Radon (full or 2pi/3 range) half fan beam, "
                        "Landweber-200 / CG-50 / TV-100, float32, normest included",
            "batched_recon_per_s": 64 / t_b, "plain_graph_recon_per_s": 64 / t_pg,
            "plain_direct_recon_per_s": 64 / t_pd, "speedup_vs_plain_direct": t_pd / t_b,
            "speedup_vs_plain_graph": t_pg / t_b,
            "batched_gpixel_angle_per_s": pa / t_b / 1e9,
            "plain_direct_gpixel_angle_per_s": pa / t_pd / 1e9,
            "pixel_angles_projected": pa, "max_rel_err_vs_per_call": err,
            "max_rel_err_vs_fp64": err64,
            "fp64_reference": f"float64 per-call solves of every {fp64_every}th problem "
                              f"({len(range(0, len(solved), fp64_every))} of {len(solved)}) "
                              f"with the batch's norm estimates, {t64:.1f} s",
            "timing": "wall clock around the whole solve, synchronised"}


def extra_autograd(device, order="F"):
    """Gradient step through Radon projections and an unrolled TV reconstruction.

    16 float32 512 x 512 images (one stack in ``order``, independent slices),
    360 angles in [0, pi), 725 detectors.  loss = ||A x - y||^2 + ||TV_20(A x) - x_true||^2
    with TV_20 = 20 primal-dual iterations (mu = 20) checkpointed every 5;
    a step is the forward pass plus ``loss.backward()``.
    """
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import autograd as ga
    from gratopy_gb300.phantom import random_ellipse_image

    nz = 16
    ps = gg.ProjectionSettings(device, gg.RADON, (512, 512), 360, n_detectors=725)
    truth = np.stack([random_ellipse_image(SEED + k, (512, 512), count=10, dtype="float32").T
                      for k in range(nz)], -1)
    x_true = gg.core.empty((512, 512, nz), torch.float32, order, device)
    x_true.copy_(torch.from_numpy(np.ascontiguousarray(truth)))
    y = gg.forwardprojection(x_true, ps)
    gen = torch.Generator(device=device).manual_seed(SEED)
    y += 0.01 * float(y.abs().max()) * torch.randn(y.shape, generator=gen, device=device)
    nrm = gg.normest(ps, 50, x0=np.ones(ps.img_shape))
    x = (0.5 * x_true).detach().requires_grad_(True)

    def step():
        x.grad = None
        yh = ga.forward_project(x, ps)
        u = ga.tv_unrolled(yh, ps, 20.0, number_iterations=20, checkpoint_every=5,
                           slice_thickness=0.0, norm_estimate=nrm)
        loss = ((yh - y) ** 2).sum() + ((u - x_true) ** 2).sum()
        loss.backward()

    _event_times(step, 2)
    t = statistics.median(_event_times(step, 5))
    # projections per step: A x, 2 per TV iteration forward, the same again in
    # the checkpoint replay, 2 per adjoint iteration, A^T for the data term
    projections = 1 + 2 * 20 + 2 * 20 + 2 * 20 + 1
    pa = 512 * 512 * 360 * nz
    return {"workload": f"16 x 512^2 Radon stack ({order} order), 360 angles [0,pi), 725 "
                        "detectors; ||Ax-y||^2 + ||TV20(Ax)-x||^2, checkpoint every 5, "
                        "forward+backward",
            "steps_per_s": 1.0 / t, "ms_per_step": t * 1e3, "projections_per_step": projections,
            "gpixel_angle_per_s": projections * pa / t / 1e9}


def extra_large_stack(device, iterations=3, adjoint_iterations=5, order="F"):
    """2048 x 2048 x 64 fan-beam stack: TV primal-dual and its adjoint, per iteration.

    1440 angles over [0, 2pi), 2900 detectors, RE = 1000, R = 2000, detector
    width 2000, automatic image width, mu = 50, slice thickness 1; stack in
    ``order`` (F: each slice a plane; C: slices fastest, 4 slices per float4
    load; the projections carry 4 slices per thread either way).  A full
    500-iteration reconstruction with a differentiable backward through the
    last 50 iterations is extrapolated from the measured per-iteration times:
    500 TV iterations + 50 x (replay + adjoint).
    """
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import autograd as ga
    from gratopy_gb300.phantom import random_ellipse_volume

    nz = 64
    ps = gg.ProjectionSettings(device, gg.FANBEAM, (2048, 2048), 1440, n_detectors=2900,
                               detector_width=2000.0, R=2000.0, RE=1000.0)
    vol = random_ellipse_volume(device, (2048, 2048), nz, seed=SEED, order=order)
    sino = gg.forwardprojection(vol, ps)
    del vol
    nrm = gg.normest(ps, 50)
    tv = lambda k: gg.total_variation(sino, ps, 50.0, k, norm_estimate=nrm)  # noqa: E731
    tv(1)
    t_tv = _event_times(lambda: tv(iterations), 1)[0] / iterations
    f = sino.detach().requires_grad_(True)

    def unrolled():
        u = ga.tv_unrolled(f, ps, 50.0, number_iterations=adjoint_iterations,
                           checkpoint_every=adjoint_iterations, slice_thickness=1.0,
                           norm_estimate=nrm)
        u.sum().backward()

    t_fb = _event_times(unrolled, 1)[0]
    # forward pass of the unrolled run = adjoint_iterations TV iterations; the
    # backward replays them and runs the adjoint iterations
    t_back_iter = (t_fb - adjoint_iterations * t_tv) / adjoint_iterations
    pa = 2048 * 2048 * 1440 * nz
    del f, sino
    torch.cuda.empty_cache()
    return {"workload": f"fanbeam 2048^2 x 64 slices float32 {order} order, 1440 angles, "
                        "2900 detectors, RE=1000, R=2000; TV mu=50, slice thickness 1",
            "tv_ms_per_iteration": t_tv * 1e3,
            "tv_gpixel_angle_per_s": 2 * pa / t_tv / 1e9,
            "backward_ms_per_iteration": t_back_iter * 1e3,
            "extrapolated_500_tv_plus_50_backward_s": 500 * t_tv + 50 * t_back_iter,
            "measured": f"{iterations} TV iterations; {adjoint_iterations} unrolled iterations "
                        "forward + backward"}


def extra_large_stack_full(device, iterations=500, backward_iterations=50, checkpoint_every=5):
    """The large-stack workload as configured, measured end to end: 500 TV
    iterations on the 2048 x 2048 x 64 fan-beam stack (F order) with the
    differentiation truncated to the last 50 iterations (states checkpointed
    every 5), then the backward pass of sum(U); wall time of each part (CUDA
    events) and the peak device memory of the whole run."""
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import autograd as ga
    from gratopy_gb300.phantom import random_ellipse_volume

    nz = 64
    ps = gg.ProjectionSettings(device, gg.FANBEAM, (2048, 2048), 1440, n_detectors=2900,
                               detector_width=2000.0, R=2000.0, RE=1000.0)
    vol = random_ellipse_volume(device, (2048, 2048), nz, seed=SEED, order="F")
    sino = gg.forwardprojection(vol, ps)
    del vol
    nrm = gg.normest(ps, 50)
    torch.cuda.synchronize(device)
    torch.cuda.reset_peak_memory_stats(device)
    f = sino.detach().requires_grad_(True)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record()
    u = ga.tv_unrolled(f, ps, 50.0, number_iterations=iterations,
                       checkpoint_every=checkpoint_every, slice_thickness=1.0,
                       norm_estimate=nrm, backward_iterations=backward_iterations)
    ev[1].record()
    u.sum().backward()
    ev[2].record()
    torch.cuda.synchronize(device)
    t_fwd = ev[0].elapsed_time(ev[1]) * 1e-3
    t_bwd = ev[1].elapsed_time(ev[2]) * 1e-3
    peak = torch.cuda.max_memory_allocated(device)
    finite = bool(torch.isfinite(f.grad).all())
    del f, u, sino
    torch.cuda.empty_cache()
    return {"workload": "fanbeam 2048^2 x 64 slices float32 F order, 1440 angles, 2900 "
                        "detectors, RE=1000, R=2000; TV mu=50, slice thickness 1; "
                        f"{iterations} iterations, backward through the last "
                        f"{backward_iterations} (checkpoint every {checkpoint_every})",
            "tv_forward_s": t_fwd, "backward_s": t_bwd, "total_s": t_fwd + t_bwd,
            "tv_ms_per_iteration": t_fwd / iterations * 1e3,
            "peak_device_memory_gb": peak / 1e9, "gradient_finite": finite}


EXTRAS = {
    "radon256": lambda device, ps, res: extra_radon256(device, res["flush"]),
    "cg50": lambda device, ps, res: extra_cg50(device, ps, res["img"]),
    "batched": lambda device, ps, res: extra_batched(device),
    "batched_small": lambda device, ps, res: extra_batched(device, small=True),
    "autograd": lambda device, ps, res: extra_autograd(device),
    "autograd_c": lambda device, ps, res: extra_autograd(device, order="C"),
    "large_stack": lambda device, ps, res: extra_large_stack(device),
    "large_stack_c": lambda device, ps, res: extra_large_stack(device, order="C"),
    "large_stack_full": lambda device, ps, res: extra_large_stack_full(device),
}


# left out of the default run: the C-ordered large stack (its x-walk strides
# 64 x 2048 floats per pixel and runs 3x slower than the F-ordered stack) and
# the full 500-iteration large-stack run (about four minutes)
DEFAULT_EXTRAS = [e for e in EXTRAS if e not in ("large_stack_c", "large_stack_full")]


def launches_per_step(ps):
    """Kernels of one forward + backprojection.  With quarter-turn maps and
    scratch bound, the forward first gathers each pixel's orbit into one
    float4 and the orbit backprojection (even sides) first interleaves the
    sinogram rows: one more launch each."""
    g = ps.gr_geometry(np.float32)
    if g.sym != 4 or not g.work:
        return 2
    return 4 if ps.img_shape[0] % 2 == 0 else 3


def cpu_baseline_sample(max_seconds=12.0, gpu_outputs=None):
    """Time the oracle (restated reference kernels) on this host's cores.

    With ``gpu_outputs = (sino, back)`` -- the GPU's float32 forward
    projection of the workload image and the backprojection of that
    sinogram, from the timed run -- the same leg also checks them against
    the float64 oracle: forward against A x, backprojection against
    A*(A x), relative L2 errors (the parity tests' bound is 1e-5).
    """
    from oracle import oracle as O
    from tests.helpers import host_settings

    ps = host_settings(WORKLOAD)
    img = make_image()
    O.forward(img, ps)  # builds and loads the library outside the timing
    reps, t0 = 0, time.perf_counter()
    while True:
        sino = O.forward(img, ps)
        O.backward(sino, ps)
        reps += 1
        if time.perf_counter() - t0 >= max_seconds or reps >= 50:
            break
    dt = time.perf_counter() - t0
    value = 2 * pixel_angles() * reps / dt / 1e9
    out = {"value": value, "unit": UNIT, "cores": O.threads(), "kind": "port",
           "sample": f"{reps} forward+back steps of the full workload, {dt:.1f} s wall"}
    if gpu_outputs is not None:
        g_sino, g_back = gpu_outputs
        ref_sino = O.forward(np.asfortranarray(img, dtype=np.float64), ps)
        ref_back = O.backward(np.asfortranarray(g_sino, dtype=np.float64), ps)

        def rel(a, b):
            return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))

        out["parity"] = {"fwd_rel_err_vs_fp64_oracle": rel(g_sino, ref_sino),
                         "bwd_rel_err_vs_fp64_oracle": rel(g_back, ref_back),
                         "tolerance": 1e-5,
                         "what": "the timed run's float32 outputs against the float64 oracle on "
                                 "the same inputs (backprojection of the GPU sinogram)"}
    return out


def reference_arm(args):
    """The oracle -- the C restatement of gratopy's OpenCL kernels, the reference's
    own kernels needing an OpenCL runtime this machine lacks -- on all host
    cores: ``warmup`` untimed and ``steps`` timed steps of forward + back.

    A step projects the whole workload; when ``steps`` full steps would take
    longer than about two minutes, every step projects an evenly spaced
    subset of the angles instead (the same image and detector), and the
    metric counts the pixel-angles actually processed.
    """
    from oracle import oracle as O
    from tests.helpers import host_settings

    ps = host_settings(WORKLOAD)
    img = make_image()
    Nx, Ny = WORKLOAD["img_shape"]

    def step(p):
        O.backward(O.forward(img, p), p)

    t0 = time.perf_counter()
    step(ps)  # also loads the library
    t_full = time.perf_counter() - t0
    stride = max(1, int(np.ceil(t_full * args.steps / 120.0)))
    sample = ps
    if stride > 1:
        sample = host_settings(dict(WORKLOAD, angles=np.asarray(ps.angles)[::stride]))
    for _ in range(args.warmup):
        step(sample)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step(sample)
    dt = time.perf_counter() - t0
    units = 2 * Nx * Ny * sample.n_angles
    value = units * args.steps / dt / 1e9
    desc = ("the full workload" if stride == 1 else
            f"{sample.n_angles} of the 360 angles (every {stride}th)")
    base = {"value": value, "unit": UNIT, "cores": O.threads(), "kind": "port",
            "sample": f"{args.steps} timed forward+back steps of {desc}, {dt:.1f} s wall"}
    return {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic: seeded random ellipses",
            "config": config_block(), "cpu_baseline": base,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gratopy_gb300", choices=["gratopy_gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--splits", default="",
                    help="pin the launch shapes as FWD,BWD (each 1, 2, 4 or 8) instead of "
                         "autotuning them")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the secondary workloads")
    ap.add_argument("--extras", default="all",
                    help="comma list of secondary workloads: " + ",".join(EXTRAS)
                    + " (or all: every one but large_stack_c and large_stack_full)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        args.steps = max(1, args.steps)
        print(json.dumps(reference_arm(args)))
        return

    import torch

    if world > 1:
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    res = run_gpu(args, rank, world, device)

    steps = args.steps
    units = 2 * pixel_angles() * world
    value = units * steps / res["total"] / 1e9
    e2e_piped = 2 * pixel_angles() * world * steps / res["e2e_piped"] / 1e9
    e2e_serial = 2 * pixel_angles() * world * steps / res["e2e_serial"] / 1e9
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    hbm, hbm_kind = peaks()
    ps = res["ps"]
    Ns, Na = ps.sinogram_shape
    Nx, Ny = ps.img_shape
    compulsory = (Nx * Ny + Ns * Na) * 4
    fwd, bwd = statistics.mean(res["t_fwd"]), statistics.mean(res["t_bwd"])
    # single fan-beam slices with quarter-turn maps run the orbit kernels (the
    # backprojection's orbits need an even side)
    quarter = ps.gr_geometry(np.float32).sym == 4
    fwd_name = "fan_fwd_quarter" if quarter else "fan_fwd_fast"
    if quarter and Nx % 2 == 0:  # with scratch bound, from the interleaved row copy
        bwd_name = "fan_bwd_orbit_rows" if ps.gr_geometry(np.float32).work else "fan_bwd_orbit"
    else:
        bwd_name = "fan_bwd_fast"
    dom, t_dom = (fwd_name, fwd) if fwd >= bwd else (bwd_name, bwd)
    # DRAM traffic and issue utilisation of the dominant kernel from the
    # committed ncu summary of this workload (one capture, not this run)
    traffic, issue = None, None
    km_file = ROOT / "profiles" / "kernel_metrics.json"
    if km_file.exists():
        try:
            km = json.loads(km_file.read_text()).get(dom, {})
            traffic = km.get("dram_bytes_per_launch")
            issue = km.get("issue_active_pct")
        except (OSError, ValueError):
            pass
    # The projections are sparse gathers bound by L1 load throughput and
    # instruction issue, not by HBM: the roofline divides the algorithmic
    # gather bytes (2 nonzero weights x 4 B per pixel-angle) by the measured
    # L1 load rate; the HBM figures (compulsory bytes: one read of the input,
    # one write of the output) are kept beside it.
    l1 = l1_load_peak(device)
    gather_bytes = 8 * pixel_angles()
    gather = gather_bytes / t_dom / 1e9
    hbm_achieved = compulsory / t_dom / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": res["total"] / steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded random ellipses (10 per image)",
        "config": config_block(),
        "parallelism": f"replicas{world}",
        "fwd_gpixel_angle_per_s": pixel_angles() / fwd / 1e9,
        "bwd_gpixel_angle_per_s": pixel_angles() / bwd / 1e9,
        "roofline": {"bound": "l1", "kernel": dom, "achieved": gather, "peak": l1,
                     "unit": "GB/s", "frac": gather / l1, "traffic": traffic,
                     "algorithmic_bytes": gather_bytes,
                     "peak_source": "measured in this run: gr_probe_l1_bandwidth (float4 loads "
                                    "of an L1-resident buffer, every SM)",
                     "hbm": {"achieved": hbm_achieved, "peak": hbm, "frac": hbm_achieved / hbm,
                             "algorithmic_bytes": compulsory,
                             "peak_source": f"{hbm_kind}: MEASURED_PEAKS.json hbm_gbs"},
                     "issue_active_pct_ncu": issue,
                     "traffic_source": "ncu capture of this workload (profiles/kernel_metrics.json)",
                     "note": "the timed forward includes its orbit-copy pre-pass (one small "
                             "kernel); DRAM traffic is the compulsory bytes plus the copy"},
        "e2e": {"value": e2e_serial, "unit": UNIT, "h2d_bytes_per_step": res["h2d"],
                "d2h_bytes_per_step": res["d2h"],
                "mode": "public API, one stream: the image uploaded from pinned host memory, "
                        "forward + backprojection, the backprojection read back into pinned "
                        "host memory, every step; L2 flushed before every step (outside the "
                        "events)",
                "pipelined_value": e2e_piped,
                "pipelined_mode": "the same steps alternating between two streams, so one "
                                  "step's copies overlap the other's projections; inputs rotate "
                                  f"through {res['e2e_buffers']} buffers (more than twice the "
                                  "L2), no flush"},
        "gpu_launches": launches_per_step(ps) * steps,
        "clocks": res["clocks"],
    }
    line["tuned_splits"] = res["tuned"]
    wanted = [] if args.no_extras else (
        DEFAULT_EXTRAS if args.extras == "all" else [e for e in args.extras.split(",") if e])
    for name in wanted:
        if name not in EXTRAS:
            raise SystemExit(f"unknown extra workload {name!r}; choose from {', '.join(EXTRAS)}")
        line[name] = EXTRAS[name](device, ps, res)
    if not args.no_cpu_baseline:
        outs = (res["sino"].cpu().numpy(), res["back"].cpu().numpy())
        line["cpu_baseline"] = cpu_baseline_sample(gpu_outputs=outs)
        line["parity"] = line["cpu_baseline"].pop("parity")
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
