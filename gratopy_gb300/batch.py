"""Batched reconstruction of many small problems in shared persistent launches.

Each problem is a float32 2-D sinogram with its own ``ProjectionSettings``
(Radon or fan beam, any image size and angle count) and its own solver:
Landweber, conjugate gradients or total variation -- the same iterations as
:func:`gratopy_gb300.landweber`, :func:`gratopy_gb300.conjugate_gradients`
and :func:`gratopy_gb300.total_variation`.  Every phase of an iteration is a
persistent launch over a (problem, tile) work list that covers all problems
still running, so the GPU is filled by the batch rather than by any one
problem.  Problems of at least 4 * 2^20 pixel-angles whose angle set has an
orbit symmetry (fan beam: Na a multiple of 4 over the full circle; parallel
beam: Na even over [0, pi); a square centred image) project over the orbits,
as the per-call form does, gathering the orbit members (the batch keeps no
copies): their tiles go to separate launches per geometry kind.  Smaller
problems keep the per-angle tiles: their orbit tiles measured slower in the
batch (the small mix of ``heterogeneous_problems``, sides 32-128: 609
against 654 reconstructions/s), where the extra launches per iteration and
the smaller quadrant tiles cost more than the shared geometry saves.  Landweber and TV problems first run ``normest`` (batched as
well; one host synchronisation reads all norms), CG problems start at once.
The iteration sequence is captured in CUDA graphs, one per range of
iterations in which the set of running problems is constant.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from . import core

_SOLVERS = {"landweber": _lib.GR_SOLVER_LANDWEBER, "cg": _lib.GR_SOLVER_CG,
            "tv": _lib.GR_SOLVER_TV}
_RAYS_PER_LANE_GROUP = 4  # detector bins per lane group of the float32 forward kernel
_ORBIT_ANGLE_GROUPS = 8  # angle groups of the batched orbit backprojection
_ORBIT_MIN_PIXEL_ANGLES = 4 << 20  # smaller problems keep the per-angle tiles


@dataclass
class Problem:
    """One reconstruction of the batch."""

    settings: core.ProjectionSettings
    sino: torch.Tensor                 # (Ns, Na) float32 on the batch device
    solver: str                        # "landweber" | "cg" | "tv"
    iterations: int
    mu: float = 20.0                   # TV regularisation weight
    w: float = 1.0                     # Landweber relaxation
    stepsize_weighting: float = 10.0   # TV step weighting
    fwd_split: int = 8                 # lanes per group of detector bins (autotuned)
    norm_estimate: float | None = None
    normest_x0: np.ndarray | None = field(default=None, repr=False)  # normest start vector
    result: torch.Tensor | None = field(default=None, repr=False)


def _f32(v) -> float:
    return float(np.float32(v))


class BatchedReconstruction:
    """Run a list of :class:`Problem` s together on one GPU."""

    def __init__(self, problems, device=None, normest_iterations=50, seed=0, use_graph=True,
                 graph_chunk=25, autotune=False, orbit_min_pixel_angles=_ORBIT_MIN_PIXEL_ANGLES):
        self.problems = list(problems)
        self.orbit_min_pixel_angles = orbit_min_pixel_angles
        if autotune:
            # per-geometry forward split from the autotuner; the per-call
            # projections of the same settings use it too
            from . import autotune as _at

            for pr in self.problems:
                pr.fwd_split = _at.tune(pr.settings, np.float32)["fwd_split"]
        self.device = core._device_of(device)
        self.normest_iterations = normest_iterations
        self.use_graph = use_graph
        self.graph_chunk = graph_chunk
        self.rng = np.random.default_rng(seed)
        if _lib.raw("gr_batch_problem_size")() != ctypes.sizeof(_lib.GrBatchProblem):
            raise RuntimeError("gr_batch_problem layout mismatch between library and binding")
        # persistent grids: 0 lets the library size one wave of resident blocks
        self.grid_fwd = self.grid_bwd = self.grid_ew = 0
        self._build()

    # ------------------------------------------------------------ setup
    def _build(self):
        dev = self.device
        P = len(self.problems)
        self.desc = (_lib.GrBatchProblem * P)()
        self.buffers = []
        for k, pr in enumerate(self.problems):
            ps = pr.settings
            if pr.solver not in _SOLVERS:
                raise ValueError(f"unknown solver {pr.solver!r}")
            if tuple(pr.sino.shape) != tuple(ps.sinogram_shape) or pr.sino.dtype != torch.float32:
                raise ValueError("batched problems are float32 2-D sinograms of the settings' shape")
            if pr.fwd_split not in (1, 2, 4, 8):
                raise ValueError("fwd_split must be 1, 2, 4 or 8")
            f = core.empty(ps.sinogram_shape, torch.float32, "F", dev)
            f.copy_(pr.sino)
            Nx, Ny = ps.img_shape
            Ns, Na = ps.sinogram_shape
            t = ps.device_tables(np.float32)
            d = self.desc[k]
            d.kind = _lib.GR_FANBEAM if ps.is_fan else _lib.GR_RADON
            d.Nx, d.Ny, d.Ns, d.Na = Nx, Ny, Ns, Na
            d.solver = _SOLVERS[pr.solver]
            d.fwd_split = pr.fwd_split
            self._tiles(d, ps, pr.fwd_split)
            geo = np.asarray(ps.struct["geo_dict"][np.dtype("float32")], dtype=np.float32)
            vals = ([geo[0], geo[1]] if not ps.is_fan
                    else [geo[0], geo[1], geo[2], geo[3], geo[4], geo[5], geo[10]])
            for i, v in enumerate(vals):
                d.geo[i] = float(v)
            bufs = {
                "f": f,
                "img": core.zeros(ps.img_shape, torch.float32, "F", dev),
                "s1": core.zeros(ps.sinogram_shape, torch.float32, "F", dev),
                "s2": core.zeros(ps.sinogram_shape, torch.float32, "F", dev),
                "i1": core.zeros(ps.img_shape, torch.float32, "F", dev),
                "i2": core.zeros(ps.img_shape, torch.float32, "F", dev),
                "v4": torch.zeros(4 * Nx * Ny if pr.solver == "tv" else 4, dtype=torch.float32,
                                  device=dev),
                "sc": torch.zeros(_lib.SC_COUNT, dtype=torch.float64, device=dev),
                "fwd_part": torch.zeros(d.fwd_tiles_x * d.fwd_tiles_y, dtype=torch.float64,
                                        device=dev),
                "bwd_part": torch.zeros(max(d.bwd_tiles_x * d.bwd_tiles_y,
                                            d.obwd_tiles_x * d.obwd_tiles_y),
                                        dtype=torch.float64, device=dev),
                "tables": t,
            }
            self.buffers.append(bufs)
            d.ofs = t["ofs"].data_ptr()
            d.sdpd = t["sdpd"].data_ptr() if ps.is_fan else None
            d.w = t["w"].data_ptr()
            for name in ("f", "img", "s1", "s2", "i1", "i2", "v4", "sc", "fwd_part", "bwd_part"):
                setattr(d, name, bufs[name].data_ptr())
            d.cg_c = ps.delta_x**2 / ps.delta_s
        self._desc_dev = torch.empty(ctypes.sizeof(self.desc), dtype=torch.uint8, device=dev)
        self._upload_desc()

    def _tiles(self, d, ps, fwd_split):
        """Tile counts of problem descriptor ``d``: the per-angle tiles, or the
        orbit tiles where the library runs the orbit kernels for this
        geometry (``gr_orbit_kinds``), checked against the library's own
        block counts."""
        Nx, Ny = ps.img_shape
        Ns, Na = ps.sinogram_shape
        g = _lib.GrGeometry.from_buffer_copy(ps.gr_geometry(np.float32))
        g.work, g.work_bytes = None, 0
        g.fwd_split, g.bwd_split = fwd_split, _ORBIT_ANGLE_GROUPS
        d.orbit = int(_lib.raw("gr_orbit_kinds")(ctypes.byref(g), 1))
        if Nx * Ny * Na < self.orbit_min_pixel_angles:
            d.orbit = 0
        d.sym = g.sym
        for m in range(3):
            for k in range(6):
                d.sym_map[m][k] = g.sym_map[m][k]
        rays_per_block = (32 // fwd_split) * 4 * _RAYS_PER_LANE_GROUP
        d.fwd_tiles_x, d.fwd_tiles_y = -(-Ns // rays_per_block), Na
        d.bwd_tiles_x, d.bwd_tiles_y = -(-Nx // 32), -(-Ny // 8)
        d.obwd_tiles_x = d.obwd_tiles_y = 0
        if d.orbit & 1:
            # 128-thread blocks over a pair of base angles; 2 x fwd_split
            # lanes per group of 4 bins (fan beam, every bin) or 4 x fwd_split
            # (parallel beam, bins below ceil(Ns / 2))
            lanes = (2 if ps.is_fan else 4) * fwd_split
            bins = (32 // lanes) * 2 * _RAYS_PER_LANE_GROUP
            covered = Ns if ps.is_fan else (Ns + 1) // 2
            base = Na // 4 if ps.is_fan else Na // 2
            d.fwd_tiles_x, d.fwd_tiles_y = -(-covered // bins), -(-base // 2)
            want = int(_lib.raw("gr_forward_partials")(ctypes.byref(g), 1))
            if want != d.fwd_tiles_x * d.fwd_tiles_y:
                raise RuntimeError("orbit forward tiles disagree with the library's launch grid")
        if d.orbit & 2:
            # 32 x 1 quadrant tiles, 8 angle groups
            half = Nx // 2
            d.obwd_tiles_x, d.obwd_tiles_y = -(-half // 32), half
            want = int(_lib.raw("gr_backward_partials")(ctypes.byref(g), 1, _lib.GR_ORDER_F))
            if want != d.obwd_tiles_x * d.obwd_tiles_y:
                raise RuntimeError("orbit backprojection tiles disagree with the library's grid")

    def _upload_desc(self):
        host = torch.frombuffer(bytearray(bytes(self.desc)), dtype=torch.uint8)
        self._desc_dev.copy_(host)

    def _items(self, ids, kind):
        items = []
        for k in ids:
            d = self.desc[k]
            if kind == "fwd":
                n = d.fwd_tiles_x * d.fwd_tiles_y
            elif kind == "bwd":
                n = (d.obwd_tiles_x * d.obwd_tiles_y if d.orbit & 2
                     else d.bwd_tiles_x * d.bwd_tiles_y)
            elif kind == "img":  # 32 x 8 pixel tiles of the whole image
                n = d.bwd_tiles_x * d.bwd_tiles_y
            else:  # sinogram chunks of 256 bins
                n = -(-(d.Ns * d.Na) // 256)
            items.append(np.stack([np.full(n, k, np.int32), np.arange(n, dtype=np.int32)], 1))
        if not items:
            return torch.zeros(0, dtype=torch.int32, device=self.device), 0
        arr = np.concatenate(items).astype(np.int32)
        # interleave problems so that the persistent blocks see a mix of sizes
        order = np.argsort(np.concatenate([np.arange(len(a)) / max(1, len(a)) for a in items]),
                           kind="stable")
        arr = np.ascontiguousarray(arr[order])
        return torch.from_numpy(arr.reshape(-1)).to(self.device), len(arr)

    def _proj_lists(self, ids, fwd):
        """Work lists of a projection phase: (entry point, geometry kind or
        None, items) for the per-angle tiles and for each kind's orbit
        tiles; empty lists left out."""
        bit = 1 if fwd else 2
        kind = "fwd" if fwd else "bwd"
        plain = [k for k in ids if not self.desc[k].orbit & bit]
        out = [("gr_batch_forward" if fwd else "gr_batch_backward", None,
                self._items(plain, kind))]
        name = "gr_batch_forward_orbit" if fwd else "gr_batch_backward_orbit"
        for geom in (_lib.GR_RADON, _lib.GR_FANBEAM):
            sel = [k for k in ids if self.desc[k].orbit & bit and self.desc[k].kind == geom]
            out.append((name, geom, self._items(sel, kind)))
        return [e for e in out if e[2][1]]

    # ---------------------------------------------------------- launches
    def _launch(self, name, lists, mode, grid, geom=None):
        items, n = lists
        if n == 0:
            return
        extra = () if geom is None else (geom,)
        _lib.call(name, ctypes.c_void_p(self._desc_dev.data_ptr()), ctypes.c_void_p(items.data_ptr()),
                  n, mode, *extra, grid, core._stream_ptr(self.device))

    def _project(self, lists, mode, grid):
        for name, geom, items in lists:
            self._launch(name, items, mode, grid, geom)

    def _scalars(self, ids, mode, phase):
        t, n = ids
        if n:
            _lib.call("gr_batch_scalars", ctypes.c_void_p(self._desc_dev.data_ptr()),
                      ctypes.c_void_p(t.data_ptr()), n, mode, phase, core._stream_ptr(self.device))

    def _ids(self, ids):
        arr = np.asarray(list(ids), dtype=np.int32)
        return torch.from_numpy(arr).to(self.device), len(arr)

    def _iterate_chunk(self, body, n):
        if n <= 0:
            return
        if not self.use_graph or n < 2:
            for _ in range(n):
                body()
            return
        chunk = min(n, self.graph_chunk)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            for _ in range(chunk):
                body()
        reps, rem = divmod(n, chunk)
        for _ in range(reps):
            graph.replay()
        for _ in range(rem):
            body()

    # --------------------------------------------------------------- run
    def run(self):
        """Run every problem to its iteration count; returns the reconstructions."""
        P = len(self.problems)
        dev = self.device
        with torch.cuda.device(dev):
            # ---- normest for Landweber and TV problems
            need = [k for k, pr in enumerate(self.problems)
                    if pr.solver in ("landweber", "tv") and pr.norm_estimate is None]
            if need:
                st = core._stream_ptr(dev)
                dot = torch.empty(int(_lib.raw("gr_dot_partials_count")()), dtype=torch.float64,
                                  device=dev)
                for k in need:
                    pr = self.problems[k]
                    x0 = pr.normest_x0
                    if x0 is None:
                        x0 = self.rng.standard_normal(pr.settings.img_shape)
                    x0 = np.asarray(x0, dtype=np.float32)
                    img = self.buffers[k]["img"]
                    img.copy_(torch.from_numpy(np.ascontiguousarray(x0.T)).T)
                    # the start vector's sum, reduced as normest reduces it
                    _lib.call("gr_sum_values_partials", core._ptr(dot), core._ptr(img),
                              _lib.GR_F32, img.numel(), st)
                    _lib.call("gr_sum_partials",
                              ctypes.c_void_p(self.buffers[k]["sc"].data_ptr() + 8 * _lib.SC_SUM),
                              core._ptr(dot), dot.numel(), st)
                img_l, fwd_l, bwd_l = (self._items(need, "img"), self._proj_lists(need, True),
                                       self._proj_lists(need, False))
                ids = self._ids(need)
                M = _lib.GR_BATCH_NORMEST

                def normest_step():
                    self._launch("gr_batch_image_step", img_l, M, self.grid_ew)
                    self._project(fwd_l, M, self.grid_fwd)
                    self._project(bwd_l, M, self.grid_bwd)
                    self._scalars(ids, M, 1)

                # normest returns the sum taken at the start of its last
                # iteration; that iteration's projections do not change it
                self._iterate_chunk(normest_step, self.normest_iterations - 1)
                sums = torch.stack([self.buffers[k]["sc"][_lib.SC_SUM] for k in need]).cpu().numpy()
                for k, s in zip(need, sums):
                    self.problems[k].norm_estimate = float(np.sqrt(s))
            # ---- solver scalars and state initialisation
            for k, pr in enumerate(self.problems):
                d, b = self.desc[k], self.buffers[k]
                ps = pr.settings
                if pr.solver == "landweber":
                    d.a0 = -_f32(pr.w / pr.norm_estimate**2)
                    b["img"].zero_()
                elif pr.solver == "tv":
                    sigma = 1.0 / np.sqrt(13) * pr.stepsize_weighting
                    tau = 1.0 / np.sqrt(13) / pr.stepsize_weighting
                    mu = pr.mu * pr.norm_estimate**2 * ps.delta_x
                    mu = mu / (sigma + mu)
                    d.a0, d.a1, d.a2 = _f32(sigma), _f32(sigma / pr.norm_estimate), _f32(mu)
                    d.a3, d.a4 = _f32(tau), _f32(1.0 / pr.norm_estimate)
                    for name in ("img", "i1", "v4", "s1"):
                        b[name].zero_()
                else:
                    b["img"].zero_()
                    b["s2"].copy_(b["f"])  # d = f - A 0
            self._upload_desc()
            cg = [k for k, pr in enumerate(self.problems) if pr.solver == "cg"]
            if cg:
                self._project(self._proj_lists(cg, False), _lib.GR_BATCH_CG_INIT, self.grid_bwd)
                self._scalars(self._ids(cg), _lib.GR_BATCH_CG_INIT, 1)
            # ---- main iterations, one graph per range of constant active set
            bounds = sorted({0} | {pr.iterations for pr in self.problems})
            M = _lib.GR_BATCH_MAIN
            for lo, hi in zip(bounds[:-1], bounds[1:]):
                active = [k for k, pr in enumerate(self.problems) if pr.iterations > lo]
                img_ids = [k for k in active if self.problems[k].solver in ("cg", "tv")]
                cg_ids = [k for k in active if self.problems[k].solver == "cg"]
                img_l = self._items(img_ids, "img")
                fwd_l, bwd_l = self._proj_lists(active, True), self._proj_lists(active, False)
                sino_l = self._items(cg_ids, "sino")
                cgi = self._ids(cg_ids)

                def step(img_l=img_l, fwd_l=fwd_l, bwd_l=bwd_l, sino_l=sino_l, cgi=cgi):
                    self._launch("gr_batch_image_step", img_l, M, self.grid_ew)
                    self._project(fwd_l, M, self.grid_fwd)
                    self._scalars(cgi, M, 0)
                    self._launch("gr_batch_sino_step", sino_l, M, self.grid_ew)
                    self._project(bwd_l, M, self.grid_bwd)
                    self._scalars(cgi, M, 1)

                self._iterate_chunk(step, hi - lo)
        for k, pr in enumerate(self.problems):
            pr.result = self.buffers[k]["img"]
        return [pr.result for pr in self.problems]

    def launches_per_iteration(self) -> int:
        """Kernel launches per batched iteration with every problem running:
        image step, alpha, sinogram step and beta, and one forward and one
        backprojection launch per tile family present (per-angle tiles,
        parallel-beam orbit tiles, fan-beam orbit tiles)."""
        ids = range(len(self.problems))
        return 4 + len(self._proj_lists(ids, True)) + len(self._proj_lists(ids, False))


def heterogeneous_problems(count=64, seed=0, device=None, landweber_iterations=200,
                           cg_iterations=50, tv_iterations=100, sizes=(128, 192, 256, 384, 512),
                           angle_range=(60, 720), mu=20.0):
    """The heterogeneous batch workload, seeded.

    Image side from ``sizes``, angle count uniform in ``angle_range``; half the
    problems are Radon (angles on [0, pi) or the limited range [0, 2pi/3)),
    half fan beam (RE uniform in [150, 300], R = 2 RE, detector width R,
    automatic image width); solvers cycle Landweber / CG / TV.  Sinograms are
    forward projections of seeded random-ellipse images plus 1% Gaussian
    noise.
    """
    from .phantom import random_ellipse_image

    dev = core._device_of(device)
    rng = np.random.default_rng(seed)
    problems = []
    for k in range(count):
        N = int(rng.choice(sizes))
        Na = int(rng.integers(angle_range[0], angle_range[1] + 1))
        if k % 2 == 0:
            if rng.random() < 0.5:
                angles = Na
            else:
                angles = [(Na, 0.0, 2 * np.pi / 3)]
            ps = core.ProjectionSettings(dev, core.RADON, (N, N), angles)
        else:
            RE = float(rng.uniform(150, 300))
            R = 2 * RE
            ps = core.ProjectionSettings(dev, core.FANBEAM, (N, N), Na,
                                         n_detectors=int(np.ceil(1.42 * N)), detector_width=R,
                                         R=R, RE=RE)
        img = random_ellipse_image(int(rng.integers(1 << 30)), (N, N), dtype="float32").T
        img_d = core.empty((N, N), torch.float32, "F", dev)
        img_d.copy_(torch.from_numpy(np.ascontiguousarray(img.T)).T)
        sino = core.forwardprojection(img_d, ps)
        noise = torch.from_numpy(rng.standard_normal(ps.sinogram_shape[::-1]).astype(np.float32))
        sino += 0.01 * float(sino.abs().max()) * noise.to(dev).T
        solver = ("landweber", "cg", "tv")[k % 3]
        iters = {"landweber": landweber_iterations, "cg": cg_iterations, "tv": tv_iterations}[solver]
        problems.append(Problem(ps, sino, solver, iters, mu=mu))
    return problems


def solve_plain(problems, use_graph=False):
    """Reference timing form: each problem through the per-call API, one after another."""
    out = []
    for pr in problems:
        if pr.solver == "landweber":
            out.append(core.landweber(pr.sino, pr.settings, pr.iterations, w=pr.w,
                                      norm_estimate=pr.norm_estimate, use_graph=use_graph))
        elif pr.solver == "cg":
            out.append(core.conjugate_gradients(pr.sino, pr.settings, pr.iterations,
                                                use_graph=use_graph))
        else:
            out.append(core.total_variation(pr.sino, pr.settings, pr.mu, pr.iterations,
                                            stepsize_weighting=pr.stepsize_weighting,
                                            norm_estimate=pr.norm_estimate, use_graph=use_graph))
    return out


def _main(argv=None):
    """Run one seeded heterogeneous batch and print its wall time (``python -m gratopy_gb300.batch``)."""
    import argparse
    import json
    import time

    ap = argparse.ArgumentParser(description=_main.__doc__)
    ap.add_argument("--count", type=int, default=64)
    ap.add_argument("--small", action="store_true", help="sides 32..128, 30..180 angles")
    ap.add_argument("--runs", type=int, default=1)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args(argv)
    dev = core._device_of(None)
    kw = dict(sizes=(32, 48, 64, 96, 128), angle_range=(30, 180)) if args.small else {}
    probs = heterogeneous_problems(args.count, seed=args.seed, device=dev, **kw)
    times = []
    for _ in range(args.runs):
        fresh = [Problem(p.settings, p.sino, p.solver, p.iterations, mu=p.mu) for p in probs]
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        BatchedReconstruction(fresh, dev).run()
        torch.cuda.synchronize(dev)
        times.append(time.perf_counter() - t0)
    print(json.dumps({"problems": args.count, "small": args.small, "seconds": times,
                      "recon_per_s": args.count / min(times)}))


if __name__ == "__main__":
    _main()
