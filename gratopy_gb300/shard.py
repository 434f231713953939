"""Multi-GPU sharding: one process per GPU, stacks split along z, batches split by problem.

What couples the units of the path decides what the ranks exchange:

* slices of a stack under Landweber (given the norm estimate) and separate
  batched problems are independent: each rank runs its share, no exchange;
* one CG problem over a stack couples its slices only through five scalars
  (<p,p>, <f,f>, <Wq,q>, <d,d>, <snew,snew>, gratopy.py:2449-2551): each
  rank reduces its own slices in float64 and a sum all-reduce of those
  numbers combines them, twice per iteration;
* TV with ``slice_thickness > 0`` couples neighbouring slices through the
  z-gradient (total_variation.cl:54-93, :108-148): each rank keeps one ghost
  slice on each interior side, refreshed every iteration -- Ubar from the
  rank above before the dual step, V from the rank below before the primal
  step (the only values of a neighbour that its own slices read).

The solver drivers are written against small backends, so the same
sequencing runs on the GPU kernels (:class:`KernelCG`, :class:`KernelTV`)
or on any other implementation of the steps; the collectives are
``torch.distributed`` calls (NCCL for device tensors, gloo for host tensors).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from . import core


# ---------------------------------------------------------------- partitions


def slice_ranges(nz: int, world: int, align: int = 4) -> list[tuple[int, int]]:
    """Contiguous slice ranges ``[z0, z1)`` per rank: whole groups of ``align``
    slices (the projections carry 4 slices per thread), spread as evenly as
    possible, earlier ranks taking the extra group.  Ranks may get none."""
    if nz < 0 or world < 1 or align < 1:
        raise ValueError("nz >= 0, world >= 1, align >= 1 required")
    groups = -(-nz // align)
    q, r = divmod(groups, world)
    out, g0 = [], 0
    for k in range(world):
        g1 = g0 + q + (1 if k < r else 0)
        out.append((min(nz, g0 * align), min(nz, g1 * align)))
        g0 = g1
    return out


@dataclass(frozen=True)
class HaloRange:
    """Slices a rank holds for a coupled (TV) solve: owned ``[own0, own1)``
    plus one ghost slice on each side that has a neighbour."""

    lo: int
    hi: int
    own0: int
    own1: int

    @property
    def ghost_below(self) -> bool:
        return self.lo < self.own0

    @property
    def ghost_above(self) -> bool:
        return self.hi > self.own1


def halo_ranges(nz: int, world: int, align: int = 4) -> list[HaloRange]:
    ranges = slice_ranges(nz, world, align)
    if any(z1 <= z0 for z0, z1 in ranges):
        raise ValueError(f"{nz} slices give some of {world} ranks no slice; use fewer ranks")
    return [HaloRange(z0 - (1 if k > 0 else 0), z1 + (1 if k < world - 1 else 0), z0, z1)
            for k, (z0, z1) in enumerate(ranges)]


def partition_costs(costs, world: int) -> list[list[int]]:
    """Deterministic longest-processing-time assignment of weighted units to
    ranks: heaviest first, each to the least-loaded rank (lowest rank on ties)."""
    load = [0.0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i)):
        k = min(range(world), key=lambda r: (load[r], r))
        out[k].append(i)
        load[k] += float(costs[i])
    return [sorted(v) for v in out]


def problem_cost(problem, normest_iterations: int = 50) -> float:
    """Projection work of a batched problem in pixel-angles (two projections
    per iteration, normest included for Landweber and TV)."""
    Nx, Ny = problem.settings.img_shape
    Na = problem.settings.sinogram_shape[1]
    its = problem.iterations + (normest_iterations if problem.solver in ("landweber", "tv") else 0)
    return 2.0 * Nx * Ny * Na * its


def partition_problems(problems, world: int) -> list[list[int]]:
    return partition_costs([problem_cost(p) for p in problems], world)


# --------------------------------------------------------------- collectives


def _dist_ready(group) -> bool:
    return torch.distributed.is_available() and torch.distributed.is_initialized() and (
        torch.distributed.get_world_size(group) > 1)


def all_reduce_sum(t: torch.Tensor, group=None) -> torch.Tensor:
    """In-place float64 sum over the ranks of ``group`` (identity on one rank)."""
    if _dist_ready(group):
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM, group=group)
    return t


def exchange_planes(send: torch.Tensor | None, send_to: int | None, recv: torch.Tensor | None,
                    recv_from: int | None, group=None) -> None:
    """Send one plane to a neighbour and receive one from the other (both optional)."""
    if not _dist_ready(group):
        return
    reqs = []
    if send is not None and send_to is not None:
        reqs.append(torch.distributed.isend(send.contiguous(), send_to, group=group))
    buf = None
    if recv is not None and recv_from is not None:
        buf = torch.empty_like(recv).contiguous()
        reqs.append(torch.distributed.irecv(buf, recv_from, group=group))
    for r in reqs:
        r.wait()
    if buf is not None:
        recv.copy_(buf)


def _rank_world(group):
    if _dist_ready(group):
        return torch.distributed.get_rank(group), torch.distributed.get_world_size(group)
    return 0, 1


# -------------------------------------------------------------- CG, sharded


def cg_sharded(backend, number_iterations: int, epsilon: float = 0.0, group=None):
    """CG on the normal equations over the union of the ranks' slices.

    The backend holds this rank's slices and returns float64 tensors of local
    partial scalars; this driver sums them over the ranks at the points
    where gratopy's CG needs a global scalar.  An ``epsilon`` stop needs the
    residual on the host, one synchronisation per iteration.
    """
    init = backend.init()                       # [<p,p>, <f,f>] over local slices
    all_reduce_sum(init, group)
    backend.set_init(init)
    for _ in range(number_iterations):
        qwq = backend.forward()                 # [<W q, q>]
        all_reduce_sum(qwq, group)
        backend.alpha(qwq)
        pair = backend.backward()               # [<d,d>, <snew,snew>]
        all_reduce_sum(pair, group)
        backend.beta(pair, epsilon)
        backend.update_p()
        if epsilon > 0 and backend.stopped():
            break
    return backend.result()


class KernelCG:
    """CG steps on this rank's slices with the library kernels (float32/64 stacks).

    With one rank this is exactly :func:`gratopy_gb300.conjugate_gradients`
    (same kernels, same partial sums in the same order).
    """

    def __init__(self, sino: torch.Tensor, ps, x0: torch.Tensor | None = None):
        core._check_tensor(sino, "sino")
        self.sino, self.ps = sino, ps
        self.order = core.order_of(sino)
        self.dims = core._img_shape_for(sino, ps)
        dev = self.dev = sino.device
        self.x = core.zeros(self.dims, sino.dtype, self.order, dev)
        if x0 is not None:
            self.x.copy_(x0)
        ndt = core._np_dtype(sino.dtype)
        self.g = ps.gr_geometry(ndt)
        self.w = ps.device_tables(ndt)["w"]
        self.Nz = core._nz(sino)
        self.of = core._oflag(self.order)
        self.d = core.zeros(sino.shape, sino.dtype, self.order, dev)
        self.r = core.empty(sino.shape, sino.dtype, self.order, dev)
        self.q = core.empty(sino.shape, sino.dtype, self.order, dev)
        self.p = core.empty(self.dims, sino.dtype, self.order, dev)
        self.snew = core.empty(self.dims, sino.dtype, self.order, dev)
        self.c = ps.delta_x**2 / ps.delta_s
        gp = ctypes.byref(self.g)
        self.n_fwd = int(_lib.raw("gr_forward_partials")(gp, self.Nz))
        self.n_bwd = int(_lib.raw("gr_backward_partials")(gp, self.Nz, self.of))
        self.scr = core._Scratch(dev, max(self.n_fwd, self.n_bwd))
        self.red = torch.zeros(4, dtype=torch.float64, device=dev)

    def _st(self):
        return core._stream_ptr(self.dev)

    def _slot(self, t: torch.Tensor, k: int = 0):
        return ctypes.c_void_p(t.data_ptr() + 8 * k)

    def init(self):
        st, gp, P = self._st(), ctypes.byref(self.g), core._ptr
        with torch.cuda.device(self.dev):
            _lib.call("gr_forward_residual", gp, P(self.r), P(self.x), P(self.sino), self.Nz,
                      self.of, st)
            _lib.call("gr_equ_mul_add", P(self.d), -1.0, P(self.r), core._dt(self.d),
                      self.d.numel(), st)
            _lib.call("gr_backward", gp, P(self.p), P(self.d), self.Nz, self.of, self.of, st)
            for k, (a, b) in enumerate(((self.p, self.p), (self.sino, self.sino))):
                _lib.call("gr_dot_partials", P(self.scr.dot), P(a), P(b), core._dt(a), a.numel(),
                          st)
                _lib.call("gr_sum_partials", self._slot(self.red, k), P(self.scr.dot),
                          self.scr.dot.numel(), st)
        return self.red[0:2]

    def set_init(self, totals):
        self.scr.sc[_lib.SC_SOLD] = totals[0]
        self.scr.sc[_lib.SC_FSQ] = totals[1]

    def forward(self):
        st, P = self._st(), core._ptr
        with torch.cuda.device(self.dev):
            _lib.call("gr_forward_wsq", ctypes.byref(self.g), P(self.q), P(self.p), P(self.w),
                      P(self.scr.part), P(self.scr.done), self.Nz, self.of, st)
            _lib.call("gr_sum_partials", self._slot(self.red, 0), P(self.scr.part), self.n_fwd,
                      st)
        return self.red[0:1]

    def alpha(self, qwq):
        with torch.cuda.device(self.dev):
            _lib.call("gr_cg_alpha", core._ptr(self.scr.sc), core._ptr(qwq), 1, float(self.c),
                      core._dt(self.sino), core._ptr(self.scr.done), self._st())

    def backward(self):
        st, P = self._st(), core._ptr
        with torch.cuda.device(self.dev):
            _lib.call("gr_cg_update_d", P(self.d), P(self.q), P(self.scr.sc), P(self.scr.dot),
                      core._dt(self.sino), self.d.numel(), P(self.scr.done), st)
            _lib.call("gr_sum_partials", self._slot(self.red, 1), P(self.scr.dot),
                      self.scr.dot.numel(), st)
            _lib.call("gr_backward_cg", ctypes.byref(self.g), P(self.snew), P(self.d), P(self.x),
                      P(self.p), self.scr.slot(_lib.SC_ALPHA), P(self.scr.part2),
                      P(self.scr.done), self.Nz, self.of, st)
            _lib.call("gr_sum_partials", self._slot(self.red, 2), P(self.scr.part2), self.n_bwd,
                      st)
        return self.red[1:3]

    def beta(self, pair, epsilon):
        with torch.cuda.device(self.dev):
            _lib.call("gr_cg_beta", core._ptr(self.scr.sc), self._slot(pair, 1), 1,
                      self._slot(pair, 0), 1, float(epsilon), core._dt(self.sino),
                      core._ptr(self.scr.done), self._st())

    def update_p(self):
        with torch.cuda.device(self.dev):
            _lib.call("gr_cg_update_p", core._ptr(self.p), core._ptr(self.snew),
                      core._ptr(self.scr.sc), core._dt(self.sino), self.p.numel(),
                      core._ptr(self.scr.done), self._st())

    def stopped(self) -> bool:
        return bool(self.scr.done.item())

    def result(self):
        return self.x


class EmptyCG:
    """A rank without slices: contributes zeros to every sum."""

    def __init__(self, device):
        self.red = torch.zeros(4, dtype=torch.float64, device=device)
        self.done = torch.zeros(1, dtype=torch.int32, device=device)

    def init(self):
        return self.red[0:2].zero_()

    def set_init(self, totals):
        self.sold, self.fsq = totals[0].clone(), totals[1].clone()

    def forward(self):
        return self.red[0:1].zero_()

    def alpha(self, qwq):
        pass

    def backward(self):
        return self.red[1:3].zero_()

    def beta(self, pair, epsilon):
        # the same stop test as the ranks with slices, on the summed scalars
        if epsilon > 0:
            res = torch.sqrt(pair[0] / self.fsq)
            self.done.copy_((res < epsilon).to(torch.int32).reshape(1))

    def update_p(self):
        pass

    def stopped(self) -> bool:
        return bool(self.done.item())

    def result(self):
        return None


def conjugate_gradients_sharded(sino_local, projectionsetting, number_iterations=20,
                                epsilon=0.0, x0=None, group=None):
    """gratopy's ``conjugate_gradients`` for a stack whose slices are spread
    over the ranks of ``group`` (each rank passes its own slices, e.g. the
    range :func:`slice_ranges` gives it; a rank with none passes a stack of
    zero slices); returns this rank's slices of x."""
    if sino_local.dim() == 3 and sino_local.shape[2] == 0:
        return cg_sharded(EmptyCG(sino_local.device), number_iterations, epsilon, group)
    return cg_sharded(KernelCG(sino_local, projectionsetting, x0), number_iterations, epsilon,
                      group)


# -------------------------------------------------------------- TV, sharded


def tv_sharded(backend, number_iterations: int, group=None):
    """TV primal-dual iterations with ghost-slice exchange (see module doc).

    The backend holds this rank's slices plus its ghosts and exposes planes
    ``plane(name, k)`` of its local arrays (k indexes the local stack).
    """
    rank, world = _rank_world(group)
    nz = backend.nz_local
    below = rank - 1 if backend.ghost_below else None
    above = rank + 1 if backend.ghost_above else None
    first_own = 1 if backend.ghost_below else 0
    last_own = nz - 2 if backend.ghost_above else nz - 1
    for _ in range(number_iterations):
        # Ubar: my first owned plane goes down, the plane above comes in
        exchange_planes(backend.plane("ubar", first_own), below,
                        backend.plane("ubar", nz - 1) if above is not None else None, above, group)
        backend.dual()
        # V: my last owned plane goes up, the plane below comes in
        exchange_planes(backend.plane("v", last_own), above,
                        backend.plane("v", 0) if below is not None else None, below, group)
        backend.data_dual()
        backend.primal()
    return backend.result()


class KernelTV:
    """TV steps on this rank's slices (plus ghosts) with the library kernels."""

    def __init__(self, sino_ext: torch.Tensor, ps, mu, slice_thickness, stepsize_weighting,
                 norm_estimate, ghost_below: bool, ghost_above: bool):
        from .autograd import _TVProblem

        if core.order_of(sino_ext) != "F" or sino_ext.dim() != 3:
            raise ValueError("sharded TV takes a Fortran-ordered (Ns, Na, Nz) stack")
        self.prob = _TVProblem(sino_ext, ps, mu, slice_thickness, stepsize_weighting,
                               norm_estimate)
        self.state = self.prob.new_state()
        self.nz_local = int(sino_ext.shape[2])
        self.ghost_below, self.ghost_above = ghost_below, ghost_above
        Nx, Ny = ps.img_shape
        self.plane_n = Nx * Ny

    def plane(self, name: str, k: int) -> torch.Tensor:
        n = self.plane_n
        if name == "ubar":
            return self.state.Ubar[:, :, k]
        if name == "v":
            return self.state.V[4 * n * k: 4 * n * (k + 1)]
        raise KeyError(name)

    def dual(self):
        p, s = self.prob, self.state
        Nx, Ny = p.ps.img_shape
        with torch.cuda.device(p.f.device):
            _lib.call("gr_tv_dual", core._ptr(s.V), core._ptr(s.Ubar), p.sigma, p.z,
                      core._dt(p.f), Nx, Ny, p.Nz, p.of, core._stream_ptr(p.f.device))

    def data_dual(self):
        p, s = self.prob, self.state
        with torch.cuda.device(p.f.device):
            _lib.call("gr_forward_lambda", ctypes.byref(p.g), core._ptr(s.L), core._ptr(s.Ubar),
                      core._ptr(p.f), p.sigma_l, p.mu2, p.Nz, p.of, core._stream_ptr(p.f.device))

    def primal(self):
        p, s = self.prob, self.state
        with torch.cuda.device(p.f.device):
            _lib.call("gr_backward_tv_primal", ctypes.byref(p.g), core._ptr(s.U),
                      core._ptr(s.Ubar), core._ptr(s.V), core._ptr(s.L), p.tau, p.norming, p.z,
                      p.Nz, p.of, core._stream_ptr(p.f.device))

    def result(self):
        lo = 1 if self.ghost_below else 0
        hi = self.nz_local - (1 if self.ghost_above else 0)
        return self.state.U[:, :, lo:hi]


def total_variation_sharded(sino_ext, projectionsetting, mu, number_iterations=1000,
                            slice_thickness=1.0, stepsize_weighting=10.0, norm_estimate=None,
                            halo: HaloRange | None = None, group=None):
    """gratopy's ``total_variation`` for a stack spread over the ranks of ``group``.

    ``sino_ext`` holds this rank's slices ``[halo.lo, halo.hi)`` of the data
    (owned slices plus one neighbour slice on each interior side, see
    :func:`halo_ranges`); ``norm_estimate`` must be the same on every rank.
    Returns this rank's owned slices of U.
    """
    if norm_estimate is None:
        raise ValueError("pass the same norm_estimate on every rank (e.g. normest on rank 0, broadcast)")
    rank, world = _rank_world(group)
    if halo is None:
        if world > 1:
            raise ValueError("pass this rank's HaloRange (halo_ranges(nz, world)[rank])")
        halo = halo_ranges(int(sino_ext.shape[2]), 1)[0]
    be = KernelTV(sino_ext, projectionsetting, mu, slice_thickness, stepsize_weighting,
                  norm_estimate, halo.ghost_below, halo.ghost_above)
    return tv_sharded(be, number_iterations, group)


# --------------------------------------------------------- batches, sharded


def batch_sharded(problems, device=None, group=None, **kwargs):
    """Solve this rank's share of a heterogeneous batch (no exchange).

    The problems are split over the ranks of ``group`` by
    :func:`partition_problems`; this rank runs its share as one
    :class:`~gratopy_gb300.batch.BatchedReconstruction` (``kwargs`` go to
    it) and returns ``{index: reconstruction}`` for the problems it solved.
    """
    from .batch import BatchedReconstruction

    rank, world = _rank_world(group)
    mine = partition_problems(problems, world)[rank]
    if not mine:
        return {}
    out = BatchedReconstruction([problems[i] for i in mine], device, **kwargs).run()
    return dict(zip(mine, out))
