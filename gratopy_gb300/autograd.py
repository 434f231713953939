"""Differentiation through the projections and an unrolled TV reconstruction.

gratopy has no gradients; this module adds them on top of the same kernels.

* :func:`forward_project` / :func:`back_project` -- ``torch.autograd``
  functions whose backward passes are the hand-written transposes: the
  gradient of the forward projection A is the backprojection kernel run with
  the adjoint table (A^T = dx/(ds/dx) * unit-weight backprojection), the
  gradient of gratopy's backprojection A* (adjoint in gratopy's weighted
  inner products) is the forward projection kernel with a per-angle weight
  epilogue (A*^T = (ds/dx)/dx * W A).
* :func:`tv_unrolled` -- a fixed number of iterations of gratopy's L2-TV
  primal-dual algorithm (gratopy.py:2554-2762, the same iteration as
  :func:`gratopy_gb300.total_variation`) as a differentiable function of the
  sinogram, with a hand-written adjoint: gradient/divergence adjoint pair,
  the Jacobian of the pointwise unit-ball projection, the positivity mask,
  the extrapolation step and the projections' transposes.  States are
  checkpointed every ``checkpoint_every`` iterations and the iterations in
  between are recomputed during the backward pass.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from . import core
from .core import _dt, _np_dtype, _nz, _oflag, _ptr, _stream_ptr, order_of


def _as_contiguous(t: torch.Tensor) -> torch.Tensor:
    try:
        order_of(t)
        return t
    except ValueError:
        return t.contiguous()


def transpose_forward(g: torch.Tensor, ps) -> torch.Tensor:
    """A^T g: plain (Euclidean) transpose of the forward projection."""
    g = _as_contiguous(g)
    ndt = _np_dtype(g.dtype)
    ga = ps.gr_geometry_adjoint(ndt)
    order = order_of(g)
    z = (int(g.shape[2]),) if g.dim() > 2 else ()
    out = core.empty(tuple(ps.img_shape) + z, g.dtype, order, g.device)
    with torch.cuda.device(g.device):
        _lib.call("gr_backward", ctypes.byref(ga), _ptr(out), _ptr(g), _nz(g), _oflag(order),
                  _oflag(order), _stream_ptr(g.device))
    return out


def transpose_back(h: torch.Tensor, ps) -> torch.Tensor:
    """A*^T h: plain transpose of gratopy's backprojection, (ds/dx)/dx * W A h."""
    h = _as_contiguous(h)
    ndt = _np_dtype(h.dtype)
    g = ps.gr_geometry(ndt)
    w = ps.device_tables(ndt)["w"]
    order = order_of(h)
    z = (int(h.shape[2]),) if h.dim() > 2 else ()
    out = core.empty(tuple(ps.sinogram_shape) + z, h.dtype, order, h.device)
    with torch.cuda.device(h.device):
        _lib.call("gr_forward_angle_axpy", ctypes.byref(g), _ptr(out), None, _ptr(h), _ptr(w),
                  1.0 / ps.forward_scale(ndt), _nz(h), _oflag(order),
                  _stream_ptr(h.device))
    return out


class _ForwardProjection(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, ps):
        ctx.ps = ps
        return core.forwardprojection(_as_contiguous(x.detach()), ps)

    @staticmethod
    def backward(ctx, grad):
        return transpose_forward(grad, ctx.ps), None


class _BackProjection(torch.autograd.Function):
    @staticmethod
    def forward(ctx, y, ps):
        ctx.ps = ps
        return core.backprojection(_as_contiguous(y.detach()), ps)

    @staticmethod
    def backward(ctx, grad):
        return transpose_back(grad, ctx.ps), None


def forward_project(x: torch.Tensor, ps) -> torch.Tensor:
    """Differentiable forward projection (gratopy.forwardprojection)."""
    return _ForwardProjection.apply(x, ps)


def back_project(y: torch.Tensor, ps) -> torch.Tensor:
    """Differentiable backprojection (gratopy.backprojection)."""
    return _BackProjection.apply(y, ps)


# ----------------------------------------------------------- unrolled TV


class _TVState:
    """(U, Ubar, V, Lambda) of the primal-dual iteration, in one memory order."""

    def __init__(self, img_shape, sino_shape, dtype, order, device):
        self.U = core.zeros(img_shape, dtype, order, device)
        self.Ubar = core.zeros(img_shape, dtype, order, device)
        self.V = torch.zeros(4 * self.U.numel(), dtype=dtype, device=device)
        self.L = core.zeros(sino_shape, dtype, order, device)

    def copy_from(self, other: "_TVState") -> "_TVState":
        self.U.copy_(other.U)
        self.Ubar.copy_(other.Ubar)
        self.V.copy_(other.V)
        self.L.copy_(other.L)
        return self


class _TVProblem:
    """Scalars and launch arguments of one unrolled TV run (float32 scalars, as gratopy)."""

    def __init__(self, f, ps, mu, slice_thickness, stepsize_weighting, norm_estimate):
        self.f = f
        self.ps = ps
        self.order = order_of(f)
        self.of = _oflag(self.order)
        self.Nz = _nz(f)
        self.dtype = f.dtype
        self.ndt = _np_dtype(f.dtype)
        self.g = ps.gr_geometry(self.ndt)
        self.ga = ps.gr_geometry_adjoint(self.ndt)
        self.w = ps.device_tables(self.ndt)["w"]
        self.img_shape = tuple(ps.img_shape) + ((self.Nz,) if f.dim() > 2 else ())
        if f.dim() == 2:
            slice_thickness = 0.0
        f32 = lambda v: float(np.float32(v))  # noqa: E731
        sigma = 1.0 / np.sqrt(13) * stepsize_weighting
        tau = 1.0 / np.sqrt(13) / stepsize_weighting
        mu2 = mu * norm_estimate**2 * ps.delta_x
        mu2 = mu2 / (sigma + mu2)
        self.sigma, self.tau = f32(sigma), f32(tau)
        self.sigma_l, self.mu2 = f32(sigma / norm_estimate), f32(mu2)
        self.norming, self.z = f32(1.0 / norm_estimate), f32(slice_thickness)

    def new_state(self) -> _TVState:
        return _TVState(self.img_shape, tuple(self.f.shape), self.dtype, self.order, self.f.device)

    def step(self, s: _TVState) -> None:
        """One primal-dual iteration in place (the three launches of total_variation)."""
        st = _stream_ptr(self.f.device)
        Nx, Ny = self.ps.img_shape
        gp = ctypes.byref(self.g)
        _lib.call("gr_tv_dual", _ptr(s.V), _ptr(s.Ubar), self.sigma, self.z, _dt(self.f), Nx, Ny,
                  self.Nz, self.of, st)
        _lib.call("gr_forward_lambda", gp, _ptr(s.L), _ptr(s.Ubar), _ptr(self.f), self.sigma_l,
                  self.mu2, self.Nz, self.of, st)
        _lib.call("gr_backward_tv_primal", gp, _ptr(s.U), _ptr(s.Ubar), _ptr(s.V), _ptr(s.L),
                  self.tau, self.norming, self.z, self.Nz, self.of, st)

    def adjoint_step(self, prev: _TVState, nxt: _TVState, adj: _TVState, tmp: _TVState, gf) -> None:
        """Map the adjoint of state k+1 (``adj``) to the adjoint of state k, in place.

        ``prev``/``nxt`` are the forward states k and k+1; ``tmp`` is scratch;
        ``gf`` accumulates the adjoint of the sinogram.
        """
        st = _stream_ptr(self.f.device)
        Nx, Ny = self.ps.img_shape
        n = adj.U.numel()
        gz, gu_prev = tmp.U, tmp.Ubar
        # U' = max(0, z), Ubar' = 2 U' - U
        _lib.call("gr_tv_adjoint_primal", _ptr(gz), _ptr(gu_prev), _ptr(adj.U), _ptr(adj.Ubar),
                  _ptr(nxt.U), _dt(self.f), n, st)
        # V' = P(V + sigma grad Ubar); z contains tau div V'
        _lib.call("gr_tv_adjoint_dual", _ptr(tmp.V), _ptr(adj.V), _ptr(gz), _ptr(prev.V),
                  _ptr(prev.Ubar), self.sigma, self.tau, self.z, _dt(self.f), Nx, Ny, self.Nz,
                  self.of, st)
        # z contains -tau n A* Lambda'  ->  gL1 = gL - tau n A*^T gz
        c3 = -float(self.tau) * float(self.norming) / self.ps.forward_scale(self.ndt)
        _lib.call("gr_forward_angle_axpy", ctypes.byref(self.g), _ptr(tmp.L), _ptr(adj.L), _ptr(gz),
                  _ptr(self.w), c3, self.Nz, self.of, st)
        # Lambda' = mu2 (Lambda + sigma_l (A Ubar - f)); the kernels apply the
        # two float32 factors one after the other, so the product stays unrounded
        _lib.call("gr_backward_tv_adjoint", ctypes.byref(self.ga), _ptr(adj.Ubar), _ptr(tmp.L),
                  _ptr(tmp.V), self.mu2 * self.sigma_l, self.sigma, self.z, self.Nz, self.of, st)
        _lib.call("gr_tv_adjoint_lambda", _ptr(adj.L), _ptr(gf), _ptr(tmp.L), self.mu2,
                  self.sigma_l, _dt(self.f), adj.L.numel(), st)
        adj.U.copy_(gu_prev)
        adj.V.copy_(tmp.V)


class _UnrolledTV(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f, ps, mu, iterations, checkpoint_every, slice_thickness,
                stepsize_weighting, norm_estimate, backward_iterations):
        f = _as_contiguous(f.detach())
        prob = _TVProblem(f, ps, mu, slice_thickness, stepsize_weighting, norm_estimate)
        k = max(1, int(checkpoint_every))
        # differentiate through the last `backward_iterations` iterations: the
        # state entering them is kept (the first checkpoint) and treated as
        # constant by the backward pass
        start = iterations - min(iterations, int(backward_iterations))
        state = prob.new_state()
        checkpoints = {}
        with torch.cuda.device(f.device):
            for i in range(iterations):
                if i == start:
                    checkpoints[i] = prob.new_state().copy_from(state)
                prob.step(state)
                if i + 1 > start and (i + 1 - start) % k == 0 and (i + 1) < iterations:
                    checkpoints[i + 1] = prob.new_state().copy_from(state)
            if start == iterations:
                checkpoints[start] = prob.new_state()
        ctx.prob, ctx.checkpoints, ctx.k, ctx.iterations = prob, checkpoints, k, iterations
        out = core.empty(prob.img_shape, f.dtype, prob.order, f.device)
        out.copy_(state.U)
        return out

    @staticmethod
    def backward(ctx, grad):
        prob, k, K = ctx.prob, ctx.k, ctx.iterations
        f = prob.f
        with torch.cuda.device(f.device):
            adj = prob.new_state()
            adj.U.copy_(grad)
            tmp = prob.new_state()
            gf = core.zeros(tuple(f.shape), f.dtype, prob.order, f.device)
            starts = sorted(ctx.checkpoints)
            for c in reversed(starts):
                stop = min(c + k, K)
                states = [prob.new_state().copy_from(ctx.checkpoints[c])]
                for _ in range(c, stop):
                    s = prob.new_state().copy_from(states[-1])
                    prob.step(s)
                    states.append(s)
                for j in range(stop - 1, c - 1, -1):
                    prob.adjoint_step(states[j - c], states[j - c + 1], adj, tmp, gf)
        return gf, None, None, None, None, None, None, None, None


def tv_unrolled(sino, projectionsetting, mu, number_iterations=20, checkpoint_every=5,
                slice_thickness=1.0, stepsize_weighting=10.0, norm_estimate=None,
                backward_iterations=None):
    """Differentiable ``number_iterations`` steps of gratopy's TV primal-dual method.

    Returns the primal iterate U (as :func:`gratopy_gb300.total_variation`
    does); gradients flow to ``sino``.  ``norm_estimate`` defaults to one
    :func:`gratopy_gb300.normest` call (not differentiated).
    ``backward_iterations`` (default: all) truncates the differentiation to
    the last that many iterations: the state entering them is kept as the
    first checkpoint and treated as constant, so memory and backward time
    scale with the truncated length; states are checkpointed every
    ``checkpoint_every`` iterations from there.
    """
    if norm_estimate is None:
        norm_estimate = core.normest(projectionsetting)
    last = int(number_iterations) if backward_iterations is None else int(backward_iterations)
    if last < 0:
        raise ValueError("backward_iterations must be non-negative")
    return _UnrolledTV.apply(sino, projectionsetting, float(mu), int(number_iterations),
                             int(checkpoint_every), float(slice_thickness),
                             float(stepsize_weighting), float(norm_estimate), last)
