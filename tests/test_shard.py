"""Sharding host logic on CPU: partitions, and the sharded CG / TV drivers run
on 2 and 3 gloo ranks with the float64 oracle as the per-rank backend,
against the oracle's single-process solvers on the whole stack.

The GPU backends (``KernelCG``, ``KernelTV``) run the same drivers; with one
rank they are checked against the per-call solvers in
``tests/test_gpu_shard.py``.
"""

from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from gratopy_gb300 import shard
from tests.helpers import host_settings

CFG = {
    "radon": dict(geometry="radon", img_shape=(24, 20), angles=18, n_detectors=32),
    "fan": dict(geometry="fanbeam", img_shape=(24, 24), angles=20, n_detectors=36,
                detector_width=40.0, R=70.0, RE=30.0),
}


def test_slice_ranges_cover_in_aligned_balanced_chunks():
    for nz in range(0, 70):
        for world in range(1, 6):
            r = shard.slice_ranges(nz, world)
            assert r[0][0] == 0 and r[-1][1] == nz
            assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
            sizes = [z1 - z0 for z0, z1 in r]
            # whole groups of 4 except the range holding the last slice
            assert all((z1 - z0) % 4 == 0 for z0, z1 in r if z1 < nz)
            groups = [-(-n // 4) for n in sizes]  # groups of 4 slices per rank
            assert max(groups) - min(groups) <= 1
    assert shard.slice_ranges(64, 3) == [(0, 24), (24, 44), (44, 64)]
    assert shard.slice_ranges(3, 2) == [(0, 3), (3, 3)]


def test_halo_ranges():
    h = shard.halo_ranges(6, 3, align=1)
    assert [(x.lo, x.hi, x.own0, x.own1) for x in h] == [(0, 3, 0, 2), (1, 5, 2, 4), (3, 6, 4, 6)]
    assert not h[0].ghost_below and h[0].ghost_above
    assert h[1].ghost_below and h[1].ghost_above
    with pytest.raises(ValueError):
        shard.halo_ranges(3, 2)


def test_partition_costs_is_deterministic_lpt():
    assert shard.partition_costs([5, 1, 4, 3, 3], 2) == [[0, 4], [1, 2, 3]]
    assert shard.partition_costs([], 3) == [[], [], []]
    costs = np.random.default_rng(0).uniform(1, 10, 64)
    parts = shard.partition_costs(costs, 4)
    assert sorted(i for p in parts for i in p) == list(range(64))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)


# ------------------------------------------------------------ oracle backends


class OracleCG:
    """CG steps on this rank's float64 slices with the oracle kernels."""

    def __init__(self, sino, ps):
        import torch

        from oracle import oracle as O

        self.O, self.ps, self.torch = O, ps, torch
        self.f = np.asfortranarray(sino)
        self.empty = self.f.shape[2] == 0
        dims = tuple(ps.img_shape) + (self.f.shape[2],)
        self.x = np.zeros(dims, order="F")
        self.c = ps.delta_x**2 / ps.delta_s

    def _t(self, *vals):
        return self.torch.tensor(vals, dtype=self.torch.float64)

    def init(self):
        if self.empty:
            return self._t(0.0, 0.0)
        O = self.O
        self.d = np.asfortranarray(self.f - O.forward(self.x, self.ps))
        self.p = O.backward(self.d, self.ps)
        return self._t(O.dot(self.p, self.p), O.dot(self.f, self.f))

    def set_init(self, t):
        self.sold, self.fsq = float(t[0]), float(t[1])

    def forward(self):
        if self.empty:
            return self._t(0.0)
        O = self.O
        self.q = O.forward(self.p, self.ps)
        qr = O.weight_sinogram(self.q, self.ps)
        return self._t(O.dot(qr, self.q))

    def alpha(self, t):
        self.a = np.float64(self.c * (self.sold / float(t[0])))

    def backward(self):
        if self.empty:
            return self._t(0.0, 0.0)
        O = self.O
        self.x += self.a * self.p
        self.d -= self.a * self.q
        self.snew = O.backward(self.d, self.ps)
        return self._t(O.dot(self.d, self.d), O.dot(self.snew, self.snew))

    def beta(self, t, epsilon):
        self.b = float(t[1]) / self.sold
        self.sold = float(t[1])
        self.res = np.sqrt(float(t[0]) / self.fsq)

    def update_p(self):
        if not self.empty:
            self.p = np.asfortranarray(self.b * self.p + self.snew)

    def stopped(self):
        return False

    def result(self):
        return self.x


class OracleTV:
    """TV steps on this rank's float64 slices plus ghosts with the oracle kernels
    (the step sequence of gratopy.py:2686-2717)."""

    def __init__(self, sino_ext, ps, mu, slice_thickness, norm, halo):
        import torch

        from oracle import oracle as O

        self.O, self.L, self.ps, self.torch = O, O.lib(), ps, torch
        self.f = np.asfortranarray(sino_ext)
        self.nz_local = self.f.shape[2]
        self.ghost_below, self.ghost_above = halo.ghost_below, halo.ghost_above
        Nx, Ny = ps.img_shape
        self.n = Nx * Ny
        dims = (Nx, Ny, self.nz_local)
        self.U = np.zeros(dims, order="F")
        self.U_ = np.zeros(dims, order="F")
        self.V = np.zeros(4 * self.n * self.nz_local)
        self.Lam = np.zeros(self.f.shape, order="F")
        sigma = 1.0 / np.sqrt(13) * 10.0
        tau = 1.0 / np.sqrt(13) / 10.0
        mu2 = mu * norm**2 * ps.delta_x
        mu2 = mu2 / (sigma + mu2)
        f32 = lambda v: float(np.float32(v))  # noqa: E731
        self.sigma, self.tau, self.z = f32(sigma), f32(tau), f32(slice_thickness)
        self.sigma_l, self.mu2, self.norming = f32(sigma / norm), f32(mu2), f32(1.0 / norm)

    def plane(self, name, k):
        t = self.torch.from_numpy
        if name == "ubar":
            return t(self.U_[:, :, k].T).T  # a (Nx, Ny) view of the plane
        return t(self.V[4 * self.n * k: 4 * self.n * (k + 1)])

    def _p(self, a):
        return self.O._ptr(a)

    def dual(self):
        Nx, Ny = self.ps.img_shape
        nt = self.O.threads()
        self.L.or_tv_update_v_f64(self._p(self.V), self._p(self.U_), self.sigma, self.z, Nx, Ny,
                                  self.nz_local, 0, nt)
        self.L.or_tv_normv_f64(self._p(self.V), self.n * self.nz_local, nt)

    def data_dual(self):
        KU = self.O.forward(self.U_, self.ps)
        self.L.or_tv_update_lambda_f64(self._p(self.Lam), self._p(KU), self._p(self.f),
                                       self.sigma_l, self.mu2, self.Lam.size, self.O.threads())

    def primal(self):
        Nx, Ny = self.ps.img_shape
        nt = self.O.threads()
        KST = self.O.backward(self.Lam, self.ps)
        self.L.or_tv_update_u_f64(self._p(self.U_), self._p(self.U), self._p(self.V),
                                  self._p(KST), self.tau, self.norming, self.z, Nx, Ny,
                                  self.nz_local, 0, nt)
        self.L.or_tv_extra_f64(self._p(self.U_), self._p(self.U), self.n * self.nz_local, nt)
        self.U, self.U_ = self.U_, self.U

    def result(self):
        lo = 1 if self.ghost_below else 0
        hi = self.nz_local - (1 if self.ghost_above else 0)
        return self.U[:, :, lo:hi]


# ---------------------------------------------------------------- gloo runs


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _stack(ps, nz, seed):
    from oracle import oracle as O
    from gratopy_gb300.phantom import random_ellipse_image

    Nx, Ny = ps.img_shape
    img = np.stack([random_ellipse_image(seed + k, (Ny, Nx), dtype="float64").T
                    for k in range(nz)], -1)
    img = np.asfortranarray(img)
    sino = O.forward(img, ps)
    rng = np.random.default_rng(seed)
    return np.asfortranarray(sino + 0.01 * rng.standard_normal(sino.shape))


def _worker(rank, world, port, outdir, kind, geom, nz, align, iters):
    import torch.distributed as dist

    os.environ["GR_ORACLE_THREADS"] = "1"
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        ps = host_settings(CFG[geom])
        sino = _stack(ps, nz, 7)
        if kind == "cg":
            z0, z1 = shard.slice_ranges(nz, world, align)[rank]
            out = shard.cg_sharded(OracleCG(sino[:, :, z0:z1], ps), iters)
        else:
            h = shard.halo_ranges(nz, world, align)[rank]
            be = OracleTV(sino[:, :, h.lo:h.hi], ps, 15.0, 1.0, 3.0, h)
            out = shard.tv_sharded(be, iters)
        np.save(os.path.join(outdir, f"r{rank}.npy"), np.asarray(out))
    finally:
        dist.destroy_process_group()


def _run(world, kind, geom, nz, align, iters, tmp_path):
    import torch.multiprocessing as mp

    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path), kind, geom, nz, align, iters),
             nprocs=world, join=True)
    return np.concatenate([np.load(tmp_path / f"r{k}.npy") for k in range(world)], axis=2)


@pytest.mark.parametrize("geom", ["radon", "fan"])
@pytest.mark.parametrize("world,nz,align", [(2, 5, 4), (2, 3, 4), (3, 6, 1)])
def test_cg_sharded_over_gloo_ranks_equals_whole_stack(tmp_path, geom, world, nz, align,
                                                       monkeypatch):
    from oracle import oracle as O

    monkeypatch.setenv("GR_ORACLE_THREADS", "1")
    got = _run(world, "cg", geom, nz, align, 6, tmp_path)
    ps = host_settings(CFG[geom])
    want = O.conjugate_gradients(_stack(ps, nz, 7), ps, 6)
    assert got.shape == want.shape
    assert np.linalg.norm(got - want) <= 1e-10 * np.linalg.norm(want)


@pytest.mark.parametrize("geom", ["radon", "fan"])
@pytest.mark.parametrize("world,nz,align", [(2, 5, 4), (3, 6, 1)])
def test_tv_sharded_with_ghost_slices_equals_whole_stack(tmp_path, geom, world, nz, align,
                                                        monkeypatch):
    from oracle import oracle as O

    monkeypatch.setenv("GR_ORACLE_THREADS", "1")
    got = _run(world, "tv", geom, nz, align, 8, tmp_path)
    ps = host_settings(CFG[geom])
    want = O.total_variation(_stack(ps, nz, 7), ps, 15.0, 8, slice_thickness=1.0,
                             norm_estimate=3.0)
    assert got.shape == want.shape
    assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want)
