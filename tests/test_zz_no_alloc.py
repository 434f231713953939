"""The allocation-free CG forward step agrees with the allocating one.

``gr_forward_wsq_noalloc`` exists for callers that cannot allocate device
memory where they run the CG forward step (inside a CUDA graph capture,
under another allocator's memory budget, or where cudaMalloc's implicit
synchronisation is not acceptable); it keeps its reduction partials in a
static device array of the library.  This file is collected last so that a
run stopping at the first failure has run every other test already; it also
passes on its own in a fresh process.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # same kernels and summation order: results agree to rounding noise


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("geometry", ["radon", "fan"])
@pytest.mark.parametrize("dtype_name", ["float32", "float64"])
def test_noalloc_matches_allocating_entry_point(cuda_device, geometry, dtype_name):
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import _lib

    if geometry == "radon":
        ps = gg.ProjectionSettings(cuda_device, gg.RADON, (96, 80), 60, n_detectors=128)
    else:
        ps = gg.ProjectionSettings(cuda_device, gg.FANBEAM, (96, 96), 72, n_detectors=140,
                                   detector_width=60.0, R=120.0, RE=50.0)
    tdt = getattr(torch, dtype_name)
    ndt = np.dtype(dtype_name)
    g = ps.gr_geometry(ndt)
    w = ps.device_tables(ndt)["w"]
    nz, order = 3, 0
    n_part = int(_lib.raw("gr_forward_partials")(ctypes.byref(g), nz))
    assert 0 < n_part <= 65536
    stream = ctypes.c_void_p(torch.cuda.current_stream(cuda_device).cuda_stream)
    gen = torch.Generator(device=cuda_device).manual_seed(11)

    for call in range(2):  # two calls in a row share the static scratch
        p = gg.core.empty(ps.img_shape + (nz,), tdt, "F", cuda_device)
        p.copy_(torch.rand(p.shape, generator=gen, device=cuda_device, dtype=tdt))
        q_ref = gg.core.empty(ps.sinogram_shape + (nz,), tdt, "F", cuda_device)
        partials = torch.empty(n_part, dtype=torch.float64, device=cuda_device)
        out_ref = torch.empty(1, dtype=torch.float64, device=cuda_device)
        _lib.call("gr_forward_wsq", ctypes.byref(g), _p(q_ref), _p(p), _p(w), _p(partials), None,
                  nz, order, stream)
        _lib.call("gr_sum_partials", _p(out_ref), _p(partials), n_part, stream)

        q_new = gg.core.empty(ps.sinogram_shape + (nz,), tdt, "F", cuda_device)
        out_new = torch.full((1,), float("nan"), dtype=torch.float64, device=cuda_device)
        _lib.call("gr_forward_wsq_noalloc", ctypes.byref(g), _p(q_new), _p(p), _p(w),
                  _p(out_new), nz, order, stream)
        torch.cuda.synchronize(cuda_device)
        assert torch.equal(q_new, q_ref), f"call {call}: projections differ"
        ref, new = float(out_ref.item()), float(out_new.item())
        assert abs(new - ref) <= REL_TOL * abs(ref), f"call {call}: {new} vs {ref}"


def test_noalloc_rejects_oversized_problem(cuda_device):
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import _lib

    ps = gg.ProjectionSettings(cuda_device, gg.RADON, (16, 16), 8, n_detectors=24)
    g = ps.gr_geometry(np.float32)
    big = _lib.GrGeometry.from_buffer_copy(g)
    big.Ns, big.Na = 8192, 8192  # 2^20+ partials: beyond the static array
    assert int(_lib.raw("gr_forward_partials")(ctypes.byref(big), 1)) > 65536
    buf = torch.zeros(16, device=cuda_device)
    out = torch.zeros(1, dtype=torch.float64, device=cuda_device)
    rc = _lib.raw("gr_forward_wsq_noalloc")(ctypes.byref(big), _p(buf), _p(buf), _p(buf), _p(out),
                                            1, 0, None)
    assert rc == 4  # GR_ERR_TOO_BIG, returned before any launch
    assert b"limit" in _lib.raw("gr_error_string")(rc)


@pytest.mark.parametrize("with_scratch", [True, False])
def test_noalloc_single_slice_quarter_turn_fan(cuda_device, with_scratch):
    """One slice of a quarter-turn symmetric fan geometry (square image centred
    on the axis, equispaced full-circle angles, a multiple of 4): the forward
    step runs the orbit kernel, whose block partials per slice follow its own
    grid.  With the descriptor's orbit-copy scratch bound (the copy kernel runs
    first) and without it (the orbit kernel gathers directly), two calls in a
    row match the allocating entry point."""
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import _lib

    ps = gg.ProjectionSettings(cuda_device, gg.FANBEAM, (128, 128), 360, n_detectors=192,
                               detector_width=400.0, R=400.0, RE=200.0)
    g = _lib.GrGeometry.from_buffer_copy(ps.gr_geometry(np.float32))
    assert g.sym == 4
    if not with_scratch:
        g.work, g.work_bytes = None, 0
    w = ps.device_tables(np.float32)["w"]
    n_part = int(_lib.raw("gr_forward_partials")(ctypes.byref(g), 1))
    assert 0 < n_part <= 65536
    stream = ctypes.c_void_p(torch.cuda.current_stream(cuda_device).cuda_stream)
    gen = torch.Generator(device=cuda_device).manual_seed(3)
    for call in range(2):
        p = gg.core.empty(ps.img_shape, torch.float32, "F", cuda_device)
        p.copy_(torch.rand(p.shape, generator=gen, device=cuda_device))
        q_ref = gg.core.empty(ps.sinogram_shape, torch.float32, "F", cuda_device)
        partials = torch.empty(n_part, dtype=torch.float64, device=cuda_device)
        out_ref = torch.empty(1, dtype=torch.float64, device=cuda_device)
        _lib.call("gr_forward_wsq", ctypes.byref(g), _p(q_ref), _p(p), _p(w), _p(partials), None,
                  1, 0, stream)
        _lib.call("gr_sum_partials", _p(out_ref), _p(partials), n_part, stream)
        q_new = gg.core.empty(ps.sinogram_shape, torch.float32, "F", cuda_device)
        out_new = torch.full((1,), float("nan"), dtype=torch.float64, device=cuda_device)
        _lib.call("gr_forward_wsq_noalloc", ctypes.byref(g), _p(q_new), _p(p), _p(w),
                  _p(out_new), 1, 0, stream)
        torch.cuda.synchronize(cuda_device)
        assert torch.equal(q_new, q_ref), f"call {call}: projections differ"
        ref, new = float(out_ref.item()), float(out_new.item())
        assert abs(new - ref) <= REL_TOL * abs(ref), f"call {call}: {new} vs {ref}"


def test_noalloc_rejects_invalid_sizes(cuda_device):
    """Sizes that describe no problem are a shape error, reported before the
    partial count is looked at and before any launch."""
    import torch

    import gratopy_gb300 as gg
    from gratopy_gb300 import _lib

    ps = gg.ProjectionSettings(cuda_device, gg.RADON, (16, 16), 8, n_detectors=24)
    buf = torch.zeros(16, device=cuda_device)
    out = torch.zeros(1, dtype=torch.float64, device=cuda_device)
    fn = _lib.raw("gr_forward_wsq_noalloc")
    for field, value in (("Ns", 0), ("Na", -3), ("Nx", 0)):
        bad = _lib.GrGeometry.from_buffer_copy(ps.gr_geometry(np.float32))
        setattr(bad, field, value)
        assert fn(ctypes.byref(bad), _p(buf), _p(buf), _p(buf), _p(out), 1, 0, None) == 2
    good = ps.gr_geometry(np.float32)
    assert fn(ctypes.byref(good), _p(buf), _p(buf), _p(buf), _p(out), 0, 0, None) == 2
