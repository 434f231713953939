"""The C-ABI library loads and exports every entry point the header declares.

CPU only: loading the library initialises no CUDA context, and no compute
entry point is called.
"""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "gratopy_gb300.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    return re.findall(r"^GR_API\s+[\w\s\*]*?\b(gr_\w+)\s*\(", text, flags=re.M)


@pytest.fixture(scope="module")
def library():
    from gratopy_gb300 import build

    return ctypes.CDLL(str(build.build()))


def test_header_declares_entry_points():
    names = declared_functions()
    assert len(names) >= 30
    assert len(set(names)) == len(names)
    for required in ("gr_radon_fwd", "gr_radon_bwd", "gr_fan_fwd", "gr_fan_bwd", "gr_forward",
                     "gr_backward", "gr_tv_dual", "gr_dot_partials"):
        assert required in names


def test_library_exports_every_declared_symbol(library):
    missing = [n for n in declared_functions() if not hasattr(library, n)]
    assert not missing, f"not exported: {missing}"


def test_binding_covers_header():
    from gratopy_gb300 import _lib

    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_host_only_entry_points(library):
    from gratopy_gb300 import _lib

    lib = _lib.load()
    assert lib.gr_version() == 1
    from gratopy_gb300 import build

    assert lib.gr_source_hash().decode() == build.source_hash()
    assert lib.gr_error_string(0) == b"success"
    assert b"geometry" in lib.gr_error_string(1)
    assert lib.gr_dot_partials_count() > 0
    # argument validation happens before any CUDA call
    g = _lib.GrGeometry()
    g.kind = 7
    assert lib.gr_forward(ctypes.byref(g), None, None, 1, 0, 0, None) == 1
    assert lib.gr_radon_fwd(None, None, None, None, 0, 1, 1, 1, 0, 0, None) == 1
    # quarter-turn maps are checked before the angle-count limit, so a
    # geometry with 70000 angles is rejected either way (1: bad maps, 4: too
    # many angles) and nothing reaches a launch
    fake = ctypes.c_void_p(64)
    q = _lib.GrGeometry()
    q.kind, q.dtype, q.Nx, q.Ny, q.Ns, q.Na = 1, 0, 8, 8, 4, 70000
    q.ofs, q.sdpd = fake, fake
    turn = [(0, -1, 1, 0, 7, 0), (-1, 0, 0, -1, 7, 7), (0, 1, -1, 0, 0, 7)]

    def set_maps(sym, maps):
        q.sym = sym
        for m, row in enumerate(maps):
            for k, v in enumerate(row):
                q.sym_map[m][k] = v

    def forward_rc(sym, maps):
        assert q.Na > 65535  # never a launch: every case is rejected
        set_maps(sym, maps)
        return lib.gr_forward(ctypes.byref(q), fake, fake, 1, 0, 0, None)

    assert forward_rc(4, turn) == 4
    assert forward_rc(0, [(0,) * 6] * 3) == 4
    assert forward_rc(3, turn) == 1
    assert forward_rc(4, [turn[0], turn[1], (0, 1, -1, 0, 0, 8)]) == 1  # leaves the grid
    assert forward_rc(4, [turn[0], (1, 1, 0, -1, 0, 7), turn[2]]) == 1  # not a permutation
    q.Ny = 9
    assert forward_rc(4, turn) == 1  # not square
    # scratch of the orbit kernels (float32 single slices): the forward's
    # float4 per pixel (from 16 Mi pixel-angles per projection), the
    # backprojection's float4 per base angle and bin (even sides with cyclic
    # maps, from 12 Mi pixel-angles); the larger of the two
    work = lib.gr_work_bytes

    def sized(N, Ns, Na, maps=None):
        q.Nx = q.Ny = N
        q.Ns, q.Na = Ns, Na
        c = N - 1
        set_maps(4, maps or [(0, -1, 1, 0, c, 0), (-1, 0, 0, -1, c, c), (0, 1, -1, 0, 0, c)])
        return work(ctypes.byref(q), 1)

    # (the row copy pads every base angle's row with 1 + 2 zero entries and
    # holds a 4-float4 geometry record per base angle)
    assert sized(512, 768, 360) == max(512 * 512 * 16, 90 * (768 + 3 + 4) * 16)
    assert sized(512, 4000, 400) == 100 * (4000 + 3 + 4) * 16
    assert sized(256, 384, 360) == 256 * 256 * 16  # both copies, the forward's the larger
    assert sized(192, 288, 360) == 90 * (288 + 3 + 4) * 16  # the backprojection's only
    assert sized(128, 192, 360) == 0
    # stacks (from 256 * 2^20 pixel-angles per slice): one slice's copy per
    # slice, up to 8 slices per launch pair; smaller slices keep the
    # per-angle kernels
    sized(1024, 1536, 720)
    assert work(ctypes.byref(q), 3) == 3 * 1024 * 1024 * 16
    assert work(ctypes.byref(q), 20) == 8 * 1024 * 1024 * 16
    sized(512, 768, 360)
    assert work(ctypes.byref(q), 3) == 0
    assert lib.gr_orbit_kinds(ctypes.byref(q), 3) == 0  # (no scratch bound in q)
    q.dtype = 1
    assert work(ctypes.byref(q), 1) == 0
    assert lib.gr_orbit_kinds(ctypes.byref(q), 1) == 0  # float64: per-angle kernels
    q.dtype = 0
    assert lib.gr_orbit_kinds(ctypes.byref(q), 1) == 3
    c = 511  # valid maps, not the powers of one quarter turn: the forward's only
    assert sized(512, 768, 360, [(-1, 0, 0, -1, c, c), (0, -1, 1, 0, c, 0),
                                 (0, 1, -1, 0, 0, c)]) == 512 * 512 * 16
    set_maps(0, [(0,) * 6] * 3)
    assert work(ctypes.byref(q), 1) == 0
    # block-partial counts of the fused reductions follow the orbit grids:
    # the forward runs 2 * fwd_split lanes per group of 4 bins in 128-thread
    # blocks over Na/4 base angles, one slice per launch; the backprojection
    # 32 x (8 / bwd_split) tiles of the quadrant, one slice per block
    fwd_parts, bwd_parts = lib.gr_forward_partials, lib.gr_backward_partials
    sized(512, 768, 360)
    cases = {(8, 8): (24 * 90, 8 * 256), (4, 2): (12 * 90, 8 * 64), (1, 1): (3 * 90, 8 * 32)}
    for (fs, bs), (want_f, want_b) in cases.items():
        q.fwd_split, q.bwd_split = fs, bs
        assert fwd_parts(ctypes.byref(q), 1) == want_f
        assert bwd_parts(ctypes.byref(q), 1, 0) == want_b
    # the fan-beam mirror: a reflection with an angle pairing, validated
    # with the geometry (gr_work_bytes is 0 for an invalid descriptor); the
    # mirrored forward walks half the bins with twice the lanes, so its
    # block count equals the quarter-turn forward's
    sized(512, 768, 360)
    q.fwd_split = 8
    plain_need, plain_parts = work(ctypes.byref(q), 1), fwd_parts(ctypes.byref(q), 1)
    q.mirror, q.mirror_pair = 1, 180
    for k, v in enumerate((-1, 0, 0, 1, 511, 0)):
        q.mirror_map[k] = v
    assert work(ctypes.byref(q), 1) == plain_need
    q.work, q.work_bytes = ctypes.c_void_p(1 << 20), plain_need
    assert fwd_parts(ctypes.byref(q), 1) == plain_parts == 48 * 90 // 2
    q.mirror_pair = 360  # out of range
    assert work(ctypes.byref(q), 1) == 0
    q.mirror_pair = 180
    q.mirror_map[0], q.mirror_map[3] = -1, -1  # a half turn, not a reflection
    assert work(ctypes.byref(q), 1) == 0
    q.mirror_map[3] = 1
    q.mirror_pair = -1  # no pairing
    assert work(ctypes.byref(q), 1) == 0
    q.sym, q.mirror_pair = 0, 360  # without the quarter-turn maps the mirror is ignored
    assert lib.gr_orbit_kinds(ctypes.byref(q), 1) == 0
    q.sym = 4
    q.mirror = 0
    q.work, q.work_bytes = None, 0
    sized(1024, 1536, 720)  # a stack whose slices take the orbit kernels
    q.fwd_split, q.bwd_split = 8, 8
    assert fwd_parts(ctypes.byref(q), 3) == 48 * 180 * 3
    assert bwd_parts(ctypes.byref(q), 3, 0) == 16 * 512 * 3
    q.fwd_split = q.bwd_split = 0
    assert lib.gr_forward_partials(None, 1) == 0
    # parallel beam with the half-circle orbit maps (sym = 2): accepted for
    # Radon only; the orbit kernels run when the scratch holds their copies
    # (the forward's float4 per pixel, the backprojection's mirror-interleaved
    # rows: Ns + 3 float4 per base angle), with grids over the bins
    # s < ceil(Ns/2) and base angles k < Na/2 (two per block, 4 * fwd_split
    # lanes per group) for the forward and over the quadrant for the
    # backprojection
    r = _lib.GrGeometry()
    r.kind, r.dtype, r.Nx, r.Ny, r.Ns, r.Na = 0, 0, 256, 256, 363, 180
    r.ofs = fake
    r.sym = 2
    for m, row in enumerate([(0, -1, 1, 0, 255, 0), (-1, 0, 0, -1, 255, 255),
                             (0, 1, -1, 0, 0, 255)]):
        for k, v in enumerate(row):
            r.sym_map[m][k] = v
    kinds = lib.gr_orbit_kinds
    assert kinds(ctypes.byref(r), 1) == 3  # forward and backprojection over orbits
    assert kinds(ctypes.byref(r), 2) == 0  # a stack of small slices: per-angle kernels
    assert kinds(None, 1) == 0 and kinds(ctypes.byref(r), 0) == 0
    need = work(ctypes.byref(r), 1)
    assert need == max(256 * 256 * 16, 90 * (363 + 3) * 16)
    assert work(ctypes.byref(r), 2) == 0  # stacks of slices below 32 * 2^20 pixel-angles
    r.fwd_split, r.bwd_split = 8, 8
    # the orbit kernels with or without their copies (without, they gather
    # the orbit members from the image and the sinogram): the forward 32
    # lanes per group, the backprojection 32 x 1 quadrant tiles
    orbit_fwd, orbit_bwd = -(-182 // 8) * 45, 4 * 128
    assert fwd_parts(ctypes.byref(r), 1) == orbit_fwd
    assert bwd_parts(ctypes.byref(r), 1, 0) == orbit_bwd
    r.work, r.work_bytes = ctypes.c_void_p(1 << 20), need
    assert fwd_parts(ctypes.byref(r), 1) == orbit_fwd
    assert bwd_parts(ctypes.byref(r), 1, 0) == orbit_bwd
    r.work_bytes = 90 * (363 + 3) * 16 - 16  # too small for the backprojection's copy
    assert bwd_parts(ctypes.byref(r), 1, 0) == orbit_bwd
    r.sym = 0
    assert fwd_parts(ctypes.byref(r), 1) == -(-363 // 32) * 180  # per-angle, 16 lanes per group
    assert bwd_parts(ctypes.byref(r), 1, 0) == 8 * 256  # per-angle 32 x 1 pixel tiles
    r.sym = 2
    # below 4 * 2^20 pixel-angles both gather without copies
    r.Nx = r.Ny = 128
    r.Ns, r.Na = 182, 90
    for m, row in enumerate([(0, -1, 1, 0, 127, 0), (-1, 0, 0, -1, 127, 127),
                             (0, 1, -1, 0, 0, 127)]):
        for k, v in enumerate(row):
            r.sym_map[m][k] = v
    assert work(ctypes.byref(r), 1) == 0
    assert kinds(ctypes.byref(r), 1) == 3
    r.Nx = r.Ny = 127  # odd side: the forward only
    for m, row in enumerate([(0, -1, 1, 0, 126, 0), (-1, 0, 0, -1, 126, 126),
                             (0, 1, -1, 0, 0, 126)]):
        for k, v in enumerate(row):
            r.sym_map[m][k] = v
    assert kinds(ctypes.byref(r), 1) == 1
    r.sym = 0
    assert kinds(ctypes.byref(r), 1) == 0
    r.sym = 2
    # stacks of larger slices: the orbit forward slice by slice (one slice's
    # copy per slice, up to 8 per launch pair), the per-angle backprojection
    r.Nx = r.Ny = 512
    r.Ns, r.Na = 725, 360
    for m, row in enumerate([(0, -1, 1, 0, 511, 0), (-1, 0, 0, -1, 511, 511),
                             (0, 1, -1, 0, 0, 511)]):
        for k, v in enumerate(row):
            r.sym_map[m][k] = v
    assert work(ctypes.byref(r), 3) == 3 * 512 * 512 * 16
    assert work(ctypes.byref(r), 20) == 8 * 512 * 512 * 16
    r.work_bytes = 512 * 512 * 16
    assert fwd_parts(ctypes.byref(r), 3) == -(-363 // 8) * 90 * 3
    per_angle_bwd = bwd_parts(ctypes.byref(r), 3, 0)
    r.sym = 0
    assert bwd_parts(ctypes.byref(r), 3, 0) == per_angle_bwd
    r.sym = 2
    r.kind, r.sdpd = 1, fake  # sym = 2 is for parallel beam only
    assert lib.gr_forward(ctypes.byref(r), fake, fake, 1, 0, 0, None) == 1
    # descriptors: binding layouts equal the library's
    assert lib.gr_geometry_size() == ctypes.sizeof(_lib.GrGeometry)
    assert lib.gr_batch_problem_size() == ctypes.sizeof(_lib.GrBatchProblem)
    assert lib.gr_batch_forward(None, None, 1, 0, 1, None) == 1
    assert lib.gr_batch_scalars(None, None, 1, 0, 1, None) == 1
