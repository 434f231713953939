"""ctypes binding of the C ABI in ``include/gratopy_gb300.h``.

Loads the in-tree ``gratopy_gb300/_build/libgratopy_gb300.so``.  There is no
fallback: if the library is missing the import of any compute entry point
raises, so a GPU run can never silently take another path.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libgratopy_gb300.so"

GR_F32, GR_F64 = 0, 1
GR_ORDER_F, GR_ORDER_C = 0, 1
GR_RADON, GR_FANBEAM = 0, 1
GR_OK = 0
SC_SOLD, SC_ALPHA, SC_BETA, SC_DSQ, SC_FSQ, SC_RES, SC_SUM = range(7)
SC_COUNT = 8


class GrGeometry(ctypes.Structure):
    """Mirror of ``struct gr_geometry``."""

    _fields_ = [
        ("kind", ctypes.c_int),
        ("dtype", ctypes.c_int),
        ("Nx", ctypes.c_int),
        ("Ny", ctypes.c_int),
        ("Ns", ctypes.c_int),
        ("Na", ctypes.c_int),
        ("ofs", ctypes.c_void_p),
        ("sdpd", ctypes.c_void_p),
        ("geo", ctypes.c_double * 11),
        ("fwd_split", ctypes.c_int),
        ("bwd_split", ctypes.c_int),
        ("sym", ctypes.c_int),
        ("sym_map", (ctypes.c_int * 6) * 3),
        ("mirror", ctypes.c_int), ("mirror_pair", ctypes.c_int),
        ("mirror_map", ctypes.c_int * 6),
        ("work", ctypes.c_void_p),
        ("work_bytes", ctypes.c_size_t),
    ]


class GrBatchProblem(ctypes.Structure):
    """Mirror of ``struct gr_batch_problem``."""

    _fields_ = [
        ("kind", ctypes.c_int), ("Nx", ctypes.c_int), ("Ny", ctypes.c_int),
        ("Ns", ctypes.c_int), ("Na", ctypes.c_int), ("solver", ctypes.c_int),
        ("fwd_split", ctypes.c_int), ("fwd_tiles_x", ctypes.c_int),
        ("bwd_tiles_x", ctypes.c_int), ("bwd_tiles_y", ctypes.c_int),
        ("ofs", ctypes.c_void_p), ("sdpd", ctypes.c_void_p), ("w", ctypes.c_void_p),
        ("geo", ctypes.c_float * 8),
        ("f", ctypes.c_void_p), ("img", ctypes.c_void_p), ("s1", ctypes.c_void_p),
        ("s2", ctypes.c_void_p), ("i1", ctypes.c_void_p), ("i2", ctypes.c_void_p),
        ("v4", ctypes.c_void_p), ("sc", ctypes.c_void_p), ("fwd_part", ctypes.c_void_p),
        ("bwd_part", ctypes.c_void_p),
        ("a0", ctypes.c_float), ("a1", ctypes.c_float), ("a2", ctypes.c_float),
        ("a3", ctypes.c_float), ("a4", ctypes.c_float), ("cg_c", ctypes.c_double),
        ("orbit", ctypes.c_int), ("sym", ctypes.c_int), ("fwd_tiles_y", ctypes.c_int),
        ("obwd_tiles_x", ctypes.c_int), ("obwd_tiles_y", ctypes.c_int),
        ("sym_map", (ctypes.c_int * 6) * 3),
    ]


GR_SOLVER_LANDWEBER, GR_SOLVER_CG, GR_SOLVER_TV = 0, 1, 2
GR_BATCH_NORMEST, GR_BATCH_MAIN, GR_BATCH_CG_INIT = 0, 1, 2

_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_D = ctypes.c_double
_Z = ctypes.c_size_t
_G = ctypes.POINTER(GrGeometry)

# name -> (restype, argtypes); must match include/gratopy_gb300.h
SIGNATURES = {
    "gr_error_string": (ctypes.c_char_p, [_I]),
    "gr_last_cuda_error": (_I, []),
    "gr_version": (_I, []),
    "gr_source_hash": (ctypes.c_char_p, []),
    "gr_radon_fwd": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _P]),
    "gr_radon_bwd": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _P]),
    "gr_fan_fwd": (_I, [_P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _P]),
    "gr_fan_bwd": (_I, [_P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _P]),
    "gr_forward": (_I, [_G, _P, _P, _I, _I, _I, _P]),
    "gr_backward": (_I, [_G, _P, _P, _I, _I, _I, _P]),
    "gr_forward_residual": (_I, [_G, _P, _P, _P, _I, _I, _P]),
    "gr_backward_axpy": (_I, [_G, _P, _P, _D, _I, _I, _P]),
    "gr_forward_lambda": (_I, [_G, _P, _P, _P, _F, _F, _I, _I, _P]),
    "gr_backward_tv_primal": (_I, [_G, _P, _P, _P, _P, _F, _F, _F, _I, _I, _P]),
    "gr_forward_wsq": (_I, [_G, _P, _P, _P, _P, _P, _I, _I, _P]),
    "gr_backward_cg": (_I, [_G, _P, _P, _P, _P, _P, _P, _P, _I, _I, _P]),
    "gr_backward_sum": (_I, [_G, _P, _P, _P, _I, _I, _P]),
    "gr_forward_wsq_noalloc": (_I, [_G, _P, _P, _P, _P, _I, _I, _P]),
    "gr_forward_angle_axpy": (_I, [_G, _P, _P, _P, _P, _D, _I, _I, _P]),
    "gr_backward_tv_adjoint": (_I, [_G, _P, _P, _P, _D, _F, _F, _I, _I, _P]),
    "gr_tv_adjoint_primal": (_I, [_P, _P, _P, _P, _P, _I, _Z, _P]),
    "gr_tv_adjoint_dual": (_I, [_P, _P, _P, _P, _P, _F, _F, _F, _I, _I, _I, _I, _I, _P]),
    "gr_tv_adjoint_lambda": (_I, [_P, _P, _P, _F, _F, _I, _Z, _P]),
    "gr_ellipses": (_I, [_P, _P, _I, _I, _I, _I, _I, _I, _P]),
    "gr_probe_l1_bandwidth": (_I, [_P, _P, _I, _I, _I, _P]),
    "gr_sparse_entries": (_I, [_G, _P, _P, _P, _I, _P]),
    "gr_batch_problem_size": (_Z, []),
    "gr_batch_forward": (_I, [_P, _P, _I, _I, _I, _P]),
    "gr_batch_backward": (_I, [_P, _P, _I, _I, _I, _P]),
    "gr_batch_forward_orbit": (_I, [_P, _P, _I, _I, _I, _I, _P]),
    "gr_batch_backward_orbit": (_I, [_P, _P, _I, _I, _I, _I, _P]),
    "gr_batch_image_step": (_I, [_P, _P, _I, _I, _I, _P]),
    "gr_batch_sino_step": (_I, [_P, _P, _I, _I, _I, _P]),
    "gr_batch_scalars": (_I, [_P, _P, _I, _I, _I, _P]),
    "gr_forward_partials": (_Z, [_G, _I]),
    "gr_work_bytes": (_Z, [_G, _I]),
    "gr_orbit_kinds": (_I, [_G, _I]),
    "gr_geometry_size": (_Z, []),
    "gr_backward_partials": (_Z, [_G, _I, _I]),
    "gr_weight_sinogram": (_I, [_P, _P, _P, _I, _I, _I, _I, _I, _I, _P]),
    "gr_equ_mul_add": (_I, [_P, _D, _P, _I, _Z, _P]),
    "gr_mul_add_add": (_I, [_P, _D, _P, _P, _I, _Z, _P]),
    "gr_dot_partials_count": (_Z, []),
    "gr_dot_partials": (_I, [_P, _P, _P, _I, _Z, _P]),
    "gr_sum_partials": (_I, [_P, _P, _Z, _P]),
    "gr_sum_values_partials": (_I, [_P, _P, _I, _Z, _P]),
    "gr_tv_dual": (_I, [_P, _P, _F, _F, _I, _I, _I, _I, _I, _P]),
    "gr_cg_alpha": (_I, [_P, _P, _Z, _D, _I, _P, _P]),
    "gr_cg_update_d": (_I, [_P, _P, _P, _P, _I, _Z, _P, _P]),
    "gr_cg_beta": (_I, [_P, _P, _Z, _P, _Z, _D, _I, _P, _P]),
    "gr_cg_update_p": (_I, [_P, _P, _P, _I, _Z, _P, _P]),
    "gr_scale_by_sum": (_I, [_P, _P, _I, _Z, _P]),
}

_lib = None


class GratopyCudaError(RuntimeError):
    """A C-ABI call returned an error code."""


def load():
    """Load the extension (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"gratopy_gb300 CUDA extension not built ({LIB_PATH} missing); "
                "run `python -m gratopy_gb300.build` (or __graft_entry__.build())"
            )
        lib = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        from .build import source_hash

        built, current = lib.gr_source_hash().decode(), source_hash()
        if built != current:
            raise ImportError(
                f"{LIB_PATH} was built from other sources (library {built[:16]}, sources "
                f"{current[:16]}); rebuild with `python -m gratopy_gb300.build`")
        _lib = lib
    return _lib


def call(name: str, *args) -> None:
    """Call a status-returning entry point and raise on a nonzero code."""
    rc = getattr(load(), name)(*args)
    if rc != GR_OK:
        lib = load()
        msg = lib.gr_error_string(rc).decode()
        cuda = lib.gr_last_cuda_error()
        raise GratopyCudaError(f"{name} failed: {msg} (code {rc}, cudaError {cuda})")


def raw(name: str):
    return getattr(load(), name)
