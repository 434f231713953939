"""gratopy_gb300: gratopy's projection toolbox on GB300 (sm_103a) CUDA kernels.

Exports the same public names as gratopy (``gratopy/__init__.py:21-47``);
arrays are torch CUDA tensors instead of pyopencl arrays.
"""

from ._version import __version__
from .core import (
    FAN,
    FANBEAM,
    PARALLEL,
    RADON,
    ProjectionSettings,
    backprojection,
    check_compatibility,
    conjugate_gradients,
    create_code,
    equ_mul_add,
    fanbeam,
    fanbeam_ad,
    forwardprojection,
    landweber,
    mul_add_add,
    normest,
    radon,
    radon_ad,
    total_variation,
    weight_sinogram,
)
from .geometry import fanbeam_struct, radon_struct, read_angles
from .phantom import ct_shepp_logan as phantom, easy_phantom
from . import operator  # noqa: E402

VERSION = __version__
