"""Operator API: algebra of projection operators (gratopy/operator/__init__.py)."""

from .base import IDENTITY, ZERO, Operator, OperatorArithmeticOperation
from .kernels import CUDAKernelSpec
from .projection import Fanbeam, Radon

__all__ = ["IDENTITY", "ZERO", "Operator", "OperatorArithmeticOperation", "Radon", "Fanbeam",
           "CUDAKernelSpec"]
