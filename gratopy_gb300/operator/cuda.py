"""Execution pipeline of device-backed operators.

Counterpart of gratopy's ``_OpenCLOperator`` (gratopy/operator/opencl.py:158-455):
infer the device, coerce NumPy input to a device tensor, validate the input
shape prefix, allocate (or validate) the output, invoke the projection
kernel and apply the operator's scalar.  ``queue`` arguments accept a
``torch.device``, a device string/index or a ``torch.cuda.Stream``.
"""

from __future__ import annotations

from typing import Any

import numpy as np
import torch

from .. import core
from .base import Operator


class _CUDAOperator(Operator):
    """Shared helpers of operators whose application is a CUDA kernel."""

    def __init__(self, *, name=None, kernel_spec=None, **operator_kwargs):
        from .kernels import CUDAKernelSpec

        super().__init__(name=name, **operator_kwargs)
        if kernel_spec is not None and not isinstance(kernel_spec, CUDAKernelSpec):
            raise TypeError("kernel_spec must be a CUDAKernelSpec (CUDA sources or a shared "
                            "library exporting <base_name>_forward/_backward)")
        self.kernel_spec = kernel_spec
        self._last_queue = None

    def __getstate__(self):
        state = self.__dict__.copy()
        state["_last_queue"] = None
        return state

    def _infer_queue(self, argument=None, output=None, queue=None):
        if queue is not None:
            self._last_queue = queue
            return queue
        if isinstance(argument, torch.Tensor) and argument.is_cuda:
            self._last_queue = argument.device
            return argument.device
        if isinstance(output, torch.Tensor) and output.is_cuda:
            self._last_queue = output.device
            return output.device
        if self._last_queue is not None:
            return self._last_queue
        raise ValueError(
            "No CUDA device available. Either pass an explicit queue (torch.device), provide "
            "a CUDA tensor as input, or provide an output tensor on a CUDA device."
        )

    @staticmethod
    def _coerce_argument(argument, queue) -> torch.Tensor:
        device = core._device_of(queue)
        if isinstance(argument, torch.Tensor):
            return argument if argument.device == device else argument.to(device)
        array = np.asarray(argument)
        if not array.flags["C_CONTIGUOUS"] and not array.flags["F_CONTIGUOUS"]:
            array = np.ascontiguousarray(array)
        if array.flags["C_CONTIGUOUS"]:
            return torch.from_numpy(array).to(device)
        # Fortran order: upload the reversed-axes C array, view it back
        axes = tuple(reversed(range(array.ndim)))
        return torch.from_numpy(np.ascontiguousarray(array.transpose(axes))).to(device).permute(axes)

    @staticmethod
    def _default_order(reference: torch.Tensor) -> str:
        return "C" if reference.is_contiguous() else "F"

    @staticmethod
    def _allocate_output(queue, shape, dtype, order="F", allocator=None) -> torch.Tensor:
        return core.zeros(shape, dtype, order, core._device_of(queue))

    def _expected_output_shape(self, argument_shape) -> tuple:
        if self.input_shape is None or self.output_shape is None:
            raise NotImplementedError(
                "Concrete operators must define _expected_output_shape() or "
                "set input_shape/output_shape appropriately."
            )
        return tuple(self.output_shape) + tuple(argument_shape[len(self.input_shape):])

    def _validate_argument(self, argument) -> None:
        if self.input_shape is None:
            return
        if tuple(argument.shape[0:len(self.input_shape)]) != tuple(self.input_shape):
            raise ValueError(
                f"Input shape mismatch: expected {self.input_shape}, got {tuple(argument.shape)}"
            )

    def _validate_output(self, output, argument):
        expected = self._expected_output_shape(argument.shape)
        if output.dtype != argument.dtype:
            raise ValueError(f"Output dtype mismatch: expected {argument.dtype}, got {output.dtype}")
        if tuple(output.shape) != tuple(expected):
            raise ValueError(f"Output shape mismatch: expected {expected}, got {tuple(output.shape)}")
        return output

    def _invoke(self, output, argument, queue):
        raise NotImplementedError

    def apply_to(self, argument: Any, output: Any = None, queue=None, return_event: bool = False,
                 **kwargs):
        queue = self._infer_queue(argument=argument, output=output, queue=queue)
        argument = self._coerce_argument(argument, queue)
        self._validate_argument(argument)
        if output is None:
            output = self._allocate_output(queue, self._expected_output_shape(argument.shape),
                                           argument.dtype, self._default_order(argument))
        output = self._validate_output(output, argument)
        event = self._invoke(output, argument, queue)
        if self.scalar != 1:
            output.mul_(float(self.scalar))
        if return_event:
            return output, [event]
        return output
