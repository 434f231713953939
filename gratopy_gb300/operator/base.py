"""Backend-independent operator algebra (gratopy/operator/base.py:15-359).

Operators support scalar multiples, sums (``+``, ``-``) and compositions
(``*``), track input/output shapes and apply right-to-left.  ``IDENTITY`` and
``ZERO`` are the neutral elements.  Semantics, ``repr`` strings and
exception types follow the reference.
"""

from __future__ import annotations

from copy import deepcopy
from enum import Enum
from numbers import Number
from typing import Any

import numpy as np


class OperatorArithmeticOperation(Enum):
    ADDITION = "sum"
    MULTIPLICATION = "prod"


def _compute_sum_shapes(operands):
    input_shape = None
    output_shape = None
    for op in operands:
        if op.input_shape is not None:
            if input_shape is not None and input_shape != op.input_shape:
                raise ValueError(
                    f"Input shape mismatch in sum: expected {input_shape}, "
                    f"but {op} has input shape {op.input_shape}"
                )
            input_shape = op.input_shape
        if op.output_shape is not None:
            if output_shape is not None and output_shape != op.output_shape:
                raise ValueError(
                    f"Output shape mismatch in sum: expected {output_shape}, "
                    f"but {op} has output shape {op.output_shape}"
                )
            output_shape = op.output_shape
    return input_shape, output_shape


def _compute_product_shapes(operands):
    for left, right in zip(operands[:-1], operands[1:]):
        if left.input_shape is not None and right.output_shape is not None:
            if left.input_shape != right.output_shape:
                raise ValueError(
                    f"Shape mismatch in composition: {left} expects input "
                    f"{left.input_shape}, but {right} produces {right.output_shape}"
                )
    return operands[-1].input_shape, operands[0].output_shape


class Operator:
    """Base class of all operators (leaf or composite)."""

    def __init__(self, name=None, scalar=1, state=None, arithmetic_operation=None,
                 operands=None, input_shape=None, output_shape=None):
        self.name = self.__class__.__name__ if name is None else name
        self.state = {} if state is None else state
        self._arithmetic_operation = arithmetic_operation
        self._operands = [] if operands is None else operands
        self._scalar = 1
        self.scalar = scalar
        self.input_shape = input_shape
        self.output_shape = output_shape

    # -- representation ---------------------------------------------------
    def _scalar_repr_(self) -> str:
        if self.scalar == 1:
            return ""
        text = repr(self.scalar)
        return f"({text})" if self.scalar < 0 else text

    def _composite_repr_(self) -> str:
        assert self.is_composite(), "This method is for composite operators only."
        sc = self._scalar_repr_()
        if self._arithmetic_operation == OperatorArithmeticOperation.ADDITION:
            body = " + ".join(repr(op) for op in self._operands)
            return f"{sc}*({body})" if sc else body
        if self._arithmetic_operation == OperatorArithmeticOperation.MULTIPLICATION:
            body = "*".join(f"({op!r})" if op.is_composite() else repr(op) for op in self._operands)
            return f"{sc}*{body}" if sc else body
        raise ValueError(f"Unknown arithmetic operation: {self._arithmetic_operation}")

    def _repr_name_(self) -> str:
        return self.name

    def __repr__(self) -> str:
        if self.is_composite():
            return self._composite_repr_()
        sc = self._scalar_repr_()
        name = self._repr_name_()
        return f"{sc}*{name}" if sc else name

    def __eq__(self, other: Any) -> bool:
        if not isinstance(other, Operator):
            return False
        return all([
            type(self) is type(other),
            self.name == other.name,
            self.scalar == other.scalar,
            self.state == other.state,
            self._arithmetic_operation == other._arithmetic_operation,
            self._operands == other._operands,
            self.input_shape == other.input_shape,
            self.output_shape == other.output_shape,
        ])

    __hash__ = None

    # -- scalar -------------------------------------------------------------
    @property
    def scalar(self):
        return self._scalar

    @scalar.setter
    def scalar(self, value):
        if self.is_composite():
            if self._arithmetic_operation == OperatorArithmeticOperation.ADDITION:
                for child in self._operands:
                    child.scalar = child.scalar * value
            elif self._arithmetic_operation == OperatorArithmeticOperation.MULTIPLICATION:
                self._operands[0].scalar = self._operands[0].scalar * value
        else:
            self._scalar = value

    # -- application -------------------------------------------------------
    def apply_to(self, argument: Any, output: Any = None, **kwargs: Any) -> Any:
        """Apply the operator; for products only the last factor writes ``output``."""
        if self.is_composite():
            if self._arithmetic_operation == OperatorArithmeticOperation.ADDITION:
                if output is None:
                    result = self._operands[0].apply_to(argument, **kwargs)
                else:
                    result = self._operands[0].apply_to(argument, output=output, **kwargs)
                for child in self._operands[1:]:
                    result += child.apply_to(argument, **kwargs)
                return result
            if self._arithmetic_operation == OperatorArithmeticOperation.MULTIPLICATION:
                result = argument
                order = list(reversed(self._operands))
                for idx, child in enumerate(order):
                    child_out = output if idx == len(order) - 1 else None
                    result = child.apply_to(result, output=child_out, **kwargs)
                return result
        raise NotImplementedError("apply_to needs to be implemented in specialized subclasses")

    def is_composite(self) -> bool:
        return self._arithmetic_operation is not None

    # -- algebra ---------------------------------------------------------------
    def __add__(self, other: "Operator") -> "Operator":
        if not isinstance(other, Operator):
            raise TypeError(f"Cannot add {type(other)} to {type(self)}")
        if isinstance(other, _ZeroOperator):
            return self
        operands = []
        for op in (deepcopy(self), deepcopy(other)):
            if op.is_composite() and op._arithmetic_operation == OperatorArithmeticOperation.ADDITION:
                for child in op._operands:
                    child.scalar *= op.scalar
                    operands.append(child)
            else:
                operands.append(op)
        ins, outs = _compute_sum_shapes(operands)
        return Operator(name=None, scalar=1, arithmetic_operation=OperatorArithmeticOperation.ADDITION,
                        operands=operands, input_shape=ins, output_shape=outs)

    def __neg__(self) -> "Operator":
        return self.__rmul__(-1)

    def __sub__(self, other: "Operator") -> "Operator":
        return self + (-other)

    def __rmul__(self, other) -> "Operator":
        if other == 0:
            return ZERO
        if other == 1:
            return self
        op = deepcopy(self)
        op.scalar = op.scalar * other
        return op

    def __mul__(self, other):
        if not isinstance(other, Operator):
            if isinstance(other, Number):
                return self.__rmul__(other)
            return self.apply_to(other)
        if isinstance(other, _ZeroOperator):
            return other
        if isinstance(other, _IdentityOperator):
            return self
        operands = []
        scalar = 1
        for op in (deepcopy(self), deepcopy(other)):
            if op.is_composite() and op._arithmetic_operation == OperatorArithmeticOperation.MULTIPLICATION:
                operands.extend(op._operands)
            else:
                scalar *= op.scalar
                op.scalar = 1
                operands.append(op)
        ins, outs = _compute_product_shapes(operands)
        return Operator(name=None, scalar=scalar,
                        arithmetic_operation=OperatorArithmeticOperation.MULTIPLICATION,
                        operands=operands, input_shape=ins, output_shape=outs)


class _IdentityOperator(Operator):
    def __mul__(self, other):
        if isinstance(other, Operator):
            return other
        return super().__mul__(other)

    def apply_to(self, argument, output=None, **kwargs):
        result = self.scalar * argument
        if output is not None:
            output[...] = result
            return output
        return result


class _ZeroOperator(Operator):
    def __add__(self, other):
        return other

    @property
    def scalar(self):
        return self._scalar

    @scalar.setter
    def scalar(self, value):
        pass

    def apply_to(self, argument, output=None, **kwargs):
        if output is not None:
            output[...] = 0
            return output
        try:
            return 0 * argument
        except TypeError:
            pass
        try:
            return np.zeros_like(argument)
        except (ValueError, TypeError):
            pass
        raise TypeError(f"Cannot apply zero operator to {type(argument)}")


IDENTITY = _IdentityOperator(name="[Id]")
ZERO = _ZeroOperator(name="[0]")
