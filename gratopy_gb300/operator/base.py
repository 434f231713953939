"""Operator algebra: expression trees of leaves, sums and compositions.

An expression is a tree.  A *leaf* is an operator with its own ``apply_to``
(a projection, the identity, the zero map) and is the only kind of node that
holds a scalar factor.  An *inner node* is the sum or the composition of its
children and has no factor of its own; scaling it moves the factor to where
factors live -- onto every term of a sum, onto the leftmost factor of a
composition (recursively, down to leaves).  ``A + B`` and ``A * B`` build
inner nodes through one function, :func:`_combine`, which flattens nested
sums of sums and compositions of compositions, pulls the factors of leaf
factors of a composition out and puts their product on its leftmost factor,
and infers the node's input and output shapes.  :meth:`Operator.apply_to`
evaluates a tree: a sum's first term writes ``output`` and the others are
added to it; a composition applies its factors right to left and only the
last one applied writes ``output``.

What callers can observe is gratopy's (gratopy/operator/base.py:15-359): the
printed form (``5*A + 5*[Id] + (-1)*B``, ``(5*A + 5*[Id])*C``), equality,
shape propagation, the ``ValueError`` / ``TypeError`` /
``NotImplementedError`` cases and their messages, ``IDENTITY`` and ``ZERO``,
and the ``_arithmetic_operation`` / ``_operands`` attributes gratopy's tests
inspect.
"""

from __future__ import annotations

from copy import deepcopy
from enum import Enum
from numbers import Number
from typing import Any

import numpy as np


class OperatorArithmeticOperation(Enum):
    """Kind of an inner node."""

    ADDITION = "sum"
    MULTIPLICATION = "prod"


_SUM = OperatorArithmeticOperation.ADDITION
_PROD = OperatorArithmeticOperation.MULTIPLICATION


def _joined_shapes(kind, parts):
    """(input_shape, output_shape) of the sum or composition of ``parts``.

    Unknown shapes (None) are compatible with anything.  A sum needs every
    known input shape and every known output shape to agree; a composition
    needs each factor's input to be the next factor's output (factors are
    listed left to right, applied right to left).
    """
    if kind is _PROD:
        for outer, inner in zip(parts, parts[1:]):
            if (outer.input_shape is not None and inner.output_shape is not None
                    and outer.input_shape != inner.output_shape):
                raise ValueError(f"Shape mismatch in composition: {outer} expects input "
                                 f"{outer.input_shape}, but {inner} produces {inner.output_shape}")
        return parts[-1].input_shape, parts[0].output_shape
    agreed = [None, None]
    for op in parts:
        for slot, (label, shape) in enumerate((("Input", op.input_shape),
                                               ("Output", op.output_shape))):
            if shape is None:
                continue
            if agreed[slot] is not None and agreed[slot] != shape:
                raise ValueError(f"{label} shape mismatch in sum: expected {agreed[slot]}, "
                                 f"but {op} has {label.lower()} shape {shape}")
            agreed[slot] = shape
    return agreed[0], agreed[1]


def _scale_in_place(op, factor) -> None:
    """Multiply the expression ``op`` by ``factor`` where its factors live."""
    if op._arithmetic_operation is _SUM:
        for term in op._operands:
            _scale_in_place(term, factor)
    elif op._arithmetic_operation is _PROD:
        _scale_in_place(op._operands[0], factor)
    else:
        op.scalar = op.scalar * factor  # leaves decide (the zero map ignores it)


def _combine(kind, left, right):
    """The inner node ``left + right`` or ``left * right`` (on copies)."""
    parts, pulled = [], 1
    for op in (deepcopy(left), deepcopy(right)):
        if op._arithmetic_operation is kind:
            parts.extend(op._operands)  # same kind: flatten
            continue
        if kind is _PROD and not op.is_composite():
            pulled *= op.scalar  # a leaf factor's scalar moves to the front
            op.scalar = 1
        parts.append(op)
    ins, outs = _joined_shapes(kind, parts)
    node = Operator(arithmetic_operation=kind, operands=parts, input_shape=ins, output_shape=outs)
    if kind is _PROD:
        # applied even when it equals 1: a float 1.0 turns integer factors into floats
        _scale_in_place(node, pulled)
    return node


def _factor_text(value) -> str:
    """Printed form of a leaf's factor: empty for 1, parenthesised when negative."""
    if value == 1:
        return ""
    text = repr(value)
    return f"({text})" if value < 0 else text


def _render(op) -> str:
    kind = op._arithmetic_operation
    if kind is _SUM:
        return " + ".join(_render(t) for t in op._operands)
    if kind is _PROD:
        return "*".join(f"({_render(t)})" if t.is_composite() else _render(t)
                        for t in op._operands)
    if kind is not None:
        raise ValueError(f"Unknown arithmetic operation: {kind}")
    factor = _factor_text(op.scalar)
    return f"{factor}*{op._repr_name_()}" if factor else op._repr_name_()


class Operator:
    """A leaf operator, or the sum / composition of ``operands``.

    Subclasses that compute something override :meth:`apply_to` for their
    leaves; inner nodes are plain ``Operator`` instances built by ``+``,
    ``-`` and ``*``.
    """

    def __init__(self, name=None, scalar=1, state=None, arithmetic_operation=None,
                 operands=None, input_shape=None, output_shape=None):
        self.name = type(self).__name__ if name is None else name
        self.state = {} if state is None else state
        self._arithmetic_operation = arithmetic_operation
        self._operands = list(operands) if operands is not None else []
        self._scalar = 1
        self.scalar = scalar
        self.input_shape = input_shape
        self.output_shape = output_shape

    # -- factor ---------------------------------------------------------------
    @property
    def scalar(self):
        """A leaf's factor; 1 for inner nodes, which hold none."""
        return self._scalar

    @scalar.setter
    def scalar(self, value):
        # On a leaf this sets the factor; on an inner node it multiplies the
        # expression by ``value`` (the factor moves to where factors live).
        if self.is_composite():
            _scale_in_place(self, value)
        else:
            self._scalar = value

    def is_composite(self) -> bool:
        return self._arithmetic_operation is not None

    # -- printed form and equality ----------------------------------------------
    def _repr_name_(self) -> str:
        return self.name

    def __repr__(self) -> str:
        return _render(self)

    def _signature(self):
        return (type(self), self.name, self.scalar, self.state, self._arithmetic_operation,
                self._operands, self.input_shape, self.output_shape)

    def __eq__(self, other: Any) -> bool:
        if not isinstance(other, Operator):
            return False
        mine, theirs = self._signature(), other._signature()
        return mine[0] is theirs[0] and all(a == b for a, b in zip(mine[1:], theirs[1:]))

    __hash__ = None

    # -- evaluation ----------------------------------------------------------------
    def apply_to(self, argument: Any, output: Any = None, **kwargs: Any) -> Any:
        """Evaluate the expression on ``argument``.

        A sum writes its first term into ``output`` (or a new array) and adds
        the others to it; a composition applies its factors right to left and
        only the last one applied writes ``output``.  Leaves without an
        implementation raise ``NotImplementedError``.
        """
        kind = self._arithmetic_operation
        if kind is _SUM:
            first, *rest = self._operands
            total = first.apply_to(argument, output=output, **kwargs)
            for term in rest:
                total += term.apply_to(argument, **kwargs)
            return total
        if kind is _PROD:
            value = argument
            factors = self._operands[::-1]
            for k, factor in enumerate(factors):
                value = factor.apply_to(value, output=output if k == len(factors) - 1 else None,
                                        **kwargs)
            return value
        raise NotImplementedError("apply_to needs to be implemented in specialized subclasses")

    # -- algebra ----------------------------------------------------------------------
    def __add__(self, other: "Operator") -> "Operator":
        if not isinstance(other, Operator):
            raise TypeError(f"Cannot add {type(other)} to {type(self)}")
        if isinstance(other, _ZeroOperator):
            return self
        return _combine(_SUM, self, other)

    def __neg__(self) -> "Operator":
        return self.__rmul__(-1)

    def __sub__(self, other: "Operator") -> "Operator":
        return self + (-other)

    def __rmul__(self, other) -> "Operator":
        if other == 0:
            return ZERO
        if other == 1:
            return self
        scaled = deepcopy(self)
        scaled.scalar = scaled.scalar * other
        return scaled

    def __mul__(self, other):
        if isinstance(other, Operator):
            if isinstance(other, _ZeroOperator):
                return other
            if isinstance(other, _IdentityOperator):
                return self
            return _combine(_PROD, self, other)
        if isinstance(other, Number):
            return self.__rmul__(other)
        return self.apply_to(other)  # ``A * x`` applies A to data


class _IdentityOperator(Operator):
    """``[Id]``: returns its argument times its factor."""

    def __mul__(self, other):
        if isinstance(other, Operator):
            return other
        return super().__mul__(other)

    def apply_to(self, argument, output=None, **kwargs):
        value = self.scalar * argument
        if output is None:
            return value
        output[...] = value
        return output


class _ZeroOperator(Operator):
    """``[0]``: the neutral element of sums; ignores factors."""

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
        # data that cannot be multiplied by 0 gets a zero array of its shape
        attempts = ((lambda a: 0 * a, (TypeError,)), (np.zeros_like, (TypeError, ValueError)))
        for make, tolerated in attempts:
            try:
                return make(argument)
            except tolerated:
                continue
        raise TypeError(f"Cannot apply zero operator to {type(argument)}")


IDENTITY = _IdentityOperator(name="[Id]")
ZERO = _ZeroOperator(name="[0]")
