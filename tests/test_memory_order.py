"""Memory-order detection of the Python layer (CPU): ``order_of`` tells C
from Fortran order by strides, as gratopy's ``flags.c_contiguous`` /
``flags.f_contiguous`` checks do, on every shape and layout the API meets."""

from __future__ import annotations

import itertools

import pytest
import torch

from gratopy_gb300.core import order_of


def _fortran(shape):
    return torch.empty(tuple(reversed(shape))).permute(*reversed(range(len(shape))))


SHAPES = [(4, 5), (4, 5, 3), (1, 5), (4, 1), (4, 1, 3), (1, 1, 1), (3,), (2, 3, 1), (1, 3, 4)]


@pytest.mark.parametrize("shape", SHAPES)
def test_c_and_fortran_orders(shape):
    assert order_of(torch.empty(shape)) == "C"
    f = _fortran(shape)
    # C is checked first (as gratopy does): arrays that are both report C
    assert order_of(f) == ("C" if f.is_contiguous() else "F")


def test_slices_of_fortran_stacks_are_fortran():
    stack = _fortran((6, 5, 4))
    assert order_of(stack[:, :, 2]) == "F"


@pytest.mark.parametrize("perm", [p for p in itertools.permutations(range(3)) if p not in
                                  ((0, 1, 2), (2, 1, 0))])
def test_other_layouts_are_rejected(perm):
    t = torch.empty(4, 5, 6).permute(*perm)
    with pytest.raises(ValueError):
        order_of(t)


def test_strided_views_are_rejected():
    with pytest.raises(ValueError):
        order_of(torch.empty(8, 6)[::2])
    with pytest.raises(ValueError):
        order_of(_fortran((8, 6))[::2])
