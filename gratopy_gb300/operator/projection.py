"""Projection operators: :class:`Radon` and :class:`Fanbeam`.

:class:`Radon` mirrors gratopy's experimental ``gratopy/operator/projection.py``
(lines 58-396): image domain / angles / detectors descriptions, extent
placeholders, ``.T`` for the adjoint and the operator algebra of
:mod:`.base`.  :class:`Fanbeam` is a working fan-beam counterpart of the
reference's stub (projection.py:399-413), built on the same fan kernels as
the legacy API.
"""

from __future__ import annotations

from copy import copy

import numpy as np

from .. import core
from ..utilities import (
    Angles,
    Detectors,
    ExtentPlaceholder,
    ImageDomain,
    full_detector_given_image_halfcircle,
    full_image_given_detector_halfcircle,
    valid_detector_given_image_halfcircle,
    valid_image_given_detector_halfcircle,
)
from .cuda import _CUDAOperator


class _ProjectionOperator(_CUDAOperator):
    """Shared state handling of the two projection operators."""

    def __getstate__(self):
        state = super().__getstate__()
        state["_settings"] = {}
        state["projection_settings"] = None
        return state

    @property
    def image_domain(self) -> ImageDomain:
        return self.state["image_domain"]

    @property
    def angles(self) -> Angles:
        return self.state["angles"]

    @property
    def detectors(self) -> Detectors:
        return self.state["detectors"]

    @property
    def adjoint(self) -> bool:
        return self.state["adjoint"]

    @property
    def T(self):
        op = copy(self)
        op.state = copy(self.state)
        op.state["adjoint"] = not self.state["adjoint"]
        op.input_shape, op.output_shape = op.output_shape, op.input_shape
        return op

    def _set_shapes(self):
        image_shape = tuple(self.image_domain.size)
        sinogram_shape = (self.detectors.number, len(self.angles))
        if self.adjoint:
            self.input_shape, self.output_shape = sinogram_shape, image_shape
        else:
            self.input_shape, self.output_shape = image_shape, sinogram_shape

    def _settings_for(self, queue) -> core.ProjectionSettings:
        """Device tables for ``queue``'s device, built once per device."""
        dev = core._device_of(queue)
        ps = self._settings.get(dev)
        if ps is None:
            ps = self._make_settings(dev)
            self._settings[dev] = ps
        return ps

    def _invoke(self, output, argument, queue):
        ps = self._settings_for(queue)
        self.projection_settings = ps
        if self.kernel_spec is not None:
            return self._invoke_custom(ps, output, argument)
        if self.adjoint:
            return ps.backprojection(output, argument, ps)
        return ps.forwardprojection(output, argument, ps)

    def _invoke_custom(self, ps, output, argument):
        """Run the operator's custom kernel bundle with the gr_forward/gr_backward ABI."""
        import ctypes

        import torch

        from .. import _lib

        if self.adjoint:
            core.check_compatibility(output, argument, ps)
        else:
            core.check_compatibility(argument, output, ps)
        forward, backward = self.kernel_spec.functions()
        fn = backward if self.adjoint else forward
        g = ps.gr_geometry(core._np_dtype(argument.dtype))
        dev = argument.device
        with torch.cuda.device(dev):
            rc = fn(ctypes.byref(g), output.data_ptr(), argument.data_ptr(), core._nz(argument),
                    core._oflag(core.order_of(output)), core._oflag(core.order_of(argument)),
                    core._stream_ptr(dev))
        if rc != _lib.GR_OK:
            raise RuntimeError(f"kernel bundle {self.kernel_spec.base_name!r} returned {rc}")
        return core._event(dev)


class Radon(_ProjectionOperator):
    """Parallel-beam Radon transform operator (``R``) or its adjoint (``R.T``).

    ``image_domain``: int, ``(Nx, Ny)`` or :class:`ImageDomain` (extent 2.0
    by default); ``angles``: int (uniform on the half circle) or
    :class:`Angles`; ``detectors``: None (``ceil(hypot(Nx, Ny))`` pixels),
    an int, or :class:`Detectors`.  An image or detector extent may be an
    :class:`ExtentPlaceholder`; exactly one may be.
    """

    def __init__(self, image_domain, angles, detectors=None, adjoint=False, kernel_spec=None):
        if not isinstance(image_domain, ImageDomain):
            image_domain = ImageDomain(size=image_domain, extent=2.0)
        if not isinstance(angles, Angles):
            angles = Angles.uniform(number=angles, half_circle=True)
        if not isinstance(detectors, Detectors):
            if detectors is None:
                detectors = int(np.ceil(np.hypot(*image_domain.size)))
            extent = image_domain.extent
            if isinstance(extent, ExtentPlaceholder):
                extent = ExtentPlaceholder.FULL
            detectors = Detectors(number=detectors, extent=extent)
        state = {"image_domain": image_domain, "angles": angles, "detectors": detectors,
                 "adjoint": adjoint}
        super().__init__(name="Radon", state=state, kernel_spec=kernel_spec)
        self.substitute_placeholder()
        self._settings = {}
        self.projection_settings = None
        self._set_shapes()

    def _repr_name_(self) -> str:
        return "Radon.T" if self.adjoint else "Radon"

    def substitute_placeholder(self) -> None:
        """Resolve a FULL/VALID extent placeholder (projection.py:235-318)."""
        img, det = self.image_domain, self.detectors
        if isinstance(img.extent, ExtentPlaceholder) and isinstance(det.extent, ExtentPlaceholder):
            raise NotImplementedError(
                "Both the ImageDomain and Detectors use an ExtentPlaceholder. "
                "Please set at least one of the two extents to a specific "
                "value; the remaining placeholder will be resolved "
                "automatically."
            )
        if isinstance(img.extent, ExtentPlaceholder):
            Mx, My = img.center
            Md = det.center
            Nx, Ny = img.size
            c = Nx / Ny
            Dd = float(det.extent)
            M = (Md, Mx, My)
            if img.extent == ExtentPlaceholder.FULL:
                result = full_image_given_detector_halfcircle(M, Dd, c)
                meaning = ("FULL means the largest image extent such that every "
                           "ray through the image also hits the detector")
            else:
                result = valid_image_given_detector_halfcircle(M, Dd, c)
                meaning = ("VALID means the smallest image extent such that "
                           "every ray hitting the detector also passes through "
                           "the image")
            if result is None:
                raise ValueError(
                    f"Cannot resolve ExtentPlaceholder.{img.extent.name} "
                    f"for the image domain ({meaning}): no such image extent "
                    f"exists with the given detector width Dd={Dd}, detector "
                    f"center Md={Md}, and image center ({Mx}, {My}). "
                    f"Consider increasing the detector width or adjusting the "
                    f"center offsets."
                )
            Dx, Dy = result
            img.extent = max(Dx, Dy)
        if isinstance(det.extent, ExtentPlaceholder):
            Mx, My = img.center
            Md = det.center
            Nx, Ny = img.size
            extent = float(img.extent)
            Dx = extent * Nx / max(Nx, Ny)
            Dy = extent * Ny / max(Nx, Ny)
            M = (Md, Mx, My)
            if det.extent == ExtentPlaceholder.FULL:
                result = full_detector_given_image_halfcircle(M, (Dx, Dy))
                meaning = ("FULL means the smallest detector width such that "
                           "every ray through the image also hits the detector")
            else:
                result = valid_detector_given_image_halfcircle(M, (Dx, Dy))
                meaning = ("VALID means the largest detector width such that "
                           "every ray hitting the detector also passes through "
                           "the image")
            if result is None:
                raise ValueError(
                    f"Cannot resolve ExtentPlaceholder.{det.extent.name} "
                    f"for the detector ({meaning}): no such detector width "
                    f"exists with image dimensions ({Dx}, {Dy}), detector "
                    f"center Md={Md}, and image center ({Mx}, {My}). "
                    f"Consider increasing the image extent or adjusting the "
                    f"center offsets."
                )
            det.extent = result

    def _make_settings(self, device) -> core.ProjectionSettings:
        return core.ProjectionSettings(
            device, core.RADON, tuple(self.image_domain.size), np.asarray(self.angles.angles),
            n_detectors=self.detectors.number, angle_weights=np.asarray(self.angles.weights),
            detector_width=float(self.detectors.extent), image_width=float(self.image_domain.extent),
            detector_shift=self.detectors.center, midpoint_shift=tuple(self.image_domain.center))

    def apply_to(self, argument, output=None, queue=None, return_event=False, **kwargs):
        return super().apply_to(argument, output=output, queue=queue, return_event=return_event)


def _fan_detector_width(image_extent: float, R: float, RE: float) -> float:
    """Detector width whose fan just covers a square image of the given extent.

    Inverse of gratopy's automatic image width (gratopy.py:879-887):
    image_width = 2 t RE / sqrt(1 + t^2) with t = (width / 2) / R.
    """
    w = image_extent / (2.0 * RE)
    if not 0.0 < w < 1.0:
        raise ValueError("the image does not fit between source and rotation centre")
    t = w / np.sqrt(1.0 - w * w)
    return 2.0 * R * t


class Fanbeam(_ProjectionOperator):
    """Fan-beam transform operator (``F``) or its adjoint (``F.T``).

    ``source_distances``: ``(R, RE)`` -- source-to-detector and
    source-to-rotation-centre distances -- or a single ``R`` (then
    ``RE = R / 2``).  ``angles``: int (uniform on the full circle) or
    :class:`Angles`.  ``detectors``: None (``ceil(hypot(Nx, Ny))`` pixels), an
    int or :class:`Detectors`; a FULL/absent detector extent becomes the
    width whose fan just covers the image, a negative count or
    ``reversed=True`` flips the detector direction.
    """

    def __init__(self, source_distances, image_domain, angles, detectors=None, adjoint=False,
                 kernel_spec=None):
        if np.isscalar(source_distances):
            R = float(source_distances)
            RE = R / 2.0
        else:
            R, RE = (float(v) for v in source_distances)
        if not isinstance(image_domain, ImageDomain):
            image_domain = ImageDomain(size=image_domain, extent=2.0)
        if isinstance(image_domain.extent, ExtentPlaceholder):
            raise NotImplementedError("Fanbeam needs a numeric image extent")
        if not isinstance(angles, Angles):
            angles = Angles.uniform(number=angles, half_circle=False)
        if not isinstance(detectors, Detectors):
            if detectors is None:
                detectors = int(np.ceil(np.hypot(*image_domain.size)))
            detectors = Detectors(number=detectors, extent=ExtentPlaceholder.FULL)
        if isinstance(detectors.extent, ExtentPlaceholder):
            if detectors.extent != ExtentPlaceholder.FULL:
                raise NotImplementedError("Fanbeam resolves only ExtentPlaceholder.FULL detectors")
            detectors.extent = _fan_detector_width(float(image_domain.extent), R, RE)
        state = {"image_domain": image_domain, "angles": angles, "detectors": detectors,
                 "adjoint": adjoint, "R": R, "RE": RE}
        super().__init__(name="Fanbeam", state=state, kernel_spec=kernel_spec)
        self._settings = {}
        self.projection_settings = None
        self._set_shapes()

    def _repr_name_(self) -> str:
        return "Fanbeam.T" if self.adjoint else "Fanbeam"

    def _make_settings(self, device) -> core.ProjectionSettings:
        return core.ProjectionSettings(
            device, core.FANBEAM, tuple(self.image_domain.size), np.asarray(self.angles.angles),
            n_detectors=self.detectors.number, angle_weights=np.asarray(self.angles.weights),
            detector_width=float(self.detectors.extent), image_width=float(self.image_domain.extent),
            R=self.state["R"], RE=self.state["RE"], detector_shift=self.detectors.center,
            midpoint_shift=tuple(self.image_domain.center),
            reverse_detector=bool(self.detectors.reversed))
