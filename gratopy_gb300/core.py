"""gratopy's legacy API on torch CUDA tensors, backed by the sm_103a kernels.

Drop-in counterparts of ``gratopy/gratopy.py``:

* :class:`ProjectionSettings`              -- gratopy.py:1299-1756
* :func:`forwardprojection`, :func:`backprojection` -- gratopy.py:126-255
* :func:`radon`, :func:`radon_ad`, :func:`fanbeam`, :func:`fanbeam_ad`
                                           -- gratopy.py:258-377, 581-703
* :func:`weight_sinogram`, :func:`equ_mul_add`, :func:`mul_add_add`
                                           -- gratopy.py:2188-2326
* :func:`normest`, :func:`landweber`, :func:`conjugate_gradients`,
  :func:`total_variation`                  -- gratopy.py:2329-2762

``torch.Tensor`` (CUDA, float32/float64, C- or F-contiguous through its
strides) replaces ``pyopencl.array.Array``; the current CUDA stream replaces
the command queue and its events (``wait_for`` is accepted and ignored
because work on one stream is ordered).  ``queue`` may be a
``torch.device``, a device string/index, a ``torch.cuda.Stream`` or ``None``
(current CUDA device).  Validation keeps gratopy's ``assert`` messages.
Every computation runs in the CUDA extension; there is no CPU path.
"""

from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np
import torch

from . import _lib
from .geometry import fanbeam_struct, radon_struct, read_angles
from .utilities import GeometryType

PARALLEL = RADON = GeometryType.RADON
FANBEAM = FAN = GeometryType.FANBEAM

VERBOSE = False


def _progress(msg: str) -> None:
    if VERBOSE:
        sys.stdout.write(msg)


# ------------------------------------------------------------------- tensors


def _device_of(queue) -> torch.device:
    if queue is None:
        return torch.device("cuda", torch.cuda.current_device())
    if isinstance(queue, torch.device):
        return queue if queue.index is not None else torch.device("cuda", torch.cuda.current_device())
    if isinstance(queue, torch.cuda.Stream):
        return queue.device
    if isinstance(queue, int):
        return torch.device("cuda", queue)
    if isinstance(queue, str):
        return _device_of(torch.device(queue))
    dev = getattr(queue, "device", None)
    if dev is not None:
        return _device_of(dev)
    raise TypeError(f"cannot interpret {queue!r} as a CUDA device or stream")


def order_of(t: torch.Tensor) -> str:
    """'C' if C-contiguous (checked first, as gratopy does), 'F' if Fortran-contiguous."""
    if t.is_contiguous():
        return "C"
    # Fortran order: first index fastest (strides of size-1 dims do not matter)
    expected = 1
    for n, st in zip(t.shape, t.stride()):
        if n != 1 and st != expected:
            break
        expected *= n
    else:
        return "F"
    raise ValueError(
        f"tensor of shape {tuple(t.shape)} with strides {t.stride()} is neither C- nor "
        "F-contiguous"
    )


def _oflag(order: str) -> int:
    return _lib.GR_ORDER_C if order.upper() == "C" else _lib.GR_ORDER_F


def empty(shape, dtype, order: str = "F", device=None) -> torch.Tensor:
    """Uninitialised device tensor with C or Fortran memory order."""
    shape = tuple(int(s) for s in shape)
    device = _device_of(device)
    if order.upper() == "C":
        return torch.empty(shape, dtype=dtype, device=device)
    return torch.empty(shape[::-1], dtype=dtype, device=device).permute(*reversed(range(len(shape))))


def zeros(shape, dtype, order: str = "F", device=None) -> torch.Tensor:
    out = empty(shape, dtype, order, device)
    out.zero_()
    return out


def _check_tensor(t, name: str) -> None:
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor on a CUDA device, got {type(t)}")
    if not t.is_cuda:
        raise TypeError(f"{name} must live on a CUDA device (got device {t.device})")
    if t.dtype not in (torch.float32, torch.float64):
        raise TypeError(f"{name} must be float32 or float64, got {t.dtype}")


def _dt(t: torch.Tensor) -> int:
    return _lib.GR_F32 if t.dtype == torch.float32 else _lib.GR_F64


def _np_dtype(t_dtype) -> np.dtype:
    if isinstance(t_dtype, torch.dtype):
        return np.dtype("float32") if t_dtype == torch.float32 else np.dtype("float64")
    return np.dtype(t_dtype)


def _torch_dtype(dtype) -> torch.dtype:
    if isinstance(dtype, torch.dtype):
        return dtype
    return torch.float32 if np.dtype(dtype) == np.float32 else torch.float64


def _stream_ptr(device: torch.device) -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _ptr(t: torch.Tensor | None) -> ctypes.c_void_p:
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _nz(t: torch.Tensor) -> int:
    return int(t.shape[2]) if t.dim() > 2 else 1


# ------------------------------------------------------- ProjectionSettings


class ProjectionSettings:
    """Projection geometry (gratopy.py:1299-1756) with device-resident tables.

    Same constructor arguments and attributes as gratopy's class.  The
    per-angle table (``ofs``), angle weights and -- for fan beam -- the
    source-detector-pixel distances are uploaded once per precision by
    :meth:`ensure_dtype` and kept on ``self.device``.
    """

    def __init__(
        self,
        queue,
        geometry,
        img_shape,
        angles,
        n_detectors=None,
        angle_weights=None,
        detector_width=2.0,
        image_width=None,
        R=None,
        RE=None,
        detector_shift=0.0,
        midpoint_shift=(0.0, 0.0),
        reverse_detector=False,
    ):
        self.geometry = geometry
        self.queue = queue
        self._device = None
        if np.isscalar(img_shape):
            img_shape = (img_shape, img_shape)
        if len(img_shape) > 2:
            img_shape = img_shape[0:2]
        self.img_shape = tuple(int(v) for v in img_shape)

        angles, angles_diff = read_angles(angles, angle_weights, self)
        self.n_angles = len(angles)
        self.angle_weights = angles_diff
        self.angles = angles

        if n_detectors is None:
            self.n_detectors = int(np.ceil(np.hypot(img_shape[0], img_shape[1])))
        else:
            self.n_detectors = n_detectors
        self.sinogram_shape = (self.n_detectors, self.n_angles)

        self.image_width = image_width
        self.detector_shift = detector_shift
        self.midpoint_shift = midpoint_shift
        self.detector_width = detector_width
        self.R = R
        self.RE = RE
        self.reverse_detector = reverse_detector
        self.buf_upload = {}
        self._dev = {}
        self._geom = {}
        self._geom_adj = {}
        self._work_bytes = {}  # scratch bytes the projections can use, per precision
        self._work = {}  # (precision, stream) -> scratch tensor

        if self.reverse_detector and self.is_parallel:
            print(
                "WARNING, the reverse_detector argument has no impact"
                + " on the parallel beam setting. To reverse the angles,"
                + " the angles parameter can be translated by np.pi"
            )

        if self.is_fan:
            assert not ((R is None) or (RE is None)), (
                "For the Fanbeam geometry "
                + "you need to set R (the normal "
                + "distance from source to detector)"
                + " and RE (distance from source to "
                + "coordinate origin which is the "
                + "rotation center)"
            )
            self.struct = fanbeam_struct(
                queue=self.queue,
                img_shape=self.img_shape,
                angles=self.angles,
                angle_weights=self.angle_weights,
                detector_width=self.detector_width,
                source_detector_dist=self.R,
                source_origin_dist=self.RE,
                n_detectors=self.n_detectors,
                detector_shift=self.detector_shift,
                image_width=image_width,
                midpoint_shift=self.midpoint_shift,
                reverse_detector=self.reverse_detector,
            )
            self.ofs_buf = self.struct["ofs_dict"]
            self.sdpd_buf = self.struct["sdpd_dict"]
            self.image_width = self.struct["image_width"]
            self.geometry_information = self.struct["geo_dict"]
            self.angle_weights_buf = self.struct["angle_diff_dict"]
            self.angle_weights = self.angle_weights_buf[np.dtype("float")].copy()
            self.delta_x = float(self.image_width) / max(self.img_shape)
            # gratopy.py:1594 divides by the n_detectors argument (None when the
            # detector count is automatic, a TypeError there); the resolved
            # count is used here.
            self.delta_s = float(detector_width) / self.n_detectors
            self.delta_ratio = self.delta_s / self.delta_x

        if self.is_parallel:
            self.image_width = 2.0 if image_width is None else float(self.image_width)
            self.struct = radon_struct(
                queue=self.queue,
                img_shape=self.img_shape,
                angles=self.angles,
                angle_weights=self.angle_weights,
                n_detectors=self.n_detectors,
                detector_width=self.detector_width,
                image_width=self.image_width,
                midpoint_shift=self.midpoint_shift,
                detector_shift=self.detector_shift,
            )
            self.ofs_buf = self.struct["ofs_dict"]
            self.delta_x = self.image_width / max(self.img_shape)
            self.delta_s = self.detector_width / self.n_detectors
            self.delta_ratio = self.delta_s / self.delta_x
            self.geometry_information = self.struct["geo_dict"]
            self.angle_weights_buf = self.struct["angle_diff_dict"]
            self.angle_weights = self.angle_weights_buf[np.dtype("float")].copy()

    # -- geometry kind -------------------------------------------------------
    @property
    def is_parallel(self) -> bool:
        return self.geometry == GeometryType.RADON

    @property
    def is_fan(self) -> bool:
        return self.geometry == GeometryType.FANBEAM

    @property
    def geometry(self) -> GeometryType:
        return self._geometry

    @geometry.setter
    def geometry(self, value) -> None:
        self._geometry = GeometryType(value)

    @property
    def device(self) -> torch.device:
        if self._device is None:
            self._device = _device_of(self.queue)
        return self._device

    # -- dispatch (gratopy.py:1655-1685) --------------------------------------
    def forwardprojection(self, sino, img, projectionsetting, wait_for=[]):
        if self.geometry == GeometryType.RADON:
            return radon(sino, img, projectionsetting, wait_for=wait_for)
        return fanbeam(sino, img, projectionsetting, wait_for=wait_for)

    def backprojection(self, img, sino, projectionsetting, wait_for=[]):
        if self.geometry == GeometryType.RADON:
            return radon_ad(img, sino, projectionsetting, wait_for=wait_for)
        return fanbeam_ad(img, sino, projectionsetting, wait_for=wait_for)

    # -- device tables ---------------------------------------------------------
    def ensure_dtype(self, dtype) -> None:
        """Upload the tables of precision ``dtype`` to the device once."""
        dtype = _np_dtype(dtype)
        if dtype in self._dev:
            return
        tdt = _torch_dtype(dtype)
        dev = self.device
        ofs = np.ascontiguousarray(np.asarray(self.struct["ofs_dict"][dtype]).T)
        tables = {
            "ofs": torch.from_numpy(ofs.reshape(-1)).to(dev, tdt),
            "w": torch.from_numpy(np.asarray(self.struct["angle_diff_dict"][dtype]).reshape(-1)).to(dev, tdt),
        }
        if self.is_fan:
            tables["sdpd"] = torch.from_numpy(
                np.asarray(self.struct["sdpd_dict"][dtype]).reshape(-1)).to(dev, tdt)
        # table of the plain transpose A^T: the angle-weight column replaced
        # by the forward projection's scale
        adj = np.array(ofs, copy=True)
        adj[:, 6 if self.is_fan else 4] = self.forward_scale(dtype)
        tables["ofs_adj"] = torch.from_numpy(adj.reshape(-1)).to(dev, tdt)
        self._dev[dtype] = tables
        self.buf_upload[dtype] = 1
        g = _lib.GrGeometry()
        g.kind = _lib.GR_FANBEAM if self.is_fan else _lib.GR_RADON
        g.dtype = _lib.GR_F32 if dtype == np.float32 else _lib.GR_F64
        g.Nx, g.Ny = self.img_shape
        g.Ns, g.Na = self.sinogram_shape
        g.ofs = tables["ofs"].data_ptr()
        g.sdpd = tables["sdpd"].data_ptr() if self.is_fan else None
        geo = np.asarray(self.struct["geo_dict"][dtype], dtype=np.float64)
        for i, v in enumerate(geo):
            g.geo[i] = float(v)
        maps = self.quarter_maps()
        if maps is not None:
            g.sym = 4 if self.is_fan else 2
            for m, row in enumerate(maps):
                for k, v in enumerate(row):
                    g.sym_map[m][k] = int(v)
            mirror = self.mirror_map() if self.is_fan else None
            if mirror is not None:
                g.mirror, g.mirror_pair = 1, mirror[1]
                for k, v in enumerate(mirror[0]):
                    g.mirror_map[k] = int(v)
        self._geom[dtype] = g
        ga = _lib.GrGeometry.from_buffer_copy(g)
        ga.ofs = tables["ofs_adj"].data_ptr()
        self._geom_adj[dtype] = ga
        # a slice's copies, or two slices' where a stack's orbit forward takes
        # slices in pairs
        work = _lib.raw("gr_work_bytes")
        self._work_bytes[dtype] = max(int(work(ctypes.byref(g), 1)), int(work(ctypes.byref(g), 2)))

    def quarter_maps(self):
        """Index maps of the geometry's orbit symmetry (see
        :mod:`gratopy_gb300.symmetry`): the quarter-turn orbits of a fan-beam
        geometry, the half-circle orbits (quarter turn and detector mirror)
        of a parallel-beam one; None when the geometry has none.  Computed
        once."""
        if not hasattr(self, "_quarter"):
            from .symmetry import fan_quarter_maps, radon_half_maps

            find = fan_quarter_maps if self.is_fan else radon_half_maps
            self._quarter = find(self.struct, self.img_shape)
        return self._quarter

    def mirror_map(self):
        """The mirror of a fan-beam geometry (see
        :func:`gratopy_gb300.symmetry.fan_mirror_map`): ``(lookup, c0)`` with
        angle ``c0 - b`` seeing the lookup's pixel as angle ``b`` sees the
        pixel, the detector reversed; None when the geometry has none.
        Computed once."""
        if not hasattr(self, "_mirror"):
            from .symmetry import fan_mirror_map

            self._mirror = fan_mirror_map(self.struct, self.img_shape) if self.is_fan else None
        return self._mirror

    def forward_scale(self, dtype) -> float:
        """Scale the forward kernels apply after the interpolation sums, in their arithmetic.

        Radon: dx*dx/ds with dx, ds rounded to float32 (radon.cl:82-83,160);
        fan beam: dx/(ds/dx) (fanbeam.cl:254-255, with sdpd[s]/R applied per bin).
        A^T is the backprojection with this value as every angle weight.
        """
        dtype = _np_dtype(dtype)
        geo = np.asarray(self.struct["geo_dict"][dtype])
        if self.is_fan:
            return float(dtype.type(geo[10]) / dtype.type(geo[2]))
        dx = dtype.type(np.float32(geo[0]))
        ds = dtype.type(np.float32(geo[1]))
        return float(dx * dx / ds)

    def device_tables(self, dtype) -> dict:
        self.ensure_dtype(dtype)
        return self._dev[_np_dtype(dtype)]

    def gr_geometry(self, dtype, stream=None) -> _lib.GrGeometry:
        """C-ABI geometry descriptor for precision ``dtype`` (tables uploaded).

        The descriptor carries the scratch of ``stream`` (default: the current
        stream; see :meth:`_bind_work`); a descriptor kept across calls on
        several streams at once must be fetched again on each stream.
        """
        self.ensure_dtype(dtype)
        dt = _np_dtype(dtype)
        return self._bind_work(self._geom[dt], dt, stream)

    def gr_geometry_adjoint(self, dtype) -> _lib.GrGeometry:
        """Descriptor whose backprojection is the plain transpose of the forward projection."""
        self.ensure_dtype(dtype)
        dt = _np_dtype(dtype)
        return self._bind_work(self._geom_adj[dt], dt)

    def _bind_work(self, g, dt, stream=None):
        """Point ``g.work`` at this settings object's scratch for ``stream``
        (default: the current one; allocated on first use, used by the library
        stream-ordered).  During a stream capture the descriptor keeps the
        scratch bound before the capture, the one of the stream that replays
        the graph."""
        nbytes = self._work_bytes.get(dt, 0)
        if not nbytes or torch.cuda.is_current_stream_capturing():
            return g
        if stream is None:
            stream = torch.cuda.current_stream(self.device)
        key = (dt, stream.cuda_stream)
        buf = self._work.get(key)
        if buf is None:
            with torch.cuda.device(self.device):
                buf = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            self._work[key] = buf
        g.work = buf.data_ptr()
        g.work_bytes = nbytes
        return g

    def set_angle_weights(self, angle_weights) -> None:
        """Replace the angle weights and re-upload the tables (gratopy.py:1697-1756)."""
        if self.is_parallel:
            self.struct = radon_struct(
                self.queue, self.img_shape, self.angles, angle_weights=angle_weights,
                n_detectors=self.n_detectors, detector_width=self.detector_width,
                image_width=self.image_width, midpoint_shift=self.midpoint_shift,
                detector_shift=self.detector_shift)
        if self.is_fan:
            self.struct = fanbeam_struct(
                self.queue, self.img_shape, self.angles, angle_weights=angle_weights,
                detector_width=self.detector_width, source_detector_dist=self.R,
                source_origin_dist=self.RE, n_detectors=self.n_detectors,
                detector_shift=self.detector_shift, image_width=self.image_width,
                midpoint_shift=self.midpoint_shift, reverse_detector=self.reverse_detector)
        self.ofs_buf = self.struct["ofs_dict"]
        self.angle_weights_buf = self.struct["angle_diff_dict"]
        self.angle_weights = self.angle_weights_buf[np.dtype("float")].copy()
        uploaded = list(self._dev.keys())
        self._dev.clear()
        self._geom.clear()
        self._geom_adj.clear()
        for dtype in uploaded:
            self.ensure_dtype(dtype)

    def get_projection_kernel(self, sinogram, image, adjoint: bool = False) -> str:
        """Name of the gratopy kernel variant a call would use (gratopy.py:2157-2185)."""
        so = order_of(sinogram).lower()
        io = order_of(image).lower()
        return "{name}{ad}_{dt}_{o1}{o2}".format(
            name=self.geometry.value,
            ad="_ad" if adjoint else "",
            dt="float" if sinogram.dtype == torch.float32 else "double",
            o1=so if not adjoint else io,
            o2=io if not adjoint else so,
        )

    def create_sparse_matrix(self, dtype=np.dtype("float32"), order="F"):
        """Sparse COO matrix of the forward projection (gratopy.py:2014-2155).

        One device launch evaluates gratopy's single-line formula
        (radon.cl:263-341, fanbeam.cl:422-568) for the two detector bins
        around every pixel's projection; entries that are not positive are
        dropped as in the reference.  Rows index the sinogram, columns the
        image, both in the linear order ``order``.
        """
        import scipy.sparse

        dtype = _np_dtype(dtype)
        tdt = _torch_dtype(dtype)
        order = order.upper()
        if order not in ("C", "F"):
            raise ValueError("Order (contiguity) not recognized, suitable choices are 'F' or 'C'")
        Nx, Ny = self.img_shape
        Ns, Na = self.sinogram_shape
        dev = self.device
        g = self.gr_geometry(dtype)
        n = 2 * Nx * Ny * Na
        rows = torch.empty(n, dtype=torch.int64, device=dev)
        cols = torch.empty(n, dtype=torch.int64, device=dev)
        vals = torch.empty(n, dtype=tdt, device=dev)
        with torch.cuda.device(dev):
            _lib.call("gr_sparse_entries", ctypes.byref(g), _ptr(rows), _ptr(cols), _ptr(vals),
                      _oflag(order), _stream_ptr(dev))
        keep = vals > 0
        rows, cols, vals = rows[keep].cpu().numpy(), cols[keep].cpu().numpy(), vals[keep].cpu().numpy()
        return scipy.sparse.coo_matrix((vals, (rows, cols)), shape=(Ns * Na, Nx * Ny))

    def show_geometry(self, *args, **kwargs):
        raise NotImplementedError(
            "show_geometry draws with matplotlib, which this GPU build does not ship")


# ------------------------------------------------------------ legacy API


def check_compatibility(img, sino, projectionsetting) -> None:
    """Shape/dtype validation with gratopy's messages (gratopy.py:85-123)."""
    assert sino.dtype == img.dtype, (
        f"sinogram and image do not share common data type: {sino.dtype} and {img.dtype}"
    )
    assert tuple(sino.shape[0:2]) == tuple(projectionsetting.sinogram_shape), (
        f"The dimensions of the sinogram {tuple(sino.shape)} "
        f"do not match the projectionsetting's {projectionsetting.sinogram_shape}"
    )
    assert tuple(img.shape[0:2]) == tuple(projectionsetting.img_shape), (
        f"The dimensions of the image {tuple(img.shape)} do not match the "
        f"projectionsetting's {projectionsetting.img_shape}"
    )
    if len(sino.shape) > 2 and sino.shape[2] > 1:
        assert len(img.shape) > 2, "The sinogram has a third dimension but the image does not."
        assert sino.shape[2] == img.shape[2], (
            "The third dimension (z-direction) of the sinogram is "
            f"{sino.shape[2]} and the image's is {img.shape[2]}, they "
            "do not coincide."
        )
    if len(img.shape) > 2 and img.shape[2] > 1:
        assert len(sino.shape) > 2, " The sinogram has a third dimension but the image does not."


def _prepare(img, sino, ps):
    _check_tensor(img, "img")
    _check_tensor(sino, "sino")
    check_compatibility(img, sino, ps)
    if img.device != sino.device:
        raise ValueError(f"img on {img.device} and sino on {sino.device}: same device required")
    if img.dim() > 3 or sino.dim() > 3:
        raise ValueError("arrays must have 2 or 3 dimensions")
    return order_of(img), order_of(sino)


def _event(device):
    ev = torch.cuda.Event()
    ev.record(torch.cuda.current_stream(device))
    return ev


def _project(entry, out, inp, out_order, in_order, ps, event=True):
    """One projection through the settings' geometry descriptor: the tuned
    launch shape, the quarter-turn orbit kernels and the current stream's
    scratch apply.  Returns a CUDA event recorded after it, or None."""
    dev = out.device
    stream = torch.cuda.current_stream(dev)
    g = ps.gr_geometry(_np_dtype(out.dtype), stream)
    args = (entry, ctypes.byref(g), _ptr(out), _ptr(inp), _nz(out), _oflag(out_order),
            _oflag(in_order), ctypes.c_void_p(stream.cuda_stream))
    if dev.index == torch.cuda.current_device():
        _lib.call(*args)
    else:
        with torch.cuda.device(dev):
            _lib.call(*args)
    if not event:
        return None
    ev = torch.cuda.Event()
    ev.record(stream)
    return ev


def radon(sino, img, projectionsetting, wait_for=[]):
    """Radon forward projection into ``sino`` (gratopy.py:258-316); returns a CUDA event.

    The C library also has the reference kernel's own argument list
    (``gr_radon_fwd``: ofs table, geometry vector, shapes) for callers
    without a settings object; this form passes the settings' descriptor.
    """
    io, so = _prepare(img, sino, projectionsetting)
    return _project("gr_forward", sino, img, so, io, projectionsetting)


def radon_ad(img, sino, projectionsetting, wait_for=[]):
    """Radon backprojection into ``img`` (gratopy.py:319-377); returns a CUDA event."""
    io, so = _prepare(img, sino, projectionsetting)
    return _project("gr_backward", img, sino, io, so, projectionsetting)


def fanbeam(sino, img, projectionsetting, wait_for=[]):
    """Fan-beam forward projection into ``sino`` (gratopy.py:581-640)."""
    io, so = _prepare(img, sino, projectionsetting)
    return _project("gr_forward", sino, img, so, io, projectionsetting)


def fanbeam_ad(img, sino, projectionsetting, wait_for=[]):
    """Fan-beam backprojection into ``img`` (gratopy.py:643-703)."""
    io, so = _prepare(img, sino, projectionsetting)
    return _project("gr_backward", img, sino, io, so, projectionsetting)


def forwardprojection(img, projectionsetting, sino=None, wait_for=[]):
    """Forward projection of ``img`` (gratopy.py:126-187).

    A new sinogram follows the image's memory order (C if the image is
    C-contiguous, else F); a given ``sino`` is overwritten and returned.
    """
    _check_tensor(img, "img")
    if sino is None:
        z = (img.shape[2],) if img.dim() > 2 else ()
        sino = empty(tuple(projectionsetting.sinogram_shape) + z, img.dtype,
                     "C" if img.is_contiguous() else "F", img.device)
    if type(projectionsetting).forwardprojection is ProjectionSettings.forwardprojection:
        # the settings' own method without its (discarded) event
        io, so = _prepare(img, sino, projectionsetting)
        _project("gr_forward", sino, img, so, io, projectionsetting, event=False)
    else:
        projectionsetting.forwardprojection(sino, img, projectionsetting, wait_for=wait_for)
    return sino


def backprojection(sino, projectionsetting, img=None, wait_for=[]):
    """Backprojection of ``sino`` (gratopy.py:190-255)."""
    _check_tensor(sino, "sino")
    if img is None:
        z = (sino.shape[2],) if sino.dim() > 2 else ()
        img = empty(tuple(projectionsetting.img_shape) + z, sino.dtype,
                    "C" if sino.is_contiguous() else "F", sino.device)
    if type(projectionsetting).backprojection is ProjectionSettings.backprojection:
        # the settings' own method without its (discarded) event
        io, so = _prepare(img, sino, projectionsetting)
        _project("gr_backward", img, sino, io, so, projectionsetting, event=False)
    else:
        projectionsetting.backprojection(img, sino, projectionsetting, wait_for=wait_for)
    return img


def weight_sinogram(sino, projectionsetting, sino_out=None, divide=False, wait_for=[]):
    """Multiply (or divide) each projection by its angle weight (gratopy.py:2188-2266)."""
    _check_tensor(sino, "sino")
    order = "C" if sino.is_contiguous() else "F"
    order_of(sino)
    if sino_out is None:
        sino_out = empty(sino.shape, sino.dtype, order, sino.device)
    elif order_of(sino_out) != order or sino_out.shape != sino.shape:
        raise ValueError("sino_out must match sino in shape and memory order")
    dtype = _np_dtype(sino.dtype)
    t = projectionsetting.device_tables(dtype)
    with torch.cuda.device(sino.device):
        _lib.call("gr_weight_sinogram", _ptr(sino_out), _ptr(sino), _ptr(t["w"]), _dt(sino),
                  sino.shape[0], sino.shape[1], _nz(sino), _oflag(order), int(bool(divide)),
                  _stream_ptr(sino.device))
    return sino_out


def equ_mul_add(rhs, a, x, projectionsetting=None, wait_for=[]):
    """rhs += a * x over the flat memory of same-order tensors (gratopy.py:2269-2295)."""
    _check_tensor(rhs, "rhs")
    _check_tensor(x, "x")
    if rhs.numel() != x.numel() or rhs.dtype != x.dtype:
        raise ValueError("rhs and x must have the same size and dtype")
    with torch.cuda.device(rhs.device):
        _lib.call("gr_equ_mul_add", _ptr(rhs), float(a), _ptr(x), _dt(rhs), rhs.numel(),
                  _stream_ptr(rhs.device))
    return rhs


def mul_add_add(rhs, a, x, y, projectionsetting=None, wait_for=[]):
    """rhs = a * x + y over flat memory (gratopy.py:2298-2326)."""
    for name, t in (("rhs", rhs), ("x", x), ("y", y)):
        _check_tensor(t, name)
    if not (rhs.numel() == x.numel() == y.numel()):
        raise ValueError("rhs, x and y must have the same size")
    with torch.cuda.device(rhs.device):
        _lib.call("gr_mul_add_add", _ptr(rhs), float(a), _ptr(x), _ptr(y), _dt(rhs), rhs.numel(),
                  _stream_ptr(rhs.device))
    return rhs


def create_code(cl_context=None) -> str:
    """Source of the toolbox's device kernels (the CUDA translation units)."""
    csrc = Path(__file__).resolve().parent / "csrc"
    return "".join(p.read_text() for p in sorted(csrc.glob("*.cu*")))


# ------------------------------------------------------------------- solvers


class _Scratch:
    """Device scalars and reduction partials of one solver run."""

    def __init__(self, device, n_partials: int):
        self.sc = torch.zeros(_lib.SC_COUNT, dtype=torch.float64, device=device)
        self.done = torch.zeros(1, dtype=torch.int32, device=device)
        self.dot = torch.empty(int(_lib.raw("gr_dot_partials_count")()), dtype=torch.float64,
                               device=device)
        self.part = torch.empty(max(1, n_partials), dtype=torch.float64, device=device)
        self.part2 = torch.empty(max(1, n_partials), dtype=torch.float64, device=device)

    def slot(self, k: int) -> ctypes.c_void_p:
        return ctypes.c_void_p(self.sc.data_ptr() + 8 * k)


GRAPH_CHUNK = 25


def _iterate(body, n: int, device, use_graph: bool) -> None:
    """Run ``body()`` ``n`` times on the current stream.

    With ``use_graph`` the launches of up to GRAPH_CHUNK iterations are
    captured once into a CUDA graph and the graph is replayed; the remainder
    runs directly.  ``body`` must launch the same kernels with the same
    arguments every iteration and must not allocate or synchronise.
    """
    if n <= 0:
        return
    if not use_graph or n < 2 or torch.cuda.is_current_stream_capturing():
        for _ in range(n):
            body()
        return
    chunk = min(n, GRAPH_CHUNK)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        for _ in range(chunk):
            body()
    reps, rem = divmod(n, chunk)
    for _ in range(reps):
        graph.replay()
    for _ in range(rem):
        body()


def _dot_into(scr: _Scratch, slot: int, a, b, stream) -> None:
    _lib.call("gr_dot_partials", _ptr(scr.dot), _ptr(a), _ptr(b), _dt(a), a.numel(), stream)
    _lib.call("gr_sum_partials", scr.slot(slot), _ptr(scr.dot), scr.dot.numel(), stream)


def normest(projectionsetting, number_iterations=50, dtype="float32", allocator=None, x0=None,
            use_graph=True):
    """Spectral-norm estimate by power iteration (gratopy.py:2329-2377).

    The iterate is normalised by its plain sum (not its norm) before each
    application of A^T A, as in the reference; the sum is a float64 device
    reduction and the whole loop runs without host synchronisation (captured
    in a CUDA graph unless ``use_graph=False``).  The start vector is
    ``np.random.randn`` (seed numpy's global generator to reproduce it)
    unless ``x0`` is given.
    """
    ps = projectionsetting
    if number_iterations < 1:
        raise ValueError("number_iterations must be positive")
    ndt = _np_dtype(dtype)
    tdt = _torch_dtype(ndt)
    dev = ps.device
    if x0 is None:
        x0 = np.random.randn(*ps.img_shape)
    if isinstance(x0, torch.Tensor):
        img = zeros(ps.img_shape, tdt, "F", dev)
        img.copy_(x0)
    else:
        img = torch.from_numpy(np.require(np.asarray(x0), ndt, "F").T.copy()).to(dev).T
    g = ps.gr_geometry(ndt)
    sino = empty(ps.sinogram_shape, tdt, "F", dev)
    with torch.cuda.device(dev):
        st = _stream_ptr(dev)
        n_bwd = int(_lib.raw("gr_backward_partials")(ctypes.byref(g), 1, _lib.GR_ORDER_F))
        scr = _Scratch(dev, n_bwd)
        n = img.numel()
        # the sum of the start vector goes into partial 0 (the others are 0),
        # so every iteration starts by summing the same partials buffer
        scr.part.zero_()
        _lib.call("gr_sum_values_partials", _ptr(scr.dot), _ptr(img), _dt(img), n, st)
        _lib.call("gr_sum_partials", _ptr(scr.part), _ptr(scr.dot), scr.dot.numel(), st)
        gptr = ctypes.byref(g)

        def body():
            s_ = _stream_ptr(dev)
            _lib.call("gr_sum_partials", scr.slot(_lib.SC_SUM), _ptr(scr.part), n_bwd, s_)
            _lib.call("gr_scale_by_sum", _ptr(img), _ptr(scr.sc), _dt(img), n, s_)
            _lib.call("gr_forward", gptr, _ptr(sino), _ptr(img), 1, 0, 0, s_)
            _lib.call("gr_backward_sum", gptr, _ptr(img), _ptr(sino), _ptr(scr.part), 1, 0, s_)

        _iterate(body, number_iterations, dev, use_graph)
        normsqr = float(scr.sc[_lib.SC_SUM].item())
    return float(np.sqrt(normsqr))


def _img_shape_for(sino, ps):
    return tuple(ps.img_shape) + ((int(sino.shape[2]),) if sino.dim() > 2 else ())


def landweber(sino, projectionsetting, number_iterations=100, w=1.0, norm_estimate=None,
              use_graph=True):
    """Landweber (SIRT) iteration (gratopy.py:2380-2446).

    Each iteration is two fused launches: r = A u - f, then u += -w' A^T r
    with w' = w / |A|^2 rounded to the data precision.
    """
    _check_tensor(sino, "sino")
    ps = projectionsetting
    order = order_of(sino)
    if norm_estimate is None:
        norm_estimate = normest(ps)
    ndt = _np_dtype(sino.dtype)
    wq = ndt.type(w / norm_estimate**2)
    g = ps.gr_geometry(ndt)
    dev = sino.device
    Nz = _nz(sino)
    resid = empty(sino.shape, sino.dtype, order, dev)
    unew = zeros(_img_shape_for(sino, ps), sino.dtype, order, dev)
    of = _oflag(order)
    gptr = ctypes.byref(g)

    def body():
        st = _stream_ptr(dev)
        _lib.call("gr_forward_residual", gptr, _ptr(resid), _ptr(unew), _ptr(sino), Nz, of, st)
        _lib.call("gr_backward_axpy", gptr, _ptr(unew), _ptr(resid), float(-wq), Nz, of, st)

    with torch.cuda.device(dev):
        _iterate(body, number_iterations, dev, use_graph)
    _progress("\rLandweber reconstruction complete\n")
    return unew


def conjugate_gradients(sino, projectionsetting, number_iterations=20, epsilon=0.0, x0=None,
                        use_graph=True):
    """CG on the normal equations in gratopy's weighted inner products (gratopy.py:2449-2551).

    Step sizes stay on the device (float64 reductions, no host round trip);
    the early stop on ``epsilon`` is a device flag that turns the remaining
    launches into no-ops, so the iterate equals the reference's at the break.
    """
    _check_tensor(sino, "sino")
    ps = projectionsetting
    order = order_of(sino)
    dims = _img_shape_for(sino, ps)
    dev = sino.device
    if x0 is None:
        x0 = zeros(dims, sino.dtype, order, dev)
    assert order_of(x0) == order, "The data sino and initial guess x0 must have the same contiguity!"
    x = empty(dims, sino.dtype, order, dev)
    x.copy_(x0)
    ndt = _np_dtype(sino.dtype)
    g = ps.gr_geometry(ndt)
    t = ps.device_tables(ndt)
    Nz = _nz(sino)
    of = _oflag(order)
    d = zeros(sino.shape, sino.dtype, order, dev)
    r = empty(sino.shape, sino.dtype, order, dev)
    q = empty(sino.shape, sino.dtype, order, dev)
    p = empty(dims, sino.dtype, order, dev)
    snew = empty(dims, sino.dtype, order, dev)
    c = ps.delta_x**2 / ps.delta_s
    with torch.cuda.device(dev):
        st = _stream_ptr(dev)
        n_fwd = int(_lib.raw("gr_forward_partials")(ctypes.byref(g), Nz))
        n_bwd = int(_lib.raw("gr_backward_partials")(ctypes.byref(g), Nz, of))
        scr = _Scratch(dev, max(n_fwd, n_bwd))
        n_dot = scr.dot.numel()
        # d = sino - A x ; p = A^T d ; <s, s> ; <f, f>
        _lib.call("gr_forward_residual", ctypes.byref(g), _ptr(r), _ptr(x), _ptr(sino), Nz, of, st)
        _lib.call("gr_equ_mul_add", _ptr(d), -1.0, _ptr(r), _dt(d), d.numel(), st)
        _lib.call("gr_backward", ctypes.byref(g), _ptr(p), _ptr(d), Nz, of, of, st)
        _dot_into(scr, _lib.SC_SOLD, p, p, st)
        _dot_into(scr, _lib.SC_FSQ, sino, sino, st)
        gptr = ctypes.byref(g)

        def body():
            st_ = _stream_ptr(dev)
            _lib.call("gr_forward_wsq", gptr, _ptr(q), _ptr(p), _ptr(t["w"]),
                      _ptr(scr.part), _ptr(scr.done), Nz, of, st_)
            _lib.call("gr_cg_alpha", _ptr(scr.sc), _ptr(scr.part), n_fwd, float(c), _dt(sino),
                      _ptr(scr.done), st_)
            _lib.call("gr_cg_update_d", _ptr(d), _ptr(q), _ptr(scr.sc), _ptr(scr.dot), _dt(sino),
                      d.numel(), _ptr(scr.done), st_)
            _lib.call("gr_backward_cg", gptr, _ptr(snew), _ptr(d), _ptr(x), _ptr(p),
                      scr.slot(_lib.SC_ALPHA), _ptr(scr.part2), _ptr(scr.done), Nz, of, st_)
            _lib.call("gr_cg_beta", _ptr(scr.sc), _ptr(scr.part2), n_bwd, _ptr(scr.dot), n_dot,
                      float(epsilon), _dt(sino), _ptr(scr.done), st_)
            _lib.call("gr_cg_update_p", _ptr(p), _ptr(snew), _ptr(scr.sc), _dt(sino), p.numel(),
                      _ptr(scr.done), st_)

        _iterate(body, number_iterations, dev, use_graph)
    _progress("\rCG reconstruction complete\n")
    return x


def total_variation(sino, projectionsetting, mu, number_iterations=1000, slice_thickness=1.0,
                    stepsize_weighting=10.0, norm_estimate=None, use_graph=True):
    """L2-TV primal-dual (Chambolle-Pock) reconstruction (gratopy.py:2554-2762).

    Per iteration three launches: the fused dual step (gradient + unit-ball
    projection), the forward projection with the data-dual update as its
    epilogue, and the backprojection with divergence, primal step,
    positivity and extrapolation as its epilogue.  Scalars are passed as
    float32 as in the reference.  3-D data (Nz > 1) couples slices through
    the z-gradient scaled by ``slice_thickness``; the reference raises a
    TypeError on 3-D input (gratopy.py:2626-2628), this follows its evident
    intent ``img_shape + (Nz,)``.
    """
    _check_tensor(sino, "sino")
    ps = projectionsetting
    order = order_of(sino)
    if sino.dim() == 2:
        slice_thickness = 0
    img_shape = _img_shape_for(sino, ps)
    Nz = _nz(sino)
    dev = sino.device
    ndt = _np_dtype(sino.dtype)
    g = ps.gr_geometry(ndt)
    U = zeros(img_shape, sino.dtype, order, dev)
    Ubar = zeros(img_shape, sino.dtype, order, dev)
    V = torch.zeros(4 * U.numel(), dtype=sino.dtype, device=dev)
    Lamb = zeros(sino.shape, sino.dtype, order, dev)
    if norm_estimate is None:
        norm_estimate = normest(ps)
    Lsqr = 13
    sigma = 1.0 / np.sqrt(Lsqr) * stepsize_weighting
    tau = 1.0 / np.sqrt(Lsqr) / stepsize_weighting
    assert mu > 0, "Regularization parameter mu must be positive"
    mu = mu * norm_estimate**2 * ps.delta_x
    mu = mu / (sigma + mu)
    f32 = lambda v: float(np.float32(v))  # noqa: E731  (scalars are float32 kernel args)
    of = _oflag(order)
    Nx, Ny = ps.img_shape
    gptr = ctypes.byref(g)
    sig, z_d = f32(sigma), f32(slice_thickness)
    sig_l, mu_f = f32(sigma / norm_estimate), f32(mu)
    tau_f, norming = f32(tau), f32(1.0 / norm_estimate)

    def body():
        st = _stream_ptr(dev)
        _lib.call("gr_tv_dual", _ptr(V), _ptr(Ubar), sig, z_d, _dt(sino), Nx, Ny, Nz, of, st)
        _lib.call("gr_forward_lambda", gptr, _ptr(Lamb), _ptr(Ubar), _ptr(sino), sig_l, mu_f, Nz,
                  of, st)
        _lib.call("gr_backward_tv_primal", gptr, _ptr(U), _ptr(Ubar), _ptr(V), _ptr(Lamb), tau_f,
                  norming, z_d, Nz, of, st)

    with torch.cuda.device(dev):
        _iterate(body, number_iterations, dev, use_graph)
    _progress("\rTV reconstruction complete\n")
    return U
