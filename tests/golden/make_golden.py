"""Generate the golden fixtures of tests/golden/ from the gratopy reference.

Run on a machine that has a checkout of the gratopy reference, giving its
root directory (the tests only read the committed outputs and never run
this):

    python tests/golden/make_golden.py PATH/TO/gratopy-checkout

It imports gratopy's pure-NumPy host code (``pyopencl`` and ``matplotlib``
are stubbed -- no OpenCL runtime is needed for geometry tables) and writes:

* ``tables.npz``      -- radon_struct / fanbeam_struct outputs (float64 ofs,
                          geometry vector, sdpd, angles, angle weights,
                          image width) for every configuration of
                          ``configs.configs()``, produced by the reference's
                          own ``ProjectionSettings``;
* ``angles.npz``      -- reference ``read_angles`` results for the angle
                          specifications of gratopy's tests/test_radon.py:887-1116,
                          for both geometries;
* ``phantom.npz``     -- reference Shepp-Logan phantoms (ct_shepp_logan) at
                          small sizes;
* ``walnut_sinogram.npz`` -- gratopy's tests/walnut_sinogram.png decoded to its
                          raw 16-bit values (the reference reads it with
                          matplotlib as value / 65535).  The walnut data are
                          from Hamalainen et al., "Tomographic X-ray data of a
                          walnut", arXiv:1502.04064 (CC BY 4.0);
* ``placeholders.json`` -- extents resolved by the reference's
                          ``operator.Radon`` for the FULL/VALID placeholder
                          grid of gratopy's tests/test_extent_placeholder.py
                          (None where it raises ValueError);
* ``control_rng.json`` -- SHA-256 of gratopy's tests/rng.txt, which the tests
                          regenerate from ``numpy.random.default_rng(1)``.
"""

from __future__ import annotations

import hashlib
import importlib.util
import json
import struct
import sys
import types
import zlib
from pathlib import Path

import numpy as np

REF = Path(".")  # root of the gratopy checkout; set from the command line by main()
HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import configs as cfgmod  # noqa: E402


def _stub_modules():
    class _Any:
        def __init__(self, *a, **k):
            pass

    names = ["pyopencl", "pyopencl.array", "pyopencl.tools", "pyopencl.elementwise",
             "matplotlib", "matplotlib.pyplot", "matplotlib.patches", "matplotlib.axes",
             "matplotlib.figure", "matplotlib.image"]
    for n in names:
        sys.modules[n] = types.ModuleType(n)
    cl = sys.modules["pyopencl"]
    cl.array = sys.modules["pyopencl.array"]
    cl.tools = sys.modules["pyopencl.tools"]
    for attr in ("Context", "CommandQueue", "Event", "Kernel", "Buffer", "Program"):
        setattr(cl, attr, _Any)
    cl.array.Array = _Any
    cl.array.to_device = lambda queue, a, allocator=None: a
    cl.tools.AllocatorBase = _Any


def load_reference():
    _stub_modules()
    pkg = types.ModuleType("gratopy")
    pkg.__path__ = [str(REF / "gratopy")]
    sys.modules["gratopy"] = pkg
    for sub in ("_version", "utilities", "gratopy", "phantom", "operator.base", "operator.opencl",
                "operator.projection"):
        if sub.startswith("operator") and "gratopy.operator" not in sys.modules:
            opkg = types.ModuleType("gratopy.operator")
            opkg.__path__ = [str(REF / "gratopy" / "operator")]
            sys.modules["gratopy.operator"] = opkg
        spec = importlib.util.spec_from_file_location(
            f"gratopy.{sub}", REF / "gratopy" / (sub.replace(".", "/") + ".py"))
        mod = importlib.util.module_from_spec(spec)
        sys.modules[f"gratopy.{sub}"] = mod
        spec.loader.exec_module(mod)
    return sys.modules["gratopy.gratopy"], sys.modules["gratopy.phantom"]


class _Queue:
    context = None


def reference_settings(G, cfg: dict):
    cfg = dict(cfg)
    geometry = G.RADON if cfg.pop("geometry") == "radon" else G.FANBEAM
    img_shape = cfg.pop("img_shape")
    angles = cfg.pop("angles")
    return G.ProjectionSettings(_Queue(), geometry, img_shape, angles, **cfg)


def decode_png16(path: Path) -> np.ndarray:
    """Decode a non-interlaced 16-bit greyscale PNG into a uint16 array."""
    data = path.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, width, height = 8, b"", None, None
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            width, height, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
            assert depth == 16 and ctype == 0 and interlace == 0
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    bpp, stride = 2, width * 2
    out = np.zeros((height, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    for r in range(height):
        ftype = raw[r * (stride + 1)]
        line = np.frombuffer(raw, dtype=np.uint8, count=stride, offset=r * (stride + 1) + 1).astype(np.int32)
        cur = np.zeros(stride, dtype=np.int32)
        for i in range(stride):
            a = cur[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if ftype == 0:
                pred = 0
            elif ftype == 1:
                pred = a
            elif ftype == 2:
                pred = b
            elif ftype == 3:
                pred = (a + b) // 2
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            cur[i] = (line[i] + pred) & 0xFF
        out[r] = cur
        prev = cur
    return (out[:, 0::2].astype(np.uint16) << 8) | out[:, 1::2].astype(np.uint16)


def main():
    G, P = load_reference()
    tables = {}
    for name, cfg in cfgmod.configs().items():
        ps = reference_settings(G, cfg)
        s = ps.struct
        f64 = np.dtype("float64")
        tables[f"{name}/ofs"] = np.asarray(s["ofs_dict"][f64])
        tables[f"{name}/geo"] = np.asarray(s["geo_dict"][f64])
        tables[f"{name}/angles"] = np.asarray(ps.angles, dtype=np.float64)
        tables[f"{name}/weights"] = np.asarray(ps.angle_weights, dtype=np.float64)
        tables[f"{name}/image_width"] = np.float64(ps.image_width)
        tables[f"{name}/delta"] = np.array([ps.delta_x, ps.delta_s, ps.delta_ratio])
        if ps.is_fan:
            tables[f"{name}/sdpd"] = np.asarray(s["sdpd_dict"][f64]).reshape(-1)
    np.savez_compressed(HERE / "tables.npz", **tables)

    angles = {}
    for j, spec in enumerate(cfgmod.angle_variants()):
        for geom, flag in (("radon", G.RADON), ("fanbeam", G.FANBEAM)):
            for wname, w in (("auto", None), ("scalar", 1.0)):
                fake = types.SimpleNamespace(is_fan=flag == G.FANBEAM, is_parallel=flag == G.RADON)
                a, wts = G.read_angles(spec, w, fake)
                angles[f"{j}/{geom}/{wname}/angles"] = np.atleast_1d(np.asarray(a, dtype=np.float64))
                angles[f"{j}/{geom}/{wname}/weights"] = np.atleast_1d(np.asarray(wts, dtype=np.float64))
    np.savez_compressed(HERE / "angles.npz", **angles)

    ph = {}
    for shape in [(64, 64), (40, 56), (150, 150)]:
        ph[f"{shape[0]}x{shape[1]}"] = np.asarray(P.ct_shepp_logan(None, shape, dtype="float64"))
        ph[f"{shape[0]}x{shape[1]}_orig"] = np.asarray(
            P.ct_shepp_logan(None, shape, modified=False, dtype="float64"))
    np.savez_compressed(HERE / "phantom.npz", **ph)

    walnut = decode_png16(REF / "tests" / "walnut_sinogram.png")
    np.savez_compressed(HERE / "walnut_sinogram.npz", raw=walnut)

    Radon = sys.modules["gratopy.operator.projection"].Radon
    U = sys.modules["gratopy.utilities"]
    cases = []
    for side in ("detector", "image"):
        for ph in (U.ExtentPlaceholder.VALID, U.ExtentPlaceholder.FULL):
            for sr in (0.7, 1.0, 1.7):
                for dc in (0, 0.2, -0.2, 0.5, -0.5):
                    for ic in ((0.5, 0.2), (-0.5, 0.2), (0.5, -0.2), (-0.5, -0.2)):
                        Ny = int(sr * 400)
                        try:
                            if side == "detector":
                                r = Radon(U.ImageDomain(size=(400, Ny), center=ic, extent=2.0), 180,
                                          U.Detectors(number=100, center=dc, extent=ph))
                                val = float(r.detectors.extent)
                            else:
                                r = Radon(U.ImageDomain(size=(400, Ny), center=ic, extent=ph), 180,
                                          U.Detectors(number=100, center=dc, extent=2.0))
                                val = float(r.image_domain.extent)
                        except ValueError:
                            val = None
                        cases.append({"side": side, "placeholder": ph.value, "side_ratio": sr,
                                      "detector_center": dc, "image_center": list(ic), "extent": val})
    (HERE / "placeholders.json").write_text(json.dumps(cases, indent=0) + "\n")

    digest = hashlib.sha256((REF / "tests" / "rng.txt").read_bytes()).hexdigest()
    (HERE / "control_rng.json").write_text(json.dumps({"rng_txt_sha256": digest}, indent=1) + "\n")
    print("wrote", sorted(p.name for p in HERE.iterdir()))


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description="regenerate tests/golden from a gratopy checkout")
    ap.add_argument("reference", type=Path, help="root directory of the gratopy checkout")
    REF = ap.parse_args().reference.resolve()
    if not (REF / "gratopy" / "gratopy.py").exists():
        raise SystemExit(f"{REF} is not a gratopy checkout (gratopy/gratopy.py missing)")
    main()
