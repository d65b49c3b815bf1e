"""Output of the deconvolved volume: the host-side mirror of Save3dTIFF
(spim/process/fusion/export/Save3dTIFF.java:45-182).

The reference hands the fused image to ImageJ's FileSaver: a 32-bit grayscale TIFF stack (one
image file directory per z-slice, uncompressed) whose ImageJ description carries the slice
count, the display range and the calibration (the bounding box's origin divided by the
down-sampling, pixel size = the down-sampling, :99-113), or the same TIFF inside a ZIP archive
(saveAsZip, :125-133).  This module writes that layout with numpy (no imaging library), and
reads it back for checks.  The HDF5 / BigDataViewer export (ExportSpimData2HDF5) needs an HDF5
library, which this package does not ship.
"""
from __future__ import annotations

import os
import struct
import zipfile

import numpy as np

# TIFF tags
_NEW_SUBFILE, _WIDTH, _LENGTH, _BITS, _COMPRESSION, _PHOTOMETRIC = 254, 256, 257, 258, 259, 262
_DESCRIPTION, _STRIP_OFFSETS, _SAMPLES, _ROWS_PER_STRIP, _STRIP_BYTES = 270, 273, 277, 278, 279
_XRES, _YRES, _RES_UNIT, _SAMPLE_FORMAT = 282, 283, 296, 339


def _imagej_description(n_slices, vmin, vmax, pixel, origin_xyz, unit):
    lines = ["ImageJ=1.54f", f"images={n_slices}", f"slices={n_slices}", f"unit={unit}",
             f"spacing={pixel!r}", f"min={vmin!r}", f"max={vmax!r}"]
    if origin_xyz is not None:
        lines += [f"xorigin={origin_xyz[0]!r}", f"yorigin={origin_xyz[1]!r}", f"zorigin={origin_xyz[2]!r}"]
    return ("\n".join(lines) + "\n").encode("ascii") + b"\0"


def tiff_bytes(img: np.ndarray, min_max=None, pixel: float = 1.0, origin_xyz=None, unit: str = "pixel") -> bytes:
    """A big-endian 32-bit float TIFF stack of ``img`` [z, y, x], ImageJ-compatible."""
    img = np.asarray(img, dtype=np.float32)
    if img.ndim == 2:
        img = img[None]
    if img.ndim != 3:
        raise ValueError("img must be 2D or 3D")
    nz, ny, nx = img.shape
    vmin, vmax = (float(img.min()), float(img.max())) if min_max is None else (float(min_max[0]), float(min_max[1]))
    desc = _imagej_description(nz, vmin, vmax, float(pixel), origin_xyz, unit)
    data = img.astype(">f4").tobytes()
    slice_bytes = nx * ny * 4
    # layout: header, description, resolution rationals, pixel data, then one IFD per slice
    out = bytearray(b"MM\x00\x2a\x00\x00\x00\x00")
    desc_off = len(out)
    out += desc
    if len(out) & 1:
        out += b"\0"
    res_off = len(out)
    den = 1000000
    num = max(1, int(round(den / float(pixel))))
    out += struct.pack(">II", num, den)
    data_off = len(out)
    out += data
    if len(out) & 1:
        out += b"\0"
    entries_per_ifd = 15
    ifd_size = 2 + 12 * entries_per_ifd + 4
    first_ifd = len(out)
    struct.pack_into(">I", out, 4, first_ifd)
    for z in range(nz):
        ifd_off = first_ifd + z * ifd_size
        nxt = ifd_off + ifd_size if z + 1 < nz else 0
        e = [
            (_NEW_SUBFILE, 4, 1, 0),
            (_WIDTH, 4, 1, nx),
            (_LENGTH, 4, 1, ny),
            (_BITS, 3, 1, 32),
            (_COMPRESSION, 3, 1, 1),
            (_PHOTOMETRIC, 3, 1, 1),
            (_DESCRIPTION, 2, len(desc), desc_off),
            (_STRIP_OFFSETS, 4, 1, data_off + z * slice_bytes),
            (_SAMPLES, 3, 1, 1),
            (_ROWS_PER_STRIP, 4, 1, ny),
            (_STRIP_BYTES, 4, 1, slice_bytes),
            (_XRES, 5, 1, res_off),
            (_YRES, 5, 1, res_off),
            (_RES_UNIT, 3, 1, 1),
            (_SAMPLE_FORMAT, 3, 1, 3),
        ]
        ifd = bytearray(struct.pack(">H", len(e)))
        for tag, typ, cnt, val in e:
            if typ == 3:  # SHORT: left-justified in the 4-byte value field
                ifd += struct.pack(">HHIHH", tag, typ, cnt, val, 0)
            else:
                ifd += struct.pack(">HHII", tag, typ, cnt, val)
        ifd += struct.pack(">I", nxt)
        out += ifd
    return bytes(out)


def read_tiff_stack(path_or_bytes) -> tuple[np.ndarray, str]:
    """Read a TIFF stack written by :func:`tiff_bytes` (uncompressed, one strip per slice):
    (volume [z, y, x] float32, ImageJ description)."""
    if isinstance(path_or_bytes, (bytes, bytearray)):
        buf = bytes(path_or_bytes)
    else:
        with open(path_or_bytes, "rb") as f:
            buf = f.read()
    bo = {b"MM": ">", b"II": "<"}[buf[:2]]
    if struct.unpack(bo + "H", buf[2:4])[0] != 42:
        raise ValueError("not a TIFF file")
    off = struct.unpack(bo + "I", buf[4:8])[0]
    slices, desc = [], ""
    while off:
        n = struct.unpack(bo + "H", buf[off:off + 2])[0]
        tags = {}
        for i in range(n):
            tag, typ, cnt = struct.unpack(bo + "HHI", buf[off + 2 + 12 * i: off + 10 + 12 * i])
            raw = buf[off + 10 + 12 * i: off + 14 + 12 * i]
            val = struct.unpack(bo + "H", raw[:2])[0] if typ == 3 else struct.unpack(bo + "I", raw)[0]
            tags[tag] = (typ, cnt, val)
        w, h = tags[_WIDTH][2], tags[_LENGTH][2]
        if tags[_BITS][2] != 32 or tags.get(_SAMPLE_FORMAT, (0, 0, 3))[2] != 3 or tags[_COMPRESSION][2] != 1:
            raise ValueError("only uncompressed 32-bit float stacks are read")
        so = tags[_STRIP_OFFSETS][2]
        slices.append(np.frombuffer(buf[so:so + 4 * w * h], dtype=bo + "f4").reshape(h, w))
        if not desc and _DESCRIPTION in tags:
            _, cnt, doff = tags[_DESCRIPTION]
            desc = buf[doff:doff + cnt].rstrip(b"\0").decode("ascii")
        off = struct.unpack(bo + "I", buf[off + 2 + 12 * n: off + 6 + 12 * n])[0]
    return np.stack(slices).astype(np.float32), desc


class Save3dTIFF:
    """Save3dTIFF(path, compress): exportImage(img, title) writes <path>/<title>.tif (or .zip)."""

    def __init__(self, path: str, compress: bool = False):
        self.path = path
        self.compress = compress

    def exportImage(self, img: np.ndarray, title: str, bb_min_xyz=None, downsampling: float = 1.0,
                    min_max=None) -> bool:
        """``bb_min_xyz``: the bounding box's minimum; the calibration origin is -min / downsampling
        and the pixel size the down-sampling (Save3dTIFF.java:99-113)."""
        origin = None if bb_min_xyz is None else tuple(-float(m) / downsampling for m in bb_min_xyz)
        data = tiff_bytes(img, min_max=min_max, pixel=downsampling, origin_xyz=origin)
        os.makedirs(self.path, exist_ok=True)
        if self.compress:
            name = os.path.join(self.path, title + ".zip")
            with zipfile.ZipFile(name, "w", zipfile.ZIP_DEFLATED) as z:
                z.writestr(title + ".tif", data)
        else:
            name = os.path.join(self.path, title + ".tif")
            with open(name, "wb") as f:
                f.write(data)
        return True
