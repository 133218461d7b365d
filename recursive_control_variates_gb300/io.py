"""Grid and image files of the reference's scenes and outputs.

* ``.vol`` — Mitsuba's binary volume-grid format (the ``gridvolume``
  ``filename`` of experiments.py:56,63,169,175,290,297 and the final-state
  dumps of utils.py:45-60): 'VOL', version 3, encoding 1 (float32) or
  2 (float16), x/y/z resolution, channel count, bounding box (xmin, ymin,
  zmin, xmax, ymax, zmax), then the data with x fastest and channels
  innermost, little-endian.  Read and written as (Dz, Dy, Dx, C) float32
  arrays, the layout of the medium grids.
* ``.exr`` — OpenEXR single-part scanline images (reference images and
  texture dumps, utils.py:45-60,98-111).  Written uncompressed with float32
  channels; read uncompressed, ZIPS and ZIP files with half, float or uint
  channels, following the published OpenEXR file layout.
"""
from __future__ import annotations

import struct
import zlib
from dataclasses import dataclass
from pathlib import Path

import numpy as np

# ------------------------------------------------------------------ .vol
_VOL_FLOAT32 = 1
_VOL_FLOAT16 = 2


@dataclass
class VolumeGrid:
    """A grid read from a ``.vol`` file: data (Dz, Dy, Dx, C) float32 and the
    bounding box the file stores (min xyz, max xyz)."""

    data: np.ndarray
    bbox_min: tuple
    bbox_max: tuple


def read_vol(path) -> VolumeGrid:
    raw = Path(path).read_bytes()
    if len(raw) < 48 or raw[:3] != b"VOL":
        raise ValueError(f"{path}: not a .vol file")
    if raw[3] != 3:
        raise ValueError(f"{path}: .vol version {raw[3]} is not supported (version 3 is)")
    enc, xres, yres, zres, ch = struct.unpack_from("<5i", raw, 4)
    bbox = struct.unpack_from("<6f", raw, 24)
    if min(xres, yres, zres, ch) <= 0:
        raise ValueError(f"{path}: bad resolution or channel count")
    n = xres * yres * zres * ch
    if enc == _VOL_FLOAT32:
        dt = np.dtype("<f4")
    elif enc == _VOL_FLOAT16:
        dt = np.dtype("<f2")
    else:
        raise ValueError(f"{path}: .vol encoding {enc} is not supported (1 = float32, 2 = float16)")
    if len(raw) < 48 + n * dt.itemsize:
        raise ValueError(f"{path}: truncated data")
    data = np.frombuffer(raw, dt, n, 48).astype(np.float32).reshape(zres, yres, xres, ch)
    return VolumeGrid(data, tuple(bbox[:3]), tuple(bbox[3:]))


def write_vol(path, data, bbox_min=(0.0, 0.0, 0.0), bbox_max=(1.0, 1.0, 1.0)) -> None:
    """Writes a (Dz, Dy, Dx[, C]) grid as float32 ``.vol`` version 3."""
    a = np.asarray(data, np.float32)
    if a.ndim == 3:
        a = a[..., None]
    if a.ndim != 4:
        raise ValueError("grid data must have shape (Dz, Dy, Dx[, C])")
    zres, yres, xres, ch = a.shape
    head = b"VOL" + bytes([3]) + struct.pack("<5i", _VOL_FLOAT32, xres, yres, zres, ch)
    head += struct.pack("<6f", *map(float, bbox_min), *map(float, bbox_max))
    Path(path).write_bytes(head + np.ascontiguousarray(a, "<f4").tobytes())


# ------------------------------------------------------------------ .exr
_EXR_MAGIC = 20000630
_EXR_UINT, _EXR_HALF, _EXR_FLOAT = 0, 1, 2
_EXR_DTYPES = {_EXR_UINT: np.dtype("<u4"), _EXR_HALF: np.dtype("<f2"), _EXR_FLOAT: np.dtype("<f4")}
_EXR_NONE, _EXR_ZIPS, _EXR_ZIP = 0, 2, 3
_EXR_LINES = {_EXR_NONE: 1, _EXR_ZIPS: 1, _EXR_ZIP: 16}


def _attr(name: str, typ: str, value: bytes) -> bytes:
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(value)) + value


def write_exr(path, image) -> None:
    """Writes an (H, W), (H, W, 1), (H, W, 3) or (H, W, 4) image as an
    uncompressed float32 OpenEXR file (channels Y, RGB or RGBA)."""
    a = np.asarray(image, np.float32)
    if a.ndim == 2:
        a = a[..., None]
    if a.ndim != 3 or a.shape[2] not in (1, 3, 4):
        raise ValueError("image must have shape (H, W), (H, W, 1), (H, W, 3) or (H, W, 4)")
    h, w, c = a.shape
    names = {1: ["Y"], 3: ["R", "G", "B"], 4: ["R", "G", "B", "A"]}[c]
    order = sorted(range(c), key=lambda i: names[i])  # channels are stored by name
    chlist = b"".join(names[i].encode() + b"\0" + struct.pack("<i4xii", _EXR_FLOAT, 1, 1) for i in order) + b"\0"
    box = struct.pack("<4i", 0, 0, w - 1, h - 1)
    header = struct.pack("<ii", _EXR_MAGIC, 2)
    header += _attr("channels", "chlist", chlist)
    header += _attr("compression", "compression", bytes([_EXR_NONE]))
    header += _attr("dataWindow", "box2i", box)
    header += _attr("displayWindow", "box2i", box)
    header += _attr("lineOrder", "lineOrder", bytes([0]))
    header += _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
    header += _attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0))
    header += _attr("screenWindowWidth", "float", struct.pack("<f", 1.0))
    header += b"\0"
    line_bytes = w * c * 4
    first = len(header) + 8 * h
    offsets = struct.pack(f"<{h}Q", *[first + y * (8 + line_bytes) for y in range(h)])
    body = bytearray()
    planar = np.ascontiguousarray(a[:, :, order].transpose(0, 2, 1), "<f4")  # (H, C, W)
    for y in range(h):
        body += struct.pack("<ii", y, line_bytes)
        body += planar[y].tobytes()
    Path(path).write_bytes(header + offsets + bytes(body))


def _read_cstr(raw: bytes, pos: int) -> tuple[str, int]:
    end = raw.index(b"\0", pos)
    return raw[pos:end].decode(), end + 1


def _unzip_exr(data: bytes, expect: int) -> bytes:
    """zlib, then the OpenEXR predictor and byte interleave undone:
    b[i] = b[i-1] + b[i] - 128 (mod 256), then the first half of the buffer
    holds the even bytes and the second half the odd ones."""
    t = np.frombuffer(zlib.decompress(data), np.uint8).astype(np.int64)
    if t.size != expect:
        raise ValueError("EXR: decompressed chunk has the wrong size")
    t[1:] -= 128
    t = (np.cumsum(t) & 0xFF).astype(np.uint8)
    half = (t.size + 1) // 2
    out = np.empty_like(t)
    out[0::2] = t[:half]
    out[1::2] = t[half:]
    return out.tobytes()


def read_exr(path) -> np.ndarray:
    """Reads a single-part scanline OpenEXR file (uncompressed, ZIPS or
    ZIP) as float32 (H, W, C): channels R, G, B[, A] in that order when
    present, otherwise sorted by name."""
    raw = Path(path).read_bytes()
    magic, version = struct.unpack_from("<ii", raw, 0)
    if magic != _EXR_MAGIC:
        raise ValueError(f"{path}: not an OpenEXR file")
    if version & 0x200 or version & 0x1000 or version & 0x800:
        raise ValueError(f"{path}: tiled, multi-part and deep OpenEXR files are not supported")
    pos = 8
    channels, compression, window = [], None, None
    while raw[pos] != 0:
        name, pos = _read_cstr(raw, pos)
        typ, pos = _read_cstr(raw, pos)
        (size,) = struct.unpack_from("<i", raw, pos)
        pos += 4
        val = raw[pos:pos + size]
        pos += size
        if name == "channels":
            q = 0
            while val[q] != 0:
                cname, q = _read_cstr(val, q)
                ptype, _plin, xs, ys = struct.unpack_from("<iB3xii", val, q)
                q += 16
                if xs != 1 or ys != 1:
                    raise ValueError(f"{path}: subsampled channels are not supported")
                channels.append((cname, ptype))
        elif name == "compression":
            compression = val[0]
        elif name == "dataWindow":
            window = struct.unpack("<4i", val)
    pos += 1
    if compression not in _EXR_LINES:
        raise ValueError(f"{path}: compression {compression} is not supported (none, ZIPS, ZIP)")
    x0, y0, x1, y1 = window
    w, h = x1 - x0 + 1, y1 - y0 + 1
    lines = _EXR_LINES[compression]
    nchunks = (h + lines - 1) // lines
    offsets = struct.unpack_from(f"<{nchunks}Q", raw, pos)
    planes = {name: np.zeros((h, w), np.float32) for name, _ in channels}
    for off in offsets:
        ys, size = struct.unpack_from("<ii", raw, off)
        data = raw[off + 8:off + 8 + size]
        n_lines = min(lines, y1 - ys + 1)
        expect = n_lines * w * sum(_EXR_DTYPES[t].itemsize for _, t in channels)
        if compression != _EXR_NONE and size < expect:
            data = _unzip_exr(data, expect)
        q = 0
        for k in range(n_lines):
            for name, t in channels:
                dt = _EXR_DTYPES[t]
                planes[name][ys - y0 + k] = np.frombuffer(data, dt, w, q).astype(np.float32)
                q += w * dt.itemsize
    names = [n for n, _ in channels]
    order = [c for c in ("R", "G", "B", "A") if c in names] if "R" in names else sorted(names)
    return np.stack([planes[n] for n in order], axis=-1)
