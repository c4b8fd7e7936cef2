"""Minimal lossless PNG reader/writer (zlib + struct) for 8-bit gray and RGB.

The reference loads images with ``cv2.imread(path, IMREAD_GRAYSCALE)``
(planar_initer.cu:64-70, consistency.py:68-70).  cv2 sniffs the content, so a
PNG stored under a ``.jpg`` name reads back losslessly; this module does the
same without OpenCV.  When cv2 is importable and the file is not a PNG, cv2
decodes it.
"""

from __future__ import annotations

import struct
import zlib

import numpy as np

_SIG = b"\x89PNG\r\n\x1a\n"


def _chunk(tag: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def write_png(path: str, img: np.ndarray) -> None:
    """Write uint8 [H, W] (gray) or [H, W, 3] (RGB)."""
    a = np.ascontiguousarray(img)
    if a.dtype != np.uint8:
        raise ValueError("write_png expects uint8")
    if a.ndim == 2:
        ctype, ch = 0, 1
    elif a.ndim == 3 and a.shape[2] == 3:
        ctype, ch = 2, 3
    else:
        raise ValueError("write_png expects [H, W] or [H, W, 3]")
    h, w = a.shape[:2]
    raw = np.concatenate([np.zeros((h, 1), np.uint8), a.reshape(h, w * ch)], axis=1).tobytes()
    ihdr = struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)
    with open(path, "wb") as f:
        f.write(_SIG + _chunk(b"IHDR", ihdr) + _chunk(b"IDAT", zlib.compress(raw, 6)) + _chunk(b"IEND", b""))


def _unfilter(data: bytes, h: int, w: int, bpp: int) -> np.ndarray:
    stride = w * bpp
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    pos = 0
    for y in range(h):
        ft = data[pos]
        line = np.frombuffer(data, np.uint8, stride, pos + 1).astype(np.int32)
        pos += 1 + stride
        if ft == 0:
            cur = line
        elif ft == 1:
            cur = line.copy()
            for x in range(bpp, stride):
                cur[x] = (cur[x] + cur[x - bpp]) & 0xFF
        elif ft == 2:
            cur = (line + prev) & 0xFF
        elif ft == 3:
            cur = line.copy()
            for x in range(stride):
                left = cur[x - bpp] if x >= bpp else 0
                cur[x] = (cur[x] + ((left + prev[x]) >> 1)) & 0xFF
        elif ft == 4:
            cur = line.copy()
            for x in range(stride):
                a = cur[x - bpp] if x >= bpp else 0
                b = prev[x]
                c = prev[x - bpp] if x >= bpp else 0
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (cur[x] + pr) & 0xFF
        else:
            raise ValueError(f"bad PNG filter {ft}")
        out[y] = cur
        prev = cur
    return out


def read_png(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        blob = f.read()
    if blob[:8] != _SIG:
        raise ValueError(f"{path} is not a PNG")
    pos, idat, hdr = 8, [], None
    while pos < len(blob):
        (n,) = struct.unpack(">I", blob[pos:pos + 4])
        tag = blob[pos + 4:pos + 8]
        data = blob[pos + 8:pos + 8 + n]
        pos += 12 + n
        if tag == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", data)
        elif tag == b"IDAT":
            idat.append(data)
        elif tag == b"IEND":
            break
    w, h, depth, ctype, _, _, interlace = hdr
    if depth != 8 or interlace != 0 or ctype not in (0, 2, 4, 6):
        raise ValueError("only 8-bit non-interlaced gray/RGB(A) PNGs are supported")
    ch = {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
    px = _unfilter(zlib.decompress(b"".join(idat)), h, w, ch).reshape(h, w, ch)
    return px[..., 0] if ch == 1 else px


def imread_gray(path: str) -> np.ndarray:
    """uint8 [H, W] like cv2.imread(path, cv2.IMREAD_GRAYSCALE)."""
    with open(path, "rb") as f:
        is_png = f.read(8) == _SIG
    if not is_png:
        try:
            import cv2  # noqa: F401
        except ImportError as e:
            raise RuntimeError(f"{path}: only PNG content can be read without OpenCV") from e
        import cv2

        img = cv2.imread(path, cv2.IMREAD_GRAYSCALE)
        if img is None:
            raise RuntimeError(f"cannot read {path}")
        return img
    px = read_png(path)
    if px.ndim == 2:
        return px
    rgb = px[..., :3].astype(np.float64)
    # ITU-R BT.601 luma, rounded, the conversion cv2 uses for RGB -> gray
    return np.clip(np.rint(0.299 * rgb[..., 0] + 0.587 * rgb[..., 1] + 0.114 * rgb[..., 2]), 0, 255).astype(np.uint8)
