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


def _read_png(path: str):
    """(pixels, set of chunk tags) of an 8-bit PNG."""
    with open(path, "rb") as f:
        blob = f.read()
    if blob[:8] != _SIG:
        raise ValueError(f"{path} is not a PNG")
    pos, idat, hdr, tags = 8, [], None, set()
    while pos < len(blob):
        (n,) = struct.unpack(">I", blob[pos:pos + 4])
        tag = blob[pos + 4:pos + 8]
        data = blob[pos + 8:pos + 8 + n]
        pos += 12 + n
        tags.add(tag)
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
    return (px[..., 0] if ch == 1 else px), tags


def read_png(path: str) -> np.ndarray:
    return _read_png(path)[0]


# libpng's RGB -> gray weights as OpenCV's PNG decoder requests them for
# IMREAD_GRAYSCALE (png_set_rgb_to_gray(png, 1, 0.299, 0.587)): the 1e-5 fixed
# point values 29900 and 58700 scaled to 1/32768 with truncation, blue the rest.
PNG_GRAY_RED, PNG_GRAY_GREEN = 29900 * 32768 // 100000, 58700 * 32768 // 100000  # 9797, 19234
PNG_GRAY_BLUE = 32768 - PNG_GRAY_RED - PNG_GRAY_GREEN  # 3737


def png_rgb_to_gray(r: np.ndarray, g: np.ndarray, b: np.ndarray) -> np.ndarray:
    """libpng's 8-bit RGB -> gray step without gamma correction
    (png_do_rgb_to_gray): the weighted sum shifted right by 15, truncated;
    equal channels come through unchanged (the sum gives the same value)."""
    acc = (PNG_GRAY_RED * r.astype(np.int64) + PNG_GRAY_GREEN * g.astype(np.int64) +
           PNG_GRAY_BLUE * b.astype(np.int64))
    return (acc >> 15).astype(np.uint8)


def imread_gray(path: str) -> np.ndarray:
    """uint8 [H, W] like cv2.imread(path, cv2.IMREAD_GRAYSCALE).

    PNG content is decoded here.  A colour PNG is reduced to gray with
    libpng's integer transform (png_rgb_to_gray), which is what OpenCV's PNG
    decoder asks libpng for; that holds for files without colour-space
    chunks, where libpng applies no gamma correction.  A colour PNG with a
    gAMA, sRGB or iCCP chunk would go through libpng's gamma tables, which
    this reader does not restate: cv2 decodes it when importable, otherwise
    the call fails.  (Neither OpenCV nor libpng is present to pin the
    transform against; gray PNGs, the synthetic scenes' format, need none.)
    """
    with open(path, "rb") as f:
        is_png = f.read(8) == _SIG
    if is_png:
        px, tags = _read_png(path)
        if px.ndim == 2:
            return px
        if px.shape[2] == 2:  # gray + alpha: the alpha is stripped
            return np.ascontiguousarray(px[..., 0])
        if not tags & {b"gAMA", b"sRGB", b"iCCP"}:
            return png_rgb_to_gray(px[..., 0], px[..., 1], px[..., 2])
    try:
        import cv2
    except ImportError as e:
        what = "colour PNGs with colour-space chunks" if is_png else "non-PNG content"
        raise RuntimeError(f"{path}: {what} can only be read with OpenCV") from e
    img = cv2.imread(path, cv2.IMREAD_GRAYSCALE)
    if img is None:
        raise RuntimeError(f"cannot read {path}")
    return img
