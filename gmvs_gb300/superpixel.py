"""Superpixel extraction of the segmentation preprocessing on the GB300.

Mirrors gmvs/scripts/extract_superpixel.py: ``extract_superpixel(image)``
(lines 55-74) and ``seg_func(image_dir, save_dir, mask_dir, var_windlen,
var_thresh, var_thresh2)`` (lines 77-126), whose ``segid_npy`` output the
fusion scripts load (mvs_fusion_segmentaion.py:367).  One call of
``gmvs_superpixels`` does the per-pixel stages on the device (resize,
Gaussian smoothing, edge weights, nearest resize back, morphological close,
mask, variance map) and the Felzenszwalb merge, a sequential scan, on the
calling thread; ``extract_many`` runs several images at once, one stream
and workspace per worker thread (ctypes releases the GIL during the call).

Inputs are BGR uint8 [H, W, 3] as cv2.imread returns them (numpy or a CUDA
tensor) and, for the variance filter, the gray uint8 [H, W] image.  The
script's segrgb visualisation (random colours) is not written.
"""

from __future__ import annotations

import ctypes
import os
import threading
from concurrent.futures import ThreadPoolExecutor
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _abi
from ._abi import check, gmvs_superpixel_params, lib


def default_params(**overrides) -> gmvs_superpixel_params:
    p = gmvs_superpixel_params()
    lib().gmvs_superpixel_default_params(ctypes.byref(p))
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def bgr_to_gray(image: np.ndarray) -> np.ndarray:
    """The gray image cv2.imread(path, IMREAD_GRAYSCALE) gives for a colour
    PNG whose cv2.imread(path) is `image` (BGR uint8): libpng's integer
    transform, as imageio.imread_gray applies it."""
    from .imageio import png_rgb_to_gray

    return png_rgb_to_gray(image[..., 2], image[..., 1], image[..., 0])


def _device_u8(a, shape, name: str, dev: torch.device) -> torch.Tensor:
    t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a))
    if t.dtype != torch.uint8 or tuple(t.shape) != tuple(shape):
        raise RuntimeError(f"{name} must be uint8 {tuple(shape)}, got {t.dtype} {tuple(t.shape)}")
    return t.to(dev, non_blocking=False).contiguous()


class Extractor:
    """One stream and one grow-only workspace; not shared between threads."""

    def __init__(self, device: Optional[torch.device] = None, params: Optional[gmvs_superpixel_params] = None):
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.params = params or default_params()
        self.stream = torch.cuda.Stream(self.device)
        self._ws: Optional[torch.Tensor] = None

    def _workspace(self, rows: int, cols: int):
        need = lib().gmvs_superpixel_workspace_bytes(rows, cols, ctypes.byref(self.params))
        if need == 0:
            raise _abi.GmvsError(_abi.ERR_INVALID, lib().gmvs_last_error().decode())
        if self._ws is None or self._ws.numel() < need:
            self._ws = None
            self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        return self._ws.data_ptr(), self._ws.numel()

    def run(self, image, gray=None, mask=None, outputs: Sequence[str] = ("segment", "ids", "ids_map", "var_map"),
            ) -> Dict[str, torch.Tensor]:
        """Device tensors by name: segment int32 (extract_superpixel),
        ids uint8 (closed, masked), ids_map int32 (variance-filtered),
        var_map float32 (when the variance filter is on); plus
        "num_segments" (int)."""
        rows, cols = int(image.shape[0]), int(image.shape[1])
        p = self.params
        var_on = p.var_thresh > 0 and p.var_windlen > 1
        with torch.cuda.device(self.device), torch.cuda.stream(self.stream):
            img = _device_u8(image, (rows, cols, 3), "image", self.device)
            g = None
            if var_on and ("ids_map" in outputs or "var_map" in outputs):
                if gray is None:
                    gray = bgr_to_gray(image.cpu().numpy() if isinstance(image, torch.Tensor) else image)
                g = _device_u8(gray, (rows, cols), "gray", self.device)
            m = None
            if mask is not None:
                mk = mask.cpu().numpy() if isinstance(mask, torch.Tensor) else np.asarray(mask)
                if mk.shape != (rows, cols):
                    raise RuntimeError(f"mask must be {(rows, cols)}, got {mk.shape}")
                m = _device_u8((mk == True).astype(np.uint8), (rows, cols), "mask", self.device)  # noqa: E712
            out: Dict[str, torch.Tensor] = {}
            kw = dict(device=self.device)
            if "segment" in outputs:
                out["segment"] = torch.empty((rows, cols), dtype=torch.int32, **kw)
            if "ids" in outputs:
                out["ids"] = torch.empty((rows, cols), dtype=torch.uint8, **kw)
            if "ids_map" in outputs:
                out["ids_map"] = torch.empty((rows, cols), dtype=torch.int32, **kw)
            if "var_map" in outputs and var_on:
                out["var_map"] = torch.empty((rows, cols), dtype=torch.float32, **kw)
            ptr, size = self._workspace(rows, cols)
            kept = ctypes.c_int32(0)

            def addr(t):
                return t.data_ptr() if t is not None else None

            check(lib().gmvs_superpixels(addr(img), addr(g), addr(m), rows, cols, ctypes.byref(p),
                                         addr(out.get("segment")), addr(out.get("ids")), addr(out.get("ids_map")),
                                         addr(out.get("var_map")), ctypes.byref(kept), ptr, size,
                                         _abi.stream_ptr(self.stream)))
            self.stream.synchronize()
        out["num_segments"] = int(kept.value)
        return out


_local = threading.local()


def _extractor(device=None, params=None) -> Extractor:
    ex = getattr(_local, "ex", None)
    if ex is None or (device is not None and ex.device != device):
        ex = _local.ex = Extractor(device)
    if params is not None:
        ex.params = params
    else:
        ex.params = default_params()
    return ex


def extract_superpixel(image, weight=None) -> np.ndarray:
    """extract_superpixel.py:55-74: segment labels [H, W] of a BGR uint8
    image (0 = the first segment or a dropped one)."""
    if weight is not None:
        raise NotImplementedError("extract_superpixel: weighted images are not supported (no caller passes one)")
    out = _extractor().run(image, outputs=("segment",))
    return out["segment"].cpu().numpy().astype(np.int64)


def segment_ids(image, gray=None, mask=None, var_windlen: int = 15, var_thresh: float = 0.2,
                var_thresh2: float = -1.0, device=None):
    """seg_func's segment-id map (extract_superpixel.py:80-110) of one image:
    returns (segment_ids_map, segment_ids) as numpy arrays -- int32 and uint8
    with the variance filter on, both the uint8 ids with it off, as the
    script saves them."""
    var_on = var_thresh > 0.0 and var_windlen > 1
    if var_thresh2 > 0.0 and not var_on:
        raise UnboundLocalError("seg_func: var_thresh2 needs the variance map (var_thresh > 0, var_windlen > 1)")
    p = default_params(var_windlen=int(var_windlen), var_thresh=float(var_thresh) if var_on else 0.0)
    ex = _extractor(device, p)
    want = ("ids", "ids_map", "var_map") if var_on else ("ids",)
    out = ex.run(image, gray, mask, outputs=want)
    ids = out["ids"]
    if not var_on:
        a = ids.cpu().numpy()
        return a, a
    ids_map = out["ids_map"]
    if var_thresh2 > 0.0:
        from .engine import filter_by_var_map

        with torch.cuda.stream(ex.stream):
            ids_map = filter_by_var_map(out["var_map"], ids_map, float(var_thresh2), stream=ex.stream)
        ex.stream.synchronize()
    return ids_map.cpu().numpy(), ids.cpu().numpy()


def read_bgr(path: str) -> np.ndarray:
    """cv2.imread(path) for PNG content without OpenCV (BGR uint8)."""
    from .imageio import read_png

    with open(path, "rb") as f:
        is_png = f.read(8) == b"\x89PNG\r\n\x1a\n"
    if not is_png:
        import cv2  # only for non-PNG content

        img = cv2.imread(path)
        if img is None:
            raise RuntimeError(f"cannot read {path}")
        return img
    px = read_png(path)
    if px.ndim == 2:
        px = np.repeat(px[..., None], 3, axis=2)
    return np.ascontiguousarray(px[..., 2::-1] if px.shape[2] >= 3 else np.repeat(px[..., :1], 3, axis=2))


def seg_func(image_dir: str, save_dir: str, mask_dir: Optional[str] = None, var_windlen: int = 15,
             var_thresh: float = 0.2, var_thresh2: float = -1) -> str:
    """extract_superpixel.py:77-126 for one image file: writes
    save_dir/segid_npy/<name>.npy and returns its path."""
    from .imageio import imread_gray

    filename = os.path.basename(image_dir)
    rgb = read_bgr(image_dir)
    gray = imread_gray(image_dir)
    mask = np.load(mask_dir) if mask_dir is not None else None
    ids_map, _ = segment_ids(rgb, gray, mask, var_windlen, var_thresh, var_thresh2)
    os.makedirs(os.path.join(save_dir, "segid_npy"), exist_ok=True)
    path = os.path.join(save_dir, "segid_npy", filename.replace(".png", ".npy"))
    np.save(path, ids_map)
    return path


def extract_many(images: Sequence, grays: Optional[Sequence] = None, workers: int = 4, **kw) -> List:
    """segment_ids over many images, `workers` at a time (one stream each)."""
    grays = grays if grays is not None else [None] * len(images)
    with ThreadPoolExecutor(max_workers=max(1, workers)) as ex:
        return list(ex.map(lambda ig: segment_ids(ig[0], ig[1], **kw), zip(images, grays)))
