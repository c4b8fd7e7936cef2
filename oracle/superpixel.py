"""ORACLE — TEST INFRASTRUCTURE ONLY.

CPU restatement of the superpixel preprocessing of the reference
(gmvs/scripts/extract_superpixel.py): extract_superpixel (lines 55-74) and
the segment-id map of seg_func (lines 77-113).  Only tests/ and bench.py's
cpu_baseline leg use it, as the checker.

The script's arithmetic lives in third-party libraries that are absent here:
OpenCV (cv2.resize INTER_LINEAR / INTER_NEAREST, cv2.morphologyEx
MORPH_CLOSE, cv2.boxFilter BORDER_REFLECT; unpinned in the reference) and
scikit-image (segmentation.felzenszwalb, util.img_as_float; unpinned).
Their published algorithms are restated:

* resize_linear: bilinear resampling with pixel-centre alignment,
  src = (dst + 0.5) * (src_size / dst_size) - 0.5, clamped at the edges,
  11-bit fixed-point weights rounded to nearest and a 22-bit rounding shift
  of the two-pass sum (OpenCV's INTER_LINEAR scheme for 8-bit images); an
  exact 2x reduction on both axes averages 2 x 2 blocks with rounding, as
  OpenCV switches INTER_LINEAR to INTER_AREA there.
* felzenszwalb: Felzenszwalb & Huttenlocher (IJCV 2004) on the 8-connected
  grid as scikit-image parameterises it: the image scaled to [0, 1] by
  multiplication with 1/255, Gaussian smoothing of each channel (SciPy's
  gaussian_filter, truncate 4, reflect borders, rows then columns), edge
  weight = Euclidean distance of the smoothed colours, k = scale / 255,
  edges visited in ascending weight, a merge when the weight is below
  min(Int(C1) + k/|C1|, Int(C2) + k/|C2|), the merged component rooted at
  its smaller pixel index, then a second pass over the same order merging
  across every edge whose side is below min_size, labels numbered by each
  component's first pixel in raster order.  scikit-image orders the edges
  with numpy's default (unstable) argsort, whose order among equal weights
  depends on numpy's build; here equal weights keep their edge order
  (right, down, down-right, up-right edges, each in raster order).
* The morphological close with a k x k box is a k x k maximum filter
  followed by a k x k minimum filter over the pixels inside the image.
* The box filter sums the window's rows in order, then the row sums in
  order, and scales by 1 / window area; borders reflect with the edge pixel
  repeated (fedcba|abcdefgh|hgfedcb).

What SciPy implements here is pinned against SciPy in the tests (the
Gaussian smoothing bit for bit, the close exactly, the box filter to
rounding); the rest is unpinned.
"""

from __future__ import annotations

import math

import numpy as np


def reflect_index(i: int, n: int) -> int:
    """Border index for a reflect border with the edge pixel repeated."""
    if n == 1:
        return 0
    while i < 0 or i >= n:
        i = -i - 1 if i < 0 else 2 * n - 1 - i
    return i


def _reflect_indices(n: int, lo: int, hi: int) -> np.ndarray:
    """[n, hi - lo + 1] source indices of a window [i + lo, i + hi] per i."""
    return np.array([[reflect_index(i + k, n) for k in range(lo, hi + 1)] for i in range(n)], dtype=np.int64)


# ------------------------------------------------------------------ resize --
def _linear_taps(src: int, dst: int):
    scale = 1.0 / (dst / src)
    d = np.arange(dst, dtype=np.float64)
    f = ((d + 0.5) * scale - 0.5).astype(np.float32)
    s = np.floor(f).astype(np.int64)
    f = (f - s.astype(np.float32)).astype(np.float32)
    low = s < 0
    f[low], s[low] = np.float32(0), 0
    high = s >= src - 1
    f[high], s[high] = np.float32(0), src - 1
    a0 = np.rint((np.float32(1) - f) * np.float32(2048)).astype(np.int64)
    a1 = np.rint(f * np.float32(2048)).astype(np.int64)
    s1 = np.minimum(s + 1, src - 1)
    return s, s1, a0, a1


def resize_linear(img: np.ndarray, out_rows: int, out_cols: int) -> np.ndarray:
    """uint8 [H, W, C] -> uint8 [out_rows, out_cols, C]."""
    H, W = img.shape[:2]
    x = img.astype(np.int64)
    if H == 2 * out_rows and W == 2 * out_cols:
        s = x[0::2, 0::2] + x[0::2, 1::2] + x[1::2, 0::2] + x[1::2, 1::2]
        return ((s + 2) >> 2).astype(np.uint8)
    sx0, sx1, a0, a1 = _linear_taps(W, out_cols)
    sy0, sy1, b0, b1 = _linear_taps(H, out_rows)
    rows = x[:, sx0] * a0[None, :, None] + x[:, sx1] * a1[None, :, None]  # [H, out_cols, C]
    v = rows[sy0] * b0[:, None, None] + rows[sy1] * b1[:, None, None]
    return np.clip((v + (1 << 21)) >> 22, 0, 255).astype(np.uint8)


def resize_nearest(lbl: np.ndarray, out_rows: int, out_cols: int) -> np.ndarray:
    H, W = lbl.shape
    ifx, ify = 1.0 / (out_cols / W), 1.0 / (out_rows / H)
    sx = np.minimum(np.floor(np.arange(out_cols) * ifx).astype(np.int64), W - 1)
    sy = np.minimum(np.floor(np.arange(out_rows) * ify).astype(np.int64), H - 1)
    return lbl[sy][:, sx]


# ----------------------------------------------------------- felzenszwalb --
def gaussian_weights(sigma: float, truncate: float = 4.0):
    r = int(truncate * sigma + 0.5)
    phi = [math.exp(-0.5 / (sigma * sigma) * float(k * k)) for k in range(-r, r + 1)]
    total = 0.0
    for p in phi:
        total += p
    return r, np.array([p / total for p in phi])


def _smooth_axis(a: np.ndarray, axis: int, r: int, w: np.ndarray) -> np.ndarray:
    """Symmetric 1-D correlation along `axis`: centre tap first, then the
    pairs from the outermost inwards, each pair summed before its weight."""
    a = np.moveaxis(a, axis, 0)
    idx = _reflect_indices(a.shape[0], -r, r)
    s = a[idx[:, r]] * w[r]
    for k in range(-r, 0):
        s = s + (a[idx[:, r + k]] + a[idx[:, r - k]]) * w[r + k]
    return np.moveaxis(s, 0, axis)


def gaussian_smooth(img: np.ndarray, sigma: float) -> np.ndarray:
    """float64 [H, W, C] smoothed along rows (axis 0), then columns."""
    r, w = gaussian_weights(sigma)
    if r == 0:
        return img.copy()
    return _smooth_axis(_smooth_axis(img, 0, r, w), 1, r, w)


def edge_costs(sm: np.ndarray) -> np.ndarray:
    """Euclidean colour distances of the right, down, down-right and
    up-right edges, each group in raster order, concatenated."""
    def dist(a, b):
        d = a - b
        q = d * d
        s = q[..., 0]
        for c in range(1, q.shape[-1]):
            s = s + q[..., c]
        return np.sqrt(s)
    right = dist(sm[:, 1:], sm[:, :-1])
    down = dist(sm[1:, :], sm[:-1, :])
    dright = dist(sm[1:, 1:], sm[:-1, :-1])
    uright = dist(sm[:-1, 1:], sm[1:, :-1])
    return np.concatenate([right.ravel(), down.ravel(), dright.ravel(), uright.ravel()])


def edge_endpoints(rows: int, cols: int) -> np.ndarray:
    p = np.arange(rows * cols).reshape(rows, cols)
    right = np.stack([p[:, :-1].ravel(), p[:, 1:].ravel()], 1)
    down = np.stack([p[:-1, :].ravel(), p[1:, :].ravel()], 1)
    dright = np.stack([p[:-1, :-1].ravel(), p[1:, 1:].ravel()], 1)
    uright = np.stack([p[:-1, 1:].ravel(), p[1:, :-1].ravel()], 1)
    return np.concatenate([right, down, dright, uright])


def felzenszwalb_merge(rows: int, cols: int, costs: np.ndarray, k: float, min_size: int) -> np.ndarray:
    n = rows * cols
    ends = edge_endpoints(rows, cols)
    order = np.argsort(costs, kind="stable")
    parent = list(range(n))
    size = [1] * n
    cint = [0.0] * n

    def find(a):
        r = a
        while parent[r] != r:
            r = parent[r]
        while parent[a] != r:
            parent[a], a = r, parent[a]
        return r

    cl = costs.tolist()
    el = ends.tolist()
    ol = order.tolist()
    for e in ol:
        a, b = find(el[e][0]), find(el[e][1])
        if a == b:
            continue
        c = cl[e]
        if c < min(cint[a] + k / size[a], cint[b] + k / size[b]):
            r = min(a, b)
            s = size[a] + size[b]
            parent[a] = parent[b] = r
            size[r], cint[r] = s, c
    for e in ol:
        a, b = find(el[e][0]), find(el[e][1])
        if a == b:
            continue
        if size[a] < min_size or size[b] < min_size:
            r = min(a, b)
            s = size[a] + size[b]
            parent[a] = parent[b] = r
            size[r] = s
    roots = np.array([find(i) for i in range(n)], dtype=np.int64)
    _, labels = np.unique(roots, return_inverse=True)
    return labels.reshape(rows, cols)


def felzenszwalb(img_u8: np.ndarray, scale: float = 100.0, sigma: float = 0.5, min_size: int = 5) -> np.ndarray:
    """Labels 0..n-1 of a uint8 [H, W, C] image."""
    x = img_u8.astype(np.float64) * (1.0 / 255.0)
    sm = gaussian_smooth(x, sigma)
    return felzenszwalb_merge(img_u8.shape[0], img_u8.shape[1], edge_costs(sm), float(scale) / 255.0, min_size)


def keep_large(labels: np.ndarray, seg_rows: int, seg_cols: int) -> np.ndarray:
    """extract_superpixel's relabel loop (extract_superpixel.py:64-71):
    label 0 is left alone; every other label with more than
    seg_rows * seg_cols / 128 pixels is renumbered 1, 2, ... in label order,
    the rest become 0."""
    counts = np.bincount(labels.ravel(), minlength=labels.max() + 1)
    keep = counts * 128 > seg_rows * seg_cols
    new = np.zeros(len(counts), dtype=np.int64)
    n = 1
    for i in range(1, len(counts)):
        if keep[i]:
            new[i] = n
            n += 1
    return new[labels]


def extract_superpixel(image: np.ndarray, seg_rows: int = 288, seg_cols: int = 384, scale: float = 100.0,
                       sigma: float = 0.5, min_size: int = 5) -> np.ndarray:
    """extract_superpixel.py:55-74 on a uint8 [H, W, 3] image: int [H, W]."""
    H, W = image.shape[:2]
    small = resize_linear(image, seg_rows, seg_cols)
    seg = keep_large(felzenszwalb(small, scale, sigma, min_size), seg_rows, seg_cols)
    return resize_nearest(seg, H, W)


# --------------------------------------------------------------- seg_func --
def _window_reduce(a: np.ndarray, size: int, fn) -> np.ndarray:
    lo, hi = -(size // 2), size - 1 - size // 2
    out = a.copy()
    for axis in (1, 0):
        m = np.moveaxis(out, axis, 0)
        n = m.shape[0]
        res = m.copy()
        for k in range(lo, hi + 1):
            if k == 0:
                continue
            src = np.clip(np.arange(n) + k, 0, n - 1)  # repeating the edge changes no max / min
            res = fn(res, m[src])
        out = np.moveaxis(res, 0, axis)
    return out


def close(seg: np.ndarray, size: int = 11) -> np.ndarray:
    return _window_reduce(_window_reduce(seg, size, np.maximum), size, np.minimum)


def box_mean(a: np.ndarray, wlen: int) -> np.ndarray:
    lo, hi = -(wlen // 2), wlen - 1 - wlen // 2
    ix = _reflect_indices(a.shape[1], lo, hi)
    s = a[:, ix[:, 0]]
    for k in range(1, ix.shape[1]):
        s = s + a[:, ix[:, k]]
    iy = _reflect_indices(a.shape[0], lo, hi)
    t = s[iy[:, 0]]
    for k in range(1, iy.shape[1]):
        t = t + s[iy[:, k]]
    return t * (1.0 / (wlen * wlen))


def win_var(gray: np.ndarray, wlen: int = 3) -> np.ndarray:
    """winVar (extract_superpixel.py:47-52) on float64 [H, W]."""
    m1 = box_mean(gray, wlen)
    m2 = box_mean(gray * gray, wlen)
    return np.sqrt(np.abs(m2 - m1 * m1))


def segment_ids(image: np.ndarray, gray_u8: np.ndarray, mask=None, var_windlen: int = 15, var_thresh: float = 0.2,
                seg_rows: int = 288, seg_cols: int = 384, scale: float = 100.0, sigma: float = 0.5,
                min_size: int = 5, close_size: int = 11):
    """seg_func (extract_superpixel.py:77-113) without its file IO: returns
    (segment_ids_map, segment_ids uint8, var_map float32 or None)."""
    seg = extract_superpixel(image, seg_rows, seg_cols, scale, sigma, min_size)
    ids = (close(seg, close_size) & 255).astype(np.uint8)
    if mask is not None:
        h, w = mask.shape
        ids = np.where(mask, ids, 0).astype(np.uint8)
        present = np.unique(ids)
        for sid in present[1:]:
            area = ids == sid
            if int(area.sum()) * 128 < h * w:
                ids[area] = 0
    if var_thresh > 0.0 and var_windlen > 1:
        v = win_var(gray_u8.astype(np.float64) / 255.0, var_windlen)
        with np.errstate(invalid="ignore", divide="ignore"):
            vm = (v / v.max()).astype(np.float32)
        return np.where(vm < np.float32(var_thresh), ids, 0).astype(np.int32), ids, vm
    return ids, ids, None
