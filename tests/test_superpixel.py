"""Superpixel extraction (extract_superpixel.py): the oracle pinned against
SciPy where SciPy implements the step, the library's host merge against the
oracle on the CPU, and the device pipeline against the oracle bit for bit."""

import ctypes
import os

import numpy as np
import pytest

from gmvs_gb300 import _abi
from gmvs_gb300.synthetic import indoor_image
from oracle import superpixel as osp

ndi = pytest.importorskip("scipy.ndimage")


# ------------------------------------------------------------ oracle pins --
@pytest.mark.parametrize("shape", [(37, 53, 3), (5, 4, 3), (64, 80, 3)])
def test_oracle_gaussian_equals_scipy(shape):
    x = np.random.default_rng(1).integers(0, 256, shape).astype(np.float64) * (1.0 / 255.0)
    assert np.array_equal(osp.gaussian_smooth(x, 0.5), ndi.gaussian_filter(x, sigma=[0.5, 0.5, 0]))


def test_oracle_close_equals_scipy():
    lbl = np.random.default_rng(2).integers(0, 40, (50, 61))
    for size in (1, 3, 11):
        assert np.array_equal(osp.close(lbl, size), ndi.grey_closing(lbl, size=(size, size), mode="nearest"))


def test_oracle_box_filter_matches_scipy():
    g = np.random.default_rng(3).random((40, 33))
    for wlen in (3, 15):
        assert np.abs(osp.box_mean(g, wlen) - ndi.uniform_filter(g, wlen, mode="reflect")).max() < 1e-14
    # window larger than the image: repeated reflection
    assert np.abs(osp.box_mean(g[:5, :6], 15) - ndi.uniform_filter(g[:5, :6], 15, mode="reflect")).max() < 1e-14


def test_oracle_resize_properties():
    rng = np.random.default_rng(4)
    img = rng.integers(0, 256, (48, 64, 3)).astype(np.uint8)
    assert np.array_equal(osp.resize_linear(img, 48, 64), img)  # identity
    flat = np.full((97, 131, 3), 77, np.uint8)
    assert np.array_equal(osp.resize_linear(flat, 30, 41), np.full((30, 41, 3), 77, np.uint8))
    half = osp.resize_linear(img, 24, 32)  # exact 2x: rounded 2 x 2 means
    x = img.astype(np.int64)
    assert np.array_equal(half, ((x[0::2, 0::2] + x[0::2, 1::2] + x[1::2, 0::2] + x[1::2, 1::2] + 2) >> 2))
    up = osp.resize_nearest(np.arange(12).reshape(3, 4), 6, 8)
    assert np.array_equal(up, np.repeat(np.repeat(np.arange(12).reshape(3, 4), 2, 0), 2, 1))


def test_oracle_resize_matches_torch_bilinear():
    """The restated INTER_LINEAR resize against torch's bilinear
    interpolation with the same pixel-centre mapping (align_corners=False,
    no antialiasing): within one grey level everywhere (the restatement
    rounds 11-bit fixed-point weights, torch interpolates in float), which
    pins the coordinate mapping and the border handling."""
    import torch

    rng = np.random.default_rng(6)
    for (h, w), (oh, ow) in (((1200, 1600), (288, 384)), ((97, 131), (288, 384)), ((50, 61), (33, 47))):
        img = rng.integers(0, 256, (h, w, 3)).astype(np.uint8)
        ours = osp.resize_linear(img, oh, ow).astype(np.float64)
        t = torch.from_numpy(img.astype(np.float64)).permute(2, 0, 1)[None]
        ref = torch.nn.functional.interpolate(t, size=(oh, ow), mode="bilinear", align_corners=False,
                                              antialias=False)[0].permute(1, 2, 0).numpy()
        assert np.abs(ours - ref).max() <= 1.0, (h, w, np.abs(ours - ref).max())
        assert np.abs(ours - ref).mean() <= 0.3


def test_oracle_segments_are_connected_and_large_enough():
    bgr, _ = indoor_image(60, 80, 5)
    lab = osp.felzenszwalb(bgr, 100.0, 0.5, 20)
    counts = np.bincount(lab.ravel())
    assert counts.min() >= 20
    for k in range(lab.max() + 1):
        comp, n = ndi.label(lab == k, structure=np.ones((3, 3)))
        assert n == 1
    # labels are numbered by first pixel in raster order
    first = [np.flatnonzero(lab.ravel() == k)[0] for k in range(lab.max() + 1)]
    assert first == sorted(first)


# ------------------------------------------------------ host merge (C ABI) --
def _host_labels(rows, cols, w, scale=100.0, min_size=5):
    out = np.zeros((rows, cols), np.int32)
    kept = ctypes.c_int32()
    rc = _abi.lib().gmvs_superpixel_labels_host(rows, cols, w.ctypes.data, scale, min_size, out.ctypes.data,
                                                ctypes.byref(kept))
    assert rc == 0, _abi.lib().gmvs_last_error()
    return out, kept.value


@pytest.mark.parametrize("rows,cols,seed,quant", [(96, 128, 0, None), (40, 70, 1, 8.0), (1, 57, 2, None),
                                                  (33, 1, 3, 4.0), (1, 1, 4, None), (61, 47, 5, 2.0)])
def test_host_merge_equals_oracle(gmvs_lib, rows, cols, seed, quant):
    if rows * cols > 1:
        bgr, _ = indoor_image(max(rows, 8), max(cols, 8), seed)
        sm = osp.gaussian_smooth(bgr[:rows, :cols].astype(np.float64) * (1.0 / 255.0), 0.5)
        w = osp.edge_costs(sm)
    else:
        w = np.zeros(0)
    if quant:  # many equal weights: the tie order decides
        w = np.rint(w * quant) / quant
    w = np.ascontiguousarray(w, dtype=np.float64)
    for scale, min_size in ((100.0, 5), (300.0, 20), (0.0, 0)):
        want = osp.keep_large(osp.felzenszwalb_merge(rows, cols, w, scale / 255.0, min_size), rows, cols)
        got, kept = _host_labels(rows, cols, w if w.size else np.zeros(1), scale, min_size)
        assert np.array_equal(got, want)
        assert kept == want.max()


def test_host_merge_rejects_bad_weights(gmvs_lib):
    w = np.zeros(4 * 3 + 3 * 4 + 2 * 9)
    w[3] = np.nan
    out = np.zeros((4, 4), np.int32)
    assert _abi.lib().gmvs_superpixel_labels_host(4, 4, w.ctypes.data, 100.0, 5, out.ctypes.data, None) != 0
    w[3] = -1.0
    assert _abi.lib().gmvs_superpixel_labels_host(4, 4, w.ctypes.data, 100.0, 5, out.ctypes.data, None) != 0


def test_params_and_workspace_validation(gmvs_lib):
    from gmvs_gb300 import superpixel as sp

    p = sp.default_params()
    assert (p.seg_rows, p.seg_cols, p.scale, p.sigma, p.min_size, p.close_size, p.var_windlen) == \
        (288, 384, 100.0, 0.5, 5, 11, 15)
    assert abs(p.var_thresh - 0.2) < 1e-7
    L = _abi.lib()
    assert L.gmvs_superpixel_workspace_bytes(1200, 1600, ctypes.byref(p)) > 1200 * 1600 * 8
    for bad in (dict(close_size=10), dict(sigma=5.0), dict(seg_rows=0), dict(min_size=-1)):
        assert L.gmvs_superpixel_workspace_bytes(64, 64, ctypes.byref(sp.default_params(**bad))) == 0


# ------------------------------------------------------------ device path --
def _oracle_all(bgr, gray, mask=None, **kw):
    p = dict(seg_rows=288, seg_cols=384, var_windlen=15, var_thresh=0.2)
    p.update(kw)
    seg = osp.extract_superpixel(bgr, p["seg_rows"], p["seg_cols"])
    ids_map, ids, vm = osp.segment_ids(bgr, gray, mask, **p)
    return seg, ids_map, ids, vm


CASES = [
    # rows, cols, seg_rows, seg_cols, seed: linear down, exact 2x (area), upscale, odd sizes
    (240, 320, 96, 128, 0),
    (192, 256, 96, 128, 1),
    (60, 80, 96, 128, 2),
    (157, 203, 71, 93, 3),
]


@pytest.mark.gpu
@pytest.mark.parametrize("rows,cols,sr,sc,seed", CASES)
def test_device_superpixels_equal_oracle(gmvs_lib, cuda, rows, cols, sr, sc, seed):
    from gmvs_gb300 import superpixel as sp

    bgr, gray = indoor_image(rows, cols, seed)
    ex = sp.Extractor(cuda, sp.default_params(seg_rows=sr, seg_cols=sc))
    out = ex.run(bgr, gray)
    seg, ids_map, ids, vm = _oracle_all(bgr, gray, seg_rows=sr, seg_cols=sc)
    assert np.array_equal(out["segment"].cpu().numpy(), seg)
    assert out["num_segments"] == seg.max() > 0
    assert np.array_equal(out["ids"].cpu().numpy(), ids)
    assert np.array_equal(out["var_map"].cpu().numpy(), vm)
    assert np.array_equal(out["ids_map"].cpu().numpy(), ids_map)
    assert 0 < (ids_map > 0).mean() < 1


@pytest.mark.gpu
def test_device_superpixels_full_size_default(gmvs_lib, cuda):
    from gmvs_gb300 import superpixel as sp

    bgr, gray = indoor_image(1200, 1600, 7)
    ids_map, ids = sp.segment_ids(bgr, gray)
    seg, want_map, want_ids, _ = _oracle_all(bgr, gray)
    assert np.array_equal(ids, want_ids) and np.array_equal(ids_map, want_map)
    assert np.array_equal(sp.extract_superpixel(bgr), seg)


@pytest.mark.gpu
def test_device_superpixels_mask_and_filter_off(gmvs_lib, cuda):
    from gmvs_gb300 import superpixel as sp

    bgr, gray = indoor_image(240, 320, 8)
    mask = np.ones((240, 320), bool)
    mask[:, :100] = False
    mask[200:, :] = False
    p = dict(seg_rows=96, seg_cols=128)
    ex = sp.Extractor(cuda, sp.default_params(**p))
    out = ex.run(bgr, gray, mask)
    _, ids_map, ids, _ = _oracle_all(bgr, gray, mask, **p)
    assert np.array_equal(out["ids"].cpu().numpy(), ids) and np.array_equal(out["ids_map"].cpu().numpy(), ids_map)
    # variance filter off: the ids themselves
    ex = sp.Extractor(cuda, sp.default_params(var_thresh=-1.0, **p))
    out = ex.run(bgr, None, None, outputs=("ids", "ids_map"))
    _, ids_map, ids, vm = _oracle_all(bgr, gray, None, var_thresh=-1.0, **p)
    assert vm is None and np.array_equal(out["ids"].cpu().numpy(), ids)
    assert np.array_equal(out["ids_map"].cpu().numpy(), ids.astype(np.int32))


@pytest.mark.gpu
def test_device_superpixels_flat_image(gmvs_lib, cuda):
    """One segment (label 0).  A flat gray level of 128 leaves rounding
    residue in E[g^2] - E[g]^2 (the same everywhere: the map is 1); a black
    image has an exact zero maximum and 0 / 0 passes nothing."""
    from gmvs_gb300 import superpixel as sp

    bgr = np.full((64, 80, 3), 128, np.uint8)
    ex = sp.Extractor(cuda, sp.default_params(seg_rows=32, seg_cols=40))
    for level in (128, 0):
        gray = np.full((64, 80), level, np.uint8)
        out = ex.run(bgr, gray)
        _, ids_map, ids, vm = _oracle_all(bgr, gray, seg_rows=32, seg_cols=40)
        assert out["num_segments"] == 0 and int(out["ids"].max()) == 0 and int(out["ids_map"].max()) == 0
        assert np.array_equal(out["var_map"].cpu().numpy(), vm, equal_nan=True)
    assert bool(out["var_map"].isnan().all())


@pytest.mark.gpu
def test_seg_func_files_and_threads(gmvs_lib, cuda, tmp_path):
    from gmvs_gb300 import superpixel as sp
    from gmvs_gb300.imageio import write_png

    imgs = [indoor_image(120, 160, s) for s in range(4)]
    path = os.path.join(tmp_path, "0000.png")
    write_png(path, np.ascontiguousarray(imgs[0][0][..., ::-1]))  # stored RGB, read back BGR
    npy = sp.seg_func(path, str(tmp_path))
    assert np.array_equal(sp.read_bgr(path), imgs[0][0])
    from gmvs_gb300.imageio import imread_gray

    want, _ = sp.segment_ids(imgs[0][0], imread_gray(path))
    assert np.array_equal(np.load(npy), want)
    seq = [sp.segment_ids(b, g) for b, g in imgs]
    par = sp.extract_many([b for b, _ in imgs], [g for _, g in imgs], workers=3)
    for (a0, a1), (b0, b1) in zip(seq, par):
        assert np.array_equal(a0, b0) and np.array_equal(a1, b1)
    # var_thresh2: the device filter_by_var_map on the device var map
    m2, _ = sp.segment_ids(imgs[1][0], imgs[1][1], var_thresh2=0.1)
    m1, _ = sp.segment_ids(imgs[1][0], imgs[1][1])
    assert set(np.unique(m2)) <= set(np.unique(m1))


def test_superpixels_rejects_bad_arguments_before_any_device_work(gmvs_lib):
    """NULL image, missing gray with the variance filter on, bad parameters
    and a short workspace fail with GMVS_ERR_INVALID before any CUDA call."""
    from gmvs_gb300 import superpixel as sp

    L = _abi.lib()
    p = sp.default_params()
    fake = 1 << 20  # never dereferenced: every case fails validation first
    big = L.gmvs_superpixel_workspace_bytes(64, 64, ctypes.byref(p))
    cases = [
        (None, fake, 64, 64, p, fake, big),          # NULL image
        (fake, None, 64, 64, p, fake, big),          # filter on, ids_map wanted, no gray
        (fake, fake, 0, 64, p, fake, big),           # empty image
        (fake, fake, 64, 64, sp.default_params(close_size=4), fake, big),
        (fake, fake, 64, 64, p, fake, big // 2),     # workspace too small
        (fake, fake, 64, 64, p, None, big),          # NULL workspace
    ]
    for img, gray, rows, cols, prm, ws, nbytes in cases:
        rc = L.gmvs_superpixels(img, gray, None, rows, cols, ctypes.byref(prm), None, None, fake, None, None, ws,
                                nbytes, None)
        assert rc == _abi.ERR_INVALID, L.gmvs_last_error()


def test_read_bgr_and_gray_conversion(tmp_path):
    """cv2.imread's BGR order and gray images read back as three equal
    channels; the gray conversion is libpng's, as imread_gray."""
    from gmvs_gb300 import superpixel as sp
    from gmvs_gb300.imageio import imread_gray, write_png

    rng = np.random.default_rng(9)
    rgb = rng.integers(0, 256, (13, 17, 3)).astype(np.uint8)
    p = os.path.join(tmp_path, "c.png")
    write_png(p, rgb)
    bgr = sp.read_bgr(p)
    assert np.array_equal(bgr, rgb[..., ::-1])
    assert np.array_equal(sp.bgr_to_gray(bgr), imread_gray(p))
    g = rng.integers(0, 256, (9, 11)).astype(np.uint8)
    q = os.path.join(tmp_path, "g.png")
    write_png(q, g)
    assert np.array_equal(sp.read_bgr(q), np.repeat(g[..., None], 3, axis=2))


def test_png_gray_transform():
    """libpng's 8-bit RGB -> gray weights (1/32768: 9797, 19234, 3737) and its
    truncating shift, checked by hand on a few triples; equal channels pass
    through unchanged; a colour PNG with a gAMA chunk needs OpenCV."""
    from gmvs_gb300.imageio import PNG_GRAY_BLUE, PNG_GRAY_GREEN, PNG_GRAY_RED, png_rgb_to_gray

    assert (PNG_GRAY_RED, PNG_GRAY_GREEN, PNG_GRAY_BLUE) == (9797, 19234, 3737)
    rgb = np.array([[255, 0, 0], [0, 255, 0], [0, 0, 255], [10, 200, 30], [255, 255, 254]], np.uint8)
    want = [(9797 * 255) >> 15, (19234 * 255) >> 15, (3737 * 255) >> 15,
            (9797 * 10 + 19234 * 200 + 3737 * 30) >> 15, (9797 * 255 + 19234 * 255 + 3737 * 254) >> 15]
    assert png_rgb_to_gray(rgb[:, 0], rgb[:, 1], rgb[:, 2]).tolist() == want == [76, 149, 29, 123, 254]
    v = np.arange(256, dtype=np.uint8)
    assert np.array_equal(png_rgb_to_gray(v, v, v), v)


def test_extract_superpixel_rejects_weights():
    from gmvs_gb300 import superpixel as sp

    with pytest.raises(NotImplementedError):
        sp.extract_superpixel(np.zeros((4, 4, 3), np.uint8), weight=np.ones((4, 4, 3)))
