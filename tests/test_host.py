"""Host-side product code that runs without a GPU: the C ABI loads and
exports every declared symbol, the defaults match the reference, and the
CPU routines (planar prior, Delaunay, segmentation helpers) equal the oracle."""

import os
import re

import numpy as np
import pytest

from gmvs_gb300 import _abi, imageio, synthetic

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            names += re.findall(r"GMVS_API\s+[\w\s\*]+?\b(gmvs_\w+)\s*\(", open(os.path.join(ROOT, "include", f)).read())
    return sorted(set(names))


def test_library_exports_every_declared_symbol(gmvs_lib):
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(gmvs_lib, n), n
    # every declared entry point is bound with a signature in _abi, and the
    # binding declares nothing the header does not
    assert set(names) == set(_abi.EXPORTED)


def test_struct_layouts():
    import ctypes
    assert ctypes.sizeof(_abi.gmvs_camera) == 100
    assert ctypes.sizeof(_abi.gmvs_problem) == 136


def test_default_params_match_reference(gmvs_lib):
    p = _abi.default_params()
    # PatchMatchParams defaults (gmvs/lib/include/planar_initer.hpp:13-31)
    assert (p.max_iterations, p.patch_size, p.num_images, p.max_image_size, p.radius_increment) == (3, 11, 5, 3200, 2)
    assert (p.sigma_spatial, p.sigma_color, p.top_k) == (5.0, 3.0, 4)
    assert abs(p.baseline - 0.54) < 1e-7 and (p.depth_min, p.depth_max) == (0.0, 1.0)
    assert (p.geom_consistency, p.multi_geometry, p.planar_prior, p.superpixel_filter) == (0, 0, 0, 0)
    assert p.seed == 3407


def test_errors_are_reported(gmvs_lib):
    from gmvs_gb300.planar_initer import fusion_planar_mask
    with pytest.raises(ValueError):
        fusion_planar_mask(np.zeros((3, 3), np.int32), np.zeros((3, 4), np.int32), np.zeros((3, 3, 3), np.float32),
                           3, 3)
    # a NULL argument is rejected by the library with a message
    rc = gmvs_lib.gmvs_filter_by_var_map(None, None, 2, 2, 1.0, None)
    assert rc == _abi.ERR_INVALID
    assert b"NULL" in gmvs_lib.gmvs_last_error()


def _pass1_like(small, rng):
    ref = 0
    H, W = small.hw
    depth = (small.depths[ref] * (1 + rng.normal(0, 0.002, (H, W)))).astype(np.float32)
    cost = rng.uniform(0.0, 0.3, (H, W)).astype(np.float32)
    cost[rng.random((H, W)) < 0.05] = 2.0
    return depth, cost


@pytest.mark.parametrize("spfilter", [False, True])
def test_planar_prior_equals_oracle(gmvs_lib, orc, small, spfilter):
    from gmvs_gb300.planar_initer import build_planar_prior
    from gmvs_gb300.engine import make_camera
    rng = np.random.default_rng(0)
    depth, cost = _pass1_like(small, rng)
    args = synthetic.camera_args(small, 0)
    gp, gm, gt = build_planar_prior(make_camera(*args), depth, cost, small.superpixels[0], spfilter, 0.3, 6.0)
    op, om, ot = orc.build_prior(args, depth, cost, small.superpixels[0], spfilter, 0.3, 6.0)
    assert len(gt) == len(ot) > 100
    assert np.array_equal(gt, ot)
    assert np.array_equal(gm, om)
    assert np.array_equal(gp, op)
    assert (gm > 0).mean() > 0.3


def test_delaunay_is_delaunay(orc):
    rng = np.random.default_rng(3)
    # jittered 5-pixel grid, like the support points, with many co-circular quads
    g = np.stack(np.meshgrid(np.arange(0, 200, 5), np.arange(0, 150, 5)), -1).reshape(-1, 2)
    pts = (g + rng.integers(0, 2, g.shape)).astype(np.int64)
    tris = orc.delaunay(pts, 200)
    P = pts.astype(np.float64)
    a, b, c = P[tris[:, 0]], P[tris[:, 1]], P[tris[:, 2]]
    # every triangle is counter-clockwise and non-degenerate
    area = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    assert (area > 0).all()
    # empty circumcircle (no point strictly inside), checked on a sample
    for k in rng.choice(len(tris), 200, replace=False):
        A, B, C = P[tris[k]]
        m = np.array([[A[0] - p[0], A[1] - p[1], (A[0] - p[0]) ** 2 + (A[1] - p[1]) ** 2,
                       B[0] - p[0], B[1] - p[1], (B[0] - p[0]) ** 2 + (B[1] - p[1]) ** 2,
                       C[0] - p[0], C[1] - p[1], (C[0] - p[0]) ** 2 + (C[1] - p[1]) ** 2] for p in P])
        det = (m[:, 0] * (m[:, 4] * m[:, 8] - m[:, 5] * m[:, 7]) - m[:, 1] * (m[:, 3] * m[:, 8] - m[:, 5] * m[:, 6])
               + m[:, 2] * (m[:, 3] * m[:, 7] - m[:, 4] * m[:, 6]))
        assert (det <= 1e-6).all()


def test_segmentation_helpers_equal_oracle(gmvs_lib, orc):
    from gmvs_gb300 import planar_initer as pi
    rng = np.random.default_rng(7)
    rows, cols = 60, 80
    seg = rng.integers(0, 9, (rows, cols)).astype(np.int32)
    seg[:30, :40] = 3
    planar = (rng.random((rows, cols)) < 0.3).astype(np.int32)
    n = rng.normal(size=(rows, cols, 3)).astype(np.float32)
    n[:30, :40] = [0, 0, 1]
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    for th in (10, 100):
        assert np.array_equal(pi.fusion_planar_mask(seg, planar, n, rows, cols, th),
                              orc.fusion_planar_mask(seg, planar, n, rows, cols, th))
    var = rng.random((rows, cols)).astype(np.float32)
    assert np.array_equal(pi.filter_by_var_map(var, seg, 0.5), orc.filter_by_var_map(var, seg, 0.5))
    for win in (3, 5):
        assert np.array_equal(pi.sliding_window_normal(planar, n, win), orc.sliding_window_normal(planar, n, win))


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    g = rng.integers(0, 256, (37, 53), dtype=np.uint8)
    c = rng.integers(0, 256, (21, 19, 3), dtype=np.uint8)
    imageio.write_png(str(tmp_path / "g.jpg"), g)
    imageio.write_png(str(tmp_path / "c.png"), c)
    assert np.array_equal(imageio.imread_gray(str(tmp_path / "g.jpg")), g)
    assert np.array_equal(imageio.read_png(str(tmp_path / "c.png")), c)


def _read_camera(path):
    # restates gmvs/consistency.py:13-24
    tok = open(path).read().split()
    E = np.array([float(x) for x in tok[1:17]]).reshape(4, 4)
    return [float(x) for x in tok[18:27]], E[:3, :3].reshape(9).tolist(), E[:3, 3].tolist(), \
        (float(tok[27]), float(tok[30]))


def _read_pairs(path):
    # restates gmvs/scripts/launch.py:22-50
    lines = open(path).read().split("\n")
    out = []
    for i in range(int(lines[0])):
        ref = int(lines[i * 2 + 1])
        s = lines[i * 2 + 2].split(" ")
        out.append((ref, [int(s[j * 2 + 1]) for j in range(int(s[0])) if float(s[j * 2 + 2]) >= 0]))
    return out


def test_scene_files_use_reference_layout(tmp_path, small):
    synthetic.write_scene(small, str(tmp_path))
    K, R, t, (dmin, dmax) = _read_camera(str(tmp_path / "cams" / "0002_cam.txt"))
    assert np.allclose(np.array(K).reshape(3, 3), small.K[2]) and np.allclose(np.array(R).reshape(3, 3), small.R[2])
    assert np.allclose(t, small.t[2]) and (dmin, dmax) == small.depth_range
    assert _read_pairs(str(tmp_path / "pair.txt")) == small.problems
    assert np.array_equal(imageio.imread_gray(str(tmp_path / "images" / "0003.jpg")), small.images[3])
    assert np.load(str(tmp_path / "superpixels" / "0001.npy")).dtype == np.uint8


def test_launch_parameters_are_validated_on_the_host(gmvs_lib):
    """gmvs_plan_workspace_bytes rejects launch parameters out of range before
    any CUDA call (0 bytes and a message): the half-sweep split (0, 1 or 2
    kernels after the first), the tile width and the tile height."""
    import ctypes

    view = (_abi.gmvs_view_pass * 1)()
    for field, value, words in (("split_sweep", 3, b"split_sweep must be 0, 1 or 2"),
                                ("tile_w", 24, b"tile_w must be 0, 16 or 32"),
                                ("tile_h", 9, b"tile_h must be in [0, 8]")):
        p = _abi.default_params()
        setattr(p, field, value)
        assert gmvs_lib.gmvs_plan_workspace_bytes(view, 1, ctypes.byref(p)) == 0
        assert words in gmvs_lib.gmvs_last_error()
