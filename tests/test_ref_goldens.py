"""Pins the oracle (CPU) and the CUDA path (GPU) to golden vectors produced
by the reference's own module-B kernels (tests/golden/make_ref_goldens.py)."""

import os

import numpy as np
import pytest

from gmvs_gb300 import synthetic

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "ref_goldens.npz")

# The reference chains the homography in fp32; the oracle forms it in FP64
# (like the CUDA path).  Well-conditioned costs agree within 1e-4; windows
# whose source variance is near the 1e-5 floor amplify fp32 rounding (the
# reference's own fp32 result differs from its FP64 evaluation by up to
# 3.6e-4 there), so the bound is 1e-4 on 99.9% of the pixels and the FP64
# bound 1e-3 everywhere.
NCC_TOL, NCC_FRAC, NCC_MAX = 1e-4, 0.999, 1e-3


def assert_ncc_close(c, ref):
    err = np.abs(c - ref)
    assert np.mean(err <= NCC_TOL) >= NCC_FRAC, f"{np.mean(err <= NCC_TOL):.5f} within {NCC_TOL}"
    assert err.max() <= NCC_MAX, f"max {err.max():.3g}"


@pytest.fixture(scope="module")
def golden():
    if not os.path.exists(GOLDEN):
        pytest.skip("reference goldens not generated")
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_ref_goldens import golden_inputs
    return dict(np.load(GOLDEN)), golden_inputs()


def _cams(sc, ids):
    return [synthetic.camera_args(sc, i) for i in ids]


def _oracle_init_cost(orc, sc, hyp_d, hyp_n, src):
    ids = [0] + list(src)
    p = orc.make_params(sampler=0, init_kind=2, sweep_kind=2, max_iterations=0,
                        depth_min=sc.depth_range[0] * 0.6, depth_max=sc.depth_range[1] * 1.2)
    _, _, c, _ = orc.run_pass(_cams(sc, ids), sc.images[ids].astype(np.float32), p, depths=hyp_d[ids],
                              ref_normal=hyp_n[0])
    return c


@pytest.mark.parametrize("j", [1, 2, 3, 4])
def test_oracle_ncc_matches_reference(orc, golden, j):
    g, (sc, hyp_d, hyp_n, _, _) = golden
    c = _oracle_init_cost(orc, sc, hyp_d, hyp_n, [j])
    assert_ncc_close(c, g[f"ncc_view{j}"])


def test_oracle_initial_cost_matches_reference(orc, golden):
    g, (sc, hyp_d, hyp_n, _, _) = golden
    c = _oracle_init_cost(orc, sc, hyp_d, hyp_n, [1, 2, 3, 4])
    assert_ncc_close(c, g["ncc_all"])


def _agree(d, n, gd, gn):
    ok_d = np.abs(d - gd) <= 0.005 * np.abs(gd)
    cos = np.sum(n * gn, -1) / np.maximum(np.linalg.norm(n, axis=-1) * np.linalg.norm(gn, axis=-1), 1e-12)
    return float(np.mean(ok_d & (np.degrees(np.arccos(np.clip(cos, -1, 1))) <= 1.0)))


def test_oracle_geom_pass_close_to_reference(orc, golden):
    """Different random streams (Philox vs curand XORWOW) make pixel
    trajectories differ, so the comparison is statistical: the same accuracy
    against ground truth (within one percentage point) and most pixels
    agreeing (measured: 89.91% vs 89.93% of the pixels within 0.5% of ground
    truth, 94.7% agreement)."""
    g, (sc, _, _, nd, nn) = golden
    ids = [0, 1, 2, 3, 4]
    p = orc.make_params(sampler=0, init_kind=2, sweep_kind=2, max_iterations=2,
                        depth_min=sc.depth_range[0] * 0.6, depth_max=sc.depth_range[1] * 1.2, stream_id=0)
    d, n, c, _ = orc.run_pass(_cams(sc, ids), sc.images[ids].astype(np.float32), p, depths=nd[ids], ref_normal=nn[0])
    gt = sc.depths[0]
    acc = lambda x: float(np.mean(np.abs(x - gt) <= 0.005 * gt))
    assert abs(acc(d) - acc(g["geom_depth"])) <= 0.01
    assert np.mean(np.abs(d - g["geom_depth"]) <= 0.005 * np.abs(g["geom_depth"])) >= 0.9


def check_fusion_against_reference(outs, masks, g, hits):
    """Masks bit-exact, the same fused pixels, and equal values up to the
    reference's FMA rounding except where several reference pixels wrote the
    same output pixel (the reference races there)."""
    assert np.array_equal(masks, g["fuse_masks"])
    for k, (d, h) in enumerate(zip(outs, hits)):
        rd = g[f"fuse_depth{k}"]
        assert np.array_equal(d > 0, rd > 0)
        single = (h == 1) & (rd > 0)
        rel = np.abs(d - rd)[single] / rd[single]
        assert rel.max() <= 1e-5, (k, rel.max())


def test_oracle_fusion_matches_reference(orc, golden):
    g, (sc, _, _, nd, nn) = golden
    V, H, W = nd.shape
    masks = np.zeros((V, H, W), np.uint8)
    outs, hits = [], []
    for k, (ref, src) in enumerate(sc.problems):
        ids = [ref] + src
        d, n, _, h = orc.fuse(_cams(sc, ids), ref, src, nd[ids], nn[ids], masks, 3, with_hits=True)
        outs.append(d)
        hits.append(h)
    check_fusion_against_reference(outs, masks, g, hits)


@pytest.mark.gpu
@pytest.mark.parametrize("j", [1, 2, 3, 4])
def test_cuda_ncc_matches_reference(gmvs_lib, cuda, golden, j):
    import torch
    from gmvs_gb300.src import PatchMatcher, load_camera, load_problem
    g, (sc, hyp_d, hyp_n, _, _) = golden
    pm = PatchMatcher()
    pm.params.max_iterations = 0
    cams = [load_camera(*synthetic.camera_args(sc, i)) for i in range(sc.num_views)]
    probs = [load_problem(0, [j])] + [load_problem(i, [0]) for i in range(1, sc.num_views)]
    pm.add_samples(probs, cams, torch.from_numpy(sc.images.astype(np.float32)), torch.from_numpy(hyp_d),
                   torch.from_numpy(hyp_n), torch.zeros(sc.images.shape))
    _, _, c = pm.run_patch_match(0, False)
    assert_ncc_close(c.cpu().numpy(), g[f"ncc_view{j}"])


@pytest.mark.gpu
def test_cuda_fusion_matches_reference(gmvs_lib, orc, cuda, golden):
    import torch
    from gmvs_gb300.src import Fuser, load_camera, load_problem
    g, (sc, _, _, nd, nn) = golden
    V, H, W = nd.shape
    cams = [load_camera(*synthetic.camera_args(sc, i)) for i in range(V)]
    probs = [load_problem(r, s) for r, s in sc.problems]
    masks = torch.zeros((V, H, W), dtype=torch.bool, device=cuda)
    fu = Fuser()
    fu.load_samples(probs, cams, torch.from_numpy(nd), torch.from_numpy(nn), masks)
    outs = [fu.run_fusion(k, 3)[0].cpu().numpy() for k in range(V)]
    om = np.zeros((V, H, W), np.uint8)
    hits = []
    for ref, src in sc.problems:
        ids = [ref] + src
        hits.append(orc.fuse(_cams(sc, ids), ref, src, nd[ids], nn[ids], om, 3, with_hits=True)[3])
    check_fusion_against_reference(outs, masks.cpu().numpy().astype(np.uint8), g, hits)
