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


def assert_ncc_close(c, ref, exact=None):
    """Within NCC_TOL on NCC_FRAC of the pixels; elsewhere within NCC_MAX or,
    given the FP64 costs `exact`, closer to them than the reference is."""
    err = np.abs(c - ref)
    assert np.mean(err <= NCC_TOL) >= NCC_FRAC, f"{np.mean(err <= NCC_TOL):.5f} within {NCC_TOL}"
    if exact is None:
        assert err.max() <= NCC_MAX, f"max {err.max():.3g}"
    else:
        far = err > NCC_TOL
        assert np.all(np.abs(c - exact)[far] <= np.abs(ref - exact)[far]), "an outlier is not the reference's"


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


def test_oracle_ncc_outliers_are_reference_rounding(orc, golden):
    """Where this path and the reference differ by more than 1e-4, this
    path is the one closer to the FP64 evaluation of the same window (the
    reference chains the homography in fp32)."""
    g, (sc, hyp_d, hyp_n, _, _) = golden
    ids = [0, 1, 2, 3, 4]
    cams = _cams(sc, ids)
    imgs = sc.images[ids].astype(np.float32)
    # the camera-frame hypotheses module B forms from (depth, world normal)
    # (TransformNormal2RefCam, GetDistance2Origin: patch_match.cu:97-134, 329-339)
    R = sc.R[0].astype(np.float32)
    n_c = np.einsum("ij,hwj->hwi", R, hyp_n[0]).astype(np.float32)
    K = sc.K[0].astype(np.float32)
    ys, xs = np.mgrid[0:sc.hw[0], 0:sc.hw[1]]
    X0 = (hyp_d[0] * (xs.astype(np.float32) - K[0, 2])) / K[0, 0]
    X1 = (hyp_d[0] * (ys.astype(np.float32) - K[1, 2])) / K[1, 1]
    w = -((n_c[..., 0] * X0 + n_c[..., 1] * X1) + n_c[..., 2] * hyp_d[0])
    pl = np.concatenate([n_c, w[..., None]], -1).astype(np.float32)
    ours, _, _ = orc.ncc_costs(cams, imgs, pl, orc.make_params(sampler=0))
    exact, _, _ = orc.ncc_costs(cams, imgs, pl, orc.make_params(sampler=0), fp64=True)
    n_out = 0
    for j in (1, 2, 3, 4):
        ref = g[f"ncc_view{j}"]
        far = np.abs(ours[j - 1] - ref) > NCC_TOL
        n_out += int(far.sum())
        assert np.all(np.abs(ours[j - 1] - exact[j - 1])[far] <= np.abs(ref - exact[j - 1])[far]), j
        assert np.abs(ours[j - 1] - exact[j - 1]).max() <= 2.5e-4
    assert n_out <= 0.001 * 4 * ref.size


def _agreement(d, n, gd, gn):
    d, n, gd, gn = (np.asarray(a, np.float64) for a in (d, n, gd, gn))
    ok_d = np.abs(d - gd) <= 0.005 * np.abs(gd)
    cos = np.sum(n * gn, -1) / np.maximum(np.linalg.norm(n, axis=-1) * np.linalg.norm(gn, axis=-1), 1e-12)
    ok_n = np.degrees(np.arccos(np.clip(cos, -1, 1))) <= 1.0
    return float(np.mean(ok_d)), float(np.mean(ok_d & ok_n))


def check_geom_pass(ours, ours_other_seed, g, gt, prefix="geom", margin=0.02):
    """Different random streams (Philox vs curand XORWOW) and the reference's
    own race (two runs of the reference with the same seed differ) make the
    comparison statistical: the same accuracy against ground truth within a
    point, and depth / depth + normal agreement with the reference no lower
    than the agreement that different streams allow — the reference against
    its own rerun, this path against itself with another seed — less
    `margin`."""
    gd, gn = g[f"{prefix}_depth"], g[f"{prefix}_normal"]
    acc = lambda x: float(np.mean(np.abs(np.asarray(x, np.float64) - gt) <= 0.005 * gt))
    assert abs(acc(ours[0]) - acc(gd)) <= 0.01, (acc(ours[0]), acc(gd))
    vs_ref = _agreement(ours[0], ours[1], gd, gn)
    ceil_ours = _agreement(ours_other_seed[0], ours_other_seed[1], ours[0], ours[1])
    ceil_ref = _agreement(g[f"{prefix}_rerun_depth"], g[f"{prefix}_rerun_normal"], gd, gn) \
        if f"{prefix}_rerun_depth" in g else ceil_ours
    for k in (0, 1):
        assert vs_ref[k] >= min(ceil_ours[k], ceil_ref[k]) - margin, (k, vs_ref, ceil_ours, ceil_ref)
    return vs_ref, ceil_ours, ceil_ref


def _oracle_geom(orc, sc, nd, nn, seed):
    ids = [0, 1, 2, 3, 4]
    p = orc.make_params(sampler=0, init_kind=2, sweep_kind=2, max_iterations=2,
                        depth_min=sc.depth_range[0] * 0.6, depth_max=sc.depth_range[1] * 1.2, stream_id=0, seed=seed)
    d, n, _, _ = orc.run_pass(_cams(sc, ids), sc.images[ids].astype(np.float32), p, depths=nd[ids], ref_normal=nn[0])
    return d, n


def test_oracle_geom_pass_close_to_reference(orc, golden):
    g, (sc, _, _, nd, nn) = golden
    check_geom_pass(_oracle_geom(orc, sc, nd, nn, 3407), _oracle_geom(orc, sc, nd, nn, 1), g,
                    sc.depths[0].astype(np.float64))


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
