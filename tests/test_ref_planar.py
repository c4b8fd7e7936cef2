"""Pins the texture path (module A: the random and planar-prior passes of
PlanarInit) to golden vectors from the reference's own module-A kernels,
gmvs/lib/src/patch_match_kernel.cu compiled from the reference sources and
launched with PlanarInit::run_patch_match's sequence
(tests/golden/make_ref_goldens.py, ref_goldens_planar.npz).  The oracle is
checked on the CPU and the CUDA path (through the C ABI) on the GPU.

NCC of given hypotheses.  The reference builds module A with --use_fast_math
(approximate exp, division and square root) and chains the homography in
fp32; the texture unit then quantises each sample's interpolation weights to
8 bits, so a last-bit change of a projected coordinate can move a sample by
up to 1/256 of a grey-level step.  No restatement reproduces the fast-math
rounding, so the bound is statistical: within 1e-4 on >= 97 % of the pixels
per source view and >= 99 % for the top-k initial cost, within 1e-3 on
>= 99.9 %.  The same module built without fast math and without fused
multiply-adds (ref_planar_ieee.cubin) is the reference's operation chain in
IEEE fp32.  The oracle's restatement of that chain (ncc_costs(ref_chain=True))
matches it within 1e-4 on every pixel (median difference 3e-6: the oracle's
exp is its own, not CUDA's expf), which pins the texture emulation and the
NCC arithmetic themselves; and the reference's two builds differ from each
other by more than 1e-4 on 1-1.6 % of the pixels — the same fraction, within
a point, by which this implementation differs from the fast-math build.

Passes.  The random streams differ (Philox here, curand XORWOW there) and
the reference is not even reproducible against itself: it reads same-colour
neighbours while they are rewritten, so two runs of the same seed differ.
Pixel agreement is therefore compared with the ceiling that different
random streams allow — the reference against its own rerun, and this
implementation against itself with another seed — and the accuracy against
ground truth is compared directly.
"""

import os
import sys

import numpy as np
import pytest

from gmvs_gb300 import synthetic

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "ref_goldens_planar.npz")
sys.path.insert(0, os.path.join(HERE, "golden"))

TAGS = ["s", "c1"]
# NCC of given hypotheses against the fast-math module (see the module docstring)
VIEW_TOL, VIEW_FRAC, ALL_FRAC, LOOSE_TOL, LOOSE_FRAC = 1e-4, 0.97, 0.99, 1e-3, 0.999
# the oracle's restatement of the reference's chain against the IEEE build of the same source
IEEE_TOL = 1e-4
# passes: accuracy against ground truth within ACC_TOL, agreement within
# AGREE_MARGIN of the random-stream ceiling
ACC_TOL, AGREE_MARGIN = 0.015, 0.02


@pytest.fixture(scope="module")
def golden():
    if not os.path.exists(GOLDEN):
        pytest.skip("module-A goldens not generated")
    import make_ref_goldens as mrg

    return dict(np.load(GOLDEN)), dict(mrg.planar_scenes()), mrg


def planes_from_depth(sc, ref, depth, n_c):
    """Camera-frame planes (n, w) with w = -(n . X), X = Get3DPoint(depth), in
    the reference's fp32 operation order (GetDistance2Origin,
    patch_match_kernel.cu:86-124)."""
    f32 = np.float32
    K = sc.K[ref].astype(f32)
    H, W = sc.hw
    ys, xs = np.mgrid[0:H, 0:W]
    X0 = (depth * (xs.astype(f32) - K[0, 2])) / K[0, 0]
    X1 = (depth * (ys.astype(f32) - K[1, 2])) / K[1, 1]
    w = -((n_c[..., 0] * X0 + n_c[..., 1] * X1) + n_c[..., 2] * depth)
    return np.concatenate([n_c, w[..., None]], -1).astype(f32)


def depth_range(sc):
    return sc.depth_range[0] * 0.6, sc.depth_range[1] * 1.2  # planar_init.py:149-150


def check_ncc(costs_by_view, init_cost, g, tag):
    """Per-view costs [N, H, W] and the top-k initial cost against the goldens."""
    for j in (1, 2, 3, 4):
        fast = g[f"{tag}_ncc_view{j}"]
        err = np.abs(costs_by_view[j - 1] - fast)
        assert np.mean(err <= VIEW_TOL) >= VIEW_FRAC, (tag, j, np.mean(err <= VIEW_TOL))
        assert np.mean(err <= LOOSE_TOL) >= LOOSE_FRAC, (tag, j, np.mean(err <= LOOSE_TOL))
        # no further from the fast-math build than the reference's own IEEE build is (within a point)
        own = np.mean(np.abs(g[f"{tag}_ieee_ncc_view{j}"] - fast) <= VIEW_TOL)
        assert np.mean(err <= VIEW_TOL) >= own - 0.01, (tag, j, np.mean(err <= VIEW_TOL), own)
    err = np.abs(init_cost - g[f"{tag}_ncc_all"])
    assert np.mean(err <= VIEW_TOL) >= ALL_FRAC, (tag, np.mean(err <= VIEW_TOL))
    assert np.mean(err <= LOOSE_TOL) >= LOOSE_FRAC, (tag, np.mean(err <= LOOSE_TOL))


def agreement(d, n, gd, gn):
    """(fraction with depth within 0.5 %, fraction with depth within 0.5 % and normal within 1 degree)."""
    d, n, gd, gn = (np.asarray(a, np.float64) for a in (d, n, gd, gn))
    ok_d = np.abs(d - gd) <= 0.005 * np.abs(gd)
    cos = np.sum(n * gn, -1) / np.maximum(np.linalg.norm(n, axis=-1) * np.linalg.norm(gn, axis=-1), 1e-12)
    ok_n = np.degrees(np.arccos(np.clip(cos, -1, 1))) <= 1.0
    return float(np.mean(ok_d)), float(np.mean(ok_d & ok_n))


def accuracy(d, gt):
    return float(np.mean(np.abs(np.asarray(d, np.float64) - gt) <= 0.005 * gt))


def check_pass(ours, ours_other_seed, ref_planes, ref_rerun, gt):
    """ours / ours_other_seed: (depth, normal) with two seeds; ref_planes /
    ref_rerun: [H, W, 4] (world normal, depth) of two reference runs (no
    rerun: the ceiling is this implementation's own)."""
    rd, rn = ref_planes[..., 3].astype(np.float64), ref_planes[..., :3].astype(np.float64)
    assert abs(accuracy(ours[0], gt) - accuracy(rd, gt)) <= ACC_TOL, (accuracy(ours[0], gt), accuracy(rd, gt))
    vs_ref = agreement(ours[0], ours[1], rd, rn)
    ceiling_ours = agreement(ours_other_seed[0], ours_other_seed[1], ours[0], ours[1])
    ceiling_ref = ceiling_ours if ref_rerun is None else agreement(ref_rerun[..., 3], ref_rerun[..., :3], rd, rn)
    for k in (0, 1):
        assert vs_ref[k] >= min(ceiling_ref[k], ceiling_ours[k]) - AGREE_MARGIN, (k, vs_ref, ceiling_ref,
                                                                                   ceiling_ours)
    return vs_ref, ceiling_ref, ceiling_ours


def _cams(sc, ids):
    return [synthetic.camera_args(sc, i) for i in ids]


# ------------------------------------------------------------------ oracle --
@pytest.mark.parametrize("tag", TAGS)
def test_oracle_reference_chain_matches_ieee_build(orc, golden, tag):
    g, scenes, mrg = golden
    sc = scenes[tag]
    _, depth, n_c, _ = mrg.mixed_hypotheses(sc, 0, 11)
    ids = [0, 1, 2, 3, 4]
    pl = planes_from_depth(sc, 0, depth, n_c)
    c, ic, _ = orc.ncc_costs(_cams(sc, ids), sc.images[ids].astype(np.float32), pl, orc.make_params(sampler=1),
                             ref_chain=True)
    for j in (1, 2, 3, 4):
        err = np.abs(c[j - 1] - g[f"{tag}_ieee_ncc_view{j}"])
        assert err.max() <= IEEE_TOL, (tag, j, err.max(), np.mean(err > 0))
    assert np.abs(ic - g[f"{tag}_ieee_ncc_all"]).max() <= IEEE_TOL


@pytest.mark.parametrize("tag", TAGS)
def test_oracle_texture_ncc_matches_reference(orc, golden, tag):
    g, scenes, mrg = golden
    sc = scenes[tag]
    _, depth, n_c, _ = mrg.mixed_hypotheses(sc, 0, 11)
    ids = [0, 1, 2, 3, 4]
    pl = planes_from_depth(sc, 0, depth, n_c)
    c, ic, iv = orc.ncc_costs(_cams(sc, ids), sc.images[ids].astype(np.float32), pl, orc.make_params(sampler=1))
    check_ncc(c, ic, g, tag)
    # the selected-view bits follow the costs: equal wherever the top-k cost agrees closely
    close = np.abs(ic - g[f"{tag}_ncc_all"]) <= 1e-5
    assert np.mean(iv[close] == g[f"{tag}_ncc_all_views"][close]) >= 0.999


def _oracle_random(orc, sc, seed):
    dmin, dmax = depth_range(sc)
    ids = [0, 1, 2, 3, 4]
    p = orc.make_params(sampler=1, init_kind=0, sweep_kind=0, max_iterations=3, depth_min=dmin, depth_max=dmax,
                        seed=seed)
    d, n, _, _ = orc.run_pass(_cams(sc, ids), sc.images[ids].astype(np.float32), p)
    return d, n


def _prior_inputs(g, tag, mrg):
    table, mask = g[f"{tag}_prior_table"], g[f"{tag}_prior_mask"]
    return mrg.prior_planes(table, mask), mask.astype(np.uint32)


def _oracle_prior(orc, sc, g, tag, mrg, seed):
    dmin, dmax = depth_range(sc)
    ids = [0, 1, 2, 3, 4]
    pp, pm = _prior_inputs(g, tag, mrg)
    p = orc.make_params(sampler=1, init_kind=1, sweep_kind=1, max_iterations=3, depth_min=dmin, depth_max=dmax,
                        seed=seed, pass_index=1)
    d, n, _, _ = orc.run_pass(_cams(sc, ids), sc.images[ids].astype(np.float32), p, prior_planes=pp, prior_masks=pm,
                              init_planes=g[f"{tag}_rand_planes"], init_costs=g[f"{tag}_rand_cost"])
    return d, n


@pytest.mark.parametrize("tag", TAGS)
def test_oracle_random_pass_close_to_reference(orc, golden, tag):
    g, scenes, _ = golden
    sc = scenes[tag]
    check_pass(_oracle_random(orc, sc, 3407), _oracle_random(orc, sc, 1), g[f"{tag}_rand_planes"],
               g[f"{tag}_rand_rerun_planes"], sc.depths[0].astype(np.float64))


def test_oracle_prior_pass_close_to_reference(orc, golden):
    """The planar-prior pass from the reference's own first-pass state and
    the same prior (the reference's rerun ceiling is measured on the random
    pass; the prior pass is compared with this implementation's own
    two-seed ceiling)."""
    g, scenes, mrg = golden
    tag = "c1"
    sc = scenes[tag]
    a = _oracle_prior(orc, sc, g, tag, mrg, 3407)
    b = _oracle_prior(orc, sc, g, tag, mrg, 1)
    check_pass(a, b, g[f"{tag}_prior_planes"], None, sc.depths[0].astype(np.float64))


# -------------------------------------------------------------------- CUDA --
def _gpu_view(sc, ids, cuda, **kw):
    import torch

    from gmvs_gb300 import engine

    imgs = torch.from_numpy(sc.images[ids].astype(np.float32)).to(cuda)
    dmin, dmax = depth_range(sc)
    return engine.ViewInputs(cams=[engine.make_camera(*synthetic.camera_args(sc, i)) for i in ids],
                             images=[imgs[k] for k in range(len(ids))], depth_min=dmin, depth_max=dmax,
                             stream_id=ids[0], **kw)


@pytest.mark.gpu
@pytest.mark.parametrize("tag", TAGS)
def test_cuda_texture_ncc_matches_reference(gmvs_lib, orc, golden, cuda, tag):
    import torch

    from gmvs_gb300 import _abi, engine

    g, scenes, mrg = golden
    sc = scenes[tag]
    _, depth, n_c, _ = mrg.mixed_hypotheses(sc, 0, 11)
    ids = [0, 1, 2, 3, 4]
    pl = planes_from_depth(sc, 0, depth, n_c)
    v = _gpu_view(sc, ids, cuda)
    p = engine.params_struct(sampler=_abi.SAMPLER_TEX, staging=_abi.STAGE_F32)
    c, ic, _ = engine.ncc_costs(v, p, torch.from_numpy(pl).to(cuda), engine.Workspace())
    check_ncc(c.cpu().numpy(), ic.cpu().numpy(), g, tag)


def _cuda_pass(sc, cuda, seed, prior=None):
    import torch

    from gmvs_gb300 import _abi, engine

    ids = [0, 1, 2, 3, 4]
    kw = {}
    if prior is None:
        p = engine.params_struct(sampler=_abi.SAMPLER_TEX, init_kind=_abi.INIT_RANDOM, sweep_kind=_abi.SWEEP_PHOTO,
                                 max_iterations=3, seed=seed)
    else:
        pp, pm, ip, icst = prior
        t = lambda a, dt=torch.float32: torch.from_numpy(np.ascontiguousarray(a)).to(cuda, dt)
        kw = dict(prior_planes=t(pp), prior_masks=t(pm.astype(np.int32), torch.int32), init_planes=t(ip),
                  init_costs=t(icst))
        p = engine.params_struct(sampler=_abi.SAMPLER_TEX, init_kind=_abi.INIT_PRIOR, sweep_kind=_abi.SWEEP_PRIOR,
                                 max_iterations=3, seed=seed, pass_index=1)
    v = _gpu_view(sc, ids, cuda, **kw)
    engine.run_passes([v], p, engine.Workspace())
    return v.out_depth.cpu().numpy(), v.out_normal.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("tag", TAGS)
def test_cuda_random_pass_close_to_reference(gmvs_lib, golden, cuda, tag):
    g, scenes, _ = golden
    sc = scenes[tag]
    check_pass(_cuda_pass(sc, cuda, 3407), _cuda_pass(sc, cuda, 1), g[f"{tag}_rand_planes"],
               g[f"{tag}_rand_rerun_planes"], sc.depths[0].astype(np.float64))


@pytest.mark.gpu
def test_cuda_prior_pass_close_to_reference(gmvs_lib, golden, cuda):
    g, scenes, mrg = golden
    tag = "c1"
    sc = scenes[tag]
    pp, pm = _prior_inputs(g, tag, mrg)
    prior = (pp, pm, g[f"{tag}_rand_planes"], g[f"{tag}_rand_cost"])
    a = _cuda_pass(sc, cuda, 3407, prior)
    b = _cuda_pass(sc, cuda, 1, prior)
    check_pass(a, b, g[f"{tag}_prior_planes"], None, sc.depths[0].astype(np.float64))
