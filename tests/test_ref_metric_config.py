"""Parity at the benchmark's configurations, against golden vectors from the
reference's own kernels (tests/golden/make_ref_goldens.py):

  ref_goldens_cfg1.npz  module B on the plain small configuration (5 views
                        at 320x256, 4 sources): NCC of given hypotheses, a
                        2-iteration geometric pass, fusion of all five views;
  ref_goldens_room.npz  reference view 0 of the 20-view 1600x1200 room scene
                        with its 10 sources: NCC of given hypotheses through
                        modules A and B, the geometric pass, module A's random
                        pass and the fusion of the view (crops and digests).

Plus the CUDA path against the oracle bit for bit on that full-size view
(init and one propagation iteration of the random pass).

The NCC bounds follow tests/test_ref_goldens.py (module B) and
tests/test_ref_planar.py (module A); the passes are compared statistically
against the agreement that different random streams allow.
"""

import os
import sys

import numpy as np
import pytest

from gmvs_gb300 import synthetic

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
CFG1 = os.path.join(HERE, "golden", "ref_goldens_cfg1.npz")
ROOM = os.path.join(HERE, "golden", "ref_goldens_room.npz")

from test_ref_goldens import NCC_TOL, assert_ncc_close, check_fusion_against_reference, check_geom_pass  # noqa: E402
from test_ref_planar import ACC_TOL, VIEW_TOL, agreement, accuracy, planes_from_depth  # noqa: E402


def _cams(sc, ids):
    return [synthetic.camera_args(sc, i) for i in ids]


@pytest.fixture(scope="module")
def cfg1():
    if not os.path.exists(CFG1):
        pytest.skip("configuration-1 goldens not generated")
    import make_ref_goldens as mrg

    return dict(np.load(CFG1)), mrg.cfg1_inputs()


def _cfg1_as_small(g):
    """The cfg1 arrays under the names test_ref_goldens' helpers use."""
    out = {k[3:]: v for k, v in g.items() if k.startswith("c1_")}
    return out


# ---------------------------------------------------------- configuration 1 --
def module_b_planes(sc, ref, depth, n_world):
    """The camera-frame planes module B forms from (depth, world normal)
    (TransformNormal2RefCam + GetDistance2Origin, patch_match.cu:97-134,
    329-339), in its fp32 operation order."""
    R = sc.R[ref].astype(np.float32)
    n = n_world.astype(np.float32)
    n_c = np.stack([(R[k, 0] * n[..., 0] + R[k, 1] * n[..., 1]) + R[k, 2] * n[..., 2] for k in range(3)], -1)
    return planes_from_depth(sc, ref, depth, n_c.astype(np.float32))


def test_oracle_cfg1_ncc_matches_reference(orc, cfg1):
    """Within 1e-4 on >= 99.9 % of the pixels, and the rest closer to the
    FP64 evaluation than the reference's fp32 chain.  The oracle's
    restatement of that chain matches module B built without fused
    multiply-adds within 1e-4 on >= 99.99 % of the pixels (median 2e-6: the
    oracle's exp is its own); the reference's own two builds (with and
    without contracted multiply-adds) differ by more than 1e-4 on as many
    pixels as this path and the reference do."""
    g, (sc, hyp_d, hyp_n, _, _) = cfg1
    ids = [0, 1, 2, 3, 4]
    cams, imgs = _cams(sc, ids), sc.images[ids].astype(np.float32)
    pl = module_b_planes(sc, 0, hyp_d[0], hyp_n[0])
    _, c, _ = orc.ncc_costs(cams, imgs, pl, orc.make_params(sampler=0))
    _, exact, _ = orc.ncc_costs(cams, imgs, pl, orc.make_params(sampler=0), fp64=True)
    assert_ncc_close(c, g["c1_ncc_all"], exact)
    _, chain, _ = orc.ncc_costs(cams, imgs, pl, orc.make_params(sampler=0), ref_chain=True)
    e = np.abs(chain - g["c1_ieee_ncc_all"])
    assert np.mean(e <= NCC_TOL) >= 0.9999 and np.median(e) <= 1e-5, (np.mean(e <= NCC_TOL), np.median(e))
    own = np.mean(np.abs(g["c1_ieee_ncc_all"] - g["c1_ncc_all"]) > NCC_TOL)
    assert np.mean(np.abs(c - g["c1_ncc_all"]) > NCC_TOL) <= own + 1e-4


def _oracle_geom(orc, sc, nd, nn, seed):
    ids = [0, 1, 2, 3, 4]
    p = orc.make_params(sampler=0, init_kind=2, sweep_kind=2, max_iterations=2,
                        depth_min=sc.depth_range[0] * 0.6, depth_max=sc.depth_range[1] * 1.2, stream_id=0, seed=seed)
    d, n, _, _ = orc.run_pass(_cams(sc, ids), sc.images[ids].astype(np.float32), p, depths=nd[ids], ref_normal=nn[0])
    return d, n


def test_oracle_cfg1_geom_pass_close_to_reference(orc, cfg1):
    g, (sc, _, _, nd, nn) = cfg1
    check_geom_pass(_oracle_geom(orc, sc, nd, nn, 3407), _oracle_geom(orc, sc, nd, nn, 1), _cfg1_as_small(g),
                    sc.depths[0].astype(np.float64))


def _oracle_fusion(orc, sc, nd, nn):
    V, H, W = nd.shape
    masks = np.zeros((V, H, W), np.uint8)
    outs, hits = [], []
    for ref, src in sc.problems:
        ids = [ref] + src
        d, _, _, h = orc.fuse(_cams(sc, ids), ref, src, nd[ids], nn[ids], masks, 3, with_hits=True)
        outs.append(d)
        hits.append(h)
    return outs, masks, hits


def check_fusion_borderline(outs, masks, g, hits, prefix="c1_", frac=1e-4):
    """Against the reference as built (nvcc contracts its multiply-adds into
    fused ones, which moves the borderline consistency tests): masks and
    fused-pixel sets equal except on `frac` of the pixels."""
    gm = g[f"{prefix}fuse_masks"]
    assert np.mean(masks != gm) <= frac, np.mean(masks != gm)
    for k, d in enumerate(outs):
        rd = g[f"{prefix}fuse_depth{k}"]
        assert np.mean((d > 0) != (rd > 0)) <= frac
        both = (hits[k] == 1) & (rd > 0) & (d > 0)
        assert np.median(np.abs(d - rd)[both] / rd[both]) <= 1e-6


def test_oracle_cfg1_fusion_matches_reference(orc, cfg1):
    """Bit-exact masks and fused-pixel sets against module B's fusion built
    without fused multiply-adds (the reference's own fp32 operation order),
    and within a few borderline pixels of the build with them."""
    g, (sc, _, _, nd, nn) = cfg1
    outs, masks, hits = _oracle_fusion(orc, sc, nd, nn)
    check_fusion_against_reference(outs, masks, {k[8:]: v for k, v in g.items() if k.startswith("c1_ieee_")}, hits)
    check_fusion_borderline(outs, masks, g, hits)


def _gpu_geom(sc, nd, nn, ref, src, cuda, seed, split=1):
    import torch

    from gmvs_gb300 import _abi, engine

    ids = [ref] + list(src)
    imgs = torch.from_numpy(sc.images[ids].astype(np.float32)).to(cuda)
    dep = torch.from_numpy(nd[ids]).to(cuda)
    v = engine.ViewInputs(cams=[engine.make_camera(*synthetic.camera_args(sc, i)) for i in ids],
                          images=[imgs[k] for k in range(len(ids))], depth_min=sc.depth_range[0] * 0.6,
                          depth_max=sc.depth_range[1] * 1.2, stream_id=0, depths=[dep[k] for k in range(len(ids))],
                          ref_normal=torch.from_numpy(nn[ref]).to(cuda))
    p = engine.params_struct(init_kind=_abi.INIT_DEPTH_NORMAL, sweep_kind=_abi.SWEEP_GEOM,
                             sampler=_abi.SAMPLER_CLAMP, staging=_abi.STAGE_AUTO, max_iterations=2, seed=seed,
                             split_sweep=split)
    engine.run_passes([v], p, engine.Workspace())
    return v.out_depth.cpu().numpy(), v.out_normal.cpu().numpy()


@pytest.mark.gpu
def test_cuda_cfg1_geom_pass_and_fusion_close_to_reference(gmvs_lib, orc, cfg1, cuda):
    import torch

    from gmvs_gb300.src import Fuser, load_camera, load_problem

    g, (sc, _, _, nd, nn) = cfg1
    check_geom_pass(_gpu_geom(sc, nd, nn, 0, [1, 2, 3, 4], cuda, 3407), _gpu_geom(sc, nd, nn, 0, [1, 2, 3, 4], cuda, 1),
                    _cfg1_as_small(g), sc.depths[0].astype(np.float64))
    V, H, W = nd.shape
    masks = torch.zeros((V, H, W), dtype=torch.bool, device=cuda)
    fu = Fuser()
    fu.load_samples([load_problem(r, s) for r, s in sc.problems],
                    [load_camera(*synthetic.camera_args(sc, i)) for i in range(V)], torch.from_numpy(nd),
                    torch.from_numpy(nn), masks)
    outs = [fu.run_fusion(k, 3)[0].cpu().numpy() for k in range(V)]
    _, _, hits = _oracle_fusion(orc, sc, nd, nn)
    m = masks.cpu().numpy().astype(np.uint8)
    check_fusion_against_reference(outs, m, {k[8:]: v for k, v in g.items() if k.startswith("c1_ieee_")}, hits)
    check_fusion_borderline(outs, m, g, hits)


# ------------------------------------------------- the 1600x1200 room view --
@pytest.fixture(scope="module")
def room(cuda):
    if not os.path.exists(ROOM):
        pytest.skip("room goldens not generated")
    import make_ref_goldens as mrg

    g = dict(np.load(ROOM))
    inp = mrg.room_inputs(cuda)
    if mrg.sha(inp[0].images) != str(g["room_images_sha"]):
        pytest.fail("the room scene renders differently from the golden run (input digest mismatch)")
    return g, inp, mrg


@pytest.mark.gpu
def test_cuda_room_ncc_matches_reference(gmvs_lib, orc, room, cuda):
    """Full-size NCC of given hypotheses (the top-k initial cost over 10
    sources).  At 1600x1200 the fp32 sample coordinates themselves carry
    rounding of ~1e-4 pixel, which the textured images turn into cost
    differences above 1e-4 on a few per cent of the pixels -- for the
    reference as much as for this path: the oracle's restatement of the
    reference's own operation chain (no fused multiply-adds, IEEE exp) agrees
    with the reference only on ~96 % of the crops' pixels within 1e-4.  So
    the bound is: within 1e-4 on no fewer pixels than that restatement,
    less 1.5 points; within 1e-3 on >= 99.8 %; and, for module B, closer
    to the FP64 evaluation than the reference on average."""
    import torch

    from gmvs_gb300 import _abi, engine

    g, (sc, ref, src, depth, n_c, n_w, _, _), mrg = room
    ids = [ref] + src
    cams = _cams(sc, ids)
    imgs32 = sc.images[ids].astype(np.float32)
    imgs = torch.from_numpy(imgs32).to(cuda)
    dmin, dmax = sc.depth_range[0] * 0.6, sc.depth_range[1] * 1.2
    v = engine.ViewInputs(cams=[engine.make_camera(*synthetic.camera_args(sc, i)) for i in ids],
                          images=[imgs[k] for k in range(len(ids))], depth_min=dmin, depth_max=dmax, stream_id=ref)
    for sampler, staging, pl, key in (
            (_abi.SAMPLER_CLAMP, _abi.STAGE_QUAD_F16, module_b_planes(sc, ref, depth, n_w), "room_b_ncc_all"),
            (_abi.SAMPLER_TEX, _abi.STAGE_F32, planes_from_depth(sc, ref, depth, n_c), "room_a_ncc_all")):
        osampler = 1 if sampler == _abi.SAMPLER_TEX else 0
        p = engine.params_struct(sampler=sampler, staging=staging)
        _, ic, _ = engine.ncc_costs(v, p, torch.from_numpy(pl).to(cuda), engine.Workspace(), want_costs=False)
        c = mrg.crops(ic.cpu().numpy())
        _, chain, _ = orc.ncc_costs(cams, imgs32, pl, orc.make_params(sampler=osampler), ref_chain=True)
        ref_c = g[key]
        err = np.abs(c - ref_c)
        own = np.mean(np.abs(mrg.crops(chain) - ref_c) <= NCC_TOL)
        assert np.mean(err <= NCC_TOL) >= own - 0.015, (key, np.mean(err <= NCC_TOL), own)
        assert np.mean(err <= 1e-3) >= 0.998, (key, np.mean(err <= 1e-3))
        if key == "room_b_ncc_all":
            _, exact, _ = orc.ncc_costs(cams, imgs32, pl, orc.make_params(sampler=0), fp64=True)
            ex = mrg.crops(exact)
            assert np.abs(c - ex).mean() <= np.abs(ref_c - ex).mean()
            assert np.mean(np.abs(c - ex) <= NCC_TOL) >= np.mean(np.abs(ref_c - ex) <= NCC_TOL)


@pytest.mark.gpu
def test_cuda_room_geom_pass_close_to_reference(gmvs_lib, room, cuda):
    g, (sc, ref, src, _, _, _, nd, nn), mrg = room
    gt = sc.depths[ref].astype(np.float64)
    a = _gpu_geom(sc, nd, nn, ref, src, cuda, 3407)
    b = _gpu_geom(sc, nd, nn, ref, src, cuda, 1)
    ok = gt > 0
    acc = lambda d: float(np.mean(np.abs(d[ok] - gt[ok]) <= 0.005 * gt[ok]))
    assert abs(acc(a[0]) - float(g["room_b_geom_acc"])) <= 0.01, (acc(a[0]), float(g["room_b_geom_acc"]))
    ca = [mrg.crops(x) for x in a]
    cb = [mrg.crops(x) for x in b]
    vs_ref = agreement(ca[0], ca[1], g["room_b_geom_depth"], g["room_b_geom_normal"])
    ceiling = agreement(cb[0], cb[1], ca[0], ca[1])
    for k in (0, 1):
        assert vs_ref[k] >= ceiling[k] - 0.02, (k, vs_ref, ceiling)


@pytest.mark.gpu
def test_cuda_room_random_pass_close_to_reference(gmvs_lib, room, cuda):
    import torch

    from gmvs_gb300 import _abi, engine

    g, (sc, ref, src, _, _, _, _, _), mrg = room
    ids = [ref] + src
    imgs = torch.from_numpy(sc.images[ids].astype(np.float32)).to(cuda)
    gt = sc.depths[ref].astype(np.float64)
    outs = []
    for seed in (3407, 1):
        v = engine.ViewInputs(cams=[engine.make_camera(*synthetic.camera_args(sc, i)) for i in ids],
                              images=[imgs[k] for k in range(len(ids))], depth_min=sc.depth_range[0] * 0.6,
                              depth_max=sc.depth_range[1] * 1.2, stream_id=0)
        p = engine.params_struct(sampler=_abi.SAMPLER_TEX, init_kind=_abi.INIT_RANDOM, sweep_kind=_abi.SWEEP_PHOTO,
                                 max_iterations=3, seed=seed)
        engine.run_passes([v], p, engine.Workspace())
        outs.append((v.out_depth.cpu().numpy(), v.out_normal.cpu().numpy()))
    ok = gt > 0
    acc = float(np.mean(np.abs(outs[0][0][ok] - gt[ok]) <= 0.005 * gt[ok]))
    assert abs(acc - float(g["room_a_rand_acc"])) <= ACC_TOL, (acc, float(g["room_a_rand_acc"]))
    ca = [mrg.crops(x) for x in outs[0]]
    cb = [mrg.crops(x) for x in outs[1]]
    vs_ref = agreement(ca[0], ca[1], g["room_a_rand_depth"], g["room_a_rand_normal"])
    ceiling = agreement(cb[0], cb[1], ca[0], ca[1])
    for k in (0, 1):
        assert vs_ref[k] >= ceiling[k] - 0.02, (k, vs_ref, ceiling)


@pytest.mark.gpu
def test_cuda_room_fusion_matches_reference(gmvs_lib, orc, room, cuda):
    """Against module B's fusion built without fused multiply-adds (the
    reference's own fp32 operation order): the fused-pixel map and the
    source masks equal bit for bit (digests), fused depths equal to 1e-5
    relative on the crops except at output pixels written by several
    reference pixels.  Against the build as shipped (nvcc contracts its
    multiply-adds, moving a few borderline consistency tests): the counts
    within 0.01 % of the pixels."""
    import torch

    from gmvs_gb300 import engine

    g, (sc, ref, src, _, _, _, nd, nn), mrg = room
    ids = [ref] + src
    V, H, W = nd.shape
    masks = torch.zeros((V, H, W), dtype=torch.bool, device=cuda)
    dev_d = torch.from_numpy(nd).to(cuda)
    dev_n = torch.from_numpy(nn).to(cuda)
    d, _ = engine.fuse(engine.make_problem(ref, src), [engine.make_camera(*synthetic.camera_args(sc, i)) for i in ids],
                       [dev_d[i] for i in ids], [dev_n[i] for i in ids], masks, 3, engine.Workspace())
    d = d.cpu().numpy()
    m = masks.cpu().numpy()[ids]
    assert int((d > 0).sum()) == int(g["room_ieee_fuse_count"])
    assert mrg.sha(d > 0) == str(g["room_ieee_fuse_sha"])
    assert mrg.sha(m) == str(g["room_ieee_fuse_masks_sha"])
    assert abs(int((d > 0).sum()) - int(g["room_fuse_count"])) <= 1e-4 * H * W
    assert np.abs(m.reshape(len(ids), -1).sum(1) - g["room_fuse_masks_count"]).max() <= 1e-4 * H * W
    om = np.zeros((V, H, W), np.uint8)
    hits = orc.fuse(_cams(sc, ids), ref, src, nd[ids], nn[ids], om, 3, with_hits=True)[3]
    rd, cd, ch = g["room_ieee_fuse_depth"], mrg.crops(d), mrg.crops(hits)
    single = (ch == 1) & (rd > 0)
    assert np.array_equal(cd > 0, rd > 0)
    assert (np.abs(cd - rd)[single] / rd[single]).max() <= 1e-5


@pytest.mark.gpu
def test_cuda_room_random_pass_equals_oracle(gmvs_lib, orc, room, cuda):
    """The full-size view (1600x1200, 10 sources): initialisation and one
    propagation iteration of the texture path, CUDA against the oracle bit
    for bit."""
    import torch

    from gmvs_gb300 import _abi, engine
    from test_gpu_parity import diff_report, same_bits

    g, (sc, ref, src, _, _, _, _, _), mrg = room
    ids = [ref] + src
    imgs32 = sc.images[ids].astype(np.float32)
    imgs = torch.from_numpy(imgs32).to(cuda)
    dmin, dmax = sc.depth_range[0] * 0.6, sc.depth_range[1] * 1.2
    v = engine.ViewInputs(cams=[engine.make_camera(*synthetic.camera_args(sc, i)) for i in ids],
                          images=[imgs[k] for k in range(len(ids))], depth_min=dmin, depth_max=dmax, stream_id=ref)
    p = engine.params_struct(sampler=_abi.SAMPLER_TEX, init_kind=_abi.INIT_RANDOM, sweep_kind=_abi.SWEEP_PHOTO,
                             max_iterations=1)
    engine.run_passes([v], p, engine.Workspace())
    od, on, oc, _ = orc.run_pass(_cams(sc, ids), imgs32, orc.make_params(sampler=1, depth_min=dmin, depth_max=dmax,
                                                                         max_iterations=1, stream_id=ref))
    gd, gn, gc = v.out_depth.cpu().numpy(), v.out_normal.cpu().numpy(), v.out_cost.cpu().numpy()
    assert same_bits(gd, od) and same_bits(gn, on) and same_bits(gc, oc), \
        diff_report(depth=(gd, od), normal=(gn, on), cost=(gc, oc))
