"""Parity of the CUDA path (through the C ABI) with the oracle on the small
scene.  Both evaluate the same documented fp32 arithmetic (explicit fused
multiply-adds, correctly rounded division/reciprocal/sqrt, shared elementary
functions, the same summation order and the same Philox stream), so NCC
costs, whole passes and fusion are compared bit for bit."""

import numpy as np
import pytest
import torch

from gmvs_gb300 import _abi, engine, synthetic
from scenes import cam_args, gpu_view, gt_planes, random_planes

pytestmark = pytest.mark.gpu

# bound quoted for results that are expected to be bit-identical
NCC_TOL = 1e-4
# full-pass agreement: depth within 0.5% relative and normal within 1 degree
DEPTH_REL, NORMAL_DEG, MIN_AGREE = 0.005, 1.0, 0.99


def _bits(a):
    """float32 bit patterns with every NaN mapped to one pattern (GPU and x86
    produce different NaN payloads for the same 0/0)."""
    a = np.ascontiguousarray(a, np.float32).copy()
    a[np.isnan(a)] = np.float32("nan")
    return a.view(np.uint32)


def same_bits(a, b):
    """Equal bit for bit (NaNs equal to NaNs)."""
    return np.shape(a) == np.shape(b) and np.array_equal(_bits(a), _bits(b))


def diff_report(**pairs):
    """Which outputs differ, where first and by how much."""
    out = []
    for name, (a, b) in pairs.items():
        a = np.ascontiguousarray(a, np.float32)
        b = np.ascontiguousarray(b, np.float32)
        bad = _bits(a) != _bits(b)
        if bad.any():
            idx = np.argwhere(bad)[0]
            d = np.abs(np.nan_to_num(a) - np.nan_to_num(b))
            out.append(f"{name}: {int(bad.sum())} differ, first at {tuple(int(i) for i in idx)} "
                       f"({a[tuple(idx)]!r} vs {b[tuple(idx)]!r}), max |diff| {d.max():.3g}")
    return "; ".join(out) or "identical"

SAMPLERS = [
    ("tex", _abi.SAMPLER_TEX, _abi.STAGE_F32, 1),
    ("clamp_f32", _abi.SAMPLER_CLAMP, _abi.STAGE_F32, 0),
    ("clamp_quad_f32", _abi.SAMPLER_CLAMP, _abi.STAGE_QUAD_F32, 0),
    ("clamp_quad_f16", _abi.SAMPLER_CLAMP, _abi.STAGE_QUAD_F16, 0),
]


def mixed_hypotheses(sc, view, seed=1):
    rng = np.random.default_rng(seed)
    pl = gt_planes(sc, view)
    rp = random_planes(sc, view, rng, 0.3, 6.0)
    return np.where(rng.random(pl.shape[:2])[..., None] < 0.5, pl, rp).astype(np.float32)


def agreement(d1, n1, d2, n2):
    ok_d = np.abs(d1 - d2) <= DEPTH_REL * np.abs(d2)
    cosang = np.clip(np.sum(n1 * n2, -1) / np.maximum(np.linalg.norm(n1, axis=-1) * np.linalg.norm(n2, axis=-1),
                                                       1e-12), -1, 1)
    ok_n = np.degrees(np.arccos(cosang)) <= NORMAL_DEG
    return float(np.mean(ok_d & ok_n))


@pytest.mark.parametrize("name,sampler,staging,osampler", SAMPLERS)
def test_ncc_costs_match_oracle(gmvs_lib, orc, small, cuda, name, sampler, staging, osampler):
    ref, src = small.problems[0]
    ids = [ref] + src
    hyp = mixed_hypotheses(small, ref)
    v = gpu_view(small, ids, cuda, 0.3, 6.0)
    p = engine.params_struct(sampler=sampler, staging=staging)
    costs, ic, iv = engine.ncc_costs(v, p, torch.from_numpy(hyp).to(cuda), engine.Workspace())
    oc, oic, oiv = orc.ncc_costs(cam_args(small, ids), small.images[ids].astype(np.float32), hyp,
                                 orc.make_params(sampler=osampler))
    gc = costs.cpu().numpy()
    err = np.abs(gc - oc)
    assert np.isfinite(gc).all()
    assert same_bits(gc, oc), f"{name}: " + diff_report(costs=(gc, oc))
    assert same_bits(ic.cpu().numpy(), oic)
    assert np.array_equal(iv.cpu().numpy().view(np.uint32), oiv)


def test_ncc_costs_vs_fp64_oracle(gmvs_lib, orc, small, cuda):
    """FP16-staged texel quads with FP32 moments stay within 1e-3 of the FP64 oracle."""
    ref, src = small.problems[0]
    ids = [ref] + src
    hyp = mixed_hypotheses(small, ref, seed=2)
    v = gpu_view(small, ids, cuda, 0.3, 6.0)
    p = engine.params_struct(sampler=_abi.SAMPLER_CLAMP, staging=_abi.STAGE_QUAD_F16)
    costs, _, _ = engine.ncc_costs(v, p, torch.from_numpy(hyp).to(cuda), engine.Workspace())
    o64, _, _ = orc.ncc_costs(cam_args(small, ids), small.images[ids].astype(np.float32), hyp,
                              orc.make_params(sampler=0), fp64=True)
    assert np.abs(costs.cpu().numpy() - o64).max() <= 1e-3


def _noisy_inputs(sc, seed=3):
    rng = np.random.default_rng(seed)
    d = (sc.depths * (1.0 + rng.normal(0, 0.005, sc.depths.shape))).astype(np.float32)
    n = sc.normals + rng.normal(0, 0.02, sc.normals.shape)
    n = (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)
    return d, n


def _gpu_pass(sc, ids, dev, p, dmin, dmax, **extra):
    v = gpu_view(sc, ids, dev, dmin, dmax, **extra)
    v.allocate_outputs(with_planes=True)
    engine.run_passes([v], p, engine.Workspace())
    return (v.out_depth.cpu().numpy(), v.out_normal.cpu().numpy(), v.out_cost.cpu().numpy(),
            v.out_planes.cpu().numpy())


def test_random_pass_matches_oracle(gmvs_lib, orc, small, cuda):
    ref, src = small.problems[0]
    ids = [ref] + src
    dmin, dmax = 0.3, 6.0
    p = engine.params_struct(sampler=_abi.SAMPLER_TEX, init_kind=_abi.INIT_RANDOM, sweep_kind=_abi.SWEEP_PHOTO)
    gd, gn, gcst, _ = _gpu_pass(small, ids, cuda, p, dmin, dmax)
    od, on, ocst, _ = orc.run_pass(cam_args(small, ids), small.images[ids].astype(np.float32),
                                   orc.make_params(sampler=1, depth_min=dmin, depth_max=dmax, stream_id=ref))
    a = agreement(gd, gn, od, on)
    assert same_bits(gd, od) and same_bits(gn, on) and same_bits(gcst, ocst), \
        f"agreement {a:.6f}: " + diff_report(depth=(gd, od), normal=(gn, on), cost=(gcst, ocst))


def test_geom_pass_matches_oracle(gmvs_lib, orc, small, cuda):
    ref, src = small.problems[0]
    ids = [ref] + src
    dmin, dmax = 0.3, 6.0
    d_in, n_in = _noisy_inputs(small)
    dev_d = [torch.from_numpy(d_in[i]).to(cuda) for i in ids]
    p = engine.params_struct(sampler=_abi.SAMPLER_CLAMP, init_kind=_abi.INIT_DEPTH_NORMAL,
                             sweep_kind=_abi.SWEEP_GEOM, max_iterations=2, pass_index=2)
    gd, gn, gcst, _ = _gpu_pass(small, ids, cuda, p, dmin, dmax, depths=dev_d,
                                ref_normal=torch.from_numpy(n_in[ref]).to(cuda))
    op = orc.make_params(sampler=0, depth_min=dmin, depth_max=dmax, init_kind=2, sweep_kind=2, max_iterations=2,
                         pass_index=2, stream_id=ref)
    od, on, ocst, _ = orc.run_pass(cam_args(small, ids), small.images[ids].astype(np.float32), op,
                                   depths=d_in[ids], ref_normal=n_in[ref])
    a = agreement(gd, gn, od, on)
    assert same_bits(gd, od) and same_bits(gn, on) and same_bits(gcst, ocst), \
        f"agreement {a:.6f}: " + diff_report(depth=(gd, od), normal=(gn, on), cost=(gcst, ocst))


def test_prior_pass_matches_oracle(gmvs_lib, orc, small, cuda):
    ref, src = small.problems[0]
    ids = [ref] + src
    dmin, dmax = 0.3, 6.0
    imgs = small.images[ids].astype(np.float32)
    od1, on1, oc1, op1 = orc.run_pass(cam_args(small, ids), imgs,
                                      orc.make_params(sampler=1, depth_min=dmin, depth_max=dmax, stream_id=ref))
    planes, masks, _ = orc.build_prior(synthetic.camera_args(small, ref), od1, oc1, small.superpixels[ref], True,
                                       dmin, dmax)
    assert (masks > 0).mean() > 0.2
    p = engine.params_struct(sampler=_abi.SAMPLER_TEX, init_kind=_abi.INIT_PRIOR, sweep_kind=_abi.SWEEP_PRIOR,
                             pass_index=1)
    t = lambda a, dt=torch.float32: torch.from_numpy(np.ascontiguousarray(a)).to(device=cuda, dtype=dt)
    gd, gn, gcst, _ = _gpu_pass(small, ids, cuda, p, dmin, dmax, prior_planes=t(planes),
                                prior_masks=t(masks.view(np.int32), torch.int32), init_planes=t(op1),
                                init_costs=t(oc1))
    o = orc.make_params(sampler=1, depth_min=dmin, depth_max=dmax, init_kind=1, sweep_kind=1, pass_index=1,
                        stream_id=ref)
    od, on, ocst, _ = orc.run_pass(cam_args(small, ids), imgs, o, prior_planes=planes, prior_masks=masks,
                                   init_planes=op1, init_costs=oc1)
    a = agreement(gd, gn, od, on)
    assert same_bits(gd, od) and same_bits(gn, on) and same_bits(gcst, ocst), \
        f"agreement {a:.6f}: " + diff_report(depth=(gd, od), normal=(gn, on), cost=(gcst, ocst))


def test_batched_views_equal_single_views(gmvs_lib, small, cuda):
    """One launch chain over several reference views gives the same bits as
    one chain per view (the Philox stream is keyed by pixel and view)."""
    p = engine.params_struct(sampler=_abi.SAMPLER_CLAMP, staging=_abi.STAGE_QUAD_F16,
                             init_kind=_abi.INIT_RANDOM, sweep_kind=_abi.SWEEP_PHOTO, max_iterations=2)
    views = []
    for ref, src in small.problems[:3]:
        views.append(gpu_view(small, [ref] + src, cuda, 0.3, 6.0))
    engine.run_passes(views, p, engine.Workspace())
    for k, (ref, src) in enumerate(small.problems[:3]):
        single = gpu_view(small, [ref] + src, cuda, 0.3, 6.0)
        engine.run_passes([single], p, engine.Workspace())
        assert torch.equal(single.out_depth, views[k].out_depth)
        assert torch.equal(single.out_normal, views[k].out_normal)
        assert torch.equal(torch.nan_to_num(single.out_cost, 7.0), torch.nan_to_num(views[k].out_cost, 7.0))


def test_fusion_bit_exact(gmvs_lib, orc, small, cuda):
    d_in, n_in = _noisy_inputs(small, seed=5)
    V = small.num_views
    H, W = small.hw
    masks_o = np.zeros((V, H, W), np.uint8)
    masks_g = torch.zeros((V, H, W), dtype=torch.bool, device=cuda)
    scratch = engine.Workspace()
    dev_d = torch.from_numpy(d_in).to(cuda)
    dev_n = torch.from_numpy(n_in).to(cuda)
    for ref, src in small.problems:
        ids = [ref] + src
        od, on, ocnt = orc.fuse(cam_args(small, ids), ref, src, d_in[ids], n_in[ids], masks_o, 3)
        cnt = torch.empty((H, W), dtype=torch.int32, device=cuda)
        gd, gn = engine.fuse(engine.make_problem(ref, src),
                             [engine.make_camera(*synthetic.camera_args(small, i)) for i in ids],
                             [dev_d[i] for i in ids], [dev_n[i] for i in ids], masks_g, 3, scratch, out_count=cnt)
        assert np.array_equal(cnt.cpu().numpy(), ocnt)
        assert np.array_equal(masks_g.cpu().numpy().astype(np.uint8), masks_o)
        assert np.array_equal(gd.cpu().numpy(), od)
        assert np.array_equal(gn.cpu().numpy(), on)
    assert masks_o.any() and (ocnt >= 3).any()
