"""CUDA path against the oracle, bit for bit, away from the default shape:
the generic window path (window sizes and strides other than 11 / 2),
image sizes that do not fill whole tiles, one source view, zero iterations,
and one launch over views of uneven size and source count (the batching
form) against one launch per view."""

import numpy as np
import pytest
import torch

from gmvs_gb300 import _abi, engine, synthetic
from scenes import cam_args, gpu_view, gt_planes
from test_gpu_parity import diff_report, same_bits

pytestmark = pytest.mark.gpu


def _pass(sc, ids, cuda, p):
    v = gpu_view(sc, ids, cuda, 0.3, 6.0)
    v.allocate_outputs(with_planes=True)
    engine.run_passes([v], p, engine.Workspace())
    return v.out_depth.cpu().numpy(), v.out_normal.cpu().numpy(), v.out_cost.cpu().numpy()


def _oracle_pass(orc, sc, ids, **kw):
    od, on, oc, _ = orc.run_pass(cam_args(sc, ids), sc.images[ids].astype(np.float32),
                                 orc.make_params(depth_min=0.3, depth_max=6.0, stream_id=ids[0], **kw))
    return od, on, oc


def _check(g, o):
    assert all(same_bits(a, b) for a, b in zip(g, o)), diff_report(depth=(g[0], o[0]), normal=(g[1], o[1]),
                                                                   cost=(g[2], o[2]))


@pytest.mark.parametrize("patch,stride,sampler", [(7, 1, _abi.SAMPLER_TEX), (11, 1, _abi.SAMPLER_CLAMP),
                                                  (9, 2, _abi.SAMPLER_CLAMP), (5, 2, _abi.SAMPLER_TEX)])
def test_generic_window_pass(gmvs_lib, orc, cuda, patch, stride, sampler):
    sc = synthetic.small_scene(0, H=96, W=128)
    ref, src = sc.problems[0]
    ids = [ref] + src
    p = engine.params_struct(sampler=sampler, staging=_abi.STAGE_F32, patch_size=patch, radius_increment=stride,
                             max_iterations=2)
    _check(_pass(sc, ids, cuda, p), _oracle_pass(orc, sc, ids, sampler=1 if sampler == _abi.SAMPLER_TEX else 0,
                                                 patch_size=patch, radius_increment=stride, max_iterations=2))


@pytest.mark.parametrize("H,W", [(67, 93), (33, 17), (130, 161)])
def test_ragged_image_sizes(gmvs_lib, orc, cuda, H, W):
    sc = synthetic.small_scene(1, H=H, W=W)
    ref, src = sc.problems[0]
    ids = [ref] + src
    p = engine.params_struct(sampler=_abi.SAMPLER_CLAMP, staging=_abi.STAGE_QUAD_F16, max_iterations=2)
    _check(_pass(sc, ids, cuda, p), _oracle_pass(orc, sc, ids, sampler=0, max_iterations=2))


def test_one_source_and_zero_iterations(gmvs_lib, orc, cuda):
    sc = synthetic.small_scene(2, H=64, W=80)
    ref, src = sc.problems[0]
    ids = [ref, src[0]]
    p = engine.params_struct(sampler=_abi.SAMPLER_TEX, max_iterations=2)
    _check(_pass(sc, ids, cuda, p), _oracle_pass(orc, sc, ids, sampler=1, max_iterations=2))
    ids = [ref] + src
    p = engine.params_struct(sampler=_abi.SAMPLER_TEX, max_iterations=0)
    _check(_pass(sc, ids, cuda, p), _oracle_pass(orc, sc, ids, sampler=1, max_iterations=0))


def test_uneven_batch_equals_single_launches(gmvs_lib, cuda):
    """Views of different sizes and source counts in one launch per stage."""
    scenes = [synthetic.small_scene(0, H=96, W=128), synthetic.small_scene(3, H=80, W=112),
              synthetic.small_scene(4, H=120, W=96)]
    picks = [(0, 4), (1, 2), (2, 3), (0, 1)]  # (scene, number of sources)
    p = engine.params_struct(sampler=_abi.SAMPLER_CLAMP, staging=_abi.STAGE_QUAD_F16, max_iterations=2)
    views, refs = [], []
    for k, (si, n) in enumerate(picks):
        sc = scenes[si]
        ref, src = sc.problems[k % len(sc.problems)]
        ids = [ref] + list(src)[:n]
        refs.append((sc, ids))
        views.append(gpu_view(sc, ids, cuda, 0.3, 6.0))
        views[-1].allocate_outputs(with_planes=True)
    engine.run_passes(views, p, engine.Workspace())
    for v, (sc, ids) in zip(views, refs):
        single = gpu_view(sc, ids, cuda, 0.3, 6.0)
        single.allocate_outputs(with_planes=True)
        engine.run_passes([single], p, engine.Workspace())
        for a, b in ((single.out_depth, v.out_depth), (single.out_normal, v.out_normal),
                     (single.out_planes, v.out_planes)):
            assert torch.equal(torch.nan_to_num(a, 7.0), torch.nan_to_num(b, 7.0))


@pytest.mark.parametrize("scene", ["small", "room"])
def test_staging_modes_agree(gmvs_lib, cuda, scene):
    """fp32 rows, fp32 quads and fp16 quads hold the same taps of 8-bit
    images, so whole geometric passes agree bit for bit."""
    if scene == "small":
        sc = synthetic.small_scene(0, H=128, W=160)
    else:
        sc = synthetic.room_scene(0, H=240, W=320, num_views=20, device=cuda)
    ref, src = sc.problems[0]
    ids = [ref] + list(src)
    rng = np.random.default_rng(3)
    d = (sc.depths * (1.0 + rng.normal(0, 0.005, sc.depths.shape))).astype(np.float32)
    n = sc.normals + rng.normal(0, 0.02, sc.normals.shape)
    n = (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)
    outs = []
    for staging in (_abi.STAGE_F32, _abi.STAGE_QUAD_F32, _abi.STAGE_QUAD_F16):
        p = engine.params_struct(sampler=_abi.SAMPLER_CLAMP, staging=staging, init_kind=_abi.INIT_DEPTH_NORMAL,
                                 sweep_kind=_abi.SWEEP_GEOM, max_iterations=2, pass_index=2)
        v = gpu_view(sc, ids, cuda, 0.3, 13.0, depths=[torch.from_numpy(d[i]).to(cuda) for i in ids],
                     ref_normal=torch.from_numpy(n[ref]).to(cuda))
        v.allocate_outputs(with_planes=True)
        engine.run_passes([v], p, engine.Workspace())
        outs.append((v.out_depth.cpu().numpy(), v.out_normal.cpu().numpy(), v.out_cost.cpu().numpy()))
    for o in outs[1:]:
        _check(o, outs[0])


@pytest.mark.parametrize("kind", ["random", "prior", "geom"])
def test_split_half_sweeps_equal_single_kernel(gmvs_lib, cuda, kind):
    """A half-sweep as two kernels (neighbour hypotheses, then the rest) or
    three (neighbour hypotheses and the current plane, then view selection
    and the refinement planes, then the refinement) computes exactly what
    the single kernel does."""
    sc = synthetic.small_scene(0, H=128, W=160)
    views = [sc.problems[0], sc.problems[1]]
    rng = np.random.default_rng(3)
    d = (sc.depths * (1.0 + rng.normal(0, 0.005, sc.depths.shape))).astype(np.float32)
    n = sc.normals + rng.normal(0, 0.02, sc.normals.shape)
    n = (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)
    prior = {}
    if kind == "prior":
        # a prior over every pixel: the restricted-cost branches everywhere
        t = lambda a, dt=torch.float32: torch.from_numpy(np.ascontiguousarray(a)).to(device=cuda, dtype=dt)
        for ref, _ in views:
            pl = gt_planes(sc, ref)
            prior[ref] = dict(prior_planes=t(pl), prior_masks=t(np.full(pl.shape[:2], 1, np.int32), torch.int32),
                              init_planes=t(pl), init_costs=t(np.full(pl.shape[:2], 0.5, np.float32)))
    outs = []
    for split in (0, 1, 2):
        if kind == "random":
            p = engine.params_struct(sampler=_abi.SAMPLER_TEX, max_iterations=3, split_sweep=split)
        elif kind == "prior":
            p = engine.params_struct(sampler=_abi.SAMPLER_TEX, init_kind=_abi.INIT_PRIOR, sweep_kind=_abi.SWEEP_PRIOR,
                                     pass_index=1, split_sweep=split)
        else:
            p = engine.params_struct(sampler=_abi.SAMPLER_CLAMP, init_kind=_abi.INIT_DEPTH_NORMAL,
                                     sweep_kind=_abi.SWEEP_GEOM, max_iterations=2, pass_index=2, split_sweep=split)
        vs = []
        for ref, src in views:
            ids = [ref] + list(src)
            extra = {"random": {}, "prior": prior.get(ref, {})}.get(kind) if kind != "geom" else dict(
                depths=[torch.from_numpy(d[i]).to(cuda) for i in ids], ref_normal=torch.from_numpy(n[ref]).to(cuda))
            v = gpu_view(sc, ids, cuda, 0.3, 6.0, **extra)
            v.allocate_outputs(with_planes=True)
            vs.append(v)
        engine.run_passes(vs, p, engine.Workspace())
        outs.append([(v.out_depth.cpu().numpy(), v.out_normal.cpu().numpy(), v.out_cost.cpu().numpy()) for v in vs])
    for split in (1, 2):
        for a, b in zip(outs[0], outs[split]):
            _check(b, a)


def test_texture_arrays_equal_pitched_textures(gmvs_lib, orc, cuda):
    """Module A's CUDA-array textures filter exactly like the pitched ones."""
    sc = synthetic.small_scene(0, H=96, W=128)
    ref, src = sc.problems[0]
    ids = [ref] + src
    outs = [_pass(sc, ids, cuda, engine.params_struct(sampler=_abi.SAMPLER_TEX, max_iterations=2, tex_storage=t))
            for t in (0, 1)]
    _check(outs[1], outs[0])
    _check(outs[1], _oracle_pass(orc, sc, ids, sampler=1, max_iterations=2))


@pytest.mark.parametrize("num_src", [17, 32])
def test_many_sources(gmvs_lib, orc, cuda, num_src):
    """More than 16 source views (the second half of the view-selection draw
    counters) up to the maximum, GMVS_MAX_NGB = 32 (every bit of the
    selection masks, the widest neighbour-cost matrices): the random pass
    with the texture sampler, and the geometric pass with fp16 texel quads
    as one kernel and split in two, against the oracle bit for bit."""
    sc = synthetic.room_scene(0, H=72, W=96, num_views=num_src + 1, device=cuda)
    ids = list(range(num_src + 1))
    dmin, dmax = sc.depth_range
    p = engine.params_struct(sampler=_abi.SAMPLER_TEX, max_iterations=2)
    v = gpu_view(sc, ids, cuda, dmin, dmax)
    v.allocate_outputs(with_planes=True)
    engine.run_passes([v], p, engine.Workspace())
    g = (v.out_depth.cpu().numpy(), v.out_normal.cpu().numpy(), v.out_cost.cpu().numpy())
    od, on, oc, _ = orc.run_pass(cam_args(sc, ids), sc.images[ids].astype(np.float32),
                                 orc.make_params(sampler=1, depth_min=dmin, depth_max=dmax, stream_id=0,
                                                 max_iterations=2))
    _check(g, (od, on, oc))
    assert (v.out_depth > 0).float().mean().item() > 0.5

    rng = np.random.default_rng(4)
    d = (sc.depths * (1.0 + rng.normal(0, 0.005, sc.depths.shape))).astype(np.float32)
    n = sc.normals + rng.normal(0, 0.02, sc.normals.shape)
    n = (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)
    op = orc.make_params(sampler=0, depth_min=dmin, depth_max=dmax, init_kind=2, sweep_kind=2, max_iterations=2,
                         pass_index=2, stream_id=0)
    o = orc.run_pass(cam_args(sc, ids), sc.images[ids].astype(np.float32), op, depths=d[ids], ref_normal=n[0])[:3]
    for split in (0, 1):
        p = engine.params_struct(sampler=_abi.SAMPLER_CLAMP, staging=_abi.STAGE_QUAD_F16,
                                 init_kind=_abi.INIT_DEPTH_NORMAL, sweep_kind=_abi.SWEEP_GEOM, max_iterations=2,
                                 pass_index=2, split_sweep=split)
        v = gpu_view(sc, ids, cuda, dmin, dmax, depths=[torch.from_numpy(d[i]).to(cuda) for i in ids],
                     ref_normal=torch.from_numpy(n[0]).to(cuda))
        v.allocate_outputs(with_planes=True)
        engine.run_passes([v], p, engine.Workspace())
        _check((v.out_depth.cpu().numpy(), v.out_normal.cpu().numpy(), v.out_cost.cpu().numpy()), o)
