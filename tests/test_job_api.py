"""The scene-level C API (gmvs_ctx_* / gmvs_job_* / gmvs_pass_* /
gmvs_export): argument checks on the CPU, and on the GPU the whole
reconstruction through the C ABI equal to the Python pipeline's."""

import ctypes

import numpy as np
import pytest

from gmvs_gb300 import _abi


def test_job_api_rejects_bad_arguments(gmvs_lib):
    L = _abi.lib()
    job = ctypes.c_void_p()
    cam = (_abi.gmvs_camera * 1)()
    prob = (_abi.gmvs_problem * 1)()
    # no context, no cameras, no images: nothing reaches the device
    assert L.gmvs_job_create(None, cam, 1, 8, 8, 1 << 20, None, prob, 1, ctypes.byref(job)) == _abi.ERR_INVALID
    assert L.gmvs_job_create(1 << 20, None, 1, 8, 8, 1 << 20, None, prob, 1, ctypes.byref(job)) == _abi.ERR_INVALID
    assert L.gmvs_ctx_last_error(None, ctypes.create_string_buffer(8), 8) == _abi.ERR_INVALID
    assert L.gmvs_pass_random_prior(None, None, 0, None, None) == _abi.ERR_INVALID
    assert L.gmvs_pass_geom(None, None, 0, None, None, None, None) == _abi.ERR_INVALID
    assert L.gmvs_job_fuse(None, None, 0, 3, None, None) == _abi.ERR_INVALID
    assert L.gmvs_export(None, 0, 0, None, None, None, None) == _abi.ERR_INVALID
    assert L.gmvs_ctx_create(0, None) == _abi.ERR_INVALID


@pytest.mark.gpu
def test_job_api_equals_python_pipeline(gmvs_lib, cuda):
    import torch

    from gmvs_gb300 import engine, synthetic
    from gmvs_gb300.pipeline import ScenePipeline, scene_inputs_from_synthetic

    L = _abi.lib()
    sc = synthetic.room_scene(0, H=240, W=320, num_views=8, num_src=4, device=cuda)
    inp = scene_inputs_from_synthetic(sc, cuda)
    V, H, W = inp.images.shape
    pipe = ScenePipeline(inp, geom_iters=2, geom_consistent=3, mode="batched")
    pipe.run()
    torch.cuda.synchronize()

    ctx, job = ctypes.c_void_p(), ctypes.c_void_p()
    assert L.gmvs_ctx_create(0, ctypes.byref(ctx)) == 0
    cams = (_abi.gmvs_camera * V)(*inp.cams)
    probs = (_abi.gmvs_problem * len(inp.problems))(*[engine.make_problem(r, s) for r, s in inp.problems])
    sp = np.ascontiguousarray(inp.superpixels)
    images = inp.images.contiguous()
    rc = L.gmvs_job_create(ctx, cams, V, H, W, images.data_ptr(), sp.ctypes.data, probs, len(inp.problems),
                           ctypes.byref(job))
    assert rc == 0, L.gmvs_last_error()

    def same(a, b):  # bit for bit, NaN where the other has NaN
        na, nb = a.isnan(), b.isnan()
        return torch.equal(na, nb) and torch.equal(a[~na], b[~nb])

    def err():
        buf = ctypes.create_string_buffer(512)
        L.gmvs_ctx_last_error(ctx, buf, 512)
        return buf.value.decode()

    try:
        p = engine.params_struct()
        assert L.gmvs_pass_random_prior(job, None, 0, ctypes.byref(p), None) == 0, err()
        g = engine.params_struct(max_iterations=2)
        for _ in range(2):
            assert L.gmvs_pass_geom(job, None, 0, ctypes.byref(g), None, None, None) == 0, err()
        assert L.gmvs_job_fuse(job, None, 0, 3, None, None) == 0, err()
        last = 1  # random -> buffer 0, prior -> 1, geometric passes -> 0, then 1
        d = torch.empty((H, W), dtype=torch.float32, device=cuda)
        n = torch.empty((H, W, 3), dtype=torch.float32, device=cuda)
        c = torch.empty((H, W), dtype=torch.float32, device=cuda)
        fused = 0
        for ref, _ in inp.problems:
            assert L.gmvs_export(job, ref, 0, d.data_ptr(), n.data_ptr(), c.data_ptr(), None) == 0, err()
            torch.cuda.synchronize()
            assert same(d, pipe.depth[last][ref]) and same(n, pipe.normal[last][ref])
            assert same(c, pipe.cost[last][ref])
            assert L.gmvs_export(job, ref, 1, d.data_ptr(), n.data_ptr(), None, None) == 0, err()
            torch.cuda.synchronize()
            assert same(d, pipe.fused_depth[ref])
            assert torch.allclose(n, pipe.fused_normal[ref], atol=1e-6, rtol=0)
            fused += int((d > 0).sum())
        assert fused > 0.1 * H * W  # fusion masks what earlier views fused: later views fuse fewer pixels
        # host outputs and error paths through the context
        hd = np.empty((H, W), np.float32)
        assert L.gmvs_export(job, inp.problems[0][0], 1, hd.ctypes.data, None, None, None) == 0, err()
        assert np.array_equal(hd, pipe.fused_depth[inp.problems[0][0]].cpu().numpy())
        assert L.gmvs_export(job, V, 0, d.data_ptr(), None, None, None) == _abi.ERR_INVALID
        assert "no such view" in err()
        assert L.gmvs_export(job, 0, 1, None, None, c.data_ptr(), None) == _abi.ERR_INVALID
        twice = (ctypes.c_int32 * 2)(0, 0)
        assert L.gmvs_pass_geom(job, twice, 2, ctypes.byref(g), None, None, None) == _abi.ERR_INVALID
        assert "twice" in err()
        shared = (_abi.gmvs_problem * 2)(probs[0], probs[0])
        other = ctypes.c_void_p()
        assert L.gmvs_job_create(ctx, cams, V, H, W, images.data_ptr(), None, shared, 2,
                                 ctypes.byref(other)) == _abi.ERR_INVALID
    finally:
        L.gmvs_job_destroy(job)
        L.gmvs_ctx_destroy(ctx)


@pytest.mark.gpu
def test_job_api_rejects_bad_problems(gmvs_lib, cuda):
    """A source view equal to its reference view, or listed twice, is refused
    at gmvs_job_create, before any pass runs (the fusion would refuse the
    first only at the end)."""
    from gmvs_gb300 import engine

    L = _abi.lib()
    ctx, job = ctypes.c_void_p(), ctypes.c_void_p()
    assert L.gmvs_ctx_create(0, ctypes.byref(ctx)) == 0
    try:
        cams = (_abi.gmvs_camera * 3)()
        for c in cams:
            c.height, c.width = 8, 8
        for src, why in (([1, 0], "equals the reference view"), ([1, 2, 1], "listed twice")):
            probs = (_abi.gmvs_problem * 1)(engine.make_problem(0, src))
            rc = L.gmvs_job_create(ctx, cams, 3, 8, 8, 1 << 20, None, probs, 1, ctypes.byref(job))
            assert rc == _abi.ERR_INVALID and not job.value
            buf = ctypes.create_string_buffer(512)
            L.gmvs_ctx_last_error(ctx, buf, 512)
            assert why in buf.value.decode(), buf.value
    finally:
        L.gmvs_ctx_destroy(ctx)
