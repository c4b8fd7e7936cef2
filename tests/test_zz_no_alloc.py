"""gmvs_fuse_fixed_scratch (fusion with library-owned scratch, no device
allocation) against gmvs_fuse with caller scratch, through the C ABI.

Collected last on purpose: it must give the same results in a fresh process
and after every other test has run in the same process."""

import ctypes

import numpy as np
import pytest

from gmvs_gb300 import _abi, engine, synthetic


def _noisy_inputs(sc, seed):
    rng = np.random.default_rng(seed)
    d = (sc.depths * (1.0 + rng.normal(0, 0.005, sc.depths.shape))).astype(np.float32)
    n = sc.normals + rng.normal(0, 0.02, sc.normals.shape)
    return d, (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)


def _fuse_args(sc, ref, src, dev_d, dev_n, masks, out_depth, out_normal, out_count):
    ids = [ref] + list(src)
    H, W = sc.hw
    a = _abi.gmvs_fuse_view()
    a.height, a.width, a.num_views = H, W, int(masks.shape[0])
    a.problem = engine.make_problem(ref, list(src))
    for j, i in enumerate(ids):
        a.cams[j] = engine.make_camera(*synthetic.camera_args(sc, i))
        a.depths[j] = dev_d[i].data_ptr()
        a.normals[j] = dev_n[i].data_ptr()
    a.masks = masks.data_ptr()
    a.geom_consistent = 3
    a.out_depth, a.out_normal, a.out_count = out_depth.data_ptr(), out_normal.data_ptr(), out_count.data_ptr()
    return a


@pytest.mark.gpu
def test_fixed_scratch_matches_caller_scratch(gmvs_lib, small, cuda):
    import torch

    L = _abi.lib()
    d_in, n_in = _noisy_inputs(small, seed=5)
    V = small.num_views
    H, W = small.hw
    dev_d = torch.from_numpy(d_in).to(cuda)
    dev_n = torch.from_numpy(n_in).to(cuda)
    masks_ref = torch.zeros((V, H, W), dtype=torch.bool, device=cuda)
    masks_fix = torch.zeros((V, H, W), dtype=torch.bool, device=cuda)
    scratch = torch.empty(L.gmvs_fuse_scratch_bytes(H, W), dtype=torch.uint8, device=cuda)
    stream = _abi.stream_ptr()
    fused = 0
    # two fixed-scratch calls in a row on different views: the second finds
    # the shared scratch as the first left it
    for ref, src in small.problems[:2]:
        outs = []
        for masks, fixed in ((masks_ref, False), (masks_fix, True)):
            od = torch.full((H, W), 7.0, device=cuda)
            on = torch.full((H, W, 3), 7.0, device=cuda)
            oc = torch.full((H, W), 7, dtype=torch.int32, device=cuda)
            a = _fuse_args(small, ref, src, dev_d, dev_n, masks, od, on, oc)
            if fixed:
                rc = L.gmvs_fuse_fixed_scratch(ctypes.byref(a), stream)
            else:
                rc = L.gmvs_fuse(ctypes.byref(a), scratch.data_ptr(), scratch.numel(), stream)
            _abi.check(rc)
            outs.append((od.cpu().numpy(), on.cpu().numpy(), oc.cpu().numpy()))
        (rd, rn, rcnt), (fd, fn, fcnt) = outs
        assert np.array_equal(fcnt, rcnt)
        assert np.array_equal(fd, rd)
        assert np.array_equal(fn, rn)
        assert torch.equal(masks_fix, masks_ref)
        fused += int((rcnt >= 3).sum())
    assert fused > 0 and masks_ref.any()


@pytest.mark.gpu
def test_fixed_scratch_at_its_limit_then_smaller(gmvs_lib, small, cuda):
    """A view of exactly GMVS_FUSE_FIXED_MAX_PIXELS (2048 x 2048) fills the
    whole array; a smaller view afterwards finds a stale tail beyond its own
    pixels, which it never reads.  Both equal gmvs_fuse with caller scratch."""
    import torch

    L = _abi.lib()
    big = synthetic.small_scene(3, H=2048, W=2048, device=cuda)
    assert big.hw[0] * big.hw[1] == _abi.FUSE_FIXED_MAX_PIXELS
    stream = _abi.stream_ptr()
    for sc, (ref, src) in ((big, big.problems[0]), (small, small.problems[3])):
        d_in, n_in = _noisy_inputs(sc, seed=8)
        V = sc.num_views
        H, W = sc.hw
        dev_d = torch.from_numpy(d_in).to(cuda)
        dev_n = torch.from_numpy(n_in).to(cuda)
        scratch = torch.empty(L.gmvs_fuse_scratch_bytes(H, W), dtype=torch.uint8, device=cuda)
        outs, all_masks = [], []
        for fixed in (False, True):
            masks = torch.zeros((V, H, W), dtype=torch.bool, device=cuda)
            od = torch.full((H, W), 7.0, device=cuda)
            on = torch.full((H, W, 3), 7.0, device=cuda)
            oc = torch.full((H, W), 7, dtype=torch.int32, device=cuda)
            a = _fuse_args(sc, ref, src, dev_d, dev_n, masks, od, on, oc)
            if fixed:
                rc = L.gmvs_fuse_fixed_scratch(ctypes.byref(a), stream)
            else:
                rc = L.gmvs_fuse(ctypes.byref(a), scratch.data_ptr(), scratch.numel(), stream)
            _abi.check(rc)
            outs.append((od.cpu().numpy(), on.cpu().numpy(), oc.cpu().numpy()))
            all_masks.append(masks)
        (rd, rn, rcnt), (fd, fn, fcnt) = outs
        assert np.array_equal(fcnt, rcnt) and np.array_equal(fd, rd) and np.array_equal(fn, rn)
        assert torch.equal(all_masks[0], all_masks[1])
        assert int((rcnt >= 3).sum()) > 0


def test_fixed_scratch_rejects_oversized_views(gmvs_lib):
    # the size check comes before any CUDA call, so this runs without a GPU
    a = _abi.gmvs_fuse_view()
    a.height, a.width = 2048, 2049
    assert 2048 * 2049 > _abi.FUSE_FIXED_MAX_PIXELS
    rc = _abi.lib().gmvs_fuse_fixed_scratch(ctypes.byref(a), None)
    assert rc == _abi.ERR_INVALID
    msg = _abi.lib().gmvs_last_error().decode()
    assert "exceeds the fixed scratch" in msg and str(_abi.FUSE_FIXED_MAX_PIXELS) in msg
