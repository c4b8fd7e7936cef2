"""Device segment statistics (fusion_planar_mask, filter_by_var_map,
sliding_window_normal) against the oracle, bit for bit, on superpixel maps
that reach every branch of the reference's decisions."""

import numpy as np
import pytest
import torch

from gmvs_gb300 import _abi, engine
from gmvs_gb300 import planar_initer as pi
from gmvs_gb300.synthetic import superpixel_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rows,cols,seed", [(240, 320, 0), (1200, 1600, 1), (37, 53, 2)])
def test_device_segment_statistics_equal_oracle(gmvs_lib, orc, cuda, rows, cols, seed):
    seg, planar, n, var = superpixel_case(rows, cols, seed)
    t = lambda a: torch.from_numpy(a).to(cuda)
    ws = engine.Workspace(cuda)
    for th in (10, 100):
        want = orc.fusion_planar_mask(seg, planar, n, rows, cols, th)
        got = engine.fusion_planar_mask(t(seg), t(planar), t(n), th, workspace=ws).cpu().numpy()
        assert np.array_equal(got, want)
        if rows >= 240:  # every branch reached
            assert (want == 300).any() and (want > 300).any() and ((want > 0) & (want < 300)).any()
    for thr in (0.2, 0.45):
        want = orc.filter_by_var_map(var, seg, thr)
        assert np.array_equal(engine.filter_by_var_map(t(var), t(seg), thr, workspace=ws).cpu().numpy(), want)
    for win in (1, 3, 7):
        want = orc.sliding_window_normal(planar, n, win)
        got = engine.sliding_window_normal(t(planar), t(n), win).cpu().numpy()
        assert np.array_equal(got, want, equal_nan=True)


def test_module_a_mirror_runs_device_path_for_cuda_tensors(gmvs_lib, cuda):
    seg, planar, n, var = superpixel_case(96, 128, 3)
    t = lambda a: torch.from_numpy(a).to(cuda)
    got = pi.fusion_planar_mask(t(seg), t(planar), t(n), 96, 128, 20)
    assert got.is_cuda and np.array_equal(got.cpu().numpy(), pi.fusion_planar_mask(seg, planar, n, 96, 128, 20))
    got = pi.filter_by_var_map(t(var), t(seg), 0.3)
    assert got.is_cuda and np.array_equal(got.cpu().numpy(), pi.filter_by_var_map(var, seg, 0.3))
    got = pi.sliding_window_normal(t(planar), t(n), 5)
    assert got.is_cuda and np.array_equal(got.cpu().numpy(), pi.sliding_window_normal(planar, n, 5))


def test_edge_cases(gmvs_lib, orc, cuda):
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    rows, cols = 16, 24
    zeros = np.zeros((rows, cols), np.int32)
    n = np.tile(np.array([0, 0, 1], np.float32), (rows, cols, 1))
    var = np.ones((rows, cols), np.float32)
    # only segment 0, and a max_seg_id above the largest id
    assert not engine.fusion_planar_mask(t(zeros), t(zeros), t(n), 1, max_seg_id=9).any()
    assert not engine.filter_by_var_map(t(var), t(zeros), 2.0, max_seg_id=9).any()
    one = np.ones((rows, cols), np.int32)
    assert np.array_equal(engine.fusion_planar_mask(t(one), t(zeros), t(n), 10).cpu().numpy(),
                          orc.fusion_planar_mask(one, zeros, n, rows, cols, 10))
    # an id above max_seg_id is an error, not an out-of-bounds write
    with pytest.raises(_abi.GmvsError):
        engine.fusion_planar_mask(t(one * 5), t(zeros), t(n), 10, max_seg_id=3)
    with pytest.raises(_abi.GmvsError):
        engine.filter_by_var_map(t(var), t(-one), 1.0, max_seg_id=3)
