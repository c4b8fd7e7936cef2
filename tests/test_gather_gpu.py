"""Point gather of the fusion scripts on the device against the numpy
restatement (oracle/gather.py): the same points in the same raster order,
coordinates within 1e-5 relative of the float64 values, the view-normal test
identical except for dot products within 1e-6 of the threshold."""

import math

import numpy as np
import pytest
import torch

from gmvs_gb300 import engine, synthetic
from oracle import gather as og

pytestmark = pytest.mark.gpu


def _inputs(seed, H=256, W=320):
    sc = synthetic.small_scene(seed, H=H, W=W)
    rng = np.random.default_rng(seed)
    depth = sc.depths[0].astype(np.float32)
    depth[rng.random(depth.shape) < 0.2] = 0.0                 # unfused pixels
    n = sc.normals[0] + rng.normal(0, 0.3, sc.normals[0].shape)
    n = (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)
    R, t = sc.R[0], sc.t[0]
    pose = np.eye(4)
    pose[:3, :3] = R.T
    pose[:3, 3] = -R.T @ t                                      # camera-to-world
    return depth, n, sc.K[0], pose


@pytest.mark.parametrize("seed,angle", [(0, 80.0), (1, 60.0), (2, 89.0)])
def test_gather_matches_restatement(gmvs_lib, cuda, seed, angle):
    depth, n, K, pose = _inputs(seed)
    thr = math.cos(angle / 180 * math.pi)
    pts, fac, od, on = engine.gather_points(torch.from_numpy(depth).to(cuda), torch.from_numpy(n).to(cuda), K, pose,
                                            thr)
    a32, f32, d32, n32, dot32 = og.gather_points(depth, n, K, pose, thr, np.float32)
    a64, f64, _, _, dot64 = og.gather_points(depth, n, K, pose, thr, np.float64)
    pts, fac = pts.cpu().numpy(), fac.cpu().numpy()
    assert pts.shape == a32.shape
    scale = np.maximum(np.abs(a64[:, :3]), 1.0)
    assert np.max(np.abs(pts[:, :3] - a64[:, :3]) / scale) < 1e-5
    assert np.array_equal(pts[:, 3:], a32[:, 3:])
    tie = np.abs(dot64 - thr) < 1e-6
    assert abs(len(fac) - len(f32)) <= int(tie.sum())
    if not tie.any():
        assert np.array_equal(fac[:, 3:], f32[:, 3:])
        assert np.array_equal(od.cpu().numpy(), d32) and np.array_equal(on.cpu().numpy(), n32)
    assert 0 < len(fac) < len(pts)


def test_gather_edge_cases(gmvs_lib, cuda):
    K = np.array([[100, 0, 16], [0, 100, 12], [0, 0, 1]], np.float32)
    z = torch.zeros((24, 32), device=cuda)
    nz = torch.zeros((24, 32, 3), device=cuda)
    pts, fac, od, on = engine.gather_points(z, nz, K, np.eye(4), 0.5)
    assert len(pts) == 0 and len(fac) == 0 and not od.any()
    # one pixel, one point
    d = torch.zeros((1, 1), device=cuda) + 2.0
    n = torch.tensor([[[0.0, 0.0, -1.0]]], device=cuda)
    pts, fac, _, _ = engine.gather_points(d, n, np.eye(3), np.eye(4), 0.5)
    assert pts.shape == (1, 6) and len(fac) == 1
    assert torch.allclose(pts[0, :3], torch.tensor([0.0, 0.0, 2.0], device=cuda))
