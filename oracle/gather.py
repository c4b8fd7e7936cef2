"""CPU restatement (numpy) of the fusion scripts' point gather, test
infrastructure only: gmvs/scripts/mvs_fusion_segmentaion.py:195-236.

Per view: ray directions d = ((x - cx) / fx, (y - cy) / fy, 1) rotated by the
camera-to-world rotation (`dirs_ @ rot_mat.T`), points o + depth * d for
depth > 0 in raster order (torch boolean indexing), the view-normal test
dot(-d, n) > cos(angle), and the depth/normal map keeping only the pixels
that pass it.  `dtype` float32 follows the script's arithmetic step by
step; float64 gives the exact values."""

from __future__ import annotations

import numpy as np


def gather_points(depth, normal, K, pose, cos_thresh, dtype=np.float32):
    H, W = depth.shape
    K = np.asarray(K, np.float64).reshape(3, 3)
    P = np.asarray(pose, np.float64).reshape(4, 4)
    f = lambda v: np.asarray(v, dtype)
    yy, xx = np.mgrid[0:H, 0:W].astype(dtype)
    dx = (xx - f(K[0, 2])) / f(K[0, 0])
    dy = (yy - f(K[1, 2])) / f(K[1, 1])
    R = f(P[:3, :3])
    o = f(P[:3, 3])
    dirs = np.stack([R[i, 0] * dx + R[i, 1] * dy + R[i, 2] for i in range(3)], -1).reshape(-1, 3)
    d = f(depth).reshape(-1)
    n = f(normal).reshape(-1, 3)
    valid = d > 0
    pts = o[None, :] + d[valid, None] * dirs[valid]
    dot = (-dirs[valid, 0]) * n[valid, 0] + (-dirs[valid, 1]) * n[valid, 1] + (-dirs[valid, 2]) * n[valid, 2]
    facing = dot > f(cos_thresh)
    allp = np.concatenate([pts, n[valid]], 1)
    keep = np.zeros(H * W, bool)
    keep[np.flatnonzero(valid)[facing]] = True
    od = np.where(keep, d, 0).reshape(H, W).astype(dtype)
    on = np.where(keep[:, None], n, 0).reshape(H, W, 3).astype(dtype)
    return allp, allp[facing], od, on, dot
