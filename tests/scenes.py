"""Scene helpers shared by the tests (ground-truth planes, argument packing)."""

from __future__ import annotations

import numpy as np

from gmvs_gb300 import synthetic


def cam_args(sc: synthetic.Scene, ids):
    return [synthetic.camera_args(sc, i) for i in ids]


def gt_planes(sc: synthetic.Scene, view: int) -> np.ndarray:
    """Camera-frame planes (n, d) of the ground truth of `view` [H, W, 4]."""
    H, W = sc.hw
    K, R = sc.K[view], sc.R[view]
    d = sc.depths[view].astype(np.float64)
    ys, xs = np.mgrid[0:H, 0:W]
    X = np.stack([(xs - K[0, 2]) / K[0, 0] * d, (ys - K[1, 2]) / K[1, 1] * d, d], -1)
    n = sc.normals[view].astype(np.float64) @ R.T
    w = -np.sum(n * X, -1)
    return np.concatenate([n, w[..., None]], -1).astype(np.float32)


def random_planes(sc: synthetic.Scene, view: int, rng: np.random.Generator, dmin: float, dmax: float) -> np.ndarray:
    """Random camera-frame planes facing the camera, depth uniform in [dmin, dmax]."""
    H, W = sc.hw
    K = sc.K[view]
    d = rng.uniform(dmin, dmax, size=(H, W))
    n = rng.normal(size=(H, W, 3))
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    ys, xs = np.mgrid[0:H, 0:W]
    X = np.stack([(xs - K[0, 2]) / K[0, 0] * d, (ys - K[1, 2]) / K[1, 1] * d, d], -1)
    flip = np.sum(n * X, -1) > 0
    n[flip] = -n[flip]
    w = -np.sum(n * X, -1)
    return np.concatenate([n, w[..., None]], -1).astype(np.float32)


def gpu_view(sc: synthetic.Scene, ids, dev, dmin, dmax, **kw):
    """engine.ViewInputs of reference ids[0] with sources ids[1:] on `dev`."""
    import torch

    from gmvs_gb300 import engine

    imgs = torch.from_numpy(sc.images[ids].astype(np.float32)).to(dev)
    cams = [engine.make_camera(*synthetic.camera_args(sc, i)) for i in ids]
    return engine.ViewInputs(cams=cams, images=[imgs[k] for k in range(len(ids))], depth_min=dmin, depth_max=dmax,
                             stream_id=ids[0], **kw)
