"""View selection of the COLMAP conversion on the device: the pairwise
scores of calc_score (gmvs/scripts/colmap2mvs.py:324-357) for all image
pairs in one launch, and the top-k source selection that the script writes
to pair.txt (colmap2mvs.py:505-523)."""

from __future__ import annotations

import ctypes
from typing import List, Sequence

import numpy as np
import torch

from . import _abi
from ._abi import check, lib


def calc_scores(point_ids: Sequence[np.ndarray], xyz: np.ndarray, centers: np.ndarray,
                device=None) -> np.ndarray:
    """Score matrix [V, V] (symmetric, zero diagonal).  point_ids: per image
    the point3D id of each keypoint (-1 = none); xyz: float64 [P, 3] indexed
    by point id; centers: float64 [V, 3] camera centres."""
    dev = device or torch.device("cuda", torch.cuda.current_device())
    V = len(point_ids)
    lists = [np.sort(np.asarray(a, np.int64)[np.asarray(a) >= 0]) for a in point_ids]
    if any(len(a) and a[-1] >= len(xyz) for a in lists):
        raise ValueError("a point id is beyond xyz")
    off = np.zeros(V + 1, np.int64)
    off[1:] = np.cumsum([len(a) for a in lists])
    ids = np.concatenate(lists).astype(np.int32) if off[-1] else np.zeros(1, np.int32)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_off, d_ids = t(off), t(ids)
    d_xyz, d_c = t(np.asarray(xyz, np.float64).reshape(-1, 3)), t(np.asarray(centers, np.float64).reshape(V, 3))
    scores = torch.empty((V, V), dtype=torch.float32, device=dev)
    check(lib().gmvs_view_scores(d_off.data_ptr(), d_ids.data_ptr(), V, d_xyz.data_ptr(), int(d_xyz.shape[0]),
                                 d_c.data_ptr(), scores.data_ptr(), _abi.stream_ptr()))
    return scores.cpu().numpy().astype(np.float64)


def select_views(score: np.ndarray, num_view: int) -> List[List[tuple]]:
    """Per image the num_view best (source index, score), best first, as the
    script's argsort(...)[::-1][:num_view]."""
    out = []
    for i in range(score.shape[0]):
        order = np.argsort(score[i])[::-1][:num_view]
        out.append([(int(k), float(score[i, k])) for k in order])
    return out
