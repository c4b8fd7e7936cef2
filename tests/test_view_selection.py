"""View-selection scores (calc_score of the COLMAP conversion) on the
device against the CPU restatement, exactly, on a synthetic sparse model:
keypoints without points (-1), pairs with no shared points, and pairs whose
75th-percentile triangulation angle is below 1 degree (score zeroed)."""

import numpy as np
import pytest

from oracle import view_selection as ov


def sparse_model(V=24, P=4000, seed=0):
    rng = np.random.default_rng(seed)
    xyz = rng.normal(size=(P, 3)) * np.array([3.0, 1.0, 3.0])
    ang = 2 * np.pi * np.arange(V) / V
    centers = np.stack([8 * np.cos(ang), np.zeros(V), 8 * np.sin(ang)], 1)
    centers[1] = centers[0] + np.array([0.01, 0.0, 0.0])  # a near-duplicate camera: angles < 1 degree
    ids = []
    for i in range(V):
        d = centers[i] / np.linalg.norm(centers[i])
        seen = np.flatnonzero(((xyz - centers[i]) @ -d) > 6.0)   # points in front, roughly
        seen = rng.permutation(seen)[: rng.integers(200, 900)]
        kp = np.concatenate([seen, -np.ones(rng.integers(0, 50), np.int64)])
        ids.append(rng.permutation(kp))
    ids[5] = np.full(30, -1)                                     # an image without points
    return ids, xyz, centers


def test_oracle_selection_semantics():
    ids, xyz, c = sparse_model(V=6, P=500)
    s = ov.score_matrix(ids, xyz, c)
    assert np.allclose(s, s.T) and (np.diag(s) == 0).all()
    assert (s[5] == 0).all()


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [0, 1])
def test_device_scores_equal_oracle(gmvs_lib, cuda, seed):
    from gmvs_gb300 import view_selection as vs

    ids, xyz, c = sparse_model(seed=seed)
    want = ov.score_matrix(ids, xyz, c)
    got = vs.calc_scores(ids, xyz, c, cuda)
    assert np.array_equal(got, want)
    assert want[0, 1] == 0 and (want > 0).sum() > 20
    assert vs.select_views(got, 10) == vs.select_views(want, 10)


@pytest.mark.gpu
def test_device_scores_edge_cases(gmvs_lib, cuda):
    from gmvs_gb300 import view_selection as vs

    xyz = np.zeros((1, 3))
    assert vs.calc_scores([np.array([-1])], xyz, np.zeros((1, 3)), cuda).shape == (1, 1)
    with pytest.raises(ValueError):
        vs.calc_scores([np.array([3]), np.array([3])], xyz, np.zeros((2, 3)), cuda)
