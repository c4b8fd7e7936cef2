"""CPU restatement of the view-selection score of the COLMAP conversion,
test infrastructure only: calc_score (gmvs/scripts/colmap2mvs.py:324-357)
and the top-k selection that writes pair.txt (colmap2mvs.py:505-523).

calc_score(i, j): the points of image i (its point3D_ids, in order, -1 for
keypoints without a point) that also appear in image j; for each, the
triangulation angle in degrees between the two camera centres seen from the
point; score = their number, or 0 when the 75th-percentile angle
(sorted(angles)[int(0.75 * n)]) is below 1 degree."""

from __future__ import annotations

import numpy as np


def calc_score(ids_i, ids_j, xyz, center_i, center_j) -> float:
    set_j = set(int(x) for x in ids_j)
    shared = [int(it) for it in ids_i if int(it) in set_j]
    score = 0
    angles = []
    for pid in shared:
        if pid == -1:
            continue
        p = xyz[pid]
        a, b = center_i - p, center_j - p
        theta = (180 / np.pi) * np.arccos(np.dot(a, b) / np.linalg.norm(a) / np.linalg.norm(b))
        angles.append(theta)
        score += 1
    if angles:
        if sorted(angles)[int(len(angles) * 0.75)] < 1:
            score = 0.0
    return float(score)


def score_matrix(point_ids, xyz, centers) -> np.ndarray:
    """point_ids: per image an int array (-1 = no point); xyz [P, 3] float64
    indexed by point id; centers [V, 3] float64."""
    V = len(point_ids)
    s = np.zeros((V, V))
    for i in range(V):
        for j in range(i + 1, V):
            s[i, j] = s[j, i] = calc_score(point_ids[i], point_ids[j], xyz, centers[i], centers[j])
    return s
