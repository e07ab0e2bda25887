"""KeyframeSelector (host utility of the Python module): the SE(3) distance
against an independent restatement (scipy's rotation vector and the
left-Jacobian V of SE(3), solved rather than inverted in closed form), and
the keyframe rule."""
import os
import sys

import numpy as np
import pytest
from scipy.spatial.transform import Rotation

from mrfmap_gb300 import _build


@pytest.fixture(scope="module")
def G():
    path = _build.build_pymodule()
    sys.path.insert(0, os.path.dirname(path))
    import GVDBPyModules
    return GVDBPyModules


def _pose(rotvec, t):
    P = np.eye(4, dtype=np.float32)
    P[:3, :3] = Rotation.from_rotvec(rotvec).as_matrix()
    P[:3, 3] = t
    return P


def _ref_distance(A, B):
    D = np.linalg.inv(A.astype(np.float64)) @ B.astype(np.float64)
    w = Rotation.from_matrix(D[:3, :3]).as_rotvec()
    th = np.linalg.norm(w)
    W = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-8:
        V = np.eye(3)
    else:
        V = np.eye(3) + (1 - np.cos(th)) / th ** 2 * W + (th - np.sin(th)) / th ** 3 * W @ W
    u = np.linalg.solve(V, D[:3, 3])
    return th, np.linalg.norm(u)


def test_distance_matches_independent_restatement(G):
    ks = G.KeyframeSelector(0.1, 0.1)
    rng = np.random.default_rng(0)
    cases = [(np.zeros(3), np.zeros(3), np.zeros(3), np.zeros(3)),          # identity
             (np.zeros(3), np.zeros(3), np.array([1e-7, 0, 0]), np.array([0.1, 0, 0])),  # tiny angle
             (np.zeros(3), np.zeros(3), np.array([0, 0, np.pi - 1e-7]), np.array([0, 1.0, 0]))]  # near pi
    for _ in range(50):
        cases.append((rng.normal(0, 1, 3), rng.normal(0, 2, 3), rng.normal(0, 1, 3), rng.normal(0, 2, 3)))
    for r1, t1, r2, t2 in cases:
        A, B = _pose(r1, t1), _pose(r2, t2)
        rot, trans = ks.compute_rot_trans(A, B)
        er, et = _ref_distance(A, B)
        assert rot == pytest.approx(er, abs=2e-5, rel=2e-5)
        assert trans == pytest.approx(et, abs=2e-4, rel=2e-4)
        assert ks.compute_distance(0.0, 0.0, A, B) == pytest.approx(rot + trans, rel=1e-6)


def test_keyframe_rule(G):
    ks = G.KeyframeSelector(0.1, 0.1)
    P0 = _pose(np.zeros(3), np.zeros(3))
    assert ks.is_keyframe(P0)
    assert not ks.is_keyframe(_pose([0.05, 0, 0], [0.05, 0, 0]))   # within both thresholds
    assert ks.is_keyframe(_pose([0.05, 0, 0], [0.2, 0, 0]))        # translated far enough
    assert ks.is_keyframe(_pose([0.3, 0, 0], [0.0, 0, 0]))         # rotated far enough
    assert ks.num_keyframes() == 3
    ks.set_thresh(1.0, 1.0)
    assert not ks.is_keyframe(_pose([0.3, 0, 0], [0.5, 0, 0]))
