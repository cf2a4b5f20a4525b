"""Skinning data of the synthetic body: the joint transforms reproduce its pose, through the
oracle's restatement of SMPL's lbs.  CPU only."""
import numpy as np

from oracle.oracle import lbs
from xrtailor_gb300 import scenes


def test_joint_transforms_reproduce_the_pose():
    body = scenes.TubeBody(seed=5)
    rest, outer, joints, weights = body.skin()
    for t in (0.0, 0.37, 1.5):
        x = lbs(rest, outer, joints, weights, body.joint_transforms(t))
        np.testing.assert_allclose(x, body.pose(t), atol=2e-6)


def test_lbs_blends_influences_in_csr_order():
    rng = np.random.default_rng(0)
    rest = rng.normal(size=(5, 3)).astype(np.float32)
    outer = np.array([0, 1, 3, 3, 4, 6], np.uint32)        # vertex 2 has no influence
    joints = np.array([0, 0, 1, 1, 0, 1], np.uint32)
    weights = np.array([1.0, 0.25, 0.75, 1.0, 0.5, 0.5], np.float32)
    T = rng.normal(size=(2, 12)).astype(np.float32)
    out = lbs(rest, outer, joints, weights, T)
    M = [np.vstack([T[j].reshape(3, 4), [0, 0, 0, 1]]).astype(np.float64) for j in range(2)]
    for v in range(5):
        want = np.zeros(3)
        for k in range(outer[v], outer[v + 1]):
            want += weights[k] * (M[joints[k]] @ np.append(rest[v], 1.0))[:3]
        np.testing.assert_allclose(out[v], want, rtol=1e-5, atol=1e-6)
    assert (out[2] == 0).all()
