"""Obstacle skinning on the device (xrt_set_obstacle_skinning): the skinned targets equal the
oracle's restatement of SMPL's lbs bit for bit, and frames driven by joint transforms equal frames
driven by those targets set from the host."""
import numpy as np
import pytest

from oracle.oracle import lbs
from tests.helpers import bits
from xrtailor_gb300 import ClothSolver, XrtError, scenes

pytestmark = pytest.mark.gpu


def _solver(body, n=24, skinning=True):
    cloth = scenes.grid_cloth(n, 0.6, origin=(-0.3, body.height + 0.02, -0.3), jitter=1e-3, seed=2)
    cloth.fixed_indices = scenes.two_corner_pins(n)
    p = scenes._params(num_substeps=4, num_iterations=4, num_collision_passes=4,
                       bend_compliance=100.0)
    s = ClothSolver(p)
    s.add_cloth(cloth)
    s.add_obstacle(body.mesh)
    s.start()
    if skinning:
        rest, outer, joints, weights = body.skin()
        s.set_obstacle_skinning(rest, outer, joints, weights, body.bones)
    return s


def test_skinned_targets_match_the_oracle(xrt):
    body = scenes.TubeBody(seed=7)
    s = _solver(body)
    rest, outer, joints, weights = body.skin()
    for f in range(3):
        T = body.joint_transforms((f + 1) / 60.0)
        s.set_joint_transforms(T)
        s.step()
        # the frame commits its targets as the obstacle's positions
        want = lbs(rest, outer, joints, weights, T)
        np.testing.assert_array_equal(bits(s.obstacle_positions()), bits(want))


def test_skinned_frames_equal_frames_with_host_targets(xrt):
    body = scenes.TubeBody(seed=8)
    a = _solver(body, skinning=True)
    b = _solver(body, skinning=False)
    rest, outer, joints, weights = body.skin()
    for f in range(4):
        T = body.joint_transforms((f + 1) / 60.0)
        a.set_joint_transforms(T)
        b.set_obstacle_targets(lbs(rest, outer, joints, weights, T))
        a.step()
        b.step()
    np.testing.assert_array_equal(bits(a.host_positions()), bits(b.host_positions()))


def test_batched_skinning_numbers_joints_across_instances(xrt):
    bodies = [scenes.TubeBody(seed=11), scenes.TubeBody(seed=12, radius=0.12)]
    p = scenes._params(num_substeps=2, num_iterations=2, num_collision_passes=2)
    s = ClothSolver(p)
    for k, body in enumerate(bodies):
        cloth = scenes.grid_cloth(16 + 4 * k, 0.5, origin=(-0.25, body.height + 0.02, -0.25),
                                  seed=k)
        s.add_instance(cloth, body.mesh)
    s.start()
    parts = [b.skin() for b in bodies]
    rest = np.concatenate([q[0] for q in parts])
    outer = np.concatenate([[0], np.cumsum(np.concatenate([np.diff(q[1]) for q in parts]))])
    joints = np.concatenate([q[2] + k * bodies[0].bones for k, q in enumerate(parts)])
    weights = np.concatenate([q[3] for q in parts])
    s.set_obstacle_skinning(rest, outer.astype(np.uint32), joints.astype(np.uint32), weights,
                            2 * bodies[0].bones)
    T = np.concatenate([b.joint_transforms(0.25 + k) for k, b in enumerate(bodies)])
    s.set_joint_transforms(T)
    s.step()
    np.testing.assert_array_equal(bits(s.obstacle_positions()),
                                  bits(lbs(rest, outer, joints, weights, T)))


def test_skinning_errors(xrt):
    body = scenes.TubeBody(seed=9)
    s = _solver(body, skinning=False)
    rest, outer, joints, weights = body.skin()
    with pytest.raises(XrtError):
        s.set_joint_transforms(body.joint_transforms(0.0))          # skinning not on
    bad = joints.copy()
    bad[5] = body.bones                                             # joint out of range
    with pytest.raises(XrtError):
        s.set_obstacle_skinning(rest, outer, bad, weights, body.bones)
    bad_outer = outer.copy()
    bad_outer[3], bad_outer[4] = bad_outer[4], bad_outer[3]         # decreasing offsets
    with pytest.raises(XrtError):
        s.set_obstacle_skinning(rest, bad_outer, joints, weights, body.bones)
    s.set_obstacle_skinning(rest, outer, joints, weights, body.bones)
    with pytest.raises(XrtError):
        s.set_obstacle_targets(body.pose(0.0))                      # skinning owns the targets
    s.set_obstacle_skinning(None)
    s.set_obstacle_targets(body.pose(0.0))
    s.step()
