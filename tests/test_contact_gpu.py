"""Quality-mode self contact on the GPU against the CPU oracle: cloth LBVH, face-pair lists
(bit-exact, reference order), proximity repulsion (float-atomic sums: 1e-4 x diagonal), CCD
impacts (bit-exact per test)."""
import numpy as np
import pytest

from tests.helpers import bits, diag, make_pair, small_scene
from xrtailor_gb300 import scenes

pytestmark = pytest.mark.gpu


def _state(n=12, frames=8, seed=0, noise=0.01):
    cloth, obs = small_scene(n)
    p = scenes._params(num_substeps=2, num_iterations=3, solve_bending=0, num_collision_passes=2,
                       enable_self_collision=0)
    g, o = make_pair(p, [cloth], [obs])
    for _ in range(frames):
        g.step()
        o.step()
    x = o.host_positions()
    np.testing.assert_array_equal(bits(g.host_positions()), bits(x))
    pred = (x + np.random.default_rng(seed).normal(0, noise, x.shape)).astype(np.float32)
    g.set_predicted(pred)
    o.set_predicted(pred)
    return g, o


def test_cloth_bvh_and_pairs_match_oracle(xrt):
    g, o = _state()
    g.cloth_bvh_build()
    o.cloth_bvh_build()
    a, b = g.export_cloth_bvh(), o.export_cloth_bvh()
    for k in ("morton", "objects", "nodes", "iesc", "eesc"):
        np.testing.assert_array_equal(a[k], b[k])
    np.testing.assert_array_equal(bits(a["aabbs"]), bits(b["aabbs"]))
    ng, no = g.update_pairs(1e-6), o.update_pairs(1e-6)
    assert ng == no > 0
    np.testing.assert_array_equal(g.pairs(), o.pairs())
    a, b = g.export_cloth_bvh(), o.export_cloth_bvh()  # after Update(ccd)
    np.testing.assert_array_equal(bits(a["aabbs"]), bits(b["aabbs"]))


def test_obstacle_update_ccd_matches_oracle(xrt):
    g, o = _state()
    g.obstacle_bvh_update_ccd()
    o.obstacle_bvh_update_ccd()
    a, b = g.export_obstacle_bvh(), o.export_obstacle_bvh()
    np.testing.assert_array_equal(bits(a["aabbs"]), bits(b["aabbs"]))


def test_repulsion_matches_oracle(xrt):
    g, o = _state(seed=1, noise=0.02)
    for s in (g, o):
        s.cloth_bvh_build()
        s.update_pairs(1e-6)
    before = o.predicted()
    for it in range(3):
        g.proximity_solve(1e-4, 0.25)
        o.proximity_solve(1e-4, 0.25)
        xg, xo = g.predicted(), o.predicted()
        err = np.abs(xg.astype(np.float64) - xo).max()
        assert err <= 1e-4 * diag(xo), err
    assert np.abs(o.predicted() - before).max() > 0  # the case exercises the repulsion


def test_impacts_match_oracle(xrt):
    g, o = _state(seed=2, noise=0.03)
    for s in (g, o):
        s.cloth_bvh_build()
        s.update_pairs(1e-6)
        s.check_impacts(1e-4)
    a, b = g.impacts(), o.impacts()
    np.testing.assert_array_equal(a["nodes"], b["nodes"])
    np.testing.assert_array_equal(a["is_vf"], b["is_vf"])
    hit = b["t"] >= 0
    np.testing.assert_array_equal(a["t"] >= 0, hit)  # the set of impacts is exact
    assert hit.sum() > 0
    for k in ("t", "w", "n"):  # impact times, weights and normals
        np.testing.assert_array_equal(bits(a[k][hit]), bits(b[k][hit]))
