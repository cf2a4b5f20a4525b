"""The oracle's impact-zone collision step (ImpactZoneOptimization::CollisionStep,
impact_zone/Entry.cu:140-256) on the CPU: a state whose x0 -> x path crosses the obstacle or the
cloth itself is made crossing-free, a second step on the result finds no impact, and an impact
that free cloth vertices cannot resolve (the obstacle sweeping through a pinned vertex) is solved
at deform 1 by moving the obstacle."""
import numpy as np

from oracle.oracle import OracleSolver
from tests.helpers import small_scene
from xrtailor_gb300 import scenes


def _params(**kw):
    base = dict(num_substeps=2, num_iterations=3, solve_bending=0, num_collision_passes=2,
                enable_self_collision=0)
    base.update(kw)
    return scenes._params(**base)


def _oracle(n=12, obstacle="sphere", pins=True, **kw):
    cloth, obs = small_scene(n, obstacle=obstacle, pins=pins)
    o = OracleSolver(_params(**kw))
    o.add_cloth(cloth)
    if obs is not None:
        o.add_obstacle(obs)
    o.start()
    return o, cloth


def test_step_makes_the_obstacle_crossing_free():
    o, _ = _oracle()
    for _ in range(4):
        o.step()
    x = o.host_positions()
    pred = x.copy()
    pred[:, 1] -= 0.12  # through the sphere's cap within one step
    o.set_predicted(pred)
    st = o.collision_step()
    assert st["success"] == 1 and st["deform"] == 0
    assert st["impacts"] > 0 and st["passes"] > 1
    after = o.predicted()
    assert np.isfinite(after).all()
    moved = np.abs(after - pred).max(axis=1)
    assert moved.max() < 0.13           # vertices move back towards x0, not past it
    assert (moved > 0).sum() < len(x)   # only vertices of impact zones move
    again = o.collision_step()
    assert again == {"success": 1, "deform": 0, "passes": 1, "impacts": 0, "zones": 0, "solves": 0}


def test_step_separates_two_sheets():
    a = scenes.grid_cloth(8, 1.0, origin=(0.0, 0.50, 0.0), jitter=1e-3, seed=3)
    b = scenes.grid_cloth(8, 1.0, origin=(0.05, 0.45, 0.05), jitter=1e-3, seed=4)
    o = OracleSolver(_params())
    o.add_cloth(a)
    o.add_cloth(b)
    o.start()
    x = o.host_positions()
    nb = len(b.positions) // 3
    pred = x.copy()
    pred[-nb:, 1] += 0.1  # the lower sheet moves up through the upper one
    o.set_predicted(pred)
    st = o.collision_step()
    assert st["success"] == 1 and st["impacts"] > 0
    after = o.predicted()
    assert np.isfinite(after).all()
    # the sheets no longer cross: the lower sheet stays below the upper one where they overlap
    assert o.collision_step()["impacts"] == 0


def test_unresolvable_at_deform_0_moves_the_obstacle():
    o, cloth = _oracle(n=8)
    o.step()
    x = o.host_positions()
    ob0 = o.obstacle_positions()
    pin = x[cloth.fixed_indices[0]]
    tgt = ob0 + np.array([pin[0] - 0.5, pin[1] + 0.05, pin[2] - 0.5], np.float32)
    o.set_obstacle_targets(tgt.astype(np.float32))
    o.set_predicted(x)
    st = o.collision_step()
    # deform 0 cannot move the pinned vertex: 100 passes, then deform 1 moves obstacle vertices
    assert st["deform"] == 1 and st["success"] == 1
    assert o.collision_step()["impacts"] == 0


def test_frames_with_impact_zone_stay_finite():
    o, _ = _oracle(n=10, impact_zone=1)
    for _ in range(3):
        o.step()
    assert np.isfinite(o.host_positions()).all()
    assert np.isfinite(o.host_velocities()).all()


def test_imminent_repulsion_acts_and_stays_finite():
    xs = []
    for on in (0, 1):
        o, _ = _oracle(n=10, imminent_repulsion=on, imminent_thickness=0.05)
        for _ in range(8):  # the sheet reaches the sphere at frame 6
            o.step()
        x = o.host_positions()
        assert np.isfinite(x).all() and np.isfinite(o.host_velocities()).all()
        xs.append(x)
    assert np.abs(xs[1] - xs[0]).max() > 1e-6  # the impulses moved the cloth
