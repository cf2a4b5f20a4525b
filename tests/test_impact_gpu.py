"""The impact-zone collision step on the GPU (xrt_collision_step, include/xrt_impact.h) against
the CPU oracle's restatement of ImpactZoneOptimization::CollisionStep (impact_zone/Entry.cu):
the pass structure (passes, impacts, zones, zone solves, deform level) is equal and the positions
are bit-exact, through the obstacle, between two sheets, at deform 1 and over whole frames."""
import numpy as np
import pytest

from tests.helpers import bits, make_pair, small_scene
from xrtailor_gb300 import scenes

pytestmark = pytest.mark.gpu


def _params(**kw):
    base = dict(num_substeps=2, num_iterations=3, solve_bending=0, num_collision_passes=2,
                enable_self_collision=0)
    base.update(kw)
    return scenes._params(**base)


def _same(a, b):
    np.testing.assert_array_equal(bits(a), bits(b))


def test_collision_step_through_the_obstacle_matches_oracle(xrt):
    cloth, obs = small_scene(12)
    g, o = make_pair(_params(), [cloth], [obs])
    for _ in range(4):
        g.step()
        o.step()
    x = o.host_positions()
    _same(g.host_positions(), x)
    pred = x.copy()
    pred[:, 1] -= 0.12
    g.set_predicted(pred)
    o.set_predicted(pred)
    sg, so = g.collision_step(), o.collision_step()
    assert sg == so and sg["success"] == 1 and sg["impacts"] > 0, (sg, so)
    _same(g.predicted(), o.predicted())
    assert g.collision_step()["impacts"] == 0


def test_collision_step_between_sheets_matches_oracle(xrt):
    a = scenes.grid_cloth(16, 1.0, origin=(0.0, 0.50, 0.0), jitter=1e-3, seed=3)
    b = scenes.grid_cloth(16, 1.0, origin=(0.05, 0.45, 0.05), jitter=1e-3, seed=4)
    g, o = make_pair(_params(), [a, b], [])
    x = o.host_positions()
    nb = len(b.positions) // 3
    pred = x.copy()
    pred[-nb:, 1] += 0.1  # parallel motion: linear coplanarity polynomials in every test
    g.set_predicted(pred)
    o.set_predicted(pred)
    for s in (g, o):  # the CCD tests of the first pass
        s.cloth_bvh_build()
        s.update_pairs(1e-4)
        s.check_impacts(1e-4)
    ia, ib = g.impacts(), o.impacts()
    hit = ib["t"] >= 0
    assert hit.sum() > 1000
    for k in ("t", "w", "n"):
        _same(ia[k][hit], ib[k][hit])
    sg, so = g.collision_step(), o.collision_step()
    assert sg == so and sg["success"] == 1 and sg["impacts"] > 0, (sg, so)
    _same(g.predicted(), o.predicted())
    assert g.collision_step()["impacts"] == 0


def test_collision_step_at_deform_1_matches_oracle(xrt):
    cloth, obs = small_scene(8)
    g, o = make_pair(_params(), [cloth], [obs])
    g.step()
    o.step()
    x = o.host_positions()
    pin = x[cloth.fixed_indices[0]]
    tgt = (o.obstacle_positions() + np.array([pin[0] - 0.5, pin[1] + 0.05, pin[2] - 0.5])).astype(np.float32)
    for s in (g, o):
        s.set_obstacle_targets(tgt)
        s.set_predicted(x)
    sg, so = g.collision_step(), o.collision_step()
    assert sg == so and sg["deform"] == 1 and sg["success"] == 1, (sg, so)
    _same(g.predicted(), o.predicted())


def test_frames_with_impact_zone_match_oracle(xrt):
    cloth, obs = small_scene(12)
    p = _params(impact_zone=1, num_substeps=4, num_iterations=4)
    p.gravity[1] = -60.0  # the cloth reaches the sphere within a few frames
    g, o = make_pair(p, [cloth], [obs])
    for _ in range(6):
        g.step()
        o.step()
        _same(g.host_positions(), o.host_positions())
        _same(g.host_velocities(), o.host_velocities())
    g.synchronize()


def test_large_sheet_ends_crossing_free(xrt):
    from xrtailor_gb300 import ClothSolver
    cloth, obs = small_scene(64)
    g = ClothSolver(_params())
    g.add_cloth(cloth)
    g.add_obstacle(obs)
    g.start()
    g.step()
    x = g.host_positions()
    pred = x.copy()
    pred[:, 1] -= 0.15
    g.set_predicted(pred)
    st = g.collision_step()
    assert st["success"] == 1 and st["impacts"] > 100, st
    g.synchronize()
    assert np.isfinite(g.predicted()).all()
    assert g.collision_step()["impacts"] == 0


def test_one_large_zone_matches_oracle(xrt):
    """A 192 x 192 sheet crossing the icosphere by 0.12: one zone of about 5,600 impacts, more
    than sixteen 256-element chunks, so it is solved by 16-block clusters of 1,024 threads (four
    chunk trees at once) where the device holds them.  Sums keep the blocked order, so the pass
    statistics and positions equal the oracle's bit for bit."""
    n = 192
    cloth = scenes.grid_cloth(n, 1.0, origin=(0.0, 0.35, 0.0), jitter=1e-3, seed=1)
    cloth.fixed_indices = scenes.two_corner_pins(n)
    sphere = scenes.icosphere(2, 0.3, center=(0.5, 0.0, 0.5))
    g, o = make_pair(_params(), [cloth], [sphere])
    for _ in range(4):
        g.step()
        o.step()
    x = o.host_positions()
    _same(g.host_positions(), x)
    pred = x.copy()
    pred[:, 1] -= 0.12
    g.set_predicted(pred)
    o.set_predicted(pred)
    sg = g.collision_step(launch_shapes=True)
    so = o.collision_step()
    shapes = sg.pop("wide_solves")
    assert sg == so and sg["success"] == 1 and sg["impacts"] > 4096, (sg, so)
    assert shapes[0] + shapes[1] > 0, shapes  # the zone outgrew the 8-block clusters
    _same(g.predicted(), o.predicted())


def test_rejected_in_batched_context(xrt):
    from xrtailor_gb300 import ClothSolver
    cloth, obs = small_scene(8)
    s = ClothSolver(_params(impact_zone=1))
    s.add_instance(cloth, obs)
    with pytest.raises(RuntimeError):
        s.start()


def _diag(x):
    return float(np.linalg.norm(x.max(axis=0) - x.min(axis=0)))


def test_frames_with_imminent_repulsion_match_oracle(xrt):
    # impulses are summed with float atomics, as in the reference: 1e-4 of the diagonal
    cloth, obs = small_scene(12)
    p = _params(imminent_repulsion=1, imminent_thickness=0.05)
    g, o = make_pair(p, [cloth], [obs])
    for _ in range(8):  # the sheet reaches the sphere at frame 6
        g.step()
        o.step()
        xo = o.host_positions()
        err = float(np.abs(g.host_positions().astype(np.float64) - xo).max())
        assert err <= 1e-4 * _diag(xo), err


def test_quality_frames_match_oracle(xrt):
    # SimulateQuality's pieces together: FEM fabric, imminent and PBD repulsion, impact zones
    from xrtailor_gb300 import ClothSolver
    cloth, obs = small_scene(12)
    p = _params(imminent_repulsion=1, imminent_thickness=0.02, pbd_repulsion=1, impact_zone=1,
                num_substeps=2, num_iterations=4)
    g, o = make_pair(p, [cloth], [obs], fem=ClothSolver.fem_material())
    for _ in range(8):
        g.step()
        o.step()
        xo = o.host_positions()
        err = float(np.abs(g.host_positions().astype(np.float64) - xo).max())
        assert err <= 1e-4 * _diag(xo), err
    g.synchronize()


def test_imminent_quadratures_match_oracle(xrt):
    # the quadratures involve no atomics: bit-exact; then solves (float atomics) to 1e-4
    cloth, obs = small_scene(12)
    g, o = make_pair(_params(), [cloth], [obs])
    for _ in range(7):  # the sheet on the sphere
        g.step()
        o.step()
    x = o.host_positions()
    pred = (x + np.random.default_rng(5).normal(0, 0.01, x.shape)).astype(np.float32)
    for s in (g, o):
        s.set_predicted(pred)
        s.cloth_bvh_build()
    ng, no = g.imminent_generate(), o.imminent_generate()
    assert ng == no > 0, (ng, no)
    (an, ab), (bn, bb) = g.quads(), o.quads()
    np.testing.assert_array_equal(an, bn)
    _same(ab, bb)
    for _ in range(3):
        g.imminent_solve(0.05, 0.25, 1.0 / 120)
        o.imminent_solve(0.05, 0.25, 1.0 / 120)
    err = float(np.abs(g.predicted().astype(np.float64) - o.predicted()).max())
    assert err <= 1e-4 * _diag(x), err
    assert np.abs(o.predicted() - pred).max() > 0  # the impulses acted
