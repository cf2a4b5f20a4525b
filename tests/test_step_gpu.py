"""Parity of the Swift frame on the GPU against the CPU oracle.

Every operation on the path is an IEEE +,-,*,/,sqrt or floor in the same order on both sides (the
bend angle's arccos is one polynomial evaluated the same way on both), so frames must match bit
for bit; the tolerance of 1e-4 of the cloth's bounding-box diagonal is checked as well."""
import numpy as np
import pytest

from tests.helpers import bits, diag, make_pair, small_scene, tube_mesh
from xrtailor_gb300 import ClothSolver, XrtError, scenes

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _params(**kw):
    base = dict(num_substeps=4, num_iterations=5, stretch_compliance=1e-8, bend_compliance=1e-6,
                num_collision_passes=4)
    base.update(kw)
    return scenes._params(**base)


def _close(g, o, exact):
    xg, xo = g.host_positions(), o.host_positions()
    assert np.isfinite(xg).all()
    if exact:
        np.testing.assert_array_equal(bits(xg), bits(xo))
    err = np.abs(xg.astype(np.float64) - xo).max()
    assert err <= TOL * diag(xo), (err, diag(xo))
    return err


def test_setup_exports_match_oracle(xrt):
    cloth, obs = small_scene(20, attached=[0, 19, 210])
    g, o = make_pair(_params(), [cloth], [obs], colors_from_gpu=False)
    e1, r1 = g.edges()
    e2, r2 = o.edges()
    np.testing.assert_array_equal(e1, e2)
    np.testing.assert_array_equal(bits(r1), bits(r2))
    b1, t1 = g.bends()
    b2, t2 = o.bends()
    np.testing.assert_array_equal(b1, b2)
    np.testing.assert_array_equal(bits(t1), bits(t2))
    for k, idx in ((0, e1), (1, b1)):  # the GPU's tile schedule is a valid coloring
        col = g.coloring(k)
        assert len(col) == len(idx)
        seen = set()
        for c, verts in zip(col.tolist(), idx.tolist()):
            for v in verts:
                assert (c, v) not in seen
                seen.add((c, v))
        assert o.coloring_valid(k)  # the oracle's own greedy coloring
    for a, b in zip(g.lra(), o.lra()):
        np.testing.assert_array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))
    np.testing.assert_array_equal(g.obstacle_rtri(), o.obstacle_rtri())
    s = g.sizes()
    assert (s.num_edges, s.num_bends, s.num_lra) == (len(e2), len(b2), 3 * 400)
    assert abs(s.particle_diameter - o.particle_diameter()) == 0


@pytest.mark.parametrize("self_collision", [0, 1])
def test_frame_bit_exact_without_bending(xrt, self_collision):
    cloth, obs = small_scene(16)
    p = _params(solve_bending=0, enable_self_collision=self_collision)
    g, o = make_pair(p, [cloth], [obs], particle_diameter=0.02)
    for f in range(3):
        g.step()
        o.step()
        _close(g, o, exact=True)
    np.testing.assert_array_equal(bits(g.host_velocities()), bits(o.host_velocities()))
    np.testing.assert_array_equal(bits(g.host_normals()), bits(o.host_normals()))
    g.synchronize()


def test_contacts_and_bvh_match_oracle(xrt):
    cloth, obs = small_scene(24)
    p = _params(solve_bending=0, enable_self_collision=1, num_substeps=2, num_iterations=3)
    g, o = make_pair(p, [cloth], [obs], particle_diameter=0.02)
    for _ in range(8):  # fall onto the sphere
        g.step()
        o.step()
    _close(g, o, exact=True)
    cg, co = g.export_contacts(), o.export_contacts()
    for k in ("vf_index", "rt_index"):
        np.testing.assert_array_equal(cg[k], co[k])
    for k in ("vf_qs", "rt_qc", "ee"):
        np.testing.assert_array_equal(bits(cg[k]), bits(co[k]))
    assert (cg["vf_index"] >= 0).sum() > 0
    bg, bo = g.export_obstacle_bvh(), o.export_obstacle_bvh()
    for k in ("morton", "objects", "nodes", "iesc", "eesc"):
        np.testing.assert_array_equal(bg[k], bo[k])
    np.testing.assert_array_equal(bits(bg["aabbs"]), bits(bo["aabbs"]))
    np.testing.assert_array_equal(g.export_neighbors(), o.export_neighbors())


def test_frame_with_bending(xrt):
    # the bend angle uses the same arccos polynomial on both sides, so bending frames are exact
    cloth, obs = small_scene(16)
    g, o = make_pair(_params(), [cloth], [obs], particle_diameter=0.02)
    for _ in range(2):
        g.step()
        o.step()
        _close(g, o, exact=True)


def test_new_substep_dt_after_start_matches_oracle(xrt):
    # the tile records carry compliance / dt^2 terms: a new dt after start re-evaluates them
    cloth, obs = small_scene(16)
    g, o = make_pair(_params(), [cloth], [obs], particle_diameter=0.02)
    g.step()
    o.step()
    p = _params(num_substeps=3)
    g.set_params(p)
    o.set_params(p)
    for _ in range(2):
        g.step()
        o.step()
        _close(g, o, exact=True)


def test_small_config_one_frame(xrt):
    sc = scenes.plain_small(64)
    p = scenes.scene_params(sc)
    g, o = make_pair(p, [sc.cloth], [sc.obstacle], particle_diameter=sc.particle_diameter)
    g.step()
    o.step()
    _close(g, o, exact=True)


def test_plain_colored_launches_match_tiled(xrt):
    """The same greedy coloring run as plain per-color launches (caller-supplied coloring) and the
    default tile schedule each match the oracle given their own coloring."""
    from oracle.oracle import OracleSolver
    cloth, obs = small_scene(20)
    p = _params()
    o0 = OracleSolver(p)
    o0.add_cloth(cloth, particle_diameter=0.02)
    o0.add_obstacle(obs)
    o0.start()
    g, o = make_pair(p, [cloth], [obs], particle_diameter=0.02)
    gp = ClothSolver(p)
    gp.add_cloth(cloth, particle_diameter=0.02)
    gp.add_obstacle(obs)
    gp.set_coloring(0, o0.coloring(0))
    gp.set_coloring(1, o0.coloring(1))
    gp.start()
    for _ in range(2):
        g.step()
        o.step()
        gp.step()
        o0.step()
    _close(g, o, exact=True)
    _close(gp, o0, exact=True)
    assert gp.sizes().launches_per_frame > g.sizes().launches_per_frame


@pytest.mark.parametrize("tile", [32, 64, 200])
def test_tile_sizes_match_oracle(xrt, tile):
    """Any tile size gives a valid schedule; the oracle, run with the exported coloring, matches
    bit for bit (tiles of 32 vertices on a 24-wide grid have footprints spanning 3 tiles)."""
    cloth, obs = small_scene(24, attached=scenes.two_corner_pins(24))
    p = _params(num_substeps=2, num_iterations=4, num_collision_passes=2)
    from oracle.oracle import OracleSolver
    g = ClothSolver(p)
    g.set_tile_vertices(tile)
    g.add_cloth(cloth, particle_diameter=0.02)
    g.add_obstacle(obs)
    g.start()
    o = OracleSolver(p)
    o.add_cloth(cloth, particle_diameter=0.02)
    o.add_obstacle(obs)
    o.set_coloring(0, g.coloring(0))
    o.set_coloring(1, g.coloring(1))
    o.start()
    for _ in range(2):
        g.step()
        o.step()
    _close(g, o, exact=True)
    with pytest.raises(XrtError):
        g.set_tile_vertices(64)  # after start


def test_later_context_with_smaller_tiles(xrt):
    """A context started after another, with smaller tile footprints, must not break the first
    (the tile kernels' shared-memory limit is shared by the process)."""
    big_cloth, obs = small_scene(40)
    small_cloth, _ = small_scene(8)
    p = _params(num_substeps=2, num_iterations=3, num_collision_passes=2)
    big = ClothSolver(p)
    big.set_tile_vertices(1024)
    big.add_cloth(big_cloth, particle_diameter=0.02)
    big.add_obstacle(obs)
    big.start()
    small = ClothSolver(p)
    small.add_cloth(small_cloth, particle_diameter=0.02)
    small.start()
    for _ in range(2):
        big.step()
        small.step()
    big.synchronize()
    small.synchronize()
    assert np.isfinite(big.host_positions()).all()


@pytest.mark.parametrize("graph", [True, False])
def test_dependent_launch_is_bit_identical(xrt, graph):
    """Programmatic dependent launch changes only when kernels start, never what they compute:
    a garment-like scene (tiles, self collision, obstacle contacts, LRA) gives the same bits with
    it on and off, in graph replay and eagerly, and both match the oracle."""
    cloth, obs = small_scene(48, attached=scenes.two_corner_pins(48))
    p = _params(num_substeps=3, num_iterations=6, num_collision_passes=3)
    runs = []
    for pdl in (True, False):
        g, o = make_pair(p, [cloth], [obs], particle_diameter=0.02)
        g.set_graph_mode(graph)
        g.set_dependent_launch(pdl)
        for _ in range(3):
            g.step()
            o.step()
        _close(g, o, exact=True)
        runs.append(g.host_positions())
    np.testing.assert_array_equal(bits(runs[0]), bits(runs[1]))


def test_vertex_block_is_bit_identical(xrt):
    """The per-vertex kernels' block size (xrt_set_vertex_block, an autotuner knob) changes only
    how vertices are grouped into blocks: every block size gives the oracle's bits."""
    cloth, obs = small_scene(40, attached=scenes.two_corner_pins(40))
    p = _params(num_substeps=3, num_iterations=5, num_collision_passes=3)
    runs = []
    for block in (64, 128, 512):
        g, o = make_pair(p, [cloth], [obs], particle_diameter=0.02)
        g.set_vertex_block(block)
        for _ in range(3):
            g.step()
            o.step()
        _close(g, o, exact=True)
        runs.append(g.host_positions())
    np.testing.assert_array_equal(bits(runs[0]), bits(runs[2]))
    with pytest.raises(XrtError):
        g.set_vertex_block(100)


def test_pbd_repulsion_frame(xrt):
    cloth, obs = small_scene(14)
    p = _params(solve_bending=0, pbd_repulsion=1, pbd_thickness=1e-3, repulsion_relaxation=0.25,
                num_iterations=12, num_substeps=2)
    g, o = make_pair(p, [cloth], [obs], particle_diameter=0.02)
    for _ in range(6):
        g.step()
        o.step()
    _close(g, o, exact=False)  # repulsion deltas are float-atomic sums on the GPU


@pytest.mark.parametrize("pinned_slots", [True, False])
def test_long_range_attachments(xrt, pinned_slots):
    cloth, obs = small_scene(16, attached=[0, 15], pins=pinned_slots)
    p = _params(solve_bending=0, enable_self_collision=0, long_range_stretchiness=1.02)
    g, o = make_pair(p, [cloth], [obs])
    for _ in range(3):
        g.step()
        o.step()
        _close(g, o, exact=True)


def test_moving_obstacle_and_bindings(xrt):
    body = tube_mesh()
    cloth, _ = small_scene(12)
    # bind four cloth vertices to body triangles
    tris = body.triangles[:4]
    cloth.binded_indices = np.array([30, 40, 50, 60], np.uint32)
    cloth.bind_obstacle_tri = tris.astype(np.uint32)
    cloth.bind_barycentric = np.tile(np.array([[0.2, 0.3, 0.5]], np.float32), (4, 1))
    cloth.bind_stiffnesses = np.full(4, 0.5, np.float32)
    cloth.bind_distances = np.zeros(4, np.float32)
    p = _params(solve_bending=0, enable_self_collision=1)
    g, o = make_pair(p, [cloth], [body.mesh], particle_diameter=0.02)
    for f in range(4):
        tgt = body.pose((f + 1) / 60.0)
        g.set_obstacle_targets(tgt)
        o.set_obstacle_targets(tgt)
        g.step()
        o.step()
        _close(g, o, exact=True)
    np.testing.assert_array_equal(bits(g.obstacle_positions()), bits(o.obstacle_positions()))


def test_multiple_cloths_and_obstacles(xrt):
    c1, o1 = small_scene(10, seed=3)
    c2, _ = small_scene(8, seed=4, size=0.6)
    o2 = scenes.ground_plane(6, 2.0, height=-0.5, center=(0.5, 0.5))
    p = _params(solve_bending=0)
    g, o = make_pair(p, [c1, c2], [o1, o2], particle_diameter=0.02)
    for _ in range(2):
        g.step()
        o.step()
        _close(g, o, exact=True)


def test_no_obstacle(xrt):
    cloth, _ = small_scene(16, obstacle=None)
    p = _params(solve_bending=0, enable_self_collision=0)
    g, o = make_pair(p, [cloth], [])
    for _ in range(3):
        g.step()
        o.step()
        _close(g, o, exact=True)


def test_graph_replay_equals_eager(xrt):
    cloth, obs = small_scene(16)
    p = _params(enable_self_collision=1)
    a = ClothSolver(p)
    b = ClothSolver(p)
    for s in (a, b):
        s.add_cloth(cloth, particle_diameter=0.02)
        s.add_obstacle(obs)
        s.start()
    b.set_graph_mode(False)
    for _ in range(3):
        a.step()
        b.step()
    np.testing.assert_array_equal(bits(a.host_positions()), bits(b.host_positions()))
    assert a.sizes().launches_per_frame > 0


def test_invalid_inputs_are_rejected(xrt):
    cloth, obs = small_scene(8)
    bad = _params(num_substeps=1, num_iterations=2, num_collision_passes=3)
    with pytest.raises(XrtError):
        ClothSolver(bad)
    s = ClothSolver(_params())
    broken = scenes.grid_cloth(4, 1.0)
    broken.triangles = broken.triangles.copy()
    broken.triangles[0, 0] = 99
    with pytest.raises(XrtError):
        s.add_cloth(broken)
    s.add_cloth(cloth)
    e, _ = s.edges()
    s.set_coloring(0, np.zeros(len(e), np.uint32))  # every edge the same color: not independent
    with pytest.raises(XrtError):
        s.start()
    t = ClothSolver(_params())
    t.add_cloth(cloth)
    t.start()
    with pytest.raises(XrtError):
        t.add_obstacle(obs)
