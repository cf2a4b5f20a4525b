"""Batched form (xrt_add_instance): several garments, each against its own obstacle, in one
context.  Instance i must step bit for bit like a context that holds only cloth i and obstacle i:
the same coloring / tiles, particle hash, obstacle LBVH (a segment of the forest) and contacts.
"""
import numpy as np
import pytest

from tests.helpers import bits
from xrtailor_gb300 import ClothSolver, XrtError, scenes

pytestmark = pytest.mark.gpu


def _params(**kw):
    base = dict(num_substeps=3, num_iterations=5, stretch_compliance=1e-8, bend_compliance=1e-6,
                num_collision_passes=3, update_obstacle_animation=1)
    base.update(kw)
    return scenes._params(**base)


def _instances():
    """(cloth, obstacle or None, per-edge stretch compliance seed) of uneven sizes."""
    specs = [(20, 14, "sphere", 0.0), (24, 24, "plane", 0.4), (12, 18, None, -0.3),
             (16, 16, "sphere", 0.8)]
    out = []
    for k, (nx, ny, kind, dx) in enumerate(specs):
        cloth = scenes.rect_cloth(nx, ny, 1.0, ny / nx, origin=(dx, 0.35, 0.0), seed=10 + k)
        cloth.fixed_indices = np.array([0, nx - 1], np.uint32)
        cloth.attached_indices = np.array([0, nx - 1], np.uint32)
        obs = None
        if kind == "sphere":
            obs = scenes.icosphere(2, 0.3, center=(dx + 0.5, 0.0, 0.5 * ny / nx))
        elif kind == "plane":
            obs = scenes.ground_plane(8, 3.0, height=0.15, center=(dx + 0.5, 0.5))
        out.append((cloth, obs, k))
    return out


def _compliance(cloth, seed):
    """Per-edge stretch compliance, log-uniform in [1e-9, 1e-5] (edges in the library's order)."""
    s = ClothSolver(_params())
    s.add_cloth(cloth)
    s.start()
    ne = s.sizes().num_edges
    rng = np.random.default_rng(100 + seed)
    return np.exp(rng.uniform(np.log(1e-9), np.log(1e-5), ne)).astype(np.float32)


def _targets(obs, frame):
    """Obstacle motion: a small seeded translation per frame."""
    if obs is None:
        return None
    shift = np.array([0.01 * np.sin(0.7 * frame), -0.004 * frame, 0.006 * np.cos(frame)], np.float32)
    return (obs.positions + shift).astype(np.float32)


def _run_pair(params, frames=3, graph=True):
    inst = _instances()
    comps = [_compliance(c, k) for c, _, k in inst]
    batch = ClothSolver(params)
    for (c, o, _), comp in zip(inst, comps):
        batch.add_instance(c, o)
    batch.set_compliance(0, np.concatenate(comps))
    batch.start()
    batch.set_graph_mode(graph)
    singles = []
    for (c, o, _), comp in zip(inst, comps):
        s = ClothSolver(params)
        s.add_cloth(c)
        if o is not None:
            s.add_obstacle(o)
        s.set_compliance(0, comp)
        s.start()
        s.set_graph_mode(graph)
        singles.append(s)
    for f in range(frames):
        tg = [_targets(o, f + 1) for _, o, _ in inst]
        batch.set_obstacle_targets(np.concatenate([t for t in tg if t is not None]))
        batch.step()
        for s, t in zip(singles, tg):
            if t is not None:
                s.set_obstacle_targets(t)
            s.step()
    return inst, batch, singles


@pytest.mark.parametrize("graph", [True, False])
def test_instances_match_single_contexts(xrt, graph):
    inst, batch, singles = _run_pair(_params(), graph=graph)
    sz = batch.sizes()
    assert sz.num_instances == len(inst)
    xb = batch.host_positions()
    vb = batch.host_velocities()
    off = 0
    moved = 0.0
    for (c, _, _), s in zip(inst, singles):
        n = len(c.positions)
        xs = s.host_positions()
        np.testing.assert_array_equal(bits(xb[off:off + n]), bits(xs))
        np.testing.assert_array_equal(bits(vb[off:off + n]), bits(s.host_velocities()))
        moved = max(moved, float(np.abs(xs - c.positions).max()))
        off += n
    assert off == sz.num_vertices
    assert moved > 1e-3  # the cloths actually fell


def test_instance_particle_diameters_and_colors(xrt):
    """Each instance keeps its own particle diameter (first edge x 1.3) and its schedule."""
    inst, batch, singles = _run_pair(_params(), frames=1)
    for s in singles:
        assert s.sizes().num_instances == 1
    assert batch.sizes().particle_diameter == singles[0].sizes().particle_diameter


def test_obstacle_forest_matches_single_trees(xrt):
    inst, batch, singles = _run_pair(_params(), frames=2)
    fb = batch.export_obstacle_bvh()
    p_base = n_base = i_base = 0
    for (_, o, _), s in zip(inst, singles):
        if o is None:
            continue
        fs = s.export_obstacle_bvh()
        n = len(fs["morton"])
        nn = 2 * n - 1
        np.testing.assert_array_equal(fb["morton"][p_base:p_base + n], fs["morton"])
        np.testing.assert_array_equal(fb["objects"][p_base:p_base + n] - p_base, fs["objects"])
        np.testing.assert_array_equal(fb["nodes"][n_base:n_base + nn], fs["nodes"])
        np.testing.assert_array_equal(bits(fb["aabbs"][n_base:n_base + nn]), bits(fs["aabbs"]))
        np.testing.assert_array_equal(fb["iesc"][i_base:i_base + n - 1], fs["iesc"])
        np.testing.assert_array_equal(fb["eesc"][p_base:p_base + n], fs["eesc"])
        p_base += n
        n_base += nn
        i_base += n - 1
    assert n_base == batch.sizes().num_obstacle_bvh_nodes


def test_tiles_off_matches_too(xrt):
    """Per-color launches of a greedy coloring: the batch's coloring restricted to an instance is
    the instance's own greedy coloring."""
    inst = _instances()[:2]
    p = _params(num_substeps=2, num_iterations=4)
    batch = ClothSolver(p)
    batch.set_tile_vertices(0)
    for c, o, _ in inst:
        batch.add_instance(c, o)
    batch.start()
    singles = []
    for c, o, _ in inst:
        s = ClothSolver(p)
        s.set_tile_vertices(0)
        s.add_cloth(c)
        s.add_obstacle(o)
        s.start()
        singles.append(s)
    for _ in range(2):
        batch.step()
        for s in singles:
            s.step()
    xb = batch.host_positions()
    off = 0
    for (c, _, _), s in zip(inst, singles):
        n = len(c.positions)
        np.testing.assert_array_equal(bits(xb[off:off + n]), bits(s.host_positions()))
        off += n


def test_autotune_picks_a_timed_candidate(xrt):
    from xrtailor_gb300 import autotune
    inst = _instances()[:2]

    def make(t):
        s = ClothSolver(_params())
        s.set_tile_vertices(t)
        for c, o, _ in inst:
            s.add_instance(c, o)
        s.start()
        return s

    best, trials = autotune.tune(make, tiles=(64, 128), frames=1, warmup=1)
    assert len(trials) == 6 and all(ms > 0 for _, _, _, ms in trials)
    first = [r for r in trials if r[2] == 128]
    assert (best["tile_vertices"], best["dependent_launch"]) == min(first, key=lambda r: r[3])[:2]
    assert best["vertex_block"] in (64, 128, 256)
    assert autotune.subset(10, 4) == [0, 3, 6, 9] and autotune.subset(3, 8) == [0, 1, 2]


def test_batched_errors(xrt):
    c, o, _ = _instances()[0]
    s = ClothSolver(_params())
    s.add_cloth(c)
    with pytest.raises(XrtError):
        s.add_instance(c, o)  # merged context
    b = ClothSolver(_params())
    b.add_instance(c, o)
    with pytest.raises(XrtError):
        b.add_cloth(c)
    with pytest.raises(XrtError):
        b.add_obstacle(o)
    r = ClothSolver(_params(pbd_repulsion=1))
    r.add_instance(c, o)
    with pytest.raises(XrtError):
        r.start()  # Quality-mode repulsion is merged-mode only
