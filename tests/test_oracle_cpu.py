"""The CPU oracle checked on its own, without a GPU: known-answer tests of the primitive tests
and Morton codes, structural invariants of the LBVH, brute-force candidate sets, topology
invariants, geodesic distances against an independent Dijkstra, and the golden fixtures."""
import os

import numpy as np
import pytest

from oracle import oracle as orc
from tests.helpers import bits, prim_soup
from xrtailor_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def py_expand(v):
    r = 0
    for i in range(10):
        if (v >> i) & 1:
            r |= 1 << (3 * i)
    return r


def test_expand_bits_is_bit_interleaving(oracle_lib):
    for v in range(1024):
        assert orc.expand_bits(v) == py_expand(v)


def test_morton_code_known_answers(oracle_lib):
    assert orc.morton_code([0, 0, 0]) == 0
    assert orc.morton_code([1, 1, 1]) == 0x3FFFFFFF           # clamped to 1023 on every axis
    assert orc.morton_code([-5, 2, 0.5]) == py_expand(1023) * 2 + py_expand(512)
    rng = np.random.default_rng(0)
    for p in rng.uniform(-0.1, 1.1, size=(500, 3)).astype(np.float32):
        q = [int(min(max(np.float32(c) * np.float32(1024), 0), 1023)) for c in p]
        assert orc.morton_code(p) == py_expand(q[0]) * 4 + py_expand(q[1]) * 2 + py_expand(q[2])


def test_nearest_point_regions(oracle_lib):
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    d, q, uvw = orc.nearest_point([0.2, 0.2, 1.0], tri)           # face region
    assert d == np.float32(1.0) and np.allclose(q, [0.2, 0.2, 0]) and np.allclose(uvw, [0.6, 0.2, 0.2])
    d, q, _ = orc.nearest_point([-1, -1, 0], tri)                 # vertex a
    assert np.array_equal(q, tri[0]) and d == np.float32(np.sqrt(2))
    d, q, _ = orc.nearest_point([2, -1, 0], tri)                  # vertex b
    assert np.array_equal(q, tri[1])
    d, q, _ = orc.nearest_point([0.5, -1, 0], tri)                # edge ab
    assert np.allclose(q, [0.5, 0, 0]) and d == np.float32(1.0)
    d, q, _ = orc.nearest_point([1, 1, 0], tri)                   # edge bc
    assert np.allclose(q, [0.5, 0.5, 0])


def test_nearest_point_against_float64(oracle_lib):
    rng = np.random.default_rng(1)
    for _ in range(300):
        tri = rng.normal(size=(3, 3)).astype(np.float32)
        p = rng.normal(size=3).astype(np.float32)
        d, q, _ = orc.nearest_point(p, tri)
        # brute force over a fine barycentric grid + exact edge projections
        best = np.inf
        a, b, c = tri.astype(np.float64)
        for s, t in np.random.default_rng(2).uniform(size=(4000, 2)):
            if s + t > 1:
                s, t = 1 - s, 1 - t
            best = min(best, np.linalg.norm(a + s * (b - a) + t * (c - a) - p))
        assert d <= best + 1e-5


def test_ray_intersect_known_answers(oracle_lib):
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    assert orc.ray_intersect([0.2, 0.2, 1], [0, 0, -1], 2.0, tri) == np.float32(1.0)
    assert orc.ray_intersect([0.2, 0.2, 1], [0, 0, -1], 0.5, tri) == np.inf       # too short
    assert orc.ray_intersect([2, 2, 1], [0, 0, -1], 2.0, tri) == np.float32(3.4028235e38)
    assert orc.ray_intersect([0.2, 0.2, 1], [1, 0, 0], 2.0, tri) == np.float32(3.4028235e38)


def test_closest_segment_segment_known_answers(oracle_lib):
    d, st, cc = orc.closest_seg_seg([0, 0, 0], [1, 0, 0], [0.5, -1, 1], [0.5, 1, 1])
    assert d == np.float32(1.0) and np.allclose(st, [0.5, 0.5])
    d, st, cc = orc.closest_seg_seg([0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0])   # parallel
    assert d == np.float32(1.0) and st[0] == 0
    d, st, cc = orc.closest_seg_seg([0, 0, 0], [0, 0, 0], [1, 0, 0], [1, 2, 0])   # point-segment
    assert d == np.float32(1.0) and st[1] == 0


def test_arccos_polynomial_error_bound(oracle_lib):
    """A&S 4.4.46 as evaluated in float by the oracle and the bend kernel."""
    x = np.linspace(0.0, 1.0, 200001, dtype=np.float32)
    got = np.array([orc.acos_as(float(v)) for v in x[::97]], np.float64)
    ref = np.arccos(x[::97].astype(np.float64))
    assert np.abs(got - ref).max() < 3e-7  # 2e-8 formula error + float evaluation


def test_solve_cubic_roots(oracle_lib):
    # (x-0.2)(x-0.5)(x-0.8) = x^3 - 1.5x^2 + 0.66x - 0.08
    n, x = orc.solve_cubic(1.0, -1.5, 0.66, -0.08)
    assert n == 3 and np.allclose(np.sort(x), [0.2, 0.5, 0.8], atol=1e-5)
    n, x = orc.solve_cubic(1.0, 0.0, 1.0, -2.0)  # one real root at 1
    assert n == 1 and abs(x[0] - 1.0) < 1e-5
    # a = b = 0 (parallel motion): Newton's method from 0 on 0.4 x - 0.1, the same every call
    for _ in range(3):
        n, x = orc.solve_cubic(0.0, 0.0, 0.4, -0.1)
        assert n == 1 and x[0] == np.float32(0.1) / np.float32(0.4)


def _check_tree(t, n):
    nodes, aabbs = t["nodes"], t["aabbs"]
    ni = n - 1
    assert sorted(t["objects"].tolist()) == list(range(n))
    assert np.all(np.diff(t["morton"].astype(np.int64)) >= 0)
    for k in range(ni):
        l, r = nodes[k, 1], nodes[k, 2]
        assert nodes[l, 0] == k and nodes[r, 0] == k
        lo = np.minimum(aabbs[l, :3], aabbs[r, :3])
        hi = np.maximum(aabbs[l, 3:], aabbs[r, 3:])
        assert np.array_equal(aabbs[k, :3], lo) and np.array_equal(aabbs[k, 3:], hi)
    for i in range(n):
        assert nodes[ni + i, 3] == t["objects"][i]


@pytest.mark.parametrize("n", [1, 2, 5, 300, 4000])
def test_lbvh_structure(oracle_lib, n):
    b = orc.OracleLbvh()
    b.build(prim_soup(n, seed=n))
    t = b.export()
    _check_tree(t, n)
    # a box query covering everything returns every leaf (left-first) when n <= 256
    counts, cands = b.query(2, np.array([[-9, -9, -9, 9, 9, 9]], np.float32))
    assert counts[0] == min(n, 256)
    if n <= 256:
        assert sorted(cands[0, :n].tolist()) == list(range(n))


def test_lbvh_point_queries_equal_brute_force(oracle_lib):
    n = 3000
    p = prim_soup(n, seed=4, size=0.1)
    b = orc.OracleLbvh()
    b.build(p)
    t = b.export()
    ni = n - 1
    leaf_box = {int(t["nodes"][ni + i, 3]): t["aabbs"][ni + i] for i in range(n)}
    rng = np.random.default_rng(5)
    q = rng.uniform(-1, 1, size=(500, 3)).astype(np.float32)
    counts, cands = b.query(0, q)
    for i in range(len(q)):
        expect = {o for o, bx in leaf_box.items()
                  if np.all(q[i] > bx[:3]) and np.all(q[i] < bx[3:])}
        assert set(cands[i, : counts[i]].tolist()) == expect


def test_grid_topology_counts_and_ownership(oracle_lib):
    n = 12
    cloth = scenes.grid_cloth(n, 1.0)
    o = orc.OracleSolver(scenes._params())
    o.add_cloth(cloth)
    o.add_obstacle(cloth)  # the same grid as an obstacle exercises the R-triangle masks
    o.start()
    s = o.sizes()
    E = 2 * n * (n - 1) + (n - 1) ** 2
    assert s["num_edges"] == E and s["num_bends"] == E - 4 * (n - 1)
    assert s["num_triangles"] == 2 * (n - 1) ** 2
    assert o.coloring_valid(0) and o.coloring_valid(1)
    rt = o.obstacle_rtri()
    tri = cloth.triangles
    owned_v = np.zeros(n * n, int)
    edge_owner = {}
    for f, m in enumerate(rt):
        for k in range(3):
            if (m >> k) & 1:
                owned_v[tri[f, k]] += 1
            if (m >> (k + 3)) & 1:
                e = tuple(sorted((tri[f, k], tri[f, (k + 1) % 3])))
                edge_owner[e] = edge_owner.get(e, 0) + 1
    assert np.all(owned_v == 1)
    assert len(edge_owner) == E and set(edge_owner.values()) == {1}


def test_geodesic_lra_against_scipy(oracle_lib):
    sp = pytest.importorskip("scipy.sparse.csgraph")
    import scipy.sparse as sps
    n = 10
    cloth = scenes.grid_cloth(n, 1.0, jitter=1e-3, seed=3)
    cloth.attached_indices = np.array([0, n - 1], np.uint32)
    o = orc.OracleSolver(scenes._params())
    o.add_cloth(cloth)
    o.start()
    src, tgt, rest = o.lra()
    e, _ = o.edges()
    pos = cloth.positions.astype(np.float64)
    w = np.linalg.norm(pos[e[:, 0]] - pos[e[:, 1]], axis=1)
    g = sps.coo_matrix((w, (e[:, 0], e[:, 1])), shape=(n * n, n * n))
    d = sp.dijkstra(g, directed=False, indices=[0, n - 1])
    np.testing.assert_allclose(rest.reshape(2, -1), d, rtol=1e-5, atol=1e-6)
    assert np.array_equal(src, np.repeat(np.array([0, n - 1], np.uint32), n * n))


def test_bend_element_orientation(oracle_lib):
    """GenerateBendingElements (ClothSolverHelper.cpp:4-88): f1 = (idx1, idx2, idx3) and
    f2 = (idx2, idx1, idx4) counter-clockwise.  The reference decides the winding with a substring
    test on "a,b,c,a,b,c" that can match across numbers (e.g. "1,2" inside "1,257"); with edges
    oriented as in their first face, f1 always holds idx1 -> idx2, so the test never has to swap
    and its false positives cannot change a result.  Faces such as (257, 2, 1) exercise it."""
    from xrtailor_gb300.solver import Mesh
    pos = np.random.default_rng(0).normal(size=(258, 3)).astype(np.float32)
    tri = np.array([[257, 2, 1], [1, 2, 3], [3, 2, 12], [12, 2, 257]], np.uint32)
    for mesh in (Mesh(pos, tri), scenes.grid_cloth(9, 1.0)):
        o = orc.OracleSolver(scenes._params())
        o.add_cloth(mesh)
        o.start()
        b, th = o.bends()
        t = mesh.triangles
        assert len(b) > 0 and np.all(np.isfinite(th))
        for i1, i2, i3, i4 in b:
            def has(f, a, c, d):
                r = list(t[f])
                return any(r[k] == a and r[(k + 1) % 3] == c and r[(k + 2) % 3] == d for k in range(3))
            assert any(has(f, i1, i2, i3) for f in range(len(t)))
            assert any(has(f, i2, i1, i4) for f in range(len(t)))


def test_golden_fixtures(oracle_lib):
    """Regression pin of the oracle: outputs recorded by tests/golden/make_golden.py."""
    from tests.golden import make_golden
    for name, fn in make_golden.CASES.items():
        path = os.path.join(GOLDEN, name + ".npz")
        assert os.path.exists(path), f"missing fixture {path}"
        ref = np.load(path)
        cur = fn()
        for k in ref.files:
            a, b = ref[k], cur[k]
            if a.dtype.kind == "f" and k.startswith("approx_"):
                np.testing.assert_allclose(b, a, rtol=0, atol=1e-5, err_msg=f"{name}:{k}")
            elif a.dtype.kind == "f":
                np.testing.assert_array_equal(bits(b), bits(a), err_msg=f"{name}:{k}")
            else:
                np.testing.assert_array_equal(b, a, err_msg=f"{name}:{k}")
