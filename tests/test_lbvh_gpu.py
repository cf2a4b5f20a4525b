"""LBVH parity on the GPU: Morton codes, sorted primitive order, BVH topology, boxes, escape
tables, refit and stackless candidate lists must equal the CPU oracle bit for bit
(BVH.cu:22-722, 770-818, 957-1055)."""
import numpy as np
import pytest

from tests.helpers import bits, prim_soup

pytestmark = pytest.mark.gpu


def _pair(prims, pred=None, scr=0.0):
    from oracle.oracle import OracleLbvh
    from xrtailor_gb300 import Lbvh
    g, o = Lbvh(), OracleLbvh()
    g.build(prims, pred, scr)
    o.build(prims, pred, scr)
    return g, o


def _same_tree(g, o):
    a, b = g.export(), o.export()
    assert a["unique"] == b["unique"]
    np.testing.assert_array_equal(a["morton"], b["morton"])
    np.testing.assert_array_equal(a["objects"], b["objects"])
    np.testing.assert_array_equal(a["nodes"], b["nodes"])
    np.testing.assert_array_equal(bits(a["aabbs"]), bits(b["aabbs"]))
    np.testing.assert_array_equal(a["iesc"], b["iesc"])
    np.testing.assert_array_equal(a["eesc"], b["eesc"])
    return a


def _same_queries(g, o, kind, q):
    cg, kg = g.query(kind, q)
    co, ko = o.query(kind, q)
    np.testing.assert_array_equal(cg, co)
    for i in np.nonzero(cg)[0]:
        np.testing.assert_array_equal(kg[i, : cg[i]], ko[i, : co[i]])
    return cg


@pytest.mark.parametrize("n", [1, 2, 3, 7, 1000, 50000])
def test_build_matches_oracle(xrt, n):
    p = prim_soup(n, seed=n)
    g, o = _pair(p)
    t = _same_tree(g, o)
    if n > 1:
        assert (t["nodes"][0, 0] == 0xFFFFFFFF)  # root has no parent


def test_duplicate_codes_take_64bit_keys(xrt):
    base = prim_soup(300, seed=5)
    p = np.concatenate([base, base, base[:50]])  # identical boxes -> equal Morton codes
    g, o = _pair(p)
    t = _same_tree(g, o)
    assert not t["unique"]


def test_flat_plane_and_dilation(xrt):
    p = prim_soup(2000, seed=7, flat_axis=1)  # zero extent on y: 0/0 in the normalisation
    g, o = _pair(p, scr=0.01)
    _same_tree(g, o)


def test_pred_differs_from_v(xrt):
    p = prim_soup(3000, seed=8)
    pred = p + np.random.default_rng(9).normal(0, 0.02, p.shape).astype(np.float32)
    g, o = _pair(p, pred, scr=0.002)
    _same_tree(g, o)


def test_refit_matches_oracle(xrt):
    p = prim_soup(5000, seed=10)
    g, o = _pair(p)
    rng = np.random.default_rng(11)
    for _ in range(3):
        pred = (p + rng.normal(0, 0.03, p.shape)).astype(np.float32)
        g.refit(pred)
        o.refit(pred)
        _same_tree(g, o)


def test_queries_match_oracle(xrt):
    rng = np.random.default_rng(12)
    p = prim_soup(20000, seed=12, size=0.08)
    g, o = _pair(p)
    pts = rng.uniform(-1.0, 1.0, size=(4000, 3)).astype(np.float32)
    segs = np.concatenate([pts, pts + rng.normal(0, 0.1, pts.shape).astype(np.float32)], 1)
    lo = pts - 0.05
    boxes = np.concatenate([lo, lo + 0.1], 1).astype(np.float32)
    assert _same_queries(g, o, 0, pts).sum() > 0
    assert _same_queries(g, o, 1, segs).sum() > 0
    assert _same_queries(g, o, 2, boxes).sum() > 0


def test_candidate_truncation_at_256(xrt):
    # 600 large triangles around the origin all contain the query point's neighbourhood
    rng = np.random.default_rng(13)
    c = rng.normal(0, 0.01, size=(600, 1, 3))
    tri = c + np.array([[-1.0, -1.0, -1.0], [1.0, -1.0, 1.0], [0.0, 1.0, 0.0]])
    p = tri.astype(np.float32).reshape(600, 9)
    g, o = _pair(p)
    _same_tree(g, o)
    q = np.zeros((4, 3), np.float32)
    counts = _same_queries(g, o, 0, q)
    assert counts.max() == 256
