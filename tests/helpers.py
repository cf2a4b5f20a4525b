"""Shared helpers of the parity tests: run the CUDA library and the CPU oracle on one scene."""
import numpy as np

from xrtailor_gb300 import ClothSolver, scenes
from xrtailor_gb300.solver import Mesh


def bits(a):
    """Bit pattern of a float32 array (NaN-safe exact comparison)."""
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def diag(x):
    x = np.asarray(x, np.float64)
    return float(np.linalg.norm(x.max(0) - x.min(0)))


def small_scene(n=16, obstacle="sphere", pins=True, attached=None, seed=1, size=1.0):
    cloth = scenes.grid_cloth(n, size, origin=(0.0, 0.35, 0.0), jitter=1e-3, seed=seed)
    if pins:
        cloth.fixed_indices = scenes.two_corner_pins(n)
    if attached is not None:
        cloth.attached_indices = np.asarray(attached, np.uint32)
    obs = None
    if obstacle == "sphere":
        obs = scenes.icosphere(2, 0.3, center=(0.5 * size, 0.0, 0.5 * size))
    elif obstacle == "plane":
        obs = scenes.ground_plane(8, 3.0, height=0.2, center=(0.5, 0.5))
    return cloth, obs


def make_pair(params, cloths, obstacles=(), particle_diameter=0.0, colors_from_gpu=True,
              inv_mass=None, fem=None, tile_vertices=None):
    """Builds a ClothSolver (GPU) and an OracleSolver (CPU) with the same inputs; `fem`: an
    xrt_fem_material for both (the FEM fabric)."""
    from oracle.oracle import OracleSolver
    g = ClothSolver(params)
    o = OracleSolver(params)
    if tile_vertices is not None:
        g.set_tile_vertices(tile_vertices)
    if fem is not None:
        g.set_fem_material(fem)
        o.set_fem_material(fem)
    for c in cloths:
        g.add_cloth(c, particle_diameter=particle_diameter)
        o.add_cloth(c, particle_diameter=particle_diameter)
    for ob in obstacles:
        if ob is not None:
            g.add_obstacle(ob)
            o.add_obstacle(ob)
    if inv_mass is not None:
        g.set_inv_mass(inv_mass)
        o.set_inv_mass(inv_mass)
    g.start()
    if colors_from_gpu:
        o.set_coloring(0, g.coloring(0))
        o.set_coloring(1, g.coloring(1))
        if fem is not None:
            o.set_coloring(2, g.coloring(2))
            o.set_coloring(3, g.coloring(3))
    o.start()
    return g, o


def prim_soup(n, seed=0, spread=1.0, size=0.05, flat_axis=None):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-spread, spread, size=(n, 1, 3))
    p = c + rng.normal(0, size, size=(n, 3, 3))
    if flat_axis is not None:
        p[:, :, flat_axis] = 0.0
    return p.astype(np.float32).reshape(n, 9)


def tube_mesh(rings=10, slices=12, seed=2):
    b = scenes.TubeBody(rings=rings, slices=slices, height=0.5, radius=0.1, bones=6, seed=seed,
                        base=(0.5, -0.2, 0.5))
    return b


def _closest_on_triangles(p, a, b, c):
    """Closest points of points p (n, 3) on triangles (a, b, c) (n, 3 each), by Voronoi region
    (Ericson, Real-Time Collision Detection 5.1.5).  Returns (q (n, 3), feature (n,)): feature 0 =
    face interior, 1/2/3 = vertex a/b/c, 4/5/6 = edge ab/bc/ca."""
    ab, ac, ap = b - a, c - a, p - a
    d1, d2 = (ab * ap).sum(-1), (ac * ap).sum(-1)
    bp = p - b
    d3, d4 = (ab * bp).sum(-1), (ac * bp).sum(-1)
    cp = p - c
    d5, d6 = (ab * cp).sum(-1), (ac * cp).sum(-1)
    va, vb, vc = d3 * d6 - d5 * d4, d5 * d2 - d1 * d6, d1 * d4 - d3 * d2
    with np.errstate(divide="ignore", invalid="ignore"):
        den = 1.0 / (va + vb + vc)
        v, w = vb * den, vc * den
        q = a + ab * v[:, None] + ac * w[:, None]
        feat = np.zeros(len(p), np.int64)
        t_ab = d1 / (d1 - d3)
        t_ac = d2 / (d2 - d6)
        t_bc = (d4 - d3) / ((d4 - d3) + (d5 - d6))
    done = np.zeros(len(p), bool)

    def put(mask, point, f):
        m = mask & ~done
        q[m] = point[m]
        feat[m] = f
        done[m] = True

    put((d1 <= 0) & (d2 <= 0), a, 1)
    put((d3 >= 0) & (d4 <= d3), b, 2)
    put((vc <= 0) & (d1 >= 0) & (d3 <= 0), a + ab * t_ab[:, None], 4)
    put((d6 >= 0) & (d5 <= d6), c, 3)
    put((vb <= 0) & (d2 >= 0) & (d6 <= 0), a + ac * t_ac[:, None], 6)
    put((va <= 0) & ((d4 - d3) >= 0) & ((d5 - d6) >= 0), b + (c - b) * t_bc[:, None], 5)
    return q, feat


class MeshSignedDistance:
    """Signed distance of points to a closed, outward-oriented triangle mesh of fixed topology
    (positive outside), with the angle-weighted pseudo-normal of the closest feature deciding the
    sign (Baerentzen & Aanaes 2005).  The closest triangle is searched among the k triangles of
    nearest centroid and every triangle more than three times the median size."""

    def __init__(self, tris, k=12):
        t = np.asarray(tris, np.int64)
        self.t, self.k = t, k
        # the (face, corner) slots of each undirected edge, paired through a sort of edge keys
        lo = np.minimum(t, np.roll(t, -1, axis=1)).reshape(-1)
        hi = np.maximum(t, np.roll(t, -1, axis=1)).reshape(-1)
        key = lo * (int(t.max()) + 1) + hi
        order = np.argsort(key, kind="stable")
        _, inv = np.unique(key[order], return_inverse=True)
        self.edge_of_slot = np.empty(len(key), np.int64)
        self.edge_of_slot[order] = inv
        self.num_edges = int(inv.max()) + 1

    def __call__(self, points, verts):
        from scipy.spatial import cKDTree
        t, k = self.t, self.k
        x = np.asarray(verts, np.float64)
        p = np.asarray(points, np.float64)
        a, b, c = x[t[:, 0]], x[t[:, 1]], x[t[:, 2]]
        fn = np.cross(b - a, c - a)
        fn /= np.linalg.norm(fn, axis=1, keepdims=True)
        vn = np.zeros_like(x)
        for i, (u, v, w) in enumerate(((a, b, c), (b, c, a), (c, a, b))):
            e1, e2 = v - u, w - u
            cosang = (e1 * e2).sum(1) / (np.linalg.norm(e1, axis=1) * np.linalg.norm(e2, axis=1))
            np.add.at(vn, t[:, i], fn * np.arccos(np.clip(cosang, -1, 1))[:, None])
        esum = np.zeros((self.num_edges, 3))
        np.add.at(esum, self.edge_of_slot, np.repeat(fn, 3, axis=0))
        en = esum[self.edge_of_slot].reshape(len(t), 3, 3)  # slot j = edge (corner j, j + 1)
        cen = (a + b + c) / 3.0
        _, cand = cKDTree(cen).query(p, k=k)
        best = np.full(len(p), np.inf)
        sign = np.ones(len(p))

        def feature_normal(f, feat):
            nrm = fn[f].copy()
            for code, vi in ((1, 0), (2, 1), (3, 2)):
                m = feat == code
                nrm[m] = vn[t[f[m], vi]]
            for code, ej in ((4, 0), (5, 1), (6, 2)):
                m = feat == code
                nrm[m] = en[f[m], ej]
            return nrm

        for j in range(k):
            f = cand[:, j]
            q, feat = _closest_on_triangles(p, a[f], b[f], c[f])
            d = np.linalg.norm(p - q, axis=1)
            better = d < best
            if not better.any():
                continue
            s_ = np.where(((p - q) * feature_normal(f, feat)).sum(1) < 0, -1.0, 1.0)
            best = np.where(better, d, best)
            sign = np.where(better, s_, sign)
        # triangles much longer than the typical one (fans around a pole) can hold a point's
        # closest point while their centroid is far away: each is also tested against every point
        # within its bounding radius plus the largest distance found so far
        rad = np.max([np.linalg.norm(v - cen, axis=1) for v in (a, b, c)], axis=0)
        large = np.nonzero(rad > 3.0 * np.median(rad))[0]
        if len(large):
            near = cKDTree(p).query_ball_point(cen[large], r=rad[large] + best.max())
            pi = np.concatenate([np.asarray(l, np.int64) for l in near])
            fi = np.repeat(large, [len(l) for l in near])
            if len(pi):
                q, feat = _closest_on_triangles(p[pi], a[fi], b[fi], c[fi])
                d = np.linalg.norm(p[pi] - q, axis=1)
                s_ = np.where(((p[pi] - q) * feature_normal(fi, feat)).sum(1) < 0, -1.0, 1.0)
                order = np.lexsort((d, pi))  # by point, nearest first
                first = order[np.r_[True, pi[order][1:] != pi[order][:-1]]]
                win = d[first] < best[pi[first]]
                best[pi[first[win]]] = d[first[win]]
                sign[pi[first[win]]] = s_[first[win]]
        return sign * best


def mesh_signed_distance(points, verts, tris, k=12):
    """One-off MeshSignedDistance(tris, k)(points, verts)."""
    return MeshSignedDistance(tris, k)(points, verts)
