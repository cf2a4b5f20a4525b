"""TEST INFRASTRUCTURE — ctypes front end of the CPU oracle (oracle/_build/liboracle.so).

The oracle restates the reference's Swift-mode frame on the CPU (see oracle_step.cpp for the
file:line of every restated function).  Only tests/, the smoke check and bench.py's CPU-baseline
leg may use it, and only as the checker; the product (libxrt.so) never links or calls it.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import build as _build  # noqa: E402
from xrtailor_gb300 import _lib as L  # noqa: E402  (struct layouts of include/xrt.h only)
from xrtailor_gb300.solver import cloth_desc, obstacle_desc  # noqa: E402

_lib = None
FP, UP, IP, P = C.POINTER(C.c_float), C.POINTER(C.c_uint32), C.POINTER(C.c_int32), C.c_void_p

_SIG = {
    "orc_default_params": (None, [C.POINTER(L.SwiftParams)]),
    "orc_default_fem_material": (None, [C.POINTER(L.FemMaterial)]),
    "orc_create": (P, []), "orc_destroy": (None, [P]), "orc_num_threads": (C.c_int, []),
    "orc_set_threads": (None, [C.c_int]),
    "orc_set_params": (None, [P, C.POINTER(L.SwiftParams)]),
    "orc_add_cloth": (C.c_int, [P, C.POINTER(L.ClothDesc)]),
    "orc_add_obstacle": (C.c_int, [P, C.POINTER(L.ObstacleDesc)]),
    "orc_set_coloring": (None, [P, C.c_int, UP, C.c_uint32]),
    "orc_set_fem_material": (None, [P, C.POINTER(L.FemMaterial)]),
    "orc_set_compliance": (None, [P, C.c_int, FP, C.c_uint32]),
    "orc_set_inv_mass": (None, [P, FP, C.c_uint32]),
    "orc_start": (None, [P]), "orc_set_obstacle_targets": (None, [P, FP]),
    "orc_step_frame": (None, [P]), "orc_get_sizes": (None, [P, UP]),
    "orc_get_positions": (None, [P, FP]), "orc_get_velocities": (None, [P, FP]),
    "orc_get_normals": (None, [P, FP]), "orc_get_obstacle_positions": (None, [P, FP]),
    "orc_particle_diameter": (C.c_float, [P]),
    "orc_get_edges": (None, [P, UP, FP]), "orc_get_bends": (None, [P, UP, FP]),
    "orc_get_coloring": (None, [P, C.c_int, UP]), "orc_coloring_valid": (C.c_int, [P, C.c_int]),
    "orc_get_lra": (None, [P, UP, UP, FP]), "orc_get_rtri": (None, [P, UP]),
    "orc_export_obstacle_bvh": (None, [P, UP, UP, UP, FP, IP, IP]),
    "orc_export_contacts": (None, [P, IP, FP, IP, FP, FP]),
    "orc_export_neighbors": (None, [P, UP]), "orc_hash_now": (None, [P]),
    "orc_cloth_bvh_build": (None, [P]), "orc_obstacle_bvh_update_ccd": (None, [P]),
    "orc_update_pairs": (C.c_uint32, [P, C.c_float]),
    "orc_solve_repulsion": (None, [P, C.c_float, C.c_float]),
    "orc_check_impacts": (None, [P, C.c_float]),
    "orc_collision_step": (None, [P, C.c_float, C.c_float, IP]),
    "orc_imminent_generate": (C.c_uint32, [P]),
    "orc_get_quads": (None, [P, UP, FP]),
    "orc_imminent_solve": (None, [P, C.c_float, C.c_float, C.c_float]),
    "orc_get_pairs": (C.c_uint32, [P, UP]),
    "orc_get_impacts": (None, [P, FP, FP, FP, UP, IP]),
    "orc_set_positions_predicted": (None, [P, FP]), "orc_get_positions_predicted": (None, [P, FP]),
    "orc_export_cloth_bvh": (None, [P, UP, UP, UP, FP, IP, IP]),
    "orc_lbvh_create": (P, []), "orc_lbvh_destroy": (None, [P]),
    "orc_lbvh_build": (None, [P, FP, FP, C.c_uint32, C.c_float]),
    "orc_lbvh_refit": (None, [P, FP, C.c_uint32]),
    "orc_lbvh_export": (None, [P, UP, UP, UP, FP, IP, IP, IP]),
    "orc_lbvh_query": (None, [P, C.c_int, FP, C.c_uint32, UP, UP]),
    "orc_expand_bits": (C.c_uint32, [C.c_uint32]), "orc_morton_code": (C.c_uint32, [FP]),
    "orc_nearest_point": (C.c_float, [FP, FP, FP, FP]),
    "orc_ray_intersect": (C.c_float, [FP, FP, C.c_float, FP]),
    "orc_closest_seg_seg": (C.c_float, [FP, FP, FP, FP, FP, FP]),
    "orc_solve_cubic": (C.c_int, [C.c_float, C.c_float, C.c_float, C.c_float, FP]),
    "orc_acos_as": (C.c_float, [C.c_float]),
}


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        h = C.CDLL(path)
        for k, (r, a) in _SIG.items():
            f = getattr(h, k)
            f.restype = r
            f.argtypes = a
        _lib = h
    return _lib


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _u(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def default_params(**overrides) -> L.SwiftParams:
    """The reference's effective Swift-mode defaults (orc_default_params) with overrides; needs
    nothing from the CUDA library."""
    from xrtailor_gb300.scenes import apply_overrides
    p = L.SwiftParams()
    lib().orc_default_params(C.byref(p))
    return apply_overrides(p, **overrides)


def default_fem_material() -> L.FemMaterial:
    """FEMFabricSettings' defaults (orc_default_fem_material)."""
    m = L.FemMaterial()
    lib().orc_default_fem_material(C.byref(m))
    return m


class OracleSolver:
    """CPU restatement with the same calls as xrtailor_gb300.ClothSolver."""

    def __init__(self, params: L.SwiftParams, threads: int = 0):
        self._l = lib()
        if threads:
            self._l.orc_set_threads(int(threads))
        self._h = self._l.orc_create()
        self.params = params
        self._l.orc_set_params(self._h, C.byref(params))

    def set_params(self, params: L.SwiftParams):
        self.params = params
        self._l.orc_set_params(self._h, C.byref(params))

    def add_cloth(self, mesh, model_matrix=None, particle_diameter=0.0):
        d, keep = cloth_desc(mesh, model_matrix, particle_diameter)
        r = self._l.orc_add_cloth(self._h, C.byref(d))
        del keep
        return r

    def add_obstacle(self, mesh, model_matrix=None):
        d, keep = obstacle_desc(mesh, model_matrix)
        r = self._l.orc_add_obstacle(self._h, C.byref(d))
        del keep
        return r

    def set_coloring(self, kind, colors):
        """kind 0 stretch, 1 bend, 2 FEM strain, 3 FEM bending."""
        c = _u(colors)
        self._l.orc_set_coloring(self._h, kind, c.ctypes.data_as(UP), c.size)

    def set_fem_material(self, material=None):
        """The FEM fabric (an xrt_fem_material) or None for the Swift fabric; before start()."""
        self._l.orc_set_fem_material(self._h, C.byref(material) if material is not None else None)

    def set_compliance(self, kind, values):
        v = _f(values)
        self._l.orc_set_compliance(self._h, kind, v.ctypes.data_as(FP), v.size)

    def set_inv_mass(self, w):
        v = _f(w)
        self._l.orc_set_inv_mass(self._h, v.ctypes.data_as(FP), v.size)

    def start(self):
        self._l.orc_start(self._h)

    def set_obstacle_targets(self, pos):
        p = _f(pos).reshape(-1)
        self._l.orc_set_obstacle_targets(self._h, p.ctypes.data_as(FP))

    def step(self, frames=1):
        for _ in range(frames):
            self._l.orc_step_frame(self._h)

    fixed_update = step

    def sizes(self):
        s = np.zeros(8, np.uint32)
        self._l.orc_get_sizes(self._h, s.ctypes.data_as(UP))
        return dict(num_vertices=int(s[0]), num_edges=int(s[1]), num_triangles=int(s[2]),
                    num_bends=int(s[3]), num_lra=int(s[4]), num_obstacle_vertices=int(s[5]),
                    num_obstacle_triangles=int(s[6]), num_stretch_colors=int(s[7] & 0xFFFF),
                    num_bend_colors=int(s[7] >> 16))

    def _read(self, fn, n):
        out = np.empty((n, 3), np.float32)
        fn(self._h, out.ctypes.data_as(FP))
        return out

    def host_positions(self):
        return self._read(self._l.orc_get_positions, self.sizes()["num_vertices"])

    def host_velocities(self):
        return self._read(self._l.orc_get_velocities, self.sizes()["num_vertices"])

    def host_normals(self):
        return self._read(self._l.orc_get_normals, self.sizes()["num_vertices"])

    def obstacle_positions(self):
        return self._read(self._l.orc_get_obstacle_positions, self.sizes()["num_obstacle_vertices"])

    def particle_diameter(self):
        return self._l.orc_particle_diameter(self._h)

    def edges(self):
        n = self.sizes()["num_edges"]
        e, r = np.empty((n, 2), np.uint32), np.empty(n, np.float32)
        self._l.orc_get_edges(self._h, e.ctypes.data_as(UP), r.ctypes.data_as(FP))
        return e, r

    def bends(self):
        n = self.sizes()["num_bends"]
        b, t = np.empty((n, 4), np.uint32), np.empty(n, np.float32)
        self._l.orc_get_bends(self._h, b.ctypes.data_as(UP), t.ctypes.data_as(FP))
        return b, t

    def coloring(self, kind):
        s = self.sizes()
        n = s["num_edges"] if kind == 0 else s["num_bends"]
        c = np.empty(n, np.uint32)
        self._l.orc_get_coloring(self._h, kind, c.ctypes.data_as(UP))
        return c

    def coloring_valid(self, kind):
        return bool(self._l.orc_coloring_valid(self._h, kind))

    def lra(self):
        n = self.sizes()["num_lra"]
        s, t, r = np.empty(n, np.uint32), np.empty(n, np.uint32), np.empty(n, np.float32)
        self._l.orc_get_lra(self._h, s.ctypes.data_as(UP), t.ctypes.data_as(UP), r.ctypes.data_as(FP))
        return s, t, r

    def obstacle_rtri(self):
        m = np.empty(self.sizes()["num_obstacle_triangles"], np.uint32)
        self._l.orc_get_rtri(self._h, m.ctypes.data_as(UP))
        return m

    def export_obstacle_bvh(self):
        n = self.sizes()["num_obstacle_triangles"]
        nn = 2 * n - 1
        out = dict(morton=np.empty(n, np.uint32), objects=np.empty(n, np.uint32),
                   nodes=np.empty((nn, 4), np.uint32), aabbs=np.empty((nn, 6), np.float32),
                   iesc=np.empty(max(n - 1, 1), np.int32), eesc=np.empty(n, np.int32))
        self._l.orc_export_obstacle_bvh(self._h, out["morton"].ctypes.data_as(UP),
                                        out["objects"].ctypes.data_as(UP),
                                        out["nodes"].ctypes.data_as(UP),
                                        out["aabbs"].ctypes.data_as(FP),
                                        out["iesc"].ctypes.data_as(IP),
                                        out["eesc"].ctypes.data_as(IP))
        out["iesc"] = out["iesc"][: max(n - 1, 0)]
        return out

    def export_contacts(self):
        s = self.sizes()
        nv, ne = s["num_vertices"], s["num_edges"]
        out = dict(vf_index=np.empty(nv, np.int32), vf_qs=np.empty((nv, 3), np.float32),
                   rt_index=np.empty(nv, np.int32), rt_qc=np.empty((nv, 3), np.float32),
                   ee=np.empty((ne, 12), np.float32))
        self._l.orc_export_contacts(self._h, out["vf_index"].ctypes.data_as(IP),
                                    out["vf_qs"].ctypes.data_as(FP),
                                    out["rt_index"].ctypes.data_as(IP),
                                    out["rt_qc"].ctypes.data_as(FP), out["ee"].ctypes.data_as(FP))
        return out

    def export_neighbors(self):
        nv = self.sizes()["num_vertices"]
        out = np.empty(nv * self.params.max_neighbor_size, np.uint32)
        self._l.orc_export_neighbors(self._h, out.ctypes.data_as(UP))
        return out

    # -- Quality-mode self contact --------------------------------------------------------
    def cloth_bvh_build(self):
        self._l.orc_cloth_bvh_build(self._h)

    def obstacle_bvh_update_ccd(self):
        self._l.orc_obstacle_bvh_update_ccd(self._h)

    def update_pairs(self, thickness):
        return int(self._l.orc_update_pairs(self._h, float(thickness)))

    def proximity_solve(self, thickness, relaxation):
        self._l.orc_solve_repulsion(self._h, float(thickness), float(relaxation))

    def check_impacts(self, thickness):
        self._l.orc_check_impacts(self._h, float(thickness))

    def imminent_generate(self):
        self._nquads = int(self._l.orc_imminent_generate(self._h))
        return self._nquads

    def quads(self):
        n = getattr(self, "_nquads", 0)
        nodes = np.zeros((n, 4), np.uint32)
        bary = np.zeros((n, 4), np.float32)
        self._l.orc_get_quads(self._h, nodes.ctypes.data_as(UP), bary.ctypes.data_as(FP))
        return nodes, bary

    def imminent_solve(self, thickness, relaxation, dt):
        self._l.orc_imminent_solve(self._h, float(thickness), float(relaxation), float(dt))

    def collision_step(self, obstacle_mass=1e3, thickness=1e-4):
        st = np.zeros(8, np.int32)
        self._l.orc_collision_step(self._h, float(obstacle_mass), float(thickness),
                                   st.ctypes.data_as(IP))
        return dict(zip(("success", "deform", "passes", "impacts", "zones", "solves"),
                        (int(v) for v in st[:6])))

    def pairs(self):
        n = self._l.orc_get_pairs(self._h, None)
        out = np.empty((n, 2), np.uint32)
        self._l.orc_get_pairs(self._h, out.ctypes.data_as(UP))
        return out

    def impacts(self):
        n = 15 * self._l.orc_get_pairs(self._h, None)
        out = dict(t=np.empty(n, np.float32), w=np.empty((n, 4), np.float32),
                   n=np.empty((n, 3), np.float32), nodes=np.empty((n, 4), np.uint32),
                   is_vf=np.empty(n, np.int32))
        self._l.orc_get_impacts(self._h, out["t"].ctypes.data_as(FP), out["w"].ctypes.data_as(FP),
                                out["n"].ctypes.data_as(FP), out["nodes"].ctypes.data_as(UP),
                                out["is_vf"].ctypes.data_as(IP))
        return out

    def set_predicted(self, x):
        a = _f(x).reshape(-1)
        self._l.orc_set_positions_predicted(self._h, a.ctypes.data_as(FP))

    def predicted(self):
        return self._read(self._l.orc_get_positions_predicted, self.sizes()["num_vertices"])

    def export_cloth_bvh(self):
        n = self.sizes()["num_triangles"]
        nn = 2 * n - 1
        out = dict(morton=np.empty(n, np.uint32), objects=np.empty(n, np.uint32),
                   nodes=np.empty((nn, 4), np.uint32), aabbs=np.empty((nn, 6), np.float32),
                   iesc=np.empty(max(n - 1, 1), np.int32), eesc=np.empty(n, np.int32))
        self._l.orc_export_cloth_bvh(self._h, out["morton"].ctypes.data_as(UP),
                                     out["objects"].ctypes.data_as(UP),
                                     out["nodes"].ctypes.data_as(UP),
                                     out["aabbs"].ctypes.data_as(FP),
                                     out["iesc"].ctypes.data_as(IP), out["eesc"].ctypes.data_as(IP))
        out["iesc"] = out["iesc"][: max(n - 1, 0)]
        return out

    def close(self):
        if self._h:
            self._l.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OracleLbvh:
    def __init__(self):
        self._l = lib()
        self._h = self._l.orc_lbvh_create()
        self.n = 0

    def build(self, prims, pred=None, scr=0.0):
        a = _f(prims).reshape(-1)
        b = None if pred is None else _f(pred).reshape(-1)
        self.n = a.size // 9
        self._l.orc_lbvh_build(self._h, a.ctypes.data_as(FP),
                               None if b is None else b.ctypes.data_as(FP), self.n, float(scr))

    def refit(self, pred):
        b = _f(pred).reshape(-1)
        self._l.orc_lbvh_refit(self._h, b.ctypes.data_as(FP), self.n)

    def export(self):
        n = self.n
        nn = 2 * n - 1
        out = dict(morton=np.empty(n, np.uint32), objects=np.empty(n, np.uint32),
                   nodes=np.empty((nn, 4), np.uint32), aabbs=np.empty((nn, 6), np.float32),
                   iesc=np.empty(max(n - 1, 1), np.int32), eesc=np.empty(n, np.int32))
        u = C.c_int32()
        self._l.orc_lbvh_export(self._h, out["morton"].ctypes.data_as(UP),
                                out["objects"].ctypes.data_as(UP), out["nodes"].ctypes.data_as(UP),
                                out["aabbs"].ctypes.data_as(FP), out["iesc"].ctypes.data_as(IP),
                                out["eesc"].ctypes.data_as(IP), C.byref(u))
        out["iesc"] = out["iesc"][: max(n - 1, 0)]
        out["unique"] = bool(u.value)
        return out

    def query(self, kind, q):
        qa = _f(q).reshape(-1)
        nq = qa.size // (3 if kind == 0 else 6)
        counts = np.empty(nq, np.uint32)
        cands = np.zeros((nq, 256), np.uint32)  # slots past a query's count stay 0
        self._l.orc_lbvh_query(self._h, kind, qa.ctypes.data_as(FP), nq, counts.ctypes.data_as(UP),
                               cands.ctypes.data_as(UP))
        return counts, cands

    def close(self):
        if self._h:
            self._l.orc_lbvh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- primitive KATs ---------------------------------------------------------------------------
def lbs(rest, outer, joints, weights, transforms):
    """Linear blend skinning, SMPL's lbs kernel (src/runtime/rag_doll/smpl/cuda/body.cu:39-60),
    in float32 with the kernel's products and sums in its order: per vertex and row i, over the
    vertex's influences in CSR order, out_i += (w T[i][j]) v_j for j = 0, 1, 2, then
    out_i += w T[i][3].  Every numpy float32 operation rounds once, as the library's kernel
    (built without contraction) does.  Returns (V, 3) float32."""
    rest = np.asarray(rest, np.float32).reshape(-1, 3)
    outer = np.asarray(outer, np.int64)
    joints = np.asarray(joints, np.int64)
    w = np.asarray(weights, np.float32)
    T = np.asarray(transforms, np.float32).reshape(-1, 12)
    n = len(rest)
    deg = np.diff(outer)
    out = np.zeros((n, 3), np.float32)
    for s in range(int(deg.max()) if n else 0):
        v = np.nonzero(deg > s)[0]
        k = outer[v] + s
        wk, t, p = w[k], T[joints[k]], rest[v]
        for i in range(3):
            acc = out[v, i]
            acc = acc + (wk * t[:, 4 * i]) * p[:, 0]
            acc = acc + (wk * t[:, 4 * i + 1]) * p[:, 1]
            acc = acc + (wk * t[:, 4 * i + 2]) * p[:, 2]
            acc = acc + wk * t[:, 4 * i + 3]
            out[v, i] = acc
    return out


def expand_bits(v):
    return int(lib().orc_expand_bits(int(v)))


def morton_code(p):
    a = _f(p)
    return int(lib().orc_morton_code(a.ctypes.data_as(FP)))


def nearest_point(p, tri):
    p, t = _f(p), _f(tri).reshape(-1)
    qs, uvw = np.empty(3, np.float32), np.empty(3, np.float32)
    d = lib().orc_nearest_point(p.ctypes.data_as(FP), t.ctypes.data_as(FP), qs.ctypes.data_as(FP),
                                uvw.ctypes.data_as(FP))
    return np.float32(d), qs, uvw


def ray_intersect(o, d, length, tri):
    o, d, t = _f(o), _f(d), _f(tri).reshape(-1)
    return np.float32(lib().orc_ray_intersect(o.ctypes.data_as(FP), d.ctypes.data_as(FP),
                                              float(length), t.ctypes.data_as(FP)))


def closest_seg_seg(p1, q1, p2, q2):
    a = [_f(v) for v in (p1, q1, p2, q2)]
    st, cc = np.empty(2, np.float32), np.empty(6, np.float32)
    d = lib().orc_closest_seg_seg(*[v.ctypes.data_as(FP) for v in a], st.ctypes.data_as(FP),
                                  cc.ctypes.data_as(FP))
    return np.float32(d), st, cc


def acos_as(x):
    return float(lib().orc_acos_as(float(x)))


def solve_cubic(a, b, c, d):
    x = np.zeros(3, np.float32)
    n = lib().orc_solve_cubic(float(a), float(b), float(c), float(d), x.ctypes.data_as(FP))
    return int(n), x[:n]
