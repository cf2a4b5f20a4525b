"""Seeded synthetic scenes for the cloth step (no dataset or asset files are involved).

The reference ships demo scenes (examples/) and relies on SMPL body models that are not part of
it; these generators stand in with the shapes and sizes of the benchmark configurations:
  * grid cloth: n x n vertices over a square, two triangles per quad, 2n(n-1)+(n-1)^2 edges,
    seeded per-coordinate jitter;
  * icosphere obstacle (subdivision 3: 642 vertices / 1,280 triangles);
  * tube body with the SMPL mesh's counts (82 rings x 84 slices + 2 poles = 6,890 vertices,
    13,776 triangles), skinned rigidly to a chain of 24 bones whose joint angles are sums of 3
    seeded sinusoids (amplitude <= 0.4 rad in total per joint, 0.2-1.5 Hz);
  * tessellated ground plane.
"""
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from .solver import Mesh


def rect_cloth(nx: int, ny: int, width: float = 1.0, depth: float = 1.0,
               origin=(0.0, 0.0, 0.0), jitter: float = 1e-3, seed: int = 1) -> Mesh:
    """nx x ny grid (nx vertices along x over `width`, ny rows along z over `depth`) in the xz
    plane at height origin[1]; normal +y; vertex (i, j) = i * nx + j."""
    rng = np.random.default_rng(seed)
    hx = width / (nx - 1)
    hz = depth / (ny - 1)
    i, j = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    pos = np.stack([origin[0] + j * hx, np.full_like(i, origin[1], dtype=np.float64),
                    origin[2] + i * hz], axis=-1).reshape(-1, 3)
    if jitter > 0:
        pos = pos + rng.uniform(-jitter, jitter, size=pos.shape)
    a = (i[:-1, :-1] * nx + j[:-1, :-1]).reshape(-1)
    b = a + 1
    c = a + nx
    d = c + 1
    tri = np.empty((a.size * 2, 3), np.uint32)
    tri[0::2] = np.stack([a, c, b], -1)
    tri[1::2] = np.stack([b, c, d], -1)
    return Mesh(positions=pos.astype(np.float32), triangles=tri)


def grid_cloth(n: int, size: float = 1.0, origin=(0.0, 0.0, 0.0), jitter: float = 1e-3,
               seed: int = 1) -> Mesh:
    """n x n grid in the xz plane at height origin[1]; normal +y; vertex (i, j) = i * n + j."""
    return rect_cloth(n, n, size, size, origin, jitter, seed)


def icosphere(subdiv: int = 3, radius: float = 0.3, center=(0.0, 0.0, 0.0)) -> Mesh:
    t = (1.0 + 5 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
             (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(v, np.float64) / np.linalg.norm(v) for v in verts]
    for _ in range(subdiv):
        cache = {}
        new_faces = []

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            new_faces += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = new_faces
    pos = np.array(verts) * radius + np.asarray(center)
    return Mesh(positions=pos.astype(np.float32), triangles=np.array(faces, np.uint32))


def ground_plane(n: int = 64, size: float = 4.0, height: float = 0.0, center=(0.0, 0.0)) -> Mesh:
    m = grid_cloth(n, size, origin=(center[0] - size / 2, height, center[1] - size / 2), jitter=0.0)
    return m


@dataclass
class TubeBody:
    """Tube body with SMPL counts, rigidly skinned to a 24-bone chain along +y."""
    rings: int = 82
    slices: int = 84
    height: float = 1.2
    radius: float = 0.16
    bones: int = 24
    seed: int = 2
    base: tuple = (0.0, 0.0, 0.0)
    rest: np.ndarray = field(init=False)
    triangles: np.ndarray = field(init=False)
    bone_of: np.ndarray = field(init=False)

    def __post_init__(self):
        R, S = self.rings, self.slices
        ys = np.linspace(0.08 * self.height, 0.92 * self.height, R)
        phi = np.linspace(0, 2 * np.pi, S, endpoint=False)
        prof = self.radius * (1.0 + 0.15 * np.sin(ys / self.height * 3 * np.pi))
        ring = np.stack([np.cos(phi)[None, :] * prof[:, None],
                         np.repeat(ys[:, None], S, 1),
                         np.sin(phi)[None, :] * prof[:, None]], -1).reshape(-1, 3)
        bottom = np.array([[0.0, 0.0, 0.0]])
        top = np.array([[0.0, self.height, 0.0]])
        self.rest = np.concatenate([ring, bottom, top]) + np.asarray(self.base)
        tris = []
        for r in range(R - 1):
            for s in range(S):
                a = r * S + s
                b = r * S + (s + 1) % S
                c = a + S
                d = b + S
                tris += [(a, c, b), (b, c, d)]
        nb, nt = R * S, R * S + 1
        for s in range(S):
            tris.append((nb, s, (s + 1) % S))
            a = (R - 1) * S + s
            b = (R - 1) * S + (s + 1) % S
            tris.append((nt, b, a))
        self.triangles = np.array(tris, np.uint32)
        yl = self.rest[:, 1] - self.base[1]
        self.bone_of = np.clip((yl / self.height * self.bones).astype(int), 0, self.bones - 1)
        rng = np.random.default_rng(self.seed)
        self.amp = rng.uniform(0, 0.4 / 3, size=(self.bones, 3))
        self.freq = rng.uniform(0.2, 1.5, size=(self.bones, 3))
        self.phase = rng.uniform(0, 2 * np.pi, size=(self.bones, 3))
        self.axis = np.where(np.arange(self.bones)[:, None] % 2 == 0, [[1.0, 0.0, 0.0]],
                             [[0.0, 0.0, 1.0]])

    @property
    def mesh(self) -> Mesh:
        return Mesh(positions=self.rest.astype(np.float32), triangles=self.triangles)

    def joint_angles(self, t: float) -> np.ndarray:
        return (self.amp * np.sin(2 * np.pi * self.freq * t + self.phase)).sum(1)

    def pose(self, t: float) -> np.ndarray:
        """World positions at time t: bone b rotates by angle_b / 6 relative to bone b-1."""
        L = self.height / self.bones
        ang = self.joint_angles(t) / 6.0
        Rs, bases = [], []
        Rcur = np.eye(3)
        base = np.asarray(self.base, np.float64)
        for b in range(self.bones):
            ax = self.axis[b]
            c, s = np.cos(ang[b]), np.sin(ang[b])
            K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
            Rrel = np.eye(3) + s * K + (1 - c) * K @ K
            if b > 0:
                base = base + Rcur @ np.array([0.0, L, 0.0])
            Rcur = Rcur @ Rrel
            Rs.append(Rcur.copy())
            bases.append(base.copy())
        Rs, bases = np.array(Rs), np.array(bases)
        local = self.rest - np.asarray(self.base) - np.stack(
            [np.zeros(len(self.rest)), self.bone_of * L, np.zeros(len(self.rest))], -1)
        out = np.einsum("vij,vj->vi", Rs[self.bone_of], local) + bases[self.bone_of]
        return out.astype(np.float32)

    def skin(self):
        """Skinning data of the rigid binding: (rest (V, 3) float32, CSR outer (V + 1),
        joints (V), weights (V)); one influence of weight 1 per vertex, its bone."""
        V = len(self.rest)
        return (self.rest.astype(np.float32), np.arange(V + 1, dtype=np.uint32),
                self.bone_of.astype(np.uint32), np.ones(V, np.float32))

    def joint_transforms(self, t: float) -> np.ndarray:
        """(bones, 12) float32: bone b's global transform at time t, top three rows of the 4x4,
        row-major, so that pose(t) = R_b rest + t_b for the vertices of bone b."""
        L = self.height / self.bones
        ang = self.joint_angles(t) / 6.0
        Rcur = np.eye(3)
        base0 = np.asarray(self.base, np.float64)
        base = base0.copy()
        out = np.zeros((self.bones, 12))
        for b in range(self.bones):
            ax = self.axis[b]
            c, s = np.cos(ang[b]), np.sin(ang[b])
            K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
            Rrel = np.eye(3) + s * K + (1 - c) * K @ K
            if b > 0:
                base = base + Rcur @ np.array([0.0, L, 0.0])
            Rcur = Rcur @ Rrel
            tr = base - Rcur @ (base0 + np.array([0.0, b * L, 0.0]))
            out[b] = np.concatenate([Rcur, tr[:, None]], axis=1).reshape(-1)
        return out.astype(np.float32)


def two_corner_pins(n: int) -> np.ndarray:
    """Pins the two corners of the edge i = 0 (vertices 0 and n-1)."""
    return np.array([0, n - 1], np.uint32)


@dataclass
class Scene:
    name: str
    cloth: Mesh
    obstacle: Optional[Mesh]
    params: dict
    particle_diameter: float = 0.0
    body: Optional[TubeBody] = None
    frames: int = 1


def apply_overrides(p, **kw):
    """Sets the named fields of an xrt_swift_params (gravity as a 3-sequence); returns p."""
    for k, v in kw.items():
        if k == "gravity":
            for i in range(3):
                p.gravity[i] = v[i]
        else:
            setattr(p, k, v)
    return p


def _params(**kw):
    """xrt_swift_params: the library's defaults (xrt_default_params) with overrides."""
    from . import _lib as L
    import ctypes as C
    p = L.SwiftParams()
    L.load().xrt_default_params(C.byref(p))
    return apply_overrides(p, **kw)


def plain_small(n: int = 64, frames: int = 120) -> Scene:
    """64x64 cloth (1 m, jitter +-1e-3, two corners pinned) onto an icosphere r = 0.3 m;
    stretch 1e-8, bend 1e-6, 10 substeps x 10 iterations, self-contact thickness 2 mm."""
    cloth = grid_cloth(n, 1.0, origin=(0.0, 0.4, 0.0), jitter=1e-3, seed=1)
    cloth.fixed_indices = two_corner_pins(n)
    sphere = icosphere(3, 0.3, center=(0.5, 0.0, 0.5))
    return Scene("plain_small", cloth, sphere,
                 dict(num_substeps=10, num_iterations=10, stretch_compliance=1e-8,
                      bend_compliance=1e-6), particle_diameter=2e-3, frames=frames)


def plain_garment(n: int = 256, frames: int = 240) -> Scene:
    """256x256 cloth draped over the animated 6,890-vertex tube body; stretch, bend and LRA
    (slots = the two pinned corners) with obstacle and self contact; 20 substeps x 15 iterations."""
    body = TubeBody(seed=2)
    top = body.height
    cloth = grid_cloth(n, 1.0, origin=(-0.5, top + 0.05, -0.5), jitter=1e-3, seed=2)
    cloth.fixed_indices = two_corner_pins(n)
    cloth.attached_indices = two_corner_pins(n)
    return Scene("plain_garment", cloth, body.mesh,
                 dict(num_substeps=20, num_iterations=15, stretch_compliance=1e-8,
                      bend_compliance=1e-6), body=body, frames=frames)


def plain_heavy(n: int = 1024, frames: int = 180, seed: int = 3) -> Scene:
    """1024x1024 cloth dropped diagonally with seeded folds onto a tessellated ground plane;
    self contact 1 mm; 10 substeps x 10 iterations."""
    rng = np.random.default_rng(seed)
    cloth = grid_cloth(n, 2.0, origin=(-1.0, 0.0, -1.0), jitter=1e-4, seed=seed)
    p = cloth.positions.astype(np.float64)
    k = rng.uniform(2, 6, size=2)
    ph = rng.uniform(0, 2 * np.pi, size=2)
    p[:, 1] = 0.25 + 0.6 * (p[:, 0] + 1.0) / 2.0 + 0.05 * np.sin(k[0] * p[:, 0] + ph[0]) * np.sin(
        k[1] * p[:, 2] + ph[1])
    cloth.positions = p.astype(np.float32)
    ground = ground_plane(64, 6.0, height=0.0)
    return Scene("plain_heavy", cloth, ground,
                 dict(num_substeps=10, num_iterations=10, stretch_compliance=1e-8,
                      bend_compliance=1e-6), particle_diameter=1e-3, frames=frames)


@dataclass
class Garment:
    """One instance of the batched workload."""
    cloth: Mesh
    body: TubeBody
    nx: int
    ny: int
    stretch_compliance: float

    @property
    def num_edges(self) -> int:
        nx, ny = self.nx, self.ny
        return nx * (ny - 1) + ny * (nx - 1) + (nx - 1) * (ny - 1)


# 10 substeps x 10 iterations, bend compliance 1e-6, stretch per instance.
BATCHED_PARAMS = dict(num_substeps=10, num_iterations=10, bend_compliance=1e-6)


def batched_garments(count: int = 512, seed: int = 4, only=None) -> list:
    """`count` independent garments: vertex counts log-uniform in [2,000, 100,000], aspect
    (x : z) uniform in [0.5, 2], square cells, 1 m wide, draped 5 cm above their own tube body
    (joint motion seeded with seed + i), two corners pinned and LRA-attached; stretch compliance
    log-uniform in [1e-9, 1e-5] per instance.  `only`: build just these garment indices of the
    same draw (in that order)."""
    rng = np.random.default_rng(seed)
    V = np.exp(rng.uniform(np.log(2000.0), np.log(100000.0), count))
    aspect = rng.uniform(0.5, 2.0, count)
    comp = np.exp(rng.uniform(np.log(1e-9), np.log(1e-5), count))
    out = []
    for i in (range(count) if only is None else only):
        ny = max(2, int(round(np.sqrt(V[i] / aspect[i]))))
        nx = max(2, int(round(V[i] / ny)))
        body = TubeBody(seed=seed + i)
        depth = (ny - 1) / (nx - 1)
        cloth = rect_cloth(nx, ny, 1.0, depth, origin=(-0.5, body.height + 0.05, -0.5 * depth),
                           jitter=1e-3, seed=seed + i)
        cloth.fixed_indices = np.array([0, nx - 1], np.uint32)
        cloth.attached_indices = np.array([0, nx - 1], np.uint32)
        out.append(Garment(cloth, body, nx, ny, float(comp[i])))
    return out


def batched_grid_dims(count: int = 512, seed: int = 4) -> list:
    """(nx, ny) of each garment of batched_garments(count, seed), without building the meshes."""
    rng = np.random.default_rng(seed)
    V = np.exp(rng.uniform(np.log(2000.0), np.log(100000.0), count))
    aspect = rng.uniform(0.5, 2.0, count)
    out = []
    for i in range(count):
        ny = max(2, int(round(np.sqrt(V[i] / aspect[i]))))
        nx = max(2, int(round(V[i] / ny)))
        out.append((nx, ny))
    return out


def batched_sizes(count: int = 512, seed: int = 4) -> np.ndarray:
    """Vertex counts nx * ny of batched_garments(count, seed), without building the meshes."""
    return np.array([nx * ny for nx, ny in batched_grid_dims(count, seed)], np.int64)


# 10 substeps x 10 iterations, one collision pass per substep, no particle self-collision.
DIFF_PARAMS = dict(num_substeps=10, num_iterations=10, num_collision_passes=10,
                   enable_self_collision=0, update_obstacle_animation=0)


@dataclass
class DiffInstance:
    """One instance of the differentiation workload, with its seeded ground truth."""
    cloth: Mesh
    sphere: Mesh
    stretch_compliance: np.ndarray  # per edge, the ground truth of the target rollout
    bend_compliance: np.ndarray     # per bend
    mass: np.ndarray                # per vertex
    velocity: np.ndarray            # (V, 3) initial velocity


def diff_batch(count: int = 16, n: int = 128, seed: int = 7) -> list:
    """`count` n x n sheets (1 m, jitter 1e-3), each pinned along its top edge (row 0, the two
    corners LRA-attached) and 5 cm above its own sphere of radius 0.3 m (icosphere, 3
    subdivisions, centre offset seeded within 5 cm).  Ground truth per instance: stretch
    compliance log-uniform in [1e-8, 1e-5] per edge, bend compliance log-uniform in [10, 1000]
    per bend (about the reference's default of 100: stiffer bends fold a flat sheet, because the
    solve's normals are oriented against the rest angle's), vertex mass uniform in [0.5, 2] (the reference's unit inverse mass scale), initial
    velocity N(0, 0.05 m/s).
    Edge and bend counts are those the solver builds for an n x n grid:
    3 n^2 - 4 n + 1 edges, one bend per interior edge."""
    rng = np.random.default_rng(seed)
    out = []
    E = 3 * n * n - 4 * n + 1
    B = E - 4 * (n - 1)
    for i in range(count):
        off = rng.uniform(-0.05, 0.05, 2)
        sphere = icosphere(3, 0.3, center=(off[0], 0.0, off[1]))
        cloth = grid_cloth(n, 1.0, origin=(-0.5, 0.35, -0.5), jitter=1e-3, seed=seed + i)
        cloth.fixed_indices = np.arange(n, dtype=np.uint32)
        cloth.attached_indices = np.array([0, n - 1], np.uint32)
        out.append(DiffInstance(
            cloth, sphere,
            np.exp(rng.uniform(np.log(1e-8), np.log(1e-5), E)).astype(np.float32),
            np.exp(rng.uniform(np.log(10.0), np.log(1000.0), B)).astype(np.float32),
            rng.uniform(0.5, 2.0, n * n).astype(np.float32),
            rng.normal(0.0, 0.05, (n * n, 3)).astype(np.float32)))
    return out


def scene_params(scene: Scene, **overrides):
    kw = dict(scene.params)
    kw.update(overrides)
    return _params(**kw)
