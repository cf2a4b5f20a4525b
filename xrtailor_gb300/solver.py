"""Host-side mirror of the reference's Swift solver interface over the C ABI.

Reference interface being mirrored:
  * configuration: SwiftModeSettings and its JSON keys (xrtailor/include/xrtailor/config/Base.hpp:38-139,
    SimulationConfigParser::ParseSwift, xrtailor/src/config/SimulationConfigParser.cpp:147-245) and
    SimulationConfigParser::Apply (:421-498), which copies them into SimParams;
  * solver: ClothSolverUniversal::AddCloth / AddObstacle / Start
    (xrtailor/src/pipeline/impl/universal/ClothSolver.cpp:46-350) and ClothSolverBase::FixedUpdate ->
    SimulateSwift (xrtailor/src/pipeline/base/ClothSolverBase.cpp:147-261);
  * read-back: PhysicsMesh::HostPositions / HostNormals (xrtailor/src/physics/PhysicsMesh.cu:326-377).

Every call goes to libxrt.so; errors raise XrtError with the library's message.
"""
import ctypes as C
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _lib as L


@dataclass
class SolverSettings:  # config/Base.hpp:92-98
    num_substeps: int = 1
    num_iterations: int = 200
    max_speed: float = 1e6
    gravity: Sequence[float] = (0.0, -9.8, 0.0)
    damping: float = 0.98


@dataclass
class BasicFabricSettings:  # config/Base.hpp:38-45
    stretch_compliance: float = 0.0
    bend_compliance: float = 1e2
    relaxation_factor: float = 0.25
    long_range_stretchiness: float = 1.1
    geodesic_LRA: bool = False
    solve_bending: bool = True


@dataclass
class ParticleCollisionSettings:  # config/Base.hpp:59-66
    friction: float = 0.1
    max_neighbor_size: int = 64
    inter_leaved_hash: int = 3
    enable_self_collision: bool = True
    particle_diameter: float = 1.3
    hash_cell_size: float = 1.5


@dataclass
class SwiftModeCollisionSettings:  # config/Base.hpp:128-133
    num_collision_passes: int = 10
    sdf_collision_margin: float = 1e-2
    bvh_tolerance: float = 0.003
    self_contact: ParticleCollisionSettings = field(default_factory=ParticleCollisionSettings)


@dataclass
class SwiftModeSettings:  # config/Base.hpp:135-139
    solver: SolverSettings = field(default_factory=SolverSettings)
    fabric: BasicFabricSettings = field(default_factory=BasicFabricSettings)
    collision: SwiftModeCollisionSettings = field(default_factory=SwiftModeCollisionSettings)


def parse_swift(root: dict) -> SwiftModeSettings:
    """SimulationConfigParser::ParseSwift: reads the MODE_SWIFT scope of a simulation config."""
    if "MODE_SWIFT" not in root:
        raise ValueError("Property MODE_SWIFT not found")
    s = SwiftModeSettings()
    swift = root["MODE_SWIFT"]
    sv = swift.get("SOLVER", {})
    if "NUM_SUBSTEPS" in sv: s.solver.num_substeps = int(sv["NUM_SUBSTEPS"])
    if "NUM_ITERATIONS" in sv: s.solver.num_iterations = int(sv["NUM_ITERATIONS"])
    if "MAX_SPEED" in sv: s.solver.max_speed = float(sv["MAX_SPEED"])
    if "GRAVITY" in sv: s.solver.gravity = tuple(float(g) for g in sv["GRAVITY"])
    if "DAMPING" in sv: s.solver.damping = float(sv["DAMPING"])
    fb = swift.get("FABRIC", {})
    if "STRETCH_COMPLIANCE" in fb: s.fabric.stretch_compliance = float(fb["STRETCH_COMPLIANCE"])
    if "BEND_COMPLIANCE" in fb: s.fabric.bend_compliance = float(fb["BEND_COMPLIANCE"])
    if "RELAXATION_FACTOR" in fb: s.fabric.relaxation_factor = float(fb["RELAXATION_FACTOR"])
    if "LONG_RANGE_STRETCHINESS" in fb:
        s.fabric.long_range_stretchiness = float(fb["LONG_RANGE_STRETCHINESS"])
    if "GEODESIC_LRA" in fb: s.fabric.geodesic_LRA = bool(fb["GEODESIC_LRA"])
    if "SOLVE_BENDING" in fb: s.fabric.solve_bending = bool(fb["SOLVE_BENDING"])
    co = swift.get("COLLISION", {})
    if "NUM_COLLISION_PASSES" in co:
        s.collision.num_collision_passes = int(co["NUM_COLLISION_PASSES"])
    if "SDF_COLLISION_MARGIN" in co:
        s.collision.sdf_collision_margin = float(co["SDF_COLLISION_MARGIN"])
    if "BVH_TOLERANCE" in co: s.collision.bvh_tolerance = float(co["BVH_TOLERANCE"])
    pc = co.get("PARTICLE", {})
    sc = s.collision.self_contact
    if "FRICTION" in pc: sc.friction = float(pc["FRICTION"])
    if "MAX_NEIGHBOR_SIZE" in pc: sc.max_neighbor_size = int(pc["MAX_NEIGHBOR_SIZE"])
    if "INTER_LEAVED_HASH" in pc: sc.inter_leaved_hash = int(pc["INTER_LEAVED_HASH"])
    if "ENABLE_SELF_COLLISION" in pc: sc.enable_self_collision = bool(pc["ENABLE_SELF_COLLISION"])
    if "PARTICLE_DIAMETER" in pc: sc.particle_diameter = float(pc["PARTICLE_DIAMETER"])
    if "HASH_CELL_SIZE" in pc: sc.hash_cell_size = float(pc["HASH_CELL_SIZE"])
    return s


def apply_swift(s: SwiftModeSettings, frame_time: float = 1.0 / 60.0) -> L.SwiftParams:
    """SimulationConfigParser::Apply for SOLVER_MODE::SWIFT.

    Kept quirks: FABRIC.RELAXATION_FACTOR and FABRIC.GEODESIC_LRA are parsed but never copied into
    SimParams, whose defaults (0.25, true) stay in force; MAX_SPEED and SDF_COLLISION_MARGIN are
    copied but no Swift kernel reads them."""
    p = L.SwiftParams()
    L.load().xrt_default_params(C.byref(p))
    p.num_substeps = s.solver.num_substeps
    p.num_iterations = s.solver.num_iterations
    p.max_speed = s.solver.max_speed
    for i in range(3):
        p.gravity[i] = float(s.solver.gravity[i])
    p.damping = s.solver.damping
    p.stretch_compliance = s.fabric.stretch_compliance
    p.bend_compliance = s.fabric.bend_compliance
    p.solve_bending = int(s.fabric.solve_bending)
    p.long_range_stretchiness = s.fabric.long_range_stretchiness
    p.friction = s.collision.self_contact.friction
    p.max_neighbor_size = s.collision.self_contact.max_neighbor_size
    p.enable_self_collision = int(s.collision.self_contact.enable_self_collision)
    p.inter_leaved_hash = s.collision.self_contact.inter_leaved_hash
    p.particle_diameter = s.collision.self_contact.particle_diameter
    p.hash_cell_size = s.collision.self_contact.hash_cell_size
    p.sdf_collision_margin = s.collision.sdf_collision_margin
    p.bvh_tolerance = s.collision.bvh_tolerance
    p.num_collision_passes = s.collision.num_collision_passes
    p.frame_time = frame_time
    return p


@dataclass
class Mesh:
    """A triangle mesh plus the per-vertex lists the reference's Mesh carries."""
    positions: np.ndarray                 # (V, 3) float32, mesh space
    triangles: np.ndarray                 # (F, 3) uint32, counter-clockwise
    fixed_indices: Optional[np.ndarray] = None     # pinned (inv mass 0)
    attached_indices: Optional[np.ndarray] = None  # long-range-attachment slots
    binded_indices: Optional[np.ndarray] = None
    bind_stiffnesses: Optional[np.ndarray] = None
    bind_distances: Optional[np.ndarray] = None
    bind_obstacle_tri: Optional[np.ndarray] = None  # (B, 3) uint32
    bind_barycentric: Optional[np.ndarray] = None   # (B, 3) float32


def _f32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


def _u32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.uint32)


def cloth_desc(mesh: Mesh, model_matrix=None, particle_diameter: float = 0.0):
    """Builds an xrt_cloth_desc; returns (desc, keepalive) — keep the arrays alive while used."""
    keep = []
    pos = _f32(mesh.positions).reshape(-1)
    tri = _u32(mesh.triangles).reshape(-1)
    mm = None if model_matrix is None else _f32(np.asarray(model_matrix, np.float32).T.reshape(-1))
    fixed, att, bind = _u32(mesh.fixed_indices), _u32(mesh.attached_indices), _u32(mesh.binded_indices)
    bst, bdi = _f32(mesh.bind_stiffnesses), _f32(mesh.bind_distances)
    btri = None if mesh.bind_obstacle_tri is None else _u32(mesh.bind_obstacle_tri).reshape(-1)
    bbar = None if mesh.bind_barycentric is None else _f32(mesh.bind_barycentric).reshape(-1)
    keep += [pos, tri, mm, fixed, att, bind, bst, bdi, btri, bbar]
    d = L.ClothDesc()
    d.positions = L.fptr(pos)
    d.num_vertices = pos.size // 3
    d.triangles = L.uptr(tri)
    d.num_triangles = tri.size // 3
    d.model_matrix = L.fptr(mm)
    d.fixed_indices = L.uptr(fixed)
    d.num_fixed = 0 if fixed is None else fixed.size
    d.attached_indices = L.uptr(att)
    d.num_attached = 0 if att is None else att.size
    d.binded_indices = L.uptr(bind)
    d.bind_stiffnesses = L.fptr(bst)
    d.bind_distances = L.fptr(bdi)
    d.bind_obstacle_tri = L.uptr(btri)
    d.bind_barycentric = L.fptr(bbar)
    d.num_binded = 0 if bind is None else bind.size
    d.particle_diameter = float(particle_diameter or 0.0)
    return d, keep


def obstacle_desc(mesh: Mesh, model_matrix=None):
    pos = _f32(mesh.positions).reshape(-1)
    tri = _u32(mesh.triangles).reshape(-1)
    mm = None if model_matrix is None else _f32(np.asarray(model_matrix, np.float32).T.reshape(-1))
    d = L.ObstacleDesc()
    d.positions = L.fptr(pos)
    d.num_vertices = pos.size // 3
    d.triangles = L.uptr(tri)
    d.num_triangles = tri.size // 3
    d.model_matrix = L.fptr(mm)
    return d, [pos, tri, mm]


class ClothSolver:
    """One simulation context on one GPU (ClothSolverUniversal + ClothSolverBase)."""

    def __init__(self, params=None, device: int = 0):
        self._lib = L.load()
        self._h = C.c_void_p()
        self.device = int(device)
        L.check(self._lib.xrt_create(C.byref(self._h), int(device)), None, "xrt_create")
        if params is None:
            params = L.SwiftParams()
            self._lib.xrt_default_params(C.byref(params))
        elif isinstance(params, SwiftModeSettings):
            params = apply_swift(params)
        self.params = params
        L.check(self._lib.xrt_set_params(self._h, C.byref(params)), self._h, "xrt_set_params")

    # -- setup ------------------------------------------------------------------------------
    def set_params(self, params: L.SwiftParams):
        self.params = params
        L.check(self._lib.xrt_set_params(self._h, C.byref(params)), self._h, "xrt_set_params")

    def add_cloth(self, mesh: Mesh, model_matrix=None, particle_diameter: float = 0.0) -> int:
        d, keep = cloth_desc(mesh, model_matrix, particle_diameter)
        off = C.c_int32()
        L.check(self._lib.xrt_add_cloth(self._h, C.byref(d), C.byref(off)), self._h, "add_cloth")
        del keep
        return off.value

    def add_obstacle(self, mesh: Mesh, model_matrix=None) -> int:
        d, keep = obstacle_desc(mesh, model_matrix)
        off = C.c_int32()
        L.check(self._lib.xrt_add_obstacle(self._h, C.byref(d), C.byref(off)), self._h, "add_obstacle")
        del keep
        return off.value

    def add_instance(self, cloth: Mesh, obstacle: Mesh = None, cloth_matrix=None,
                     obstacle_matrix=None, particle_diameter: float = 0.0) -> int:
        """Batched form: an independent cloth + its own obstacle; returns the instance index."""
        d, keep = cloth_desc(cloth, cloth_matrix, particle_diameter)
        od, okeep = (None, None)
        if obstacle is not None:
            od, okeep = obstacle_desc(obstacle, obstacle_matrix)
        idx = C.c_int32()
        L.check(self._lib.xrt_add_instance(self._h, C.byref(d), C.byref(od) if od is not None
                                           else None, C.byref(idx)), self._h, "add_instance")
        del keep, okeep
        return idx.value

    def set_coloring(self, kind: int, colors):
        c = _u32(colors)
        L.check(self._lib.xrt_set_coloring(self._h, kind, L.uptr(c), c.size), self._h, "set_coloring")

    def set_compliance(self, kind: int, values):
        v = _f32(values)
        L.check(self._lib.xrt_set_compliance(self._h, kind, L.fptr(v), v.size), self._h, "set_compliance")

    def set_inv_mass(self, w):
        v = _f32(w)
        L.check(self._lib.xrt_set_inv_mass(self._h, L.fptr(v), v.size), self._h, "set_inv_mass")

    def start(self):
        L.check(self._lib.xrt_start(self._h), self._h, "start")

    # -- stepping ---------------------------------------------------------------------------
    def set_obstacle_targets(self, positions):
        p = _f32(positions).reshape(-1)
        L.check(self._lib.xrt_set_obstacle_targets(self._h, L.fptr(p)), self._h, "targets")

    @staticmethod
    def fem_material(**overrides):
        """xrt_fem_material with the reference's defaults (FEMFabricSettings) and overrides."""
        m = L.FemMaterial()
        L.load().xrt_default_fem_material(C.byref(m))
        for k, v in overrides.items():
            setattr(m, k, v)
        return m

    def set_fem_material(self, material=None, **overrides):
        """The FEM fabric (include/xrt_fem.h) in place of stretch + dihedral bend; before
        start().  `material=None` with no overrides selects the Swift fabric again."""
        m = material if material is not None else (self.fem_material(**overrides)
                                                   if overrides else None)
        L.check(self._lib.xrt_set_fem_material(self._h, C.byref(m) if m is not None else None),
                self._h, "fem material")

    def set_obstacle_skinning(self, rest=None, outer=None, joints=None, weights=None,
                              num_joints: int = 0):
        """Obstacle targets by linear blend skinning on the device (xrt_set_obstacle_skinning);
        `rest=None` turns it off."""
        if rest is None:
            L.check(self._lib.xrt_set_obstacle_skinning(self._h, None, None, None, None, 0),
                    self._h, "skinning")
            return
        r, o, j, w = _f32(rest).reshape(-1), _u32(outer), _u32(joints), _f32(weights)
        L.check(self._lib.xrt_set_obstacle_skinning(self._h, L.fptr(r), L.uptr(o), L.uptr(j),
                                                    L.fptr(w), int(num_joints)),
                self._h, "skinning")

    def set_joint_transforms(self, transforms):
        """12 floats per joint (3 x 4 row-major), host array."""
        t = _f32(transforms).reshape(-1)
        L.check(self._lib.xrt_set_joint_transforms(self._h, L.fptr(t)), self._h, "joints")

    # -- frame cache (include/xrt_cache.h) ------------------------------------------------------
    CACHE_CLOTH, CACHE_OBSTACLE, CACHE_NORMALS = 1, 2, 4

    def cache_begin(self, capacity_frames: int, cloth=True, obstacle=False, normals=False):
        """Records the following frames (SaveCache) into a pinned host store."""
        flags = (self.CACHE_CLOTH if cloth else 0) | (self.CACHE_OBSTACLE if obstacle else 0) | \
            (self.CACHE_NORMALS if normals else 0)
        L.check(self._lib.xrt_cache_begin(self._h, int(capacity_frames), flags), self._h, "cache")
        self._cache_flags = flags

    def cache_count(self) -> int:
        n = C.c_uint32()
        L.check(self._lib.xrt_cache_count(self._h, C.byref(n)), self._h, "cache")
        return n.value

    def cache_read(self, frame: int) -> dict:
        """Cached frame `frame`: the recorded arrays as (V, 3) float32 (absent ones None)."""
        s = self.sizes()
        out = dict(cloth_positions=np.empty((s.num_vertices, 3), np.float32),
                   cloth_normals=np.empty((s.num_vertices, 3), np.float32),
                   obstacle_positions=np.empty((s.num_obstacle_vertices, 3), np.float32),
                   obstacle_normals=np.empty((s.num_obstacle_vertices, 3), np.float32))
        L.check(self._lib.xrt_cache_read(self._h, int(frame),
                                         *(L.fptr(a.reshape(-1)) for a in out.values())),
                self._h, "cache_read")
        f = getattr(self, "_cache_flags", 0)
        cl, ob, nr = f & self.CACHE_CLOTH, f & self.CACHE_OBSTACLE, f & self.CACHE_NORMALS
        present = dict(cloth_positions=cl, cloth_normals=cl and nr, obstacle_positions=ob,
                       obstacle_normals=ob and nr)
        return {k: (v if present[k] else None) for k, v in out.items()}

    def cache_export_obj(self, directory: str, obstacle: bool = False):
        """OBJ sequence of the cached cloth (or obstacle) frames: directory/000000.obj ..."""
        which = self.CACHE_OBSTACLE if obstacle else self.CACHE_CLOTH
        L.check(self._lib.xrt_cache_export_obj(self._h, str(directory).encode(), which),
                self._h, "cache_export_obj")

    def cache_end(self):
        L.check(self._lib.xrt_cache_end(self._h), self._h, "cache_end")

    def set_joint_transforms_device(self, d_transforms: int):
        L.check(self._lib.xrt_set_joint_transforms_device(self._h, C.c_void_p(d_transforms)),
                self._h, "joints")

    def fixed_update(self, frames: int = 1):
        """ClothSolverBase::FixedUpdate -> SimulateSwift, `frames` times (asynchronous)."""
        L.check(self._lib.xrt_step_frames(self._h, int(frames)), self._h, "step")

    step = fixed_update

    def synchronize(self):
        L.check(self._lib.xrt_synchronize(self._h), self._h, "synchronize")

    def set_graph_mode(self, enabled: bool):
        L.check(self._lib.xrt_set_graph_mode(self._h, int(bool(enabled))), self._h, "graph mode")

    def set_tile_vertices(self, n: int):
        """Tile size of the tile-local Gauss-Seidel schedule (0: per-color launches); before
        start()."""
        L.check(self._lib.xrt_set_tile_vertices(self._h, int(n)), self._h, "tile vertices")

    def set_vertex_block(self, threads: int):
        """Threads per block of the per-vertex substep kernels (64 to 512, default 128)."""
        L.check(self._lib.xrt_set_vertex_block(self._h, int(threads)), self._h, "vertex block")

    def set_dependent_launch(self, enabled: bool):
        """Programmatic dependent launch of the substep kernels (default on)."""
        L.check(self._lib.xrt_set_dependent_launch(self._h, int(bool(enabled))), self._h,
                "dependent launch")

    def set_profiling(self, enabled, graph: bool = False):
        """CUDA-event timing of every phase; resets the totals.  Eager frames with an event pair
        around every launch, or with `graph` replayed frame graphs with an event-record node
        pair around every phase group (include/xrt.h xrt_set_profiling)."""
        mode = 0 if not enabled else (2 if graph else 1)
        L.check(self._lib.xrt_set_profiling(self._h, mode), self._h, "profiling")

    def profile(self) -> dict:
        pr = L.Profile()
        L.check(self._lib.xrt_get_profile(self._h, C.byref(pr)), self._h, "profile")
        return {name: dict(ms=pr.ms[i], launches=pr.launches[i], units=pr.units[i])
                for i, name in enumerate(L.PHASES)} | {"frames": pr.frames}

    def device_state(self):
        """(positions float4*, velocities float4*, cudaStream_t) as integers."""
        x, v, s = C.c_void_p(), C.c_void_p(), C.c_void_p()
        L.check(self._lib.xrt_get_device_state(self._h, C.byref(x), C.byref(v), C.byref(s)),
                self._h, "device state")
        return x.value, v.value, s.value

    # -- read-back --------------------------------------------------------------------------
    def sizes(self) -> L.Sizes:
        s = L.Sizes()
        L.check(self._lib.xrt_get_sizes(self._h, C.byref(s)), self._h, "sizes")
        return s

    def _read(self, fn, n):
        out = np.empty((n, 3), np.float32)
        L.check(fn(self._h, L.fptr(out)), self._h, "read")
        return out

    def host_positions(self):
        return self._read(self._lib.xrt_get_positions, self.sizes().num_vertices)

    def host_velocities(self):
        return self._read(self._lib.xrt_get_velocities, self.sizes().num_vertices)

    def host_normals(self):
        return self._read(self._lib.xrt_get_normals, self.sizes().num_vertices)

    def obstacle_positions(self):
        return self._read(self._lib.xrt_get_obstacle_positions, self.sizes().num_obstacle_vertices)

    def obstacle_normals(self):
        return self._read(self._lib.xrt_get_obstacle_normals, self.sizes().num_obstacle_vertices)

    def set_state(self, positions=None, velocities=None):
        p, v = _f32(positions), _f32(velocities)
        L.check(self._lib.xrt_set_state(self._h, L.fptr(None if p is None else p.reshape(-1)),
                                        L.fptr(None if v is None else v.reshape(-1))), self._h, "state")

    def edges(self):
        s = self.sizes()
        e = np.empty((s.num_edges, 2), np.uint32)
        r = np.empty(s.num_edges, np.float32)
        L.check(self._lib.xrt_get_edges(self._h, L.uptr(e), L.fptr(r)), self._h, "edges")
        return e, r

    def bends(self):
        s = self.sizes()
        b = np.empty((s.num_bends, 4), np.uint32)
        t = np.empty(s.num_bends, np.float32)
        L.check(self._lib.xrt_get_bends(self._h, L.uptr(b), L.fptr(t)), self._h, "bends")
        return b, t

    def coloring(self, kind: int):
        """kind 0 stretch (per edge), 1 bend (per bend element), 2 FEM strain (per cloth face),
        3 FEM bending (per bend element)."""
        s = self.sizes()
        n = {0: s.num_edges, 1: s.num_bends, 2: s.num_triangles, 3: s.num_bends}[kind]
        c = np.empty(n, np.uint32)
        L.check(self._lib.xrt_get_coloring(self._h, kind, L.uptr(c)), self._h, "coloring")
        return c

    def lra(self):
        n = self.sizes().num_lra
        src, tgt, rest = np.empty(n, np.uint32), np.empty(n, np.uint32), np.empty(n, np.float32)
        L.check(self._lib.xrt_get_lra(self._h, L.uptr(src), L.uptr(tgt), L.fptr(rest)), self._h, "lra")
        return src, tgt, rest

    def inv_mass(self):
        w = np.empty(self.sizes().num_vertices, np.float32)
        L.check(self._lib.xrt_get_inv_mass(self._h, L.fptr(w)), self._h, "inv_mass")
        return w

    def obstacle_rtri(self):
        m = np.empty(self.sizes().num_obstacle_triangles, np.uint32)
        L.check(self._lib.xrt_get_obstacle_rtri(self._h, L.uptr(m)), self._h, "rtri")
        return m

    def export_obstacle_bvh(self):
        """Obstacle LBVH; in a batched context the instances' trees one after the other (links
        and objects local to each tree, `objects` global)."""
        s = self.sizes()
        n = s.num_obstacle_triangles
        nn = s.num_obstacle_bvh_nodes or (2 * n - 1)
        ni = nn - n
        out = dict(morton=np.empty(n, np.uint32), objects=np.empty(n, np.uint32),
                   nodes=np.empty((nn, 4), np.uint32), aabbs=np.empty((nn, 6), np.float32),
                   iesc=np.empty(max(ni, 1), np.int32), eesc=np.empty(n, np.int32))
        L.check(self._lib.xrt_export_obstacle_bvh(
            self._h, L.uptr(out["morton"]), L.uptr(out["objects"]), L.uptr(out["nodes"]),
            L.fptr(out["aabbs"]), L.iptr(out["iesc"]), L.iptr(out["eesc"])), self._h, "bvh")
        out["iesc"] = out["iesc"][: max(ni, 0)]
        return out

    def export_contacts(self):
        s = self.sizes()
        nv, ne = s.num_vertices, s.num_edges
        out = dict(vf_index=np.empty(nv, np.int32), vf_qs=np.empty((nv, 3), np.float32),
                   rt_index=np.empty(nv, np.int32), rt_qc=np.empty((nv, 3), np.float32),
                   ee=np.empty((ne, 12), np.float32))
        L.check(self._lib.xrt_export_contacts(
            self._h, L.iptr(out["vf_index"]), L.fptr(out["vf_qs"]), L.iptr(out["rt_index"]),
            L.fptr(out["rt_qc"]), L.fptr(out["ee"])), self._h, "contacts")
        return out

    def export_neighbors(self):
        nv = self.sizes().num_vertices
        out = np.empty(nv * self.params.max_neighbor_size, np.uint32)
        L.check(self._lib.xrt_export_neighbors(self._h, L.uptr(out)), self._h, "neighbors")
        return out

    # -- Quality-mode self contact (include/xrt_contact.h) --------------------------------
    def cloth_bvh_build(self):
        L.check(self._lib.xrt_cloth_bvh_build(self._h), self._h, "cloth bvh")

    def obstacle_bvh_update_ccd(self):
        L.check(self._lib.xrt_obstacle_bvh_update_ccd(self._h), self._h, "obstacle bvh ccd")

    def update_pairs(self, thickness: float) -> int:
        n = C.c_uint32()
        L.check(self._lib.xrt_proximity_update_pairs(self._h, float(thickness), C.byref(n)),
                self._h, "update pairs")
        self._npairs = n.value
        return n.value

    def proximity_solve(self, thickness: float, relaxation: float):
        L.check(self._lib.xrt_proximity_solve(self._h, float(thickness), float(relaxation)),
                self._h, "proximity solve")

    def imminent_generate(self) -> int:
        """ImminentRepulsion::UpdateProximity + Generate; returns the number of quadratures."""
        n = C.c_uint32()
        L.check(self._lib.xrt_imminent_generate(self._h, C.byref(n)), self._h, "imminent")
        self._nquads = n.value
        return n.value

    def quads(self):
        n = getattr(self, "_nquads", 0)
        nodes = np.zeros((n, 4), np.uint32)
        bary = np.zeros((n, 4), np.float32)
        L.check(self._lib.xrt_export_quads(self._h, nodes.ctypes.data_as(C.POINTER(C.c_uint32)),
                                           L.fptr(bary)), self._h, "quads")
        return nodes, bary

    def imminent_solve(self, thickness: float, relaxation: float, dt: float):
        L.check(self._lib.xrt_imminent_solve(self._h, float(thickness), float(relaxation),
                                             float(dt)), self._h, "imminent solve")

    def check_impacts(self, thickness: float) -> int:
        n = C.c_uint32()
        L.check(self._lib.xrt_impacts_check(self._h, float(thickness), C.byref(n)), self._h,
                "impacts")
        self._nimpacts = n.value
        return n.value

    def pairs(self):
        out = np.empty((getattr(self, "_npairs", 0), 2), np.uint32)
        L.check(self._lib.xrt_export_pairs(self._h, L.uptr(out)), self._h, "pairs")
        return out

    def impacts(self):
        n = getattr(self, "_nimpacts", 0)
        out = dict(t=np.empty(n, np.float32), w=np.empty((n, 4), np.float32),
                   n=np.empty((n, 3), np.float32), nodes=np.empty((n, 4), np.uint32),
                   is_vf=np.empty(n, np.int32))
        L.check(self._lib.xrt_export_impacts(self._h, L.fptr(out["t"]), L.fptr(out["w"]),
                                             L.fptr(out["n"]), L.uptr(out["nodes"]),
                                             L.iptr(out["is_vf"])), self._h, "impacts")
        return out

    def export_cloth_bvh(self):
        n = self.sizes().num_triangles
        nn = 2 * n - 1
        out = dict(morton=np.empty(n, np.uint32), objects=np.empty(n, np.uint32),
                   nodes=np.empty((nn, 4), np.uint32), aabbs=np.empty((nn, 6), np.float32),
                   iesc=np.empty(max(n - 1, 1), np.int32), eesc=np.empty(n, np.int32))
        L.check(self._lib.xrt_export_cloth_bvh(
            self._h, L.uptr(out["morton"]), L.uptr(out["objects"]), L.uptr(out["nodes"]),
            L.fptr(out["aabbs"]), L.iptr(out["iesc"]), L.iptr(out["eesc"])), self._h, "cloth bvh")
        out["iesc"] = out["iesc"][: max(n - 1, 0)]
        return out

    def predicted(self):
        return self._read(self._lib.xrt_get_predicted, self.sizes().num_vertices)

    def set_predicted(self, x):
        a = _f32(x).reshape(-1)
        L.check(self._lib.xrt_set_predicted(self._h, L.fptr(a)), self._h, "set predicted")

    def collision_step(self, obstacle_mass: float = 1e3, thickness: float = 1e-4,
                       launch_shapes: bool = False) -> dict:
        """ImpactZoneOptimization::CollisionStep on the current state (include/xrt_impact.h).
        With `launch_shapes`, the dict also holds `wide_solves`: how many zone solves ran on
        16-block clusters of 256- and of 1,024-thread blocks."""
        st = L.CollisionStats()
        L.check(self._lib.xrt_collision_step(self._h, float(obstacle_mass), float(thickness),
                                             C.byref(st)), self._h, "collision step")
        out = {k: getattr(st, k) for k in ("success", "deform", "passes", "impacts", "zones",
                                           "solves")}
        if launch_shapes:
            out["wide_solves"] = (int(st.wide_solves[0]), int(st.wide_solves[1]))
        return out

    # -- adjoint (include/xrt_diff.h) ----------------------------------------------------------
    def diff_begin(self, interval_substeps=None):
        """Checkpoint the following frames for backward(): every frame, or every
        `interval_substeps` substeps (a multiple of the frame's substeps)."""
        if interval_substeps is None:
            L.check(self._lib.xrt_diff_begin(self._h), self._h, "diff_begin")
        else:
            L.check(self._lib.xrt_diff_begin_interval(self._h, int(interval_substeps)), self._h,
                    "diff_begin")

    def backward(self, dL_dx, dL_dv=None) -> dict:
        """Gradients of a loss on the final positions (and velocities) with respect to per-edge
        stretch compliance, per-bend compliance, per-vertex mass, initial velocity and initial
        position, over the frames stepped since diff_begin()."""
        s = self.sizes()
        gx = _f32(dL_dx).reshape(-1)
        gv = None if dL_dv is None else _f32(dL_dv).reshape(-1)
        out = dict(stretch_compliance=np.zeros(max(s.num_edges, 1), np.float32),
                   bend_compliance=np.zeros(max(s.num_bends, 1), np.float32),
                   mass=np.zeros(s.num_vertices, np.float32),
                   velocity=np.zeros((s.num_vertices, 3), np.float32),
                   position=np.zeros((s.num_vertices, 3), np.float32))
        g = L.Grads(L.fptr(out["stretch_compliance"]), L.fptr(out["bend_compliance"]),
                    L.fptr(out["mass"]), L.fptr(out["velocity"]), L.fptr(out["position"]))
        L.check(self._lib.xrt_backward(self._h, L.fptr(gx), L.fptr(gv), C.byref(g)), self._h,
                "backward")
        out["stretch_compliance"] = out["stretch_compliance"][: s.num_edges]
        out["bend_compliance"] = out["bend_compliance"][: s.num_bends]
        return out

    def diff_end(self):
        L.check(self._lib.xrt_diff_end(self._h), self._h, "diff_end")

    def close(self):
        if self._h:
            self._lib.xrt_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Lbvh:
    """Standalone LBVH over triangles (the reference's BVH class, BVH.cu)."""

    def __init__(self, device: int = 0):
        self._lib = L.load()
        self._h = C.c_void_p()
        L.check(self._lib.xrt_lbvh_create(C.byref(self._h), int(device)), None, "xrt_lbvh_create")
        self.n = 0

    def build(self, prims, pred=None, scr: float = 0.0):
        a = _f32(prims).reshape(-1)
        b = None if pred is None else _f32(pred).reshape(-1)
        self.n = a.size // 9
        L.check(self._lib.xrt_lbvh_build(self._h, L.fptr(a), L.fptr(b), self.n, float(scr)), None, "build")

    def refit(self, pred):
        b = _f32(pred).reshape(-1)
        L.check(self._lib.xrt_lbvh_refit(self._h, L.fptr(b), self.n), None, "refit")

    def build_device(self, d_prims: int, n: int, d_pred: int = 0, scr: float = 0.0,
                     stream: int = 0):
        """Build from device pointers (9 floats per primitive) on `stream`; no host sync."""
        self.n = int(n)
        L.check(self._lib.xrt_lbvh_build_device(self._h, C.c_void_p(d_prims),
                                                C.c_void_p(d_pred or None), self.n, float(scr),
                                                C.c_void_p(stream or None)), None, "build_device")

    def refit_device(self, d_pred: int, stream: int = 0):
        L.check(self._lib.xrt_lbvh_refit_device(self._h, C.c_void_p(d_pred), self.n,
                                                C.c_void_p(stream or None)), None, "refit_device")

    def export(self):
        n = self.n
        nn = 2 * n - 1
        out = dict(morton=np.empty(n, np.uint32), objects=np.empty(n, np.uint32),
                   nodes=np.empty((nn, 4), np.uint32), aabbs=np.empty((nn, 6), np.float32),
                   iesc=np.empty(max(n - 1, 1), np.int32), eesc=np.empty(n, np.int32))
        uniq = C.c_int32()
        L.check(self._lib.xrt_lbvh_export(self._h, L.uptr(out["morton"]), L.uptr(out["objects"]),
                                          L.uptr(out["nodes"]), L.fptr(out["aabbs"]),
                                          L.iptr(out["iesc"]), L.iptr(out["eesc"]), C.byref(uniq)),
                None, "export")
        out["iesc"] = out["iesc"][: max(n - 1, 0)]
        out["unique"] = bool(uniq.value)
        return out

    def query(self, kind: int, q):
        qa = _f32(q).reshape(-1)
        per = 3 if kind == 0 else 6
        nq = qa.size // per
        counts = np.empty(nq, np.uint32)
        cands = np.zeros((nq, 256), np.uint32)  # slots past a query's count stay 0
        L.check(self._lib.xrt_lbvh_query(self._h, int(kind), L.fptr(qa), nq, L.uptr(counts),
                                         L.uptr(cands)), None, "query")
        return counts, cands

    def close(self):
        if self._h:
            self._lib.xrt_lbvh_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
