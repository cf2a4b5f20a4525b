"""ctypes bindings of libxrt.so (the C ABI declared in include/xrt.h).

The structs below mirror include/xrt.h field for field.  Loading fails loudly when the library
has not been built: there is no Python or CPU fallback for any product entry point.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libxrt.so")

XRT_OK = 0
XRT_ERR_INVALID_CONFIG = 1001
XRT_ERR_INVALID_MESH = 1002
XRT_ERR_INVALID_ARGUMENT = 1003
XRT_ERR_STATE = 1004
XRT_ERR_CUDA = 8000
XRT_ERR_NODE_CAPACITY = 8001
XRT_ERR_EDGE_CAPACITY = 8003
XRT_ERR_FACE_CAPACITY = 8004
XRT_ERR_DEVICE_FLAG = 8100
XRT_ERR_NO_DEVICE = 8200
XRT_ERR_COLORING = 8300


class SwiftParams(C.Structure):
    _fields_ = [
        ("num_substeps", C.c_int32),
        ("num_iterations", C.c_int32),
        ("max_speed", C.c_float),
        ("gravity", C.c_float * 3),
        ("damping", C.c_float),
        ("stretch_compliance", C.c_float),
        ("bend_compliance", C.c_float),
        ("relaxation_factor", C.c_float),
        ("long_range_stretchiness", C.c_float),
        ("geodesic_lra", C.c_int32),
        ("solve_bending", C.c_int32),
        ("num_collision_passes", C.c_int32),
        ("sdf_collision_margin", C.c_float),
        ("bvh_tolerance", C.c_float),
        ("friction", C.c_float),
        ("max_neighbor_size", C.c_int32),
        ("inter_leaved_hash", C.c_int32),
        ("enable_self_collision", C.c_int32),
        ("particle_diameter", C.c_float),
        ("hash_cell_size", C.c_float),
        ("frame_time", C.c_float),
        ("update_obstacle_animation", C.c_int32),
        ("pbd_repulsion", C.c_int32),
        ("pbd_thickness", C.c_float),
        ("repulsion_relaxation", C.c_float),
        ("impact_zone", C.c_int32),
        ("impact_zone_obstacle_mass", C.c_float),
        ("impact_zone_thickness", C.c_float),
        ("imminent_repulsion", C.c_int32),
        ("imminent_thickness", C.c_float),
    ]


class CollisionStats(C.Structure):
    """xrt_collision_stats (include/xrt_impact.h)."""
    _fields_ = [
        ("success", C.c_int32),
        ("deform", C.c_int32),
        ("passes", C.c_int32),
        ("impacts", C.c_uint32),
        ("zones", C.c_uint32),
        ("solves", C.c_uint32),
        ("wide_solves", C.c_uint32 * 2),
    ]


class ClothDesc(C.Structure):
    _fields_ = [
        ("positions", C.POINTER(C.c_float)),
        ("num_vertices", C.c_uint32),
        ("triangles", C.POINTER(C.c_uint32)),
        ("num_triangles", C.c_uint32),
        ("model_matrix", C.POINTER(C.c_float)),
        ("fixed_indices", C.POINTER(C.c_uint32)),
        ("num_fixed", C.c_uint32),
        ("attached_indices", C.POINTER(C.c_uint32)),
        ("num_attached", C.c_uint32),
        ("binded_indices", C.POINTER(C.c_uint32)),
        ("bind_stiffnesses", C.POINTER(C.c_float)),
        ("bind_distances", C.POINTER(C.c_float)),
        ("bind_obstacle_tri", C.POINTER(C.c_uint32)),
        ("bind_barycentric", C.POINTER(C.c_float)),
        ("num_binded", C.c_uint32),
        ("particle_diameter", C.c_float),
    ]


class ObstacleDesc(C.Structure):
    _fields_ = [
        ("positions", C.POINTER(C.c_float)),
        ("num_vertices", C.c_uint32),
        ("triangles", C.POINTER(C.c_uint32)),
        ("num_triangles", C.c_uint32),
        ("model_matrix", C.POINTER(C.c_float)),
    ]


class Sizes(C.Structure):
    _fields_ = [
        ("num_vertices", C.c_uint32), ("num_edges", C.c_uint32), ("num_triangles", C.c_uint32),
        ("num_bends", C.c_uint32), ("num_lra", C.c_uint32), ("num_bindings", C.c_uint32),
        ("num_obstacle_vertices", C.c_uint32), ("num_obstacle_triangles", C.c_uint32),
        ("num_stretch_colors", C.c_uint32), ("num_bend_colors", C.c_uint32),
        ("launches_per_frame", C.c_uint32), ("frame_index", C.c_uint32),
        ("particle_diameter", C.c_float), ("num_instances", C.c_uint32),
        ("num_obstacle_bvh_nodes", C.c_uint32),
        ("num_stretch_tile_colors", C.c_uint32), ("num_bend_tile_colors", C.c_uint32),
        ("stretch_footprint_vertices", C.c_uint32), ("bend_footprint_vertices", C.c_uint32),
        ("reserved", C.c_uint32 * 1),
    ]


class Grads(C.Structure):
    """xrt_grads (include/xrt_diff.h): output pointers, any may be NULL."""
    _fields_ = [("stretch_compliance", C.POINTER(C.c_float)),
                ("bend_compliance", C.POINTER(C.c_float)),
                ("mass", C.POINTER(C.c_float)), ("velocity", C.POINTER(C.c_float)),
                ("position", C.POINTER(C.c_float))]


class FemMaterial(C.Structure):
    """xrt_fem_material (include/xrt_fem.h)."""
    _fields_ = [("xx_stiffness", C.c_float), ("yy_stiffness", C.c_float),
                ("xy_stiffness", C.c_float), ("xy_poisson_ratio", C.c_float),
                ("yx_poisson_ratio", C.c_float), ("bending_stiffness", C.c_float),
                ("solve_bending", C.c_int32), ("reserved", C.c_int32 * 3)]


class Profile(C.Structure):
    _fields_ = [("ms", C.c_double * 16), ("launches", C.c_uint64 * 16), ("units", C.c_uint64 * 16),
                ("frames", C.c_uint32), ("reserved", C.c_uint32 * 7)]


PHASES = ["predict_finalize", "hash", "collide", "bvh_build", "obstacle_pass", "generate",
          "stretch", "bend", "lra", "vf_solve", "ee_apply", "obstacle_commit",
          "adjoint_replay", "adjoint_stretch", "adjoint_bend", "adjoint_vertex"]

# name -> (restype, argtypes); every symbol declared in include/xrt.h
P = C.c_void_p
FP = C.POINTER(C.c_float)
UP = C.POINTER(C.c_uint32)
IP = C.POINTER(C.c_int32)
SIGNATURES = {
    "xrt_get_version": (C.c_int32, [IP]),
    "xrt_default_params": (C.c_int32, [C.POINTER(SwiftParams)]),
    "xrt_create": (C.c_int32, [C.POINTER(P), C.c_int32]),
    "xrt_destroy": (C.c_int32, [P]),
    "xrt_last_error": (C.c_char_p, [P]),
    "xrt_set_params": (C.c_int32, [P, C.POINTER(SwiftParams)]),
    "xrt_add_cloth": (C.c_int32, [P, C.POINTER(ClothDesc), IP]),
    "xrt_add_obstacle": (C.c_int32, [P, C.POINTER(ObstacleDesc), IP]),
    "xrt_add_instance": (C.c_int32, [P, C.POINTER(ClothDesc), C.POINTER(ObstacleDesc), IP]),
    "xrt_set_coloring": (C.c_int32, [P, C.c_int32, UP, C.c_uint32]),
    "xrt_set_compliance": (C.c_int32, [P, C.c_int32, FP, C.c_uint32]),
    "xrt_set_inv_mass": (C.c_int32, [P, FP, C.c_uint32]),
    "xrt_start": (C.c_int32, [P]),
    "xrt_set_obstacle_targets": (C.c_int32, [P, FP]),
    "xrt_set_obstacle_targets_device": (C.c_int32, [P, P]),
    "xrt_set_obstacle_skinning": (C.c_int32, [P, FP, UP, UP, FP, C.c_uint32]),
    # include/xrt_fem.h
    "xrt_default_fem_material": (C.c_int32, [C.POINTER(FemMaterial)]),
    "xrt_set_fem_material": (C.c_int32, [P, C.POINTER(FemMaterial)]),
    # include/xrt_cache.h
    "xrt_cache_begin": (C.c_int32, [P, C.c_uint32, C.c_int32]),
    "xrt_cache_count": (C.c_int32, [P, UP]),
    "xrt_cache_read": (C.c_int32, [P, C.c_uint32, FP, FP, FP, FP]),
    "xrt_cache_export_obj": (C.c_int32, [P, C.c_char_p, C.c_int32]),
    "xrt_cache_end": (C.c_int32, [P]),
    "xrt_set_joint_transforms": (C.c_int32, [P, FP]),
    "xrt_set_joint_transforms_device": (C.c_int32, [P, P]),
    "xrt_step_frame": (C.c_int32, [P]),
    "xrt_step_frames": (C.c_int32, [P, C.c_int32]),
    "xrt_synchronize": (C.c_int32, [P]),
    "xrt_set_graph_mode": (C.c_int32, [P, C.c_int32]),
    "xrt_set_dependent_launch": (C.c_int32, [P, C.c_int32]),
    "xrt_set_tile_vertices": (C.c_int32, [P, C.c_uint32]),
    "xrt_set_vertex_block": (C.c_int32, [P, C.c_uint32]),
    "xrt_get_sizes": (C.c_int32, [P, C.POINTER(Sizes)]),
    "xrt_set_profiling": (C.c_int32, [P, C.c_int32]),
    "xrt_get_profile": (C.c_int32, [P, C.POINTER(Profile)]),
    "xrt_phase_name": (C.c_char_p, [C.c_int32]),
    "xrt_get_positions": (C.c_int32, [P, FP]),
    "xrt_get_velocities": (C.c_int32, [P, FP]),
    "xrt_get_normals": (C.c_int32, [P, FP]),
    "xrt_get_obstacle_positions": (C.c_int32, [P, FP]),
    "xrt_get_obstacle_normals": (C.c_int32, [P, FP]),
    "xrt_set_state": (C.c_int32, [P, FP, FP]),
    "xrt_get_device_state": (C.c_int32, [P, C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
    "xrt_get_edges": (C.c_int32, [P, UP, FP]),
    "xrt_get_bends": (C.c_int32, [P, UP, FP]),
    "xrt_get_coloring": (C.c_int32, [P, C.c_int32, UP]),
    "xrt_get_lra": (C.c_int32, [P, UP, UP, FP]),
    "xrt_get_obstacle_rtri": (C.c_int32, [P, UP]),
    "xrt_get_inv_mass": (C.c_int32, [P, FP]),
    "xrt_export_obstacle_bvh": (C.c_int32, [P, UP, UP, UP, FP, IP, IP]),
    "xrt_export_contacts": (C.c_int32, [P, IP, FP, IP, FP, FP]),
    "xrt_export_neighbors": (C.c_int32, [P, UP]),
    "xrt_lbvh_create": (C.c_int32, [C.POINTER(P), C.c_int32]),
    "xrt_lbvh_destroy": (C.c_int32, [P]),
    "xrt_lbvh_build": (C.c_int32, [P, FP, FP, C.c_uint32, C.c_float]),
    "xrt_lbvh_build_device": (C.c_int32, [P, P, P, C.c_uint32, C.c_float, P]),
    "xrt_lbvh_refit": (C.c_int32, [P, FP, C.c_uint32]),
    "xrt_lbvh_refit_device": (C.c_int32, [P, P, C.c_uint32, P]),
    "xrt_lbvh_export": (C.c_int32, [P, UP, UP, UP, FP, IP, IP, IP]),
    "xrt_lbvh_query": (C.c_int32, [P, C.c_int32, FP, C.c_uint32, UP, UP]),
    "xrt_lbvh_sizes": (C.c_int32, [P, UP]),
    "xrt_lbvh_build_noalloc": (C.c_int32, [P, P, C.c_uint32, C.c_float, P, P, P, P, P, P, P]),
    # include/xrt_contact.h
    "xrt_cloth_bvh_build": (C.c_int32, [P]),
    "xrt_obstacle_bvh_update_ccd": (C.c_int32, [P]),
    "xrt_proximity_update_pairs": (C.c_int32, [P, C.c_float, UP]),
    "xrt_proximity_solve": (C.c_int32, [P, C.c_float, C.c_float]),
    "xrt_impacts_check": (C.c_int32, [P, C.c_float, UP]),
    "xrt_imminent_generate": (C.c_int32, [P, UP]),
    "xrt_export_quads": (C.c_int32, [P, UP, FP]),
    "xrt_imminent_solve": (C.c_int32, [P, C.c_float, C.c_float, C.c_float]),
    "xrt_collision_step": (C.c_int32, [P, C.c_float, C.c_float, C.POINTER(CollisionStats)]),
    "xrt_export_pairs": (C.c_int32, [P, UP]),
    "xrt_export_impacts": (C.c_int32, [P, FP, FP, FP, UP, IP]),
    "xrt_export_cloth_bvh": (C.c_int32, [P, UP, UP, UP, FP, IP, IP]),
    "xrt_get_predicted": (C.c_int32, [P, FP]),
    "xrt_set_predicted": (C.c_int32, [P, FP]),
    # include/xrt_diff.h
    "xrt_diff_begin": (C.c_int32, [P]),
    "xrt_diff_begin_interval": (C.c_int32, [P, C.c_int32]),
    "xrt_backward": (C.c_int32, [P, FP, FP, C.POINTER(Grads)]),
    "xrt_diff_end": (C.c_int32, [P]),
}

_lib = None


def load():
    """Loads libxrt.so; raises if it was not built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                           "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class XrtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"xrt status {code}: {msg}")
        self.code = code


def check(code, ctx=None, what=""):
    if code != XRT_OK:
        msg = ""
        if ctx:
            raw = load().xrt_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise XrtError(code, f"{what}: {msg}")


def fptr(a):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(FP)


def uptr(a):
    if a is None:
        return None
    assert a.dtype == np.uint32 and a.flags.c_contiguous
    return a.ctypes.data_as(UP)


def iptr(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(IP)
