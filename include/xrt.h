/*
 * xrt.h — C ABI of the GB300-native per-substep cloth step (Swift mode of XRTailor).
 *
 * The reference has no plugin/FFI API: the path is reached through the C++ class
 * ClothSolverBase (xrtailor/include/xrtailor/pipeline/base/ClothSolverBase.hpp:55-194),
 * configured through SimParams / SwiftModeSettings (xrtailor/include/xrtailor/core/Common.hpp:31-168,
 * xrtailor/include/xrtailor/config/Base.hpp:38-139) and driven by ClothSolverBase::FixedUpdate
 * (xrtailor/src/pipeline/base/ClothSolverBase.cpp:147-162).  Each entry point below names the
 * reference call it replaces.  All entry points:
 *   - take plain pointers and sizes (host pointers unless the name ends in _device),
 *   - return an xrt_status (0 = success) and never exit or abort,
 *   - run all device work on the context's own CUDA stream,
 *   - are not re-entrant per context (one host thread per context; contexts are independent).
 */
#ifndef XRT_H_
#define XRT_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XRT_API_VERSION 1

typedef int32_t xrt_status;

/* Status codes.  Numbering follows TAILOR_EXIT where a counterpart exists
 * (xrtailor/include/xrtailor/core/ErrorDefs.hpp:3-34). */
enum {
  XRT_OK = 0,
  XRT_ERR_INVALID_CONFIG = 1001,  /* INVALID_SIMULATION_CONFIG: bad parameter value */
  XRT_ERR_INVALID_MESH = 1002,    /* INVALID_CLOTH_CONFIG: bad topology / index out of range */
  XRT_ERR_INVALID_ARGUMENT = 1003,/* null pointer, size mismatch */
  XRT_ERR_STATE = 1004,           /* call out of order (e.g. step before start) */
  XRT_ERR_CUDA = 8000,            /* CUDA_INTERNAL_ERROR */
  XRT_ERR_NODE_CAPACITY = 8001,   /* NODE_POOL_RUN_OUT */
  XRT_ERR_EDGE_CAPACITY = 8003,   /* EDGE_POOL_RUN_OUT */
  XRT_ERR_FACE_CAPACITY = 8004,   /* FACE_POOL_RUN_OUT */
  XRT_ERR_DEVICE_FLAG = 8100,     /* a kernel raised the sticky device error word */
  XRT_ERR_NO_DEVICE = 8200,       /* no CUDA device / the library was not built for it */
  XRT_ERR_COLORING = 8300         /* supplied coloring is not an independent-set partition */
};

/* Solver parameters: the union of SimParams and SwiftModeSettings that the Swift step reads,
 * with the reference's *effective* defaults (xrt_default_params).  Quirks kept on purpose:
 *   relaxation_factor and geodesic_lra keep the SimParams defaults (0.25, 1) because
 *   SimulationConfigParser::Apply (src/config/SimulationConfigParser.cpp:470-494) never copies
 *   the FABRIC keys of the same names; max_speed and sdf_collision_margin are parsed but read by
 *   no Swift kernel. */
typedef struct xrt_swift_params {
  int32_t num_substeps;            /* SOLVER.NUM_SUBSTEPS (1) */
  int32_t num_iterations;          /* SOLVER.NUM_ITERATIONS (200) */
  float max_speed;                 /* SOLVER.MAX_SPEED (1e6, unused) */
  float gravity[3];                /* SOLVER.GRAVITY (0,-9.8,0) */
  float damping;                   /* SOLVER.DAMPING (0.98) */
  float stretch_compliance;        /* FABRIC.STRETCH_COMPLIANCE (0) default per-edge compliance */
  float bend_compliance;           /* FABRIC.BEND_COMPLIANCE (1e2) default per-bend compliance */
  float relaxation_factor;         /* SimParams.relaxation_factor (0.25) */
  float long_range_stretchiness;   /* FABRIC.LONG_RANGE_STRETCHINESS (1.1) */
  int32_t geodesic_lra;            /* SimParams.geodesic_LRA (1) */
  int32_t solve_bending;           /* FABRIC.SOLVE_BENDING (1) */
  int32_t num_collision_passes;    /* COLLISION.NUM_COLLISION_PASSES (10) */
  float sdf_collision_margin;      /* COLLISION.SDF_COLLISION_MARGIN (1e-2, unused) */
  float bvh_tolerance;             /* COLLISION.BVH_TOLERANCE (0.003) */
  float friction;                  /* COLLISION.PARTICLE.FRICTION (0.1) */
  int32_t max_neighbor_size;       /* COLLISION.PARTICLE.MAX_NEIGHBOR_SIZE (64) */
  int32_t inter_leaved_hash;       /* COLLISION.PARTICLE.INTER_LEAVED_HASH (3) */
  int32_t enable_self_collision;   /* COLLISION.PARTICLE.ENABLE_SELF_COLLISION (1) */
  float particle_diameter;         /* COLLISION.PARTICLE.PARTICLE_DIAMETER (1.3, x first edge length) */
  float hash_cell_size;            /* COLLISION.PARTICLE.HASH_CELL_SIZE (1.5, x particle diameter) */
  float frame_time;                /* Timer fixed_delta_time_ (1/60) */
  int32_t update_obstacle_animation; /* SimParams.update_obstacle_animation (1) */
  /* Quality-mode PBD repulsion inside the Swift frame (0 = off, the reference's Swift step).
   * When on, each frame builds the cloth LBVH and Update(ccd)s the obstacle LBVH, and every
   * iteration starts with SolveNoProximity, preceded every 10 iterations by UpdatePairs with
   * thickness 1e-6 (ClothSolverBase.cpp:276-308).  Frames then run eagerly (pair counts are
   * read back), not as a replayed graph. */
  int32_t pbd_repulsion;
  float pbd_thickness;             /* REPULSION.PBD_THICKNESS (1e-4) */
  float repulsion_relaxation;      /* REPULSION.RELAXATION_RATE (0.25) */
  /* Quality-mode impact-zone collision step at the end of every substep, after the iterations
   * and before the velocity update (ClothSolverBase.cpp:329-336, include/xrt_impact.h).  0 = off.
   * Frames then run eagerly, not as a replayed graph. */
  int32_t impact_zone;
  float impact_zone_obstacle_mass; /* IMPACT_ZONE.OBSTACLE_MASS (1e3) */
  float impact_zone_thickness;     /* IMPACT_ZONE.THICKNESS (1e-4) */
  /* Quality-mode imminent repulsion (ImminentRepulsion, 0 = off): once per frame the cloth x
   * cloth and cloth x obstacle face pairs of the x0 boxes give vertex-face and edge-edge
   * quadratures; every iteration starts with their impulses (ClothSolverBase.cpp:280-300). */
  int32_t imminent_repulsion;
  float imminent_thickness;        /* REPULSION.IMMINENT_THICKNESS (1e-3) */
} xrt_swift_params;

/* Cloth registration, mirrors ClothSolverUniversal::AddCloth(mesh, model_matrix, particle_diameter)
 * (src/pipeline/impl/universal/ClothSolver.cpp:247-350) plus the mesh's fixed / attached /
 * binded vertex lists (src/runtime/mesh/Mesh.cpp).  Positions are in mesh space; rest lengths,
 * rest angles and geodesic LRA lengths are taken from them, the simulated state from
 * model_matrix * position (InitializePositions, src/physics/ClothSolverHelper.cu:113-123). */
typedef struct xrt_cloth_desc {
  const float* positions;          /* 3 * num_vertices */
  uint32_t num_vertices;
  const uint32_t* triangles;       /* 3 * num_triangles, counter-clockwise */
  uint32_t num_triangles;
  const float* model_matrix;       /* 16 floats, column-major (glm), or NULL for identity */
  const uint32_t* fixed_indices;   /* pinned vertices: inv_mass 0 */
  uint32_t num_fixed;
  const uint32_t* attached_indices;/* long-range-attachment slots */
  uint32_t num_attached;
  const uint32_t* binded_indices;  /* binding constraints to the obstacle (SMPL/GLTF pipelines) */
  const float* bind_stiffnesses;
  const float* bind_distances;
  const uint32_t* bind_obstacle_tri; /* 3 obstacle vertex indices per binding */
  const float* bind_barycentric;   /* 3 weights per binding (SkinParam u,v,w) */
  uint32_t num_binded;
  float particle_diameter;         /* > 0: absolute; <= 0: first edge length x params multiplier */
} xrt_cloth_desc;

/* Obstacle registration, mirrors ClothSolverUniversal::AddObstacle (ClothSolver.cpp:189-245). */
typedef struct xrt_obstacle_desc {
  const float* positions;          /* 3 * num_vertices, mesh space */
  uint32_t num_vertices;
  const uint32_t* triangles;       /* 3 * num_triangles */
  uint32_t num_triangles;
  const float* model_matrix;       /* 16 floats column-major or NULL */
} xrt_obstacle_desc;

typedef struct xrt_sizes {
  uint32_t num_vertices, num_edges, num_triangles, num_bends;
  uint32_t num_lra, num_bindings;
  uint32_t num_obstacle_vertices, num_obstacle_triangles;
  uint32_t num_stretch_colors, num_bend_colors;
  uint32_t launches_per_frame;     /* kernels launched by one xrt_step_frame */
  uint32_t frame_index;
  float particle_diameter;         /* of instance 0 (merged mode: the last cloth added) */
  uint32_t num_instances;          /* 1 in merged mode */
  uint32_t num_obstacle_bvh_nodes; /* sum over instances of 2 F_i - 1 (F_i > 0) */
  /* tile-local schedule (0 when the kind runs per color) of the stretch and bend kinds, or of
   * the FEM strain and bending kinds when the FEM fabric is on: tile colors (one launch each
   * per iteration) and the summed footprint vertices of all tiles (a tile color's tiles have
   * disjoint footprints, so one launch touches footprint / tile colors vertices on average) */
  uint32_t num_stretch_tile_colors, num_bend_tile_colors;
  uint32_t stretch_footprint_vertices, bend_footprint_vertices;
  uint32_t reserved[1];
} xrt_sizes;

typedef struct xrt_ctx xrt_ctx;

/* ---- lifecycle ------------------------------------------------------------------------ */
xrt_status xrt_get_version(int32_t* api_version);
xrt_status xrt_default_params(xrt_swift_params* out);
/* Creates a context on `device`; owns a CUDA stream and all device buffers. */
xrt_status xrt_create(xrt_ctx** out, int32_t device);
xrt_status xrt_destroy(xrt_ctx* ctx);
/* Last error message of this context (NUL-terminated, owned by the context). */
const char* xrt_last_error(const xrt_ctx* ctx);

/* ---- setup ---------------------------------------------------------------------------- */
/* Global::sim_params / sim_config (core/Global.hpp:22-25) -> SetSimulationParams
 * (ClothSolverHelper.cu:16-23).  May be called again between frames.  After xrt_start, a new
 * substep time (frame_time / num_substeps) also re-evaluates the compliance terms held in the
 * constraint records (a synchronous upload, as xrt_set_compliance). */
xrt_status xrt_set_params(xrt_ctx* ctx, const xrt_swift_params* params);
/* ClothSolverUniversal::AddCloth.  out_vertex_offset receives prev_num_particles. */
xrt_status xrt_add_cloth(xrt_ctx* ctx, const xrt_cloth_desc* desc, int32_t* out_vertex_offset);
/* ClothSolverUniversal::AddObstacle. */
xrt_status xrt_add_obstacle(xrt_ctx* ctx, const xrt_obstacle_desc* desc, int32_t* out_vertex_offset);
/* Batched form: adds an independent instance, a cloth with its own obstacle (`obstacle` may be
 * NULL).  Every instance runs in the same launches as the others, but sees only itself: its own
 * particle diameter, particle-hash table (2 V_i cells) and obstacle LBVH, no contact with other
 * instances.  Instance i's frame is bit for bit that of a context holding only cloth i and
 * obstacle i.  Cloth vertices, obstacle vertices and triangles are numbered over all instances
 * in the order added (obstacle targets, exports); binding obstacle indices are local to the
 * instance's obstacle.  Per-instance compliance goes through xrt_set_compliance.  A context is
 * either batched or merged (xrt_add_cloth / xrt_add_obstacle: the reference's single mesh);
 * Quality-mode repulsion (pbd_repulsion) is merged-mode only.  No reference counterpart: the
 * reference steps one solver per scene. */
xrt_status xrt_add_instance(xrt_ctx* ctx, const xrt_cloth_desc* cloth,
                            const xrt_obstacle_desc* obstacle, int32_t* out_instance);
/* Kinds 2 and 3 are the FEM fabric's strain (one per cloth face) and isometric bending (one per
 * bend element) constraints (include/xrt_fem.h); xrt_get_coloring reports them after xrt_start.
 * Overrides the graph coloring of the stretch (kind 0) or bend (kind 1) constraints, in the
 * constraint order reported by xrt_get_edges / xrt_get_bends.  Replaces
 * GraphColoring::Paint (src/physics/graph_coloring/Base.cu:163-317), whose randomized result
 * differs run to run; parity runs feed one coloring to both sides.  Before xrt_start. */
xrt_status xrt_set_coloring(xrt_ctx* ctx, int32_t kind, const uint32_t* colors, uint32_t n);
/* Per-edge stretch / per-bend compliance (FABRIC.*_COMPLIANCE per element).  Before or after start. */
xrt_status xrt_set_compliance(xrt_ctx* ctx, int32_t kind, const float* compliance, uint32_t n);
/* Per-vertex inverse mass override (Node::inv_mass, PhysicsMeshHelper.cu:139 gives 1 / 0 pinned).
 * Before start any values; after start new masses for the free vertices (pinned stay 0). */
xrt_status xrt_set_inv_mass(xrt_ctx* ctx, const float* inv_mass, uint32_t n);
/* ClothSolverUniversal::Start (ClothSolver.cpp:46-93): normals, obstacle LBVH, R-triangles,
 * spatial hash, coloring, LRA, device upload. */
xrt_status xrt_start(xrt_ctx* ctx);

/* ---- stepping ------------------------------------------------------------------------- */
/* Sets the obstacle's target positions for the next frame (UpdateObstaclePredicted,
 * ClothSolverHelper.cu:71-97): world space, 3 * num_obstacle_vertices floats. */
xrt_status xrt_set_obstacle_targets(xrt_ctx* ctx, const float* positions);
xrt_status xrt_set_obstacle_targets_device(xrt_ctx* ctx, const float* d_positions);
/* Obstacle skinning on the device: each xrt_step_frame first computes the obstacle's targets by
 * linear blend skinning, as SMPL's lbs kernel (src/runtime/rag_doll/smpl/cuda/body.cu:39-60), on
 * the context stream, so a moving body costs one upload of its joint transforms per frame
 * instead of its vertex positions.  After xrt_start.  rest: 3 floats per obstacle vertex (the
 * shaped rest pose, obstacle numbering); influences in CSR over the obstacle vertices: outer
 * (num_obstacle_vertices + 1 offsets, outer[0] = 0), then per influence a joint index
 * (< num_joints; joints numbered across all instances of a batched context) and a weight.
 * rest = NULL turns skinning off.  While it is on, xrt_set_obstacle_targets* return
 * XRT_ERR_STATE.  Transforms start as identities. */
xrt_status xrt_set_obstacle_skinning(xrt_ctx* ctx, const float* rest, const uint32_t* outer,
                                     const uint32_t* joints, const float* weights,
                                     uint32_t num_joints);
/* Joint global transforms for the following frames: 12 floats per joint, the top three rows of
 * the 4x4 homogeneous transform, row-major (SMPL's d_joint_global_transform layout). */
xrt_status xrt_set_joint_transforms(xrt_ctx* ctx, const float* transforms);
xrt_status xrt_set_joint_transforms_device(xrt_ctx* ctx, const float* d_transforms);
/* One frame = ClothSolverBase::SimulateSwift (ClothSolverBase.cpp:171-261). Asynchronous on the
 * context stream; the first call (and the first after set_params) records the frame as a
 * CUDA graph which later calls replay. */
xrt_status xrt_step_frame(xrt_ctx* ctx);
xrt_status xrt_step_frames(xrt_ctx* ctx, int32_t num_frames);
/* Waits for the context stream and reports the sticky device error word. */
xrt_status xrt_synchronize(xrt_ctx* ctx);
/* Enables (1) / disables (0) CUDA-graph replay of frames (default 1). */
xrt_status xrt_set_graph_mode(xrt_ctx* ctx, int32_t enabled);
/* Enables (1) / disables (0) programmatic dependent launch of the substep kernels (default 1):
 * each kernel may start, and read its setup-time data, while its predecessor finishes.  Results
 * are identical either way.  No reference counterpart (a launch option of this library). */
xrt_status xrt_set_dependent_launch(xrt_ctx* ctx, int32_t enabled);
/* Tile size of the tile-local Gauss-Seidel schedule of stretch and bend constraints, in
 * consecutive vertices (default 256; halved while a tile's footprint exceeds 4,096 vertices),
 * or 0 for one launch per color of a greedy coloring.  Before xrt_start; a caller coloring
 * (xrt_set_coloring) always runs as per-color launches.  No reference counterpart (the
 * reference launches one kernel per color, BasicSolver.cu:131-134). */
xrt_status xrt_set_tile_vertices(xrt_ctx* ctx, uint32_t tile_vertices);
/* Threads per block of the per-vertex substep kernels (predict / finalize, particle collide,
 * LRA + VF and EE + ApplyDeltas): 64 to 512, a multiple of 32 (default 128).  Results are
 * identical for every value.  No reference counterpart (a launch option of this library; the
 * reference launches its per-vertex kernels with fixed 256-thread blocks). */
xrt_status xrt_set_vertex_block(xrt_ctx* ctx, uint32_t threads);

/* ---- per-phase GPU timing (replaces Timer / ScopedTimerGPU, utils/Timer.hpp:67-114) -------- */
#define XRT_NUM_PHASES 16
typedef struct xrt_profile {
  double ms[16];        /* summed CUDA-event time of the phase's launches */
  uint64_t launches[16];/* kernel launches of the phase */
  uint64_t units[16];   /* elements processed (vertices, constraints, edges, ...) */
  uint32_t frames;      /* frames accumulated */
  uint32_t reserved[7];
} xrt_profile;
/* enabled = 1: frames run eagerly with a CUDA-event pair around every launch, accumulating per
 * phase; 2: each frame is captured as a graph with an event-record node pair around every phase
 * group (one iteration's stretch launches, its bend launches, and each single launch of the
 * other phases) and replayed, so the launches inside a group keep their dependent-launch edges
 * (frames that read results back on the host run as in mode 1); 0: back to graph replay.
 * Resets the accumulators. */
xrt_status xrt_set_profiling(xrt_ctx* ctx, int32_t enabled);
xrt_status xrt_get_profile(xrt_ctx* ctx, xrt_profile* out);
/* Phase names: 0 predict_finalize, 1 hash, 2 collide, 3 bvh_build, 4 obstacle_pass, 5 generate,
 * 6 stretch, 7 bend, 8 lra, 9 vf_solve, 10 ee_apply, 11 obstacle_commit; the reverse pass
 * (xrt_backward, include/xrt_diff.h) while profiling: 12 adjoint_replay (taping re-run of each
 * frame), 13 adjoint_stretch, 14 adjoint_bend, 15 adjoint_vertex (LRA, contacts, integration). */
const char* xrt_phase_name(int32_t phase);

/* ---- state ---------------------------------------------------------------------------- */
xrt_status xrt_get_sizes(const xrt_ctx* ctx, xrt_sizes* out);
/* PhysicsMesh::HostPositions / HostNormals (PhysicsMesh.cu:326-377): 3 floats per vertex. */
xrt_status xrt_get_positions(xrt_ctx* ctx, float* out);
xrt_status xrt_get_velocities(xrt_ctx* ctx, float* out);
xrt_status xrt_get_normals(xrt_ctx* ctx, float* out);
xrt_status xrt_get_obstacle_positions(xrt_ctx* ctx, float* out);
xrt_status xrt_get_obstacle_normals(xrt_ctx* ctx, float* out);
xrt_status xrt_set_state(xrt_ctx* ctx, const float* positions, const float* velocities);
/* Device pointers to the resident state (float4 per vertex: xyz + inverse mass in w for
 * positions), valid until xrt_destroy; stream = the context's cudaStream_t. */
xrt_status xrt_get_device_state(xrt_ctx* ctx, void** d_positions_f4, void** d_velocities_f4,
                                void** stream);

/* ---- topology / parity exports --------------------------------------------------------- */
xrt_status xrt_get_edges(const xrt_ctx* ctx, uint32_t* out2, float* rest_lengths);
xrt_status xrt_get_bends(const xrt_ctx* ctx, uint32_t* out4, float* rest_angles);
xrt_status xrt_get_coloring(const xrt_ctx* ctx, int32_t kind, uint32_t* colors);
xrt_status xrt_get_lra(const xrt_ctx* ctx, uint32_t* src, uint32_t* tgt, float* rest);
xrt_status xrt_get_obstacle_rtri(const xrt_ctx* ctx, uint32_t* masks);
/* Per-vertex inverse mass as set (0 = pinned): num_vertices floats. */
xrt_status xrt_get_inv_mass(const xrt_ctx* ctx, float* out);
/* Obstacle LBVH as built at the last frame start (BVH::Construct, BVH.cu:618-722) and refit
 * by the last collision pass.  sorted_morton/sorted_objects: num_obstacle_triangles;
 * nodes: 4 int32 per node (parent, left, right, object; 0xFFFFFFFF = none), 2F-1 nodes;
 * aabbs: 6 floats per node (lower xyz, upper xyz); i_esc: F-1, e_esc: F.  Any pointer may be NULL.
 * Batched contexts: the instances' trees one after the other (num_obstacle_bvh_nodes nodes,
 * num_obstacle_bvh_nodes - F internal escapes); links and objects are local to each tree,
 * sorted_objects are global triangle ids. */
xrt_status xrt_export_obstacle_bvh(xrt_ctx* ctx, uint32_t* sorted_morton, uint32_t* sorted_objects,
                                   uint32_t* nodes, float* aabbs, int32_t* i_esc, int32_t* e_esc);
/* Contacts of the last collision pass (VFContact / RTContact / EEContact, pbd_collision/Contact.cuh):
 * vf_index/rt_index: int32 per cloth vertex (-1 = none); vf_qs/rt_qc: 3 floats per vertex;
 * ee: 12 floats per cloth edge (dist, p2 xyz, q2 xyz, s, t, fn xyz).  Any pointer may be NULL. */
xrt_status xrt_export_contacts(xrt_ctx* ctx, int32_t* vf_index, float* vf_qs, int32_t* rt_index,
                               float* rt_qc, float* ee);
/* Particle neighbor lists of the last hash (SpatialHashGPU::neighbors, strided by V,
 * terminated by 0xFFFFFFFF): max_neighbor_size * V uint32. */
xrt_status xrt_export_neighbors(xrt_ctx* ctx, uint32_t* neighbors);

/* ---- standalone LBVH (BVH class, src/physics/broad_phase/lbvh/BVH.cu) ----------------- */
typedef struct xrt_lbvh xrt_lbvh;
xrt_status xrt_lbvh_create(xrt_lbvh** out, int32_t device);
xrt_status xrt_lbvh_destroy(xrt_lbvh* bvh);
/* BVH::UpdateData + Construct(scr): prims = 9 floats (v1,v2,v3) per primitive; pred = 9 floats
 * (pred1..3) or NULL (= v).  Host pointers. */
xrt_status xrt_lbvh_build(xrt_lbvh* bvh, const float* prims, const float* pred, uint32_t n, float scr);
/* Same from device pointers on the given stream (cudaStream_t or NULL); no host sync. */
xrt_status xrt_lbvh_build_device(xrt_lbvh* bvh, const float* d_prims, const float* d_pred, uint32_t n,
                                 float scr, void* stream);
/* RefitExternalNode + AssignAABBCAS (BVH.cu:854-818 family): leaves grow by the new pred. */
xrt_status xrt_lbvh_refit(xrt_lbvh* bvh, const float* pred, uint32_t n);
xrt_status xrt_lbvh_refit_device(xrt_lbvh* bvh, const float* d_pred, uint32_t n, void* stream);
xrt_status xrt_lbvh_export(xrt_lbvh* bvh, uint32_t* sorted_morton, uint32_t* sorted_objects,
                           uint32_t* nodes, float* aabbs, int32_t* i_esc, int32_t* e_esc,
                           int32_t* morton_unique);
/* QueryDeviceStackless (BVH.cu:957-1055): kind 0 = points (3 floats), 1 = segments (6 floats),
 * 2 = boxes (6 floats: lower, upper).  counts: n; cands: n * 256 (LBVH_MAX_BUFFER_SIZE). */
xrt_status xrt_lbvh_query(xrt_lbvh* bvh, int32_t kind, const float* queries, uint32_t n,
                          uint32_t* counts, uint32_t* cands);
/* Wall-clock-free timing helper for benchmarks: the build's kernels on the given stream. */
xrt_status xrt_lbvh_sizes(const xrt_lbvh* bvh, uint32_t* num_objects);

/* LBVH build that allocates no memory.  No counterpart in the reference.
 * For callers that may not allocate GPU memory: applications that host the solver inside their
 * own frame loop (engines, DCC plugins) and forbid allocation after start-up, because
 * cudaMalloc / cudaFree can synchronise the device mid-frame or fail under memory pressure.
 * Same result as xrt_lbvh_build_device + xrt_lbvh_export, written to the caller's device
 * buffers: sorted_morton / sorted_objects (n), nodes (4 x (2n-1) uint32), aabbs (6 x (2n-1)
 * float), i_esc (n-1), e_esc (n).  d_pred may be NULL (= d_prims).  Asynchronous on `stream`.
 * Working memory is one fixed ~17 MiB device array per GPU (held from first use until exit):
 * at most 65,536 primitives (larger n -> XRT_ERR_FACE_CAPACITY).  All calls on a GPU share that
 * array; calls whose device work overlaps race, so order them on one stream.  The first call on
 * each GPU looks up the array's device address (cudaGetSymbolAddress) with that GPU current;
 * make it before any stream capture starts.  The status covers argument checks and launch
 * errors only: the build's bounded tree walks, which can trip only on a corrupt tree (for
 * instance NaN coordinates), record their error in the scratch array and are not reported;
 * pass finite coordinates. */
xrt_status xrt_lbvh_build_noalloc(const float* d_prims, const float* d_pred, uint32_t n, float scr,
                                  uint32_t* d_sorted_morton, uint32_t* d_sorted_objects,
                                  uint32_t* d_nodes, float* d_aabbs, int32_t* d_i_esc,
                                  int32_t* d_e_esc, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* XRT_H_ */
