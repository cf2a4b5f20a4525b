// context.h — host-side context of the GB300 cloth step: device buffers and the launchers that
// the C ABI (api.cpp) sequences.  One context = one CUDA stream; no globals.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/xrt.h"
#include "../../include/xrt_fem.h"
#include "../../include/xrt_impact.h"
#include "setup.h"

// Returns XRT_ERR_CUDA from the enclosing function, with the failing call in the context's error.
#define XRT_CUDA(ctxp, expr)                                                 \
  do {                                                                       \
    cudaError_t e_ = (expr);                                                 \
    if (e_ != cudaSuccess) {                                                 \
      (ctxp)->set_error(std::string(#expr) + ": " + cudaGetErrorString(e_)); \
      return XRT_ERR_CUDA;                                                   \
    }                                                                        \
  } while (0)

namespace xrt {

constexpr uint32_t kMaxCandidatesHost = 256;         // LBVH_MAX_BUFFER_SIZE
constexpr float kScalarMaxHost = 3.402823466e+38f;   // SCALAR_MAX

// Growable device buffer (cudaMalloc / cudaFree only at setup or on growth, never per frame).
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t reserve(size_t count) {
    if (count <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

// ---- radix sort (radix.cu) --------------------------------------------------------------------
struct RadixSort {
  // Keys per histogram / scatter tile, digits per pass, and histogram entries per block of the
  // multi-block scan.  Histograms of at most kSingleBlockScan entries are scanned by one block
  // and never touch `sums`.
  static constexpr uint32_t kTileKeys = 2048;
  static constexpr uint32_t kDigits = 256;
  static constexpr uint32_t kScanChunk = 4096;
  static constexpr uint32_t kSingleBlockScan = 4 * kScanChunk;
  static constexpr size_t hist_entries(size_t n) {
    return (size_t)kDigits * (n ? (n + kTileKeys - 1) / kTileKeys : 1);
  }
  static constexpr size_t sums_entries(size_t n) {
    return (hist_entries(n) + kScanChunk - 1) / kScanChunk;
  }
  DBuf<uint32_t> keys_tmp, vals_tmp, hist, sums;
  cudaError_t reserve(uint32_t n);
  // Stable LSD sort of (keys, vals) by the low `bits` bits of keys.  The result is left in
  // (keys, vals) if the number of 8-bit passes is even, else in the tmp buffers; returns the
  // buffers that hold it.
  void sort(uint32_t* keys, uint32_t* vals, uint32_t n, int bits, cudaStream_t s,
            uint32_t** out_keys, uint32_t** out_vals);
};

// ---- LBVH (lbvh.cu) ---------------------------------------------------------------------------
// One tree (a segment of a forest, see LbvhForest): node ids, child / escape links and objects
// are local to the tree, `pred` points at the tree's first primitive.
struct LbvhView {
  uint32_t n;          // primitives
  const float4* pred;  // 3 per primitive (pred1..3), original order
  const float4* lo;    // 2n-1 nodes; xyz = lower, w = left child (internal) / object (leaf)
  const float4* hi;    // 2n-1 nodes; xyz = upper, w = escape index (-1 = end)
};

// A forest of independent trees over consecutive primitive ranges (segments), in shared arrays.
// Segment s owns primitives [prim_base, prim_base + n), nodes [node_base, node_base + 2n - 1)
// (internal nodes first, then leaves, as in a single tree) and merge counters
// [internal_base, internal_base + n - 1).  Every link is local to its segment, so each segment is
// bit for bit the tree its primitives alone would give.  One segment = the classic single tree.
struct LbvhForest {
  LbvhView all;       // n = total primitives; lo / hi over all nodes
  const int4* seg;    // per segment {prim_base, n, node_base, internal_base}; unused if nseg == 1
  uint32_t nseg;
  int4 one;           // the record when nseg == 1
};

struct Lbvh {
  uint32_t n = 0;                  // total primitives
  uint32_t nodes = 0;              // total nodes (sum of 2 n_s - 1 over non-empty segments)
  uint32_t internal = 0;           // total internal nodes
  bool active = false;
  DBuf<float4> v, pred;            // 3 per primitive
  DBuf<float4> leaf_lo, leaf_hi;   // per primitive (original order) before sorting
  DBuf<float4> lo, hi;             // per node
  DBuf<int4> node;                 // parent, left, right, object (segment-local)
  DBuf<uint32_t> morton, index;    // sort inputs
  DBuf<uint32_t> skey, sval;       // segment pass of the sort (nseg > 1)
  DBuf<unsigned long long> key64;
  DBuf<uint32_t> flags;            // arrival counters of the bottom-up merge (parity)
  DBuf<int32_t> iesc, eesc;
  DBuf<float> root;                // 6 floats per segment (ordered-int encoded)
  DBuf<uint32_t> dup;              // number of equal adjacent Morton codes
  uint32_t* sorted_morton = nullptr;
  uint32_t* sorted_index = nullptr;
  RadixSort sorter;
  std::vector<int4> h_seg;         // segment records (host); empty = one segment of n
  DBuf<int4> seg;

  // Segments of the forest: primitive counts in primitive order (empty = one segment).
  // Uploads the table; call before reserve.
  cudaError_t set_segments(const std::vector<uint32_t>& counts, cudaStream_t s);
  cudaError_t reserve(uint32_t n_prims);
  // BVH::Construct(scr) on v / pred already in device memory (BVH.cu:618-722), every segment.
  void construct(float scr, cudaStream_t s, uint32_t* d_err);
  // Leaves grow by pred (already updated), internal boxes recomputed bottom-up.
  void refit_from_pred(cudaStream_t s, uint32_t* d_err);
  uint32_t nseg() const { return h_seg.empty() ? 1u : (uint32_t)h_seg.size(); }
  int4 seg_one() const { return make_int4(0, (int)n, 0, 0); }
  LbvhView view() const { return LbvhView{n, pred.p, lo.p, hi.p}; }  // single-segment trees
  LbvhForest forest() const {
    return LbvhForest{view(), seg.p, nseg(), h_seg.empty() ? seg_one() : h_seg[0]};
  }
  void release();
};

// prims from a mesh: v_k = x[idx_k] + tol * n[idx_k], pred = v (BVH::UpdateData, ccd = false)
void launch_prims_from_mesh(Lbvh& b, const float4* x, const float4* nrm, const int4* tri,
                            uint32_t nf, float tol, cudaStream_t s);
// RefitMidstep: pred_k = x1[idx_k] + tol * n1[idx_k], leaves grow, internal merge.
void launch_refit_midstep(Lbvh& b, const float4* x1, const float4* n1, const int4* tri, float tol,
                          cudaStream_t s, uint32_t* d_err);
// Standalone query kernel: candidates of points (kind 0), segments (1), boxes (2).
void launch_lbvh_query(const Lbvh& b, int kind, const float* d_q, uint32_t nq, uint32_t* d_counts,
                       uint32_t* d_cands, cudaStream_t s, uint32_t* d_err);
void launch_float9_to_float4(const float* d_in, float4* d_out, uint32_t n_prims, cudaStream_t s);

// ---- instances (batched form) -------------------------------------------------------------------
// Per-instance constants.  In merged mode (the reference's one mesh of every cloth) there is one
// instance; in the batched form instance i is cloth i with its own obstacle (segment i of the
// obstacle LBVH forest), its own particle diameter and its own slice of the particle hash table.
struct InstanceRec {
  float spacing, spacing2, d2, diameter;  // hash cell size, its square, diameter^2, diameter
  uint32_t table_base, table_size;        // hash keys of the instance: [base, base + size)
  uint32_t vertex_base, num_vertices;     // cloth vertices
};
struct InstView {
  uint32_t count;
  const InstanceRec* rec;      // count records (unused when count == 1)
  const uint32_t* of_vertex;   // cloth vertex -> instance (unused when count == 1)
  InstanceRec one;             // the record when count == 1
};

// ---- cloth state --------------------------------------------------------------------------------
struct ColorRange {
  uint32_t begin, end;
};

// ---- hand-written adjoint (diff.cu) --------------------------------------------------------------
// Between xrt_diff_begin and xrt_backward the state at every `interval`-th frame start is
// checkpointed, and every frame's obstacle targets are kept; the reverse pass walks the
// segments of `interval` frames newest first: it restores the segment's checkpoint, recomputes
// the segment's frames plainly (keeping each frame's start state), then replays each frame,
// newest first, while taping the inputs of every projection (same colors, same order: the same
// bits) and walks the tape backwards.
struct DiffState {
  bool active = false;
  uint32_t frames = 0;    // frames stepped since xrt_diff_begin
  uint32_t interval = 1;  // frames per checkpoint
  struct Checkpoint {
    DBuf<float4> x, x0, v, ox0, ox, on;
    uint32_t frame_index = 0;
  };
  std::vector<Checkpoint> ck;        // one per segment
  std::vector<DBuf<float4>> targets; // per frame: the obstacle targets at its start
  std::vector<Checkpoint> seg;       // the reverse pass's recomputed frame starts of a segment
  // execution slots grouped by color, colors in forward order
  std::vector<ColorRange> s_colors, b_colors;
  DBuf<uint32_t> s_order, b_order;
  DBuf<int2> s_gidx;  // per stretch execution slot: global vertex ids
  DBuf<int4> b_gidx;  // per bend execution slot
  // one frame of tape
  uint32_t S = 0, I = 0, P = 0;
  std::vector<int> it_pass;             // (substep, iteration) -> collision pass of the frame
  // every projection's inputs by execution slot; replayed and reversed per tile color where the
  // schedule is tiled (s_tiled / b_tiled), per color otherwise
  bool s_tiled = false, b_tiled = false;
  bool s_stage = false, b_stage = false;  // tiled reverse stages each tile's tape in shared memory
  uint32_t s_block = 256, b_block = 256;  // threads per tile block of the tiled reverse
  DBuf<float4> t_sx;                    // S x I x E x 2: stretch inputs (x with inverse mass)
  DBuf<float> t_sl;                     // S x I x E: stretch multipliers in
  DBuf<float4> t_bx;                    // S x I x B x 4: bend inputs
  DBuf<float4> t_stage, t_ee;           // S x I x V: inputs of the LRA+VF and EE launches
  DBuf<int> t_vf_idx, t_rt_idx;         // P x V
  DBuf<float4> t_vf_qs, t_rt_qc;        // P x V
  DBuf<float4> t_ee_a, t_ee_b, t_ee_c;  // P x E
  DBuf<float4> t_pred;                  // P x 3F (obstacle primitives of the pass)
  // adjoint
  DBuf<float4> G, G2, Gv, H, Gs;        // x-bar (+ inverse-mass bar in w), v-bar, temporaries
  DBuf<float> cnt;                      // tape: per iteration, each vertex's EE contact count
  DBuf<float> lam_bar, comp_bar, bcomp_bar;
  // one frame's replay + reverse as a CUDA graph (built per xrt_backward call), per starting
  // assignment of the G / G2 double buffer, with the assignment the frame leaves
  struct FrameGraph {
    cudaGraphExec_t exec = nullptr;
    float4 *g_in = nullptr, *g_out = nullptr, *g2_out = nullptr;
  };
  FrameGraph graph[2];
};

// Tile-local Gauss-Seidel schedule of one constraint kind on the device (setup::TileSchedule):
// one launch per tile color, one block per tile, local colors in shared memory.
// Largest tile footprint the tile kernels stage (512 threads x kFootPerThread in solver.cu).
constexpr uint32_t kTileMaxFootprint = 4096;

struct TiledSet {
  bool on = false;
  uint32_t num_local = 0;
  uint32_t max_foot = 0;
  uint32_t max_cons = 0;                // most constraints in one tile
  uint32_t max_step = 0;                // most constraints in one local color of one tile
  uint32_t block = 512;                 // threads per tile block (256 or 512)
  uint32_t block1 = 512;                // threads per block of the streamed (one-lane) kernels
  uint32_t resident = 0;                // tile blocks the GPU holds at once (pair-mode bound)
  std::vector<ColorRange> tile_colors;  // ranges of executed tiles per tile color
  std::vector<uint32_t> tile_color_cons;  // constraints per tile color (profiling units)
  DBuf<uint32_t> foot;                  // footprint vertices of every executed tile
  DBuf<int4> meta;                      // per executed tile {first footprint, footprint size,
                                        //  first constraint, constraint count}
  DBuf<uint32_t> lofs;                  // per executed tile: num_local + 1 offsets, tile-relative
  // Records of the forward tile kernels, one 16-byte aligned block per executed tile: the
  // constraints' footprint-local vertex ids as 16-bit values (2 per stretch constraint, 4 per
  // bend element), padded to 16 bytes, then their float2 values (rest length and
  // stretch_alpha(compliance, dt) / rest angle and bend_alpha(compliance, dt), for the dt of
  // Context::rec_dt), padded to 16 bytes: one such segment per local color, in color order,
  // copied whole or color by color.
  DBuf<uint4> rec;
  DBuf<uint32_t> rec_ofs;               // per executed tile: first uint4 of its block; + the end
  uint32_t max_seg16 = 0;               // largest local color's segment, in uint4
  uint32_t max_tile16 = 0;              // largest tile's block of color segments, in uint4
};

// uint4 units of one local color's record segment of n constraints: `arity` 16-bit ids each,
// then a float2 each, both padded to 16 bytes.
__host__ __device__ inline uint32_t color_seg16(uint32_t n, uint32_t arity) {
  return (2 * arity * n + 15) / 16 + (8 * n + 15) / 16;
}

// The XPBD compliance terms, in the reference's order of operations: alpha~ = compliance /
// (dt dt) of SolveStretch_Kernel (BasicSolverHelper.cu:105) and compliance / dt / dt of
// SolveBend_Kernel (BasicSolverHelper.cu:53).  The host evaluates them into the tile records with
// the same correctly rounded operations, so the kernels that read them get the same bits.
__host__ __device__ inline float stretch_alpha(float compliance, float dt) {
  return compliance / (dt * dt);
}
__host__ __device__ inline float bend_alpha(float compliance, float dt) {
  return compliance / dt / dt;
}


// One constraint kind of the FEM fabric: its schedule (as the stretch / bend kinds') and the
// slot-ordered vertex ids (footprint-local when tiled).
struct FemKind {
  std::vector<uint32_t> color;
  uint32_t ncolors = 0;
  TiledSet tiles;
  std::vector<uint32_t> perm, local;
  std::vector<ColorRange> ranges;
  std::vector<int4> meta;
  std::vector<uint32_t> lofs;
  DBuf<int4> idx;
};

// The FEM fabric (fem.cu, include/xrt_fem.h).
struct FemState {
  bool on = false;
  xrt_fem_material m{};
  float c00 = 0, c01 = 0, c10 = 0, c11 = 0, c22 = 0;  // orthotropic tensor entries
  FemKind strain, bend;            // strain: cloth faces; bend: the bend elements
  DBuf<float4> s_inv;              // per strain slot: inverse material matrix (glm order)
  DBuf<float> s_area;              // per strain slot
  DBuf<float> b_q;                 // per bend slot: 16 floats, row-major Hessian
  DBuf<float> b_lambda;            // per bend slot
};

// Obstacle skinning on the device (skin.cu): rest pose, CSR influences, joint transforms.
struct SkinState {
  bool on = false;
  uint32_t num_joints = 0;
  DBuf<float4> rest;        // per obstacle vertex
  DBuf<uint32_t> outer;     // num_obstacle_vertices + 1
  DBuf<uint32_t> joint;     // per influence
  DBuf<float> weight;       // per influence
  DBuf<float> transforms;   // 12 per joint (3 x 4, row-major)
};

// Frame cache (cache.cu): device staging slots, a copy stream and a pinned host store.
struct CacheState {
  static constexpr int kSlots = 3;
  bool on = false;
  uint32_t flags = 0, capacity = 0, count = 0;
  uint32_t per_frame = 0;            // floats per cached frame
  float* host = nullptr;             // pinned, capacity x per_frame
  DBuf<float> stage[kSlots];
  cudaEvent_t staged[kSlots] = {};   // packing done (context stream)
  cudaEvent_t copied[kSlots] = {};   // copy to the host done (copy stream)
  bool used[kSlots] = {};
  cudaStream_t copy = nullptr;
};

// Quality-mode self contact (proximity.cu): unified numbering, cloth first then obstacle.
struct ScanScratch {               // tile sums of the multi-block scan (proximity.cu)
  DBuf<uint32_t> sums, incl;
};

struct ProximityState {
  bool ready = false;
  ScanScratch scan;
  Lbvh cbvh;                       // cloth LBVH
  DBuf<int4> face;                 // nodes (unified) + r-triangle mask
  DBuf<int4> fedge;                // unified edge of (v_i, v_i+1)
  DBuf<float4> fn0;                // registration-time face normals
  DBuf<uint2> edge;                // unified nodes of each edge
  DBuf<int4> eadj;                 // adjacent unified faces, -1 = none
  DBuf<uint8_t> cfree;             // Node::is_free of cloth nodes
  DBuf<uint32_t> counts, incl, total;
  DBuf<uint2> pairs;
  uint32_t npairs = 0;
  DBuf<float> deltas;              // 3 per cloth node
  DBuf<int> rcounts;
  DBuf<float> imp_t;
  DBuf<float4> imp_w, imp_n;
  DBuf<uint4> imp_nodes;
  uint32_t nimpacts = 0;
  // imminent repulsion: 12 quadrature slots per face pair (9 edge-edge, 3 vertex-face) of the
  // frame; nodes.x = kNone marks an empty slot
  DBuf<uint4> qnodes;
  DBuf<float4> qbary;
  uint32_t nquads = 0;
  DBuf<float4> ov;                 // obstacle Node::v (set by the collision step; 0 before)
};

// Impact-zone collision step (impact.cu).  An impact zone: impacts (ids into the step's impact
// store) solved together, and the set of every unified node they touch.
struct HostZone {
  std::vector<uint32_t> impacts;
  std::vector<uint32_t> nodes;  // sorted, unique
  bool active = true, enabled = true;
};

struct ImpactZoneState {
  bool ready = false;
  Lbvh cbvh, obvh;                  // the step's own LBVHs over x0 -> x boxes
  DBuf<float4> cx1, ox1;            // Node::x1: positions at the start of the step
  DBuf<uint32_t> hits, hit_incl, hit_total;
  DBuf<float> new_t;                // impacts of this pass in (pair, test) order
  DBuf<uint4> new_nodes;
  DBuf<uint32_t> new_src;           // their slot in the CheckImpacts output
  DBuf<uint32_t> pick;              // compacted ids of the independent impacts
  DBuf<float4> sw, sn;              // impact store: weights, normal
  DBuf<uint4> snodes;
  uint32_t nstore = 0;
  // optimizer layout of the active zones
  DBuf<int4> zone;                  // entry begin, entry end, node begin, node end
  DBuf<uint32_t> zimp;              // store id per entry
  DBuf<int32_t> zloc;               // 4 per entry: node position, -1 = not optimized
  DBuf<uint32_t> znode;             // unified node per node position
  DBuf<uint32_t> gptr, gslot;       // per node position: its (4 entry + k) slots, ascending
  DBuf<float4> X, Xt, grad;
  DBuf<float> lambda, cc, inv_avg, partial;
  DBuf<int32_t> conv, zid;          // per zone: convergence iteration; zones in launch order
  // host side
  std::vector<uint32_t> cvf_ptr, cvf_list, ovf_ptr, ovf_list;  // node -> incident faces
  std::vector<uint4> h_snodes;
  std::vector<HostZone> zones;
};

struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  xrt_status frame_status = XRT_OK;  // first failure of an eagerly recorded frame's host steps
  xrt_swift_params params{};
  bool started = false;
  float rec_dt = 0.0f;  // the substep dt the tile records' compliance terms were evaluated for
  bool graph_enabled = true;
  cudaGraphExec_t graph_exec = nullptr;
  bool graph_dirty = true;
  uint32_t frame_index = 0;
  uint32_t launches_per_frame = 0;
  bool targets_pending = false;
  uint32_t tile_vertices = 256;  // 0: plain per-color launches of a greedy coloring
  bool pdl = true;               // programmatic dependent launch of the substep kernels
  int num_sms = 1;               // multiprocessors of the device (persistent launches)
  DBuf<uint32_t> gen_counter;    // work-queue counters of the contact-generation kernels
  // batched form: instance i = cloth i + obstacle i (xrt_add_instance)
  bool instanced = false;
  struct HostInstance {
    uint32_t vertex_base, num_vertices;      // cloth
    uint32_t overtex_base, num_overtices;    // obstacle
    uint32_t oface_base, num_ofaces;
    float diameter;
  };
  std::vector<HostInstance> instances;
  std::vector<InstanceRec> h_inst;
  DBuf<InstanceRec> inst;
  DBuf<uint32_t> vinst;          // cloth vertex -> instance (batched form only)
  InstView inst_view() const {
    return InstView{(uint32_t)h_inst.size(), inst.p, vinst.p,
                    h_inst.empty() ? InstanceRec{} : h_inst[0]};
  }

  // host copies (setup)
  struct HostCloth {
    std::vector<float> mesh_pos;    // 3 per vertex, mesh space
    std::vector<uint32_t> tri;      // local
    uint32_t offset = 0;
  };
  std::vector<HostCloth> cloths;
  std::vector<float> h_x0;          // 3 per vertex, world
  std::vector<float> h_w;           // inverse mass
  std::vector<uint32_t> h_tri;      // global
  std::vector<uint32_t> h_edges;    // 2 per edge
  std::vector<float> h_rest, h_scomp;
  std::vector<uint32_t> h_bends;    // 4 per bend
  std::vector<float> h_theta, h_bcomp;
  std::vector<uint32_t> h_scolor, h_bcolor;
  std::vector<uint32_t> pending_colors[4];  // stretch, bend, FEM strain, FEM bending
  std::vector<uint32_t> h_lra_src, h_lra_tgt;
  std::vector<float> h_lra_rest;
  struct HostBinding {
    uint32_t cloth, iu, iv, iw;
    float u, v, w, L, stiffness;
  };
  std::vector<HostBinding> h_bind;
  float particle_diameter = 0.0f;
  std::vector<uint8_t> h_cfree;     // Node::is_free (false for pinned vertices)
  std::vector<float> h_omesh;       // obstacle positions at registration (mesh space)
  std::vector<float> h_ox0;         // obstacle world positions
  std::vector<uint32_t> h_otri;
  std::vector<uint32_t> h_ortri;
  uint32_t n_scolors = 0, n_bcolors = 0;
  std::vector<ColorRange> s_ranges, b_ranges;
  std::vector<uint32_t> s_perm, b_perm;  // execution slot -> original constraint index
  std::vector<uint32_t> s_local, b_local;  // footprint-local vertex slots (tiled schedules)
  setup::TileSchedule tmp_schedule;        // scratch of xrt_start

  // sizes
  uint32_t nv = 0, ne = 0, nf = 0, nb = 0, nl = 0, nbind = 0, onv = 0, onf = 0;

  // device: cloth
  DBuf<float4> x, x_alt, x0, v, n, x_init;
  DBuf<int4> tri;                    // a, b, c, 0
  DBuf<uint32_t> vf_ptr, vf_list;    // vertex -> (face << 2 | corner), ascending faces
  DBuf<int4> s_con;                  // execution order: i0, i1, rest bits, compliance bits
  DBuf<float> s_lambda;
  DBuf<int4> b_idx;                  // execution order
  DBuf<float2> b_tc;                 // theta, compliance
  TiledSet s_tiles, b_tiles;         // when on, s_con / b_idx hold footprint-local slots
  DBuf<uint32_t> lra_ptr, lra_src;   // per target vertex, slot order
  DBuf<float> lra_rest;
  DBuf<uint32_t> lra_l_src, lra_l_tgt;  // list order (slot-major), used when a slot is free
  DBuf<float> lra_l_rest;
  std::vector<ColorRange> lra_blocks;   // list range of each slot
  bool lra_by_target = true;
  DBuf<uint32_t> bind_ptr;           // per cloth vertex -> bindings
  DBuf<float4> bind_a;               // u, v, w, L
  DBuf<int4> bind_b;                 // iu, iv, iw, stiffness bits
  DBuf<uint2> edge;                  // original edge order (EE contacts)
  DBuf<uint32_t> ve_ptr, ve_list;    // vertex -> (edge << 1 | side), ascending edges
  // contacts
  DBuf<int> vf_idx, rt_idx;
  DBuf<float4> vf_qs, rt_qc;
  DBuf<float4> ee_a, ee_b, ee_c;     // {dist, p2}, {q2, s}, {fn, t}
  // particle hash
  DBuf<uint32_t> hash_key, hash_val, cell_start, cell_end, neighbors;
  DBuf<float> stage3;  // packed xyz staging of the C ABI's host copies
  DBuf<uint8_t> ee_vflag;  // per cloth vertex: an incident edge holds an EE contact (this pass)
  uint32_t vertex_block = 128;  // threads per block of the per-vertex substep kernels
  RadixSort hash_sorter;
  // obstacle
  DBuf<float4> ox0, ox, ox1, on, on1;
  DBuf<int4> otri;                   // a, b, c, r-triangle mask
  DBuf<uint32_t> ovf_ptr, ovf_list;
  Lbvh bvh;
  ProximityState prox;
  ImpactZoneState izone;
  SkinState skin;
  CacheState cache;
  FemState fem;
  DiffState diff;
  // host copies of the tile schedules (the adjoint regroups their slots by color)
  std::vector<int4> h_tile_meta[2];
  std::vector<uint32_t> h_tile_lofs[2];
  // error word
  DBuf<uint32_t> err;
  // per-phase profiling: 1 = eager frames, an event pair around every launch; 2 = the frame
  // captured as a graph with an event-record node pair around each phase group (a phase's
  // launches of one iteration) and replayed, so the launches inside a group keep their
  // programmatic dependent launch edges
  struct ProfEvent {
    cudaEvent_t a, b;
    int phase;
    uint32_t kernels;
    uint64_t units;
  };
  int profiling = 0;
  std::vector<ProfEvent> prof_events;
  size_t prof_used = 0;
  double prof_ms[16] = {};
  uint64_t prof_launches[16] = {};
  uint64_t prof_units[16] = {};
  uint32_t prof_frames = 0;

  void set_error(const std::string& m) { last_error = m; }
};

// Profile phases of the reverse pass (after the frame's, which api.cpp names).
enum AdjointPhase { kAdjReplay = 12, kAdjStretch, kAdjBend, kAdjVertex };

// CUDA-event pair around one launch when profiling eagerly (mode 1), or around a whole phase
// group inside a captured frame (mode 2).  A launch inside a group (`member`) is timed only in
// mode 1; a group scope only in mode 2; any other scope in both.
struct Timed {
  enum Kind { kLaunch, kMember, kGroup };
  Context& c;
  size_t idx = (size_t)-1;
  Timed(Context& ctx, int phase, uint32_t kernels, uint64_t units, Kind kind = kLaunch) : c(ctx) {
    if (!c.profiling) return;
    if (kind == kMember && c.profiling != 1) return;
    if (kind == kGroup && c.profiling != 2) return;
    if (c.prof_used == c.prof_events.size()) {
      Context::ProfEvent e{};
      cudaEventCreate(&e.a);
      cudaEventCreate(&e.b);
      c.prof_events.push_back(e);
    }
    idx = c.prof_used++;
    Context::ProfEvent& e = c.prof_events[idx];
    e.phase = phase;
    e.kernels = kernels;
    e.units = units;
    record(e.a);
  }
  ~Timed() {
    if (idx != (size_t)-1) record(c.prof_events[idx].b);
  }
  void record(cudaEvent_t e) {
    // under stream capture (mode 2) the record becomes an event-record node of the graph
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (c.profiling == 2 && cudaStreamIsCapturing(c.stream, &cs) == cudaSuccess &&
        cs == cudaStreamCaptureStatusActive)
      cudaEventRecordWithFlags(e, c.stream, cudaEventRecordExternal);
    else
      cudaEventRecord(e, c.stream);
  }
};

// Adds the recorded event pairs to the per-phase sums (one more frame).
inline void collect_profile(Context& c) {
  if (!c.profiling) return;
  cudaStreamSynchronize(c.stream);
  for (size_t i = 0; i < c.prof_used; ++i) {
    const Context::ProfEvent& e = c.prof_events[i];
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e.a, e.b);
    c.prof_ms[e.phase] += ms;
    c.prof_launches[e.phase] += e.kernels;
    c.prof_units[e.phase] += e.units;
  }
  c.prof_used = 0;
  c.prof_frames++;
}

// ---- kernels (solver.cu / contact.cu / hash.cu) ---------------------------------------------------
struct FrameConst {
  float dt;
  float gx, gy, gz;
  float damping;
  float relaxation;
  float lra_stretch;
  float friction;
  float particle_diameter;
};

// Per-frame constants from the parameters (dt = frame time / substeps).
inline FrameConst frame_const(const Context& c) {
  const xrt_swift_params& p = c.params;
  FrameConst k;
  k.dt = p.frame_time / (float)p.num_substeps;
  k.gx = p.gravity[0];
  k.gy = p.gravity[1];
  k.gz = p.gravity[2];
  k.damping = p.damping;
  k.relaxation = p.relaxation_factor;
  k.lra_stretch = p.long_range_stretchiness;
  k.friction = p.friction;
  k.particle_diameter = c.particle_diameter;
  return k;
}

void launch_predict(Context& c, const FrameConst& k);
void launch_finalize_predict(Context& c, const FrameConst& k, bool predict_next, bool normals);
void launch_stretch(Context& c, const FrameConst& k, ColorRange r, bool reset_lambda);
void launch_bend(Context& c, const FrameConst& k, ColorRange r);
cudaError_t configure_tile_kernels(size_t max_smem_bytes);
// Raises a kernel's dynamic shared-memory limit on the current device to at least `bytes`.  The
// limit is process-wide, so it only ever grows (a context with smaller tiles must not lower it
// under another's launches).
cudaError_t raise_smem(const void* kern, size_t bytes);
// FEM fabric (fem.cu): slot-ordered records after the schedules are built; the launch shapes;
// one iteration's strain and bending launches (profiled under the given phases).
cudaError_t fem_upload(Context& c);
cudaError_t fem_configure(Context& c);
void launch_fem(Context& c, const FrameConst& k, bool reset_lambda, int phase_strain,
                int phase_bend);
void fem_release(Context& c);
size_t tile_smem_bytes(const TiledSet& T, size_t record_bytes);
// the forward stretch / bend kernels (bend: lane pairs or one lane)
size_t tile_smem_fwd(const TiledSet& T, bool stretch, bool whole);
// float4 -> packed xyz (12 B per element) and back (w set to `w`), for host copies.
void launch_pack_xyz(const float4* in, float* out, uint32_t n, cudaStream_t s);
void launch_unpack_xyz(const float* in, float4* out, uint32_t n, float w, cudaStream_t s);
// Sets T.block (256 / 512 threads) and T.resident; after configure_tile_kernels.
cudaError_t choose_tile_block(TiledSet& T, bool bend);
// tile-local Gauss-Seidel: all tiles of one tile color (range of executed tiles)
// tape_x / tape_l (the adjoint's recorded replay): every projection's input positions (and
// multiplier) are also written there, by execution slot.
void launch_stretch_tiles(Context& c, const FrameConst& k, ColorRange tiles, bool reset_lambda,
                          float4* tape_x = nullptr, float* tape_l = nullptr);
void launch_bend_tiles(Context& c, const FrameConst& k, ColorRange tiles,
                       float4* tape_x = nullptr);
void launch_lra(Context& c, const FrameConst& k);
// Iteration tail, each launch reads x and writes x_alt (caller swaps):
// LRA with all slots pinned (else launch_lra runs before) + VF solve ...
// `tape` (the adjoint's recorded replay): each vertex's input position is also written there;
// `tape_cnt` (launch_ee, with `tape`): each vertex's count of applied EE contacts.
void launch_stage(Context& c, const FrameConst& k, bool lra, bool contacts,
                  float4* tape = nullptr);
// ... then EE solve + ApplyDeltas + binding.
void launch_ee(Context& c, const FrameConst& k, bool contacts, bool bindings,
               float4* tape = nullptr, float* tape_cnt = nullptr);
void launch_obstacle_pass(Context& c, int step, int num_steps);
void launch_generate_contacts(Context& c);
void launch_obstacle_commit(Context& c);
// Obstacle targets from the joint transforms (skin.cu), when skinning is on.
void launch_skin(Context& c);
// Frame cache (cache.cu): records the frame just issued, when recording; frees the store.
cudaError_t cache_frame(Context& c);
void cache_release(Context& c);
void launch_vertex_normals(const float4* x, const int4* tri, const uint32_t* ptr,
                           const uint32_t* list, float4* out, uint32_t nv, cudaStream_t s);
void launch_hash(Context& c);
void launch_collide(Context& c, const FrameConst& k);  // reads x, writes x_alt; caller swaps
void launch_prims_obstacle(Context& c, float tol);

// Copies a built LBVH to host arrays in the export layout of include/xrt.h (api.cpp).
xrt_status export_lbvh(Lbvh& b, cudaStream_t s, std::string& err, uint32_t* morton, uint32_t* objs,
                       uint32_t* nodes, float* aabbs, int32_t* iesc, int32_t* eesc, int32_t* unique);

// ---- Quality-mode self contact (proximity.cu) ----------------------------------------------------
// ---- adjoint (diff.cu) ---------------------------------------------------------------------------
xrt_status diff_prepare(Context& c);     // schedule, tape and adjoint buffers
void diff_checkpoint(Context& c);        // state at the start of the next frame
// The frame's launches on the current state (api.cpp): profiled, replayed graph or eager.
xrt_status frame_core(Context& c, bool eager);
// Reverse pass over the checkpointed frames; host outputs may be null (sizes: E, B, V, 3V, 3V).
xrt_status diff_backward(Context& c, const float* dLdx, const float* dLdv, float* d_compliance,
                         float* d_bend_compliance, float* d_mass, float* d_velocity,
                         float* d_position);
void diff_release(Context& c);

xrt_status prox_prepare(Context& c);  // uploads the unified topology once (api_contact.cpp)
void launch_cloth_bvh_build(Context& c);
void launch_update_ccd(Lbvh& b, const float4* x, const float4* x0, const int4* tri, cudaStream_t s,
                       uint32_t* err);
cudaError_t prox_update_pairs(Context& c, float thickness);
cudaError_t prox_face_pairs(Context& c, const Lbvh& cloth, const Lbvh& obstacle, float thickness,
                            bool self_first = false);
// ImminentRepulsion::UpdateProximity + Generate (once per frame) and Solve (per iteration)
cudaError_t prox_imminent_generate(Context& c);
// v = (x - x0) / dt of n nodes (UpdateVelocity_Kernel, SetupObstacleNode_Kernel)
void launch_node_velocity(const float4* x, const float4* x0, float4* v, uint32_t n, float dt,
                          cudaStream_t s);
void prox_imminent_solve(Context& c, float thickness, float relaxation, float dt);
// inclusive scan of n counts (multi-block); total[0] = sum
cudaError_t scan_inclusive(ScanScratch& w, const uint32_t* in, uint32_t* out, uint32_t n,
                           uint32_t* total, cudaStream_t s);
void prox_solve(Context& c, float thickness, float relaxation);
cudaError_t prox_check_impacts(Context& c, float thickness);
// prims with ccd boxes: v_k = x0[idx_k] + tol * n[idx_k], pred_k = x[idx_k] + tol * n[idx_k]
void launch_prims_ccd(Lbvh& b, const float4* x, const float4* x0, const float4* nrm,
                      const int4* tri, uint32_t nf, float tol, cudaStream_t s);
// ImpactZoneOptimization::CollisionStep on the current cloth and obstacle x0 -> x (impact.cu)
xrt_status collision_step(Context& c, float obstacle_mass, float thickness, xrt_collision_stats* out);
void izone_release(Context& c);

}  // namespace xrt

// The opaque handle of include/xrt.h.
struct xrt_ctx {
  xrt::Context c;
};
