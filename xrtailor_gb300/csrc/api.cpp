// api.cpp — the C ABI (include/xrt.h): setup, the per-frame launch sequence of
// ClothSolverBase::SimulateSwift (src/pipeline/base/ClothSolverBase.cpp:171-261), CUDA-graph
// replay of frames, state and parity exports, and the standalone LBVH.
//
// Every entry point returns a status and never exits; CUDA failures become XRT_ERR_CUDA with the
// CUDA message in xrt_last_error.  The product path has no CPU fallback: without a device of the
// architecture this library was compiled for, xrt_create fails with XRT_ERR_NO_DEVICE.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/xrt.h"
#include "context.h"
#include "setup.h"

using xrt::collect_profile;
using xrt::ColorRange;
using xrt::Context;
using xrt::DBuf;
using xrt::Timed;


struct xrt_lbvh {
  int device = 0;
  cudaStream_t stream = nullptr;
  xrt::Lbvh b;
  DBuf<float> staging;
  DBuf<uint32_t> err;
  std::string last_error;
};

namespace {

xrt_status check_device(int device, std::string& why) {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    why = std::string("no CUDA device: ") + cudaGetErrorString(e);
    return XRT_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= count) {
    why = "device index out of range";
    return XRT_ERR_NO_DEVICE;
  }
  cudaFuncAttributes attr;
  (void)attr;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
    why = "cudaGetDeviceProperties failed";
    return XRT_ERR_NO_DEVICE;
  }
  if (prop.major != 10 || prop.minor != 3) {
    why = "this library is built for sm_103a (GB300); device is sm_" + std::to_string(prop.major) +
          std::to_string(prop.minor);
    return XRT_ERR_NO_DEVICE;
  }
  return XRT_OK;
}

template <typename T>
cudaError_t upload(DBuf<T>& d, const std::vector<T>& h, cudaStream_t s) {
  cudaError_t e = d.reserve(h.empty() ? 1 : h.size());
  if (e != cudaSuccess || h.empty()) return e;
  return cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

std::vector<float4> to_f4(const std::vector<float>& xyz, const std::vector<float>* w) {
  const size_t n = xyz.size() / 3;
  std::vector<float4> out(n);
  for (size_t i = 0; i < n; ++i)
    out[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], w ? (*w)[i] : 0.0f);
  return out;
}

xrt_status validate_params(const xrt_swift_params& p, std::string& why) {
  if (p.num_substeps < 1) why = "num_substeps must be >= 1";
  else if (p.num_iterations < 1) why = "num_iterations must be >= 1";
  else if (p.num_collision_passes < 1) why = "num_collision_passes must be >= 1";
  else if (p.num_collision_passes > p.num_substeps * p.num_iterations)
    why = "num_collision_passes exceeds num_substeps * num_iterations (the reference divides by zero)";
  else if (p.inter_leaved_hash < 1) why = "inter_leaved_hash must be >= 1";
  else if (p.max_neighbor_size < 1) why = "max_neighbor_size must be >= 1";
  else if (!(p.frame_time > 0.0f)) why = "frame_time must be > 0";
  else if (!(p.hash_cell_size > 0.0f)) why = "hash_cell_size must be > 0";
  else if (p.impact_zone && !(p.impact_zone_obstacle_mass > 0.0f))
    why = "impact_zone_obstacle_mass must be > 0";
  else if (p.impact_zone && !(p.impact_zone_thickness >= 0.0f))
    why = "impact_zone_thickness must be >= 0";
  else return XRT_OK;
  return XRT_ERR_INVALID_CONFIG;
}

enum Phase {
  kPredict = 0, kHash, kCollide, kBvhBuild, kObstaclePass, kGenerate, kStretch, kBend, kLra,
  kVfSolve, kEeApply, kObstacleCommit
};
const char* const kPhaseNames[XRT_NUM_PHASES] = {
    "predict_finalize", "hash", "collide", "bvh_build", "obstacle_pass", "generate",
    "stretch", "bend", "lra", "vf_solve", "ee_apply", "obstacle_commit",
    "adjoint_replay", "adjoint_stretch", "adjoint_bend", "adjoint_vertex"};
static_assert(xrt::kAdjReplay == 12 && xrt::kAdjVertex == XRT_NUM_PHASES - 1,
              "adjoint phases follow the frame's");

// The launch sequence of one frame (ClothSolverBase::SimulateSwift, ClothSolverBase.cpp:171-261).
void record_frame(Context& c) {
  const xrt_swift_params& p = c.params;
  const xrt::FrameConst k = xrt::frame_const(c);
  float4* const x_start = c.x.p;
  int swaps = 0;
  auto swap_x = [&]() {
    std::swap(c.x.p, c.x_alt.p);
    ++swaps;
  };
  const bool obstacle_updated = p.update_obstacle_animation && c.onf > 0;
  if (obstacle_updated) {  // UpdateObstacleAnimationFrame: UpdateData(tol 0) + Construct()
    Timed t(c, kBvhBuild, 19, c.onf);
    xrt::launch_prims_obstacle(c, 0.0f);
    c.bvh.construct(0.0f, c.stream, c.err.p);
  }
  const bool has_obstacle = c.onf > 0;
  const bool bindings = c.nbind > 0;
  const bool repulsion = p.pbd_repulsion != 0;
  const bool imminent = p.imminent_repulsion != 0;
  if (repulsion || imminent) {  // SimulateQuality: cloth LBVH per frame, the imminent
                                // quadratures, obstacle Update(ccd) (ClothSolverBase.cpp:276-293)
    xrt::launch_cloth_bvh_build(c);
    if (imminent) {
      const cudaError_t e = xrt::prox_imminent_generate(c);
      if (e != cudaSuccess && c.frame_status == XRT_OK) {
        c.set_error(std::string("imminent repulsion: ") + cudaGetErrorString(e));
        c.frame_status = XRT_ERR_CUDA;
      }
    }
    if (has_obstacle) xrt::launch_update_ccd(c.bvh, c.ox.p, c.ox0.p, c.otri.p, c.stream, c.err.p);
  }
  const int frequency = (p.num_substeps * p.num_iterations) / p.num_collision_passes;
  int cnt = 0;
  for (int s = 0; s < p.num_substeps; ++s) {
    if (s == 0) {
      Timed t(c, kPredict, 1, c.nv);
      xrt::launch_predict(c, k);
    }
    if (p.enable_self_collision && s % p.inter_leaved_hash == 0) {
      Timed t(c, kHash, 13, c.nv);
      xrt::launch_hash(c);
    }
    for (int it = 0; it < p.num_iterations; ++it) {
      if (imminent)  // ImminentRepulsion::Solve first (ClothSolverBase.cpp:296-301)
        xrt::prox_imminent_solve(c, p.imminent_thickness, p.repulsion_relaxation, k.dt);
      if (repulsion) {  // PBD repulsion at the start of the iteration (ClothSolverBase.cpp:303-313)
        if (it % 10 == 0) xrt::prox_update_pairs(c, 1e-6f);
        xrt::prox_solve(c, p.pbd_thickness, p.repulsion_relaxation);
      }
      if (p.enable_self_collision) {
        {
          Timed t(c, kCollide, 1, c.nv);
          xrt::launch_collide(c, k);
        }
        swap_x();
      }
      const int current = s * p.num_iterations + it;
      if (current % frequency == 0) {
        if (obstacle_updated) {
          Timed t(c, kObstaclePass, 2, c.onv);
          xrt::launch_obstacle_pass(c, cnt, p.num_collision_passes);
        }
        if (has_obstacle) {
          Timed t(c, kGenerate, 2, c.nv + c.ne);
          xrt::launch_generate_contacts(c);
        }
        cnt++;
      }
      if (c.fem.on) {  // FEM fabric: strain colors, then isometric bending colors (profiled as
                       // the stretch and bend phases)
        xrt::launch_fem(c, k, it == 0, kStretch, kBend);
      } else if (c.s_tiles.on) {
        Timed g(c, kStretch, (uint32_t)c.s_tiles.tile_colors.size(), c.ne, Timed::kGroup);
        for (size_t tc = 0; tc < c.s_tiles.tile_colors.size(); ++tc) {
          Timed t(c, kStretch, 1, c.s_tiles.tile_color_cons[tc], Timed::kMember);
          xrt::launch_stretch_tiles(c, k, c.s_tiles.tile_colors[tc], it == 0);
        }
      } else {
        Timed g(c, kStretch, (uint32_t)c.s_ranges.size(), c.ne, Timed::kGroup);
        for (const ColorRange& r : c.s_ranges) {
          Timed t(c, kStretch, 1, r.end - r.begin, Timed::kMember);
          xrt::launch_stretch(c, k, r, it == 0);
        }
      }
      if (p.solve_bending && !c.fem.on) {
        if (c.b_tiles.on) {
          Timed g(c, kBend, (uint32_t)c.b_tiles.tile_colors.size(), c.nb, Timed::kGroup);
          for (size_t tc = 0; tc < c.b_tiles.tile_colors.size(); ++tc) {
            Timed t(c, kBend, 1, c.b_tiles.tile_color_cons[tc], Timed::kMember);
            xrt::launch_bend_tiles(c, k, c.b_tiles.tile_colors[tc]);
          }
        } else {
          Timed g(c, kBend, (uint32_t)c.b_ranges.size(), c.nb, Timed::kGroup);
          for (const ColorRange& r : c.b_ranges) {
            Timed t(c, kBend, 1, r.end - r.begin, Timed::kMember);
            xrt::launch_bend(c, k, r);
          }
        }
      }
      // LRA and VF solve: one per-vertex Jacobi launch (LRA runs on its own first when a slot
      // vertex is free, since slot positions then change during the phase); then EE solve +
      // ApplyDeltas + binding.
      const bool lra = p.geodesic_lra && c.nl;
      if (lra && !c.lra_by_target) {
        Timed t(c, kLra, (uint32_t)c.lra_blocks.size(), c.nl);
        xrt::launch_lra(c, k);
      }
      const bool lra_fused = lra && c.lra_by_target;
      if (lra_fused || has_obstacle) {
        {
          Timed t(c, has_obstacle ? kVfSolve : kLra, 1, c.nv);
          xrt::launch_stage(c, k, lra_fused, has_obstacle);
        }
        swap_x();
      }
      if (has_obstacle || bindings) {
        {
          Timed t(c, kEeApply, 1, c.nv);
          xrt::launch_ee(c, k, has_obstacle, bindings);
        }
        swap_x();
      }
    }
    if (p.impact_zone) {  // CollisionStep after the iterations (ClothSolverBase.cpp:329-336)
      const xrt_status r = xrt::collision_step(c, p.impact_zone_obstacle_mass,
                                               p.impact_zone_thickness, nullptr);
      if (r != XRT_OK && c.frame_status == XRT_OK) c.frame_status = r;
    }
    const bool last = s + 1 == p.num_substeps;
    Timed t(c, kPredict, 1, c.nv);
    xrt::launch_finalize_predict(c, k, !last, last);
  }
  if (c.onv > 0) {
    Timed t(c, kObstacleCommit, 1, c.onv);
    xrt::launch_obstacle_commit(c);
  }
  if (swaps & 1) {  // keep the frame's state in the buffer a replayed graph starts from
    cudaMemcpyAsync(x_start, c.x.p, sizeof(float4) * c.nv, cudaMemcpyDeviceToDevice, c.stream);
    std::swap(c.x.p, c.x_alt.p);
  }
}

xrt_status capture_frame(Context& c) {
  if (c.graph_exec) {
    cudaGraphExecDestroy(c.graph_exec);
    c.graph_exec = nullptr;
  }
  cudaGraph_t graph = nullptr;
  XRT_CUDA(&c, cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
  record_frame(c);
  cudaError_t e = cudaStreamEndCapture(c.stream, &graph);
  if (e != cudaSuccess) {
    c.set_error(std::string("frame capture failed: ") + cudaGetErrorString(e));
    return XRT_ERR_CUDA;
  }
  size_t num_nodes = 0;
  cudaGraphGetNodes(graph, nullptr, &num_nodes);
  std::vector<cudaGraphNode_t> nodes(num_nodes);
  if (num_nodes) cudaGraphGetNodes(graph, nodes.data(), &num_nodes);
  uint32_t kernels = 0;
  for (auto nd : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kernels;
  }
  c.launches_per_frame = kernels;
  e = cudaGraphInstantiate(&c.graph_exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    c.set_error(std::string("graph instantiate failed: ") + cudaGetErrorString(e));
    c.graph_exec = nullptr;
    return XRT_ERR_CUDA;
  }
  c.graph_dirty = false;
  return XRT_OK;
}

// One frame captured with the profiling events of mode 2 as event-record nodes, replayed once
// and discarded; the frame graph of normal stepping is left as it is.
xrt_status profile_frame_graph(Context& c) {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  XRT_CUDA(&c, cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
  record_frame(c);
  cudaError_t e = cudaStreamEndCapture(c.stream, &graph);
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (exec) cudaGraphExecDestroy(exec);
  if (e != cudaSuccess) {
    c.prof_used = 0;
    c.set_error(std::string("profiled frame graph failed: ") + cudaGetErrorString(e));
    return XRT_ERR_CUDA;
  }
  collect_profile(c);
  return XRT_OK;
}

xrt_status require_started(Context& c) {
  if (!c.started) {
    c.set_error("call xrt_start first");
    return XRT_ERR_STATE;
  }
  return XRT_OK;
}

xrt_status read_f4(Context& c, const DBuf<float4>& d, uint32_t n, float* out) {
  if (!out) {
    c.set_error("null output pointer");
    return XRT_ERR_INVALID_ARGUMENT;
  }
  if (n) {  // packed on the device, then one copy straight into the caller's buffer
    XRT_CUDA(&c, c.stage3.reserve(3 * (size_t)n));
    xrt::launch_pack_xyz(d.p, c.stage3.p, n, c.stream);
    XRT_CUDA(&c, cudaMemcpyAsync(out, c.stage3.p, 3 * sizeof(float) * (size_t)n,
                                 cudaMemcpyDeviceToHost, c.stream));
    XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  }
  return XRT_OK;
}

}  // namespace

extern "C" {

xrt_status xrt_get_version(int32_t* v) {
  if (!v) return XRT_ERR_INVALID_ARGUMENT;
  *v = XRT_API_VERSION;
  return XRT_OK;
}

xrt_status xrt_default_params(xrt_swift_params* p) {
  if (!p) return XRT_ERR_INVALID_ARGUMENT;
  std::memset(p, 0, sizeof(*p));
  p->num_substeps = 1;
  p->num_iterations = 200;
  p->max_speed = 1e6f;
  p->gravity[0] = 0.0f;
  p->gravity[1] = -9.8f;
  p->gravity[2] = 0.0f;
  p->damping = 0.98f;
  p->stretch_compliance = 0.0f;
  p->bend_compliance = 1e2f;
  p->relaxation_factor = 0.25f;
  p->long_range_stretchiness = 1.1f;
  p->geodesic_lra = 1;
  p->solve_bending = 1;
  p->num_collision_passes = 10;
  p->sdf_collision_margin = 1e-2f;
  p->bvh_tolerance = 0.003f;
  p->friction = 0.1f;
  p->max_neighbor_size = 64;
  p->inter_leaved_hash = 3;
  p->enable_self_collision = 1;
  p->particle_diameter = 1.3f;
  p->hash_cell_size = 1.5f;
  p->frame_time = 1.0f / 60.0f;
  p->update_obstacle_animation = 1;
  p->pbd_repulsion = 0;
  p->pbd_thickness = 1e-4f;         // RepulsionSettings (config/Base.hpp:102-108)
  p->repulsion_relaxation = 0.25f;
  p->impact_zone = 0;
  p->impact_zone_obstacle_mass = 1e3f;  // ImpactZoneSettings (config/Base.hpp:115-118)
  p->impact_zone_thickness = 1e-4f;
  p->imminent_repulsion = 0;
  p->imminent_thickness = 1e-3f;        // RepulsionSettings (config/Base.hpp:102-108)
  return XRT_OK;
}

xrt_status xrt_create(xrt_ctx** out, int32_t device) {
  if (!out) return XRT_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  std::string why;
  xrt_status st = check_device(device, why);
  if (st != XRT_OK) return st;
  xrt_ctx* h = new xrt_ctx();
  Context& c = h->c;
  c.device = device;
  xrt_default_params(&c.params);
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess ||
      c.err.reserve(1) != cudaSuccess || cudaMemset(c.err.p, 0, sizeof(uint32_t)) != cudaSuccess ||
      c.gen_counter.reserve(4) != cudaSuccess ||
      cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
    delete h;
    return XRT_ERR_CUDA;
  }
  *out = h;
  return XRT_OK;
}

xrt_status xrt_destroy(xrt_ctx* h) {
  if (!h) return XRT_OK;
  Context& c = h->c;
  cudaSetDevice(c.device);
  if (c.stream) cudaStreamSynchronize(c.stream);
  if (c.graph_exec) cudaGraphExecDestroy(c.graph_exec);
  xrt::diff_release(c);
  for (auto& e : c.prof_events) {
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  DBuf<float4>* f4[] = {&c.x, &c.x_alt, &c.x0, &c.v, &c.n, &c.x_init, &c.bind_a, &c.vf_qs,
                        &c.rt_qc, &c.ee_a, &c.ee_b, &c.ee_c, &c.ox0, &c.ox, &c.ox1, &c.on, &c.on1};
  for (auto* b : f4) b->release();
  DBuf<uint32_t>* u[] = {&c.vf_ptr, &c.vf_list, &c.lra_ptr, &c.lra_src, &c.lra_l_src, &c.lra_l_tgt,
                         &c.bind_ptr, &c.ve_ptr, &c.ve_list, &c.hash_key, &c.hash_val,
                         &c.cell_start, &c.cell_end, &c.neighbors, &c.ovf_ptr,
                         &c.ovf_list, &c.err};
  for (auto* b : u) b->release();
  c.tri.release(); c.s_con.release(); c.b_idx.release(); c.bind_b.release(); c.otri.release();
  c.s_lambda.release(); c.lra_rest.release(); c.lra_l_rest.release(); c.b_tc.release();
  c.stage3.release();
  c.ee_vflag.release();
  c.edge.release(); c.vf_idx.release(); c.rt_idx.release();
  c.hash_sorter.keys_tmp.release(); c.hash_sorter.vals_tmp.release(); c.hash_sorter.hist.release();
  c.hash_sorter.sums.release();
  c.bvh.release();
  c.inst.release();
  c.vinst.release();
  c.gen_counter.release();
  c.skin.rest.release(); c.skin.outer.release(); c.skin.joint.release();
  c.skin.weight.release(); c.skin.transforms.release();
  xrt::cache_release(c);
  xrt::fem_release(c);
  xrt::izone_release(c);
  for (xrt::TiledSet* t : {&c.s_tiles, &c.b_tiles}) {
    t->foot.release();
    t->meta.release();
    t->lofs.release();
  }
  xrt::ProximityState& P = c.prox;
  P.cbvh.release();
  P.face.release(); P.fedge.release(); P.fn0.release(); P.edge.release(); P.eadj.release();
  P.cfree.release(); P.counts.release(); P.incl.release(); P.total.release(); P.pairs.release();
  P.scan.sums.release(); P.scan.incl.release();
  P.qnodes.release(); P.qbary.release(); P.ov.release();
  P.deltas.release(); P.rcounts.release(); P.imp_t.release(); P.imp_w.release(); P.imp_n.release();
  P.imp_nodes.release();
  if (c.stream) cudaStreamDestroy(c.stream);
  delete h;
  return XRT_OK;
}

const char* xrt_last_error(const xrt_ctx* h) { return h ? h->c.last_error.c_str() : "null context"; }

static xrt_status upload_constraints(Context& c);

xrt_status xrt_set_params(xrt_ctx* h, const xrt_swift_params* p) {
  if (!h || !p) return XRT_ERR_INVALID_ARGUMENT;
  std::string why;
  if (validate_params(*p, why) != XRT_OK) {
    h->c.set_error(why);
    return XRT_ERR_INVALID_CONFIG;
  }
  Context& c = h->c;
  c.params = *p;
  c.graph_dirty = true;
  // the tile records hold compliance terms of the substep dt: a new dt re-evaluates them
  if (c.started && (c.s_tiles.on || c.b_tiles.on) && xrt::frame_const(c).dt != c.rec_dt) {
    cudaSetDevice(c.device);
    XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
    return upload_constraints(c);
  }
  return XRT_OK;
}

}  // extern "C"

// Appends one cloth (validated first; nothing changes on error).  Binding obstacle indices are
// offset by `bind_base` (the instance's first obstacle vertex in the batched form).
static xrt_status add_cloth_impl(Context& c, const xrt_cloth_desc* d, uint32_t bind_base,
                                 uint32_t bind_limit, int32_t* out_offset) {
  if (d->num_vertices == 0 || d->num_triangles == 0) {
    c.set_error("empty cloth mesh");
    return XRT_ERR_INVALID_MESH;
  }
  const uint64_t total = (uint64_t)c.h_w.size() + d->num_vertices;
  if (total >= (1ull << 30)) {
    c.set_error("vertex count exceeds 2^30");
    return XRT_ERR_NODE_CAPACITY;
  }
  for (uint64_t k = 0; k < 3ull * d->num_triangles; ++k)
    if (d->triangles[k] >= d->num_vertices) {
      c.set_error("triangle index out of range");
      return XRT_ERR_INVALID_MESH;
    }
  auto check_list = [&](const uint32_t* l, uint32_t n, const char* what) {
    if (n && !l) return std::string(what) + " pointer is null";
    for (uint32_t i = 0; i < n; ++i)
      if (l[i] >= d->num_vertices) return std::string(what) + " index out of range";
    return std::string();
  };
  std::string why = check_list(d->fixed_indices, d->num_fixed, "fixed");
  if (why.empty()) why = check_list(d->attached_indices, d->num_attached, "attached");
  if (why.empty()) why = check_list(d->binded_indices, d->num_binded, "binded");
  if (why.empty() && d->num_binded && (!d->bind_obstacle_tri || !d->bind_barycentric))
    why = "binding needs bind_obstacle_tri and bind_barycentric";
  for (uint64_t k = 0; why.empty() && k < 3ull * d->num_binded; ++k)
    if (d->bind_obstacle_tri[k] >= bind_limit) why = "binding refers to a missing obstacle vertex";
  if (!why.empty()) {
    c.set_error(why);
    return XRT_ERR_INVALID_MESH;
  }
  Context::HostCloth cl;
  cl.offset = (uint32_t)c.h_w.size();
  cl.mesh_pos.assign(d->positions, d->positions + 3 * (size_t)d->num_vertices);
  cl.tri.assign(d->triangles, d->triangles + 3 * (size_t)d->num_triangles);
  std::vector<xrt::setup::V3> pos(d->num_vertices);
  for (uint32_t i = 0; i < d->num_vertices; ++i)
    pos[i] = xrt::setup::V3{d->positions[3 * i], d->positions[3 * i + 1], d->positions[3 * i + 2]};
  // InitializePositions (ClothSolverHelper.cu:113-123): x0 = model * p
  for (uint32_t i = 0; i < d->num_vertices; ++i) {
    xrt::setup::V3 q = pos[i];
    if (d->model_matrix) q = xrt::setup::transform_point(d->model_matrix, q);
    c.h_x0.push_back(q.x);
    c.h_x0.push_back(q.y);
    c.h_x0.push_back(q.z);
    c.h_w.push_back(1.0f);  // PhysicsMeshHelper.cu:139: free nodes have inverse mass 1
  }
  for (uint32_t k = 0; k < 3 * d->num_triangles; ++k) c.h_tri.push_back(d->triangles[k] + cl.offset);
  c.h_cfree.resize(c.h_w.size(), 1);
  for (uint32_t i = 0; i < d->num_fixed; ++i) {  // SetInvMass(0) + SetFree(false)
    c.h_w[cl.offset + d->fixed_indices[i]] = 0.0f;
    c.h_cfree[cl.offset + d->fixed_indices[i]] = 0;
  }
  std::vector<uint32_t> e;
  std::vector<std::vector<uint32_t>> ef;
  xrt::setup::build_edges(cl.tri, e, ef);
  for (size_t k = 0; k < e.size() / 2; ++k) {
    c.h_edges.push_back(e[2 * k] + cl.offset);
    c.h_edges.push_back(e[2 * k + 1] + cl.offset);
    c.h_rest.push_back(xrt::setup::length(xrt::setup::sub(pos[e[2 * k]], pos[e[2 * k + 1]])));
    c.h_scomp.push_back(c.params.stretch_compliance);
  }
  if (c.params.solve_bending) {
    std::vector<uint32_t> b;
    std::vector<float> th;
    xrt::setup::build_bends(pos, cl.tri, e, ef, cl.offset, b, th);
    c.h_bends.insert(c.h_bends.end(), b.begin(), b.end());
    c.h_theta.insert(c.h_theta.end(), th.begin(), th.end());
    c.h_bcomp.insert(c.h_bcomp.end(), th.size(), c.params.bend_compliance);
  }
  if (d->num_attached > 0 && c.params.geodesic_lra) {  // ClothObjectBase.cpp:79-93
    std::vector<std::vector<uint32_t>> adj(d->num_vertices);
    for (size_t k = 0; k < e.size() / 2; ++k) {
      adj[e[2 * k]].push_back(e[2 * k + 1]);
      adj[e[2 * k + 1]].push_back(e[2 * k]);
    }
    for (auto& a : adj) std::sort(a.begin(), a.end());
    for (uint32_t s = 0; s < d->num_attached; ++s) {
      const uint32_t slot = d->attached_indices[s];
      const std::vector<float> dist = xrt::setup::geodesic(pos, adj, slot);
      for (uint32_t v = 0; v < d->num_vertices; ++v) {
        c.h_lra_src.push_back(slot + cl.offset);
        c.h_lra_tgt.push_back(v + cl.offset);
        c.h_lra_rest.push_back(dist[v]);
      }
    }
  }
  for (uint32_t i = 0; i < d->num_binded; ++i) {
    Context::HostBinding b;
    b.cloth = d->binded_indices[i] + cl.offset;
    b.iu = d->bind_obstacle_tri[3 * i] + bind_base;
    b.iv = d->bind_obstacle_tri[3 * i + 1] + bind_base;
    b.iw = d->bind_obstacle_tri[3 * i + 2] + bind_base;
    b.u = d->bind_barycentric[3 * i];
    b.v = d->bind_barycentric[3 * i + 1];
    b.w = d->bind_barycentric[3 * i + 2];
    b.L = d->bind_distances ? d->bind_distances[i] : 0.0f;
    b.stiffness = d->bind_stiffnesses ? d->bind_stiffnesses[i] : 1.0f;
    c.h_bind.push_back(b);
  }
  // universal/ClothObject.hpp:36-37: first edge length x PARTICLE_DIAMETER; the last cloth wins
  if (d->particle_diameter > 0.0f)
    c.particle_diameter = d->particle_diameter;
  else
    c.particle_diameter =
        xrt::setup::length(xrt::setup::sub(pos[cl.tri[0]], pos[cl.tri[1]])) * c.params.particle_diameter;
  if (out_offset) *out_offset = (int32_t)cl.offset;
  c.cloths.push_back(std::move(cl));
  return XRT_OK;
}

static xrt_status check_obstacle(Context& c, const xrt_obstacle_desc* d) {
  for (uint64_t k = 0; k < 3ull * d->num_triangles; ++k)
    if (d->triangles[k] >= d->num_vertices) {
      c.set_error("obstacle triangle index out of range");
      return XRT_ERR_INVALID_MESH;
    }
  return XRT_OK;
}

static void add_obstacle_impl(Context& c, const xrt_obstacle_desc* d, int32_t* out_offset) {
  const uint32_t off = (uint32_t)(c.h_ox0.size() / 3);
  for (uint32_t i = 0; i < d->num_vertices; ++i) {
    xrt::setup::V3 q{d->positions[3 * i], d->positions[3 * i + 1], d->positions[3 * i + 2]};
    c.h_omesh.push_back(q.x);
    c.h_omesh.push_back(q.y);
    c.h_omesh.push_back(q.z);
    if (d->model_matrix) q = xrt::setup::transform_point(d->model_matrix, q);
    c.h_ox0.push_back(q.x);
    c.h_ox0.push_back(q.y);
    c.h_ox0.push_back(q.z);
  }
  for (uint64_t k = 0; k < 3ull * d->num_triangles; ++k) c.h_otri.push_back(d->triangles[k] + off);
  if (out_offset) *out_offset = (int32_t)off;
}

extern "C" {

xrt_status xrt_add_cloth(xrt_ctx* h, const xrt_cloth_desc* d, int32_t* out_offset) {
  if (!h || !d || !d->positions || !d->triangles) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (c.started) {
    c.set_error("xrt_add_cloth after xrt_start");
    return XRT_ERR_STATE;
  }
  if (c.instanced) {
    c.set_error("xrt_add_cloth in a batched context (use xrt_add_instance)");
    return XRT_ERR_STATE;
  }
  // bindings may name obstacle vertices added later; xrt_start checks them
  return add_cloth_impl(c, d, 0, 0xFFFFFFFFu, out_offset);
}

xrt_status xrt_add_obstacle(xrt_ctx* h, const xrt_obstacle_desc* d, int32_t* out_offset) {
  if (!h || !d || !d->positions || !d->triangles) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (c.started) {
    c.set_error("xrt_add_obstacle after xrt_start");
    return XRT_ERR_STATE;
  }
  if (c.instanced) {
    c.set_error("xrt_add_obstacle in a batched context (use xrt_add_instance)");
    return XRT_ERR_STATE;
  }
  const xrt_status st = check_obstacle(c, d);
  if (st != XRT_OK) return st;
  add_obstacle_impl(c, d, out_offset);
  return XRT_OK;
}

xrt_status xrt_add_instance(xrt_ctx* h, const xrt_cloth_desc* cloth,
                            const xrt_obstacle_desc* obstacle, int32_t* out_instance) {
  if (!h || !cloth || !cloth->positions || !cloth->triangles) return XRT_ERR_INVALID_ARGUMENT;
  if (obstacle && (!obstacle->positions || !obstacle->triangles)) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (c.started) {
    c.set_error("xrt_add_instance after xrt_start");
    return XRT_ERR_STATE;
  }
  if (!c.instanced && (!c.cloths.empty() || !c.h_ox0.empty())) {
    c.set_error("xrt_add_instance in a context that already has xrt_add_cloth / xrt_add_obstacle");
    return XRT_ERR_STATE;
  }
  if (obstacle) {
    const xrt_status st = check_obstacle(c, obstacle);
    if (st != XRT_OK) return st;
  }
  Context::HostInstance I{};
  I.vertex_base = (uint32_t)c.h_w.size();
  I.overtex_base = (uint32_t)(c.h_ox0.size() / 3);
  I.oface_base = (uint32_t)(c.h_otri.size() / 3);
  const xrt_status st =
      add_cloth_impl(c, cloth, I.overtex_base, obstacle ? obstacle->num_vertices : 0u, nullptr);
  if (st != XRT_OK) return st;
  if (obstacle) add_obstacle_impl(c, obstacle, nullptr);
  I.num_vertices = (uint32_t)c.h_w.size() - I.vertex_base;
  I.num_overtices = (uint32_t)(c.h_ox0.size() / 3) - I.overtex_base;
  I.num_ofaces = (uint32_t)(c.h_otri.size() / 3) - I.oface_base;
  I.diameter = c.particle_diameter;  // this cloth's (add_cloth_impl)
  c.instanced = true;
  if (out_instance) *out_instance = (int32_t)c.instances.size();
  c.instances.push_back(I);
  return XRT_OK;
}

xrt_status xrt_set_coloring(xrt_ctx* h, int32_t kind, const uint32_t* colors, uint32_t n) {
  if (!h || (n && !colors) || kind < 0 || kind > 3) return XRT_ERR_INVALID_ARGUMENT;
  if (h->c.started) {
    h->c.set_error("xrt_set_coloring after xrt_start");
    return XRT_ERR_STATE;
  }
  h->c.pending_colors[kind].assign(colors, colors + n);
  return XRT_OK;
}

static xrt_status upload_constraints(Context& c);

xrt_status xrt_set_compliance(xrt_ctx* h, int32_t kind, const float* comp, uint32_t n) {
  if (!h || !comp || (kind != 0 && kind != 1)) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  std::vector<float>& dst = kind == 0 ? c.h_scomp : c.h_bcomp;
  if (n != dst.size()) {
    c.set_error("compliance count does not match the constraint count");
    return XRT_ERR_INVALID_ARGUMENT;
  }
  dst.assign(comp, comp + n);
  if (c.started) {
    cudaSetDevice(c.device);
    return upload_constraints(c);
  }
  return XRT_OK;
}

xrt_status xrt_set_inv_mass(xrt_ctx* h, const float* w, uint32_t n) {
  if (!h || !w) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (n != c.h_w.size()) {
    c.set_error("inverse-mass count does not match the vertex count");
    return XRT_ERR_INVALID_ARGUMENT;
  }
  if (!c.started) {
    c.h_w.assign(w, w + n);
    return XRT_OK;
  }
  // after start: new masses for the free vertices; the set of pinned vertices (inverse mass 0)
  // fixes the LRA mode and stays as it was
  for (uint32_t i = 0; i < n; ++i)
    if ((w[i] > 0.0f) != (c.h_w[i] > 0.0f) || !(w[i] >= 0.0f)) {
      c.set_error("xrt_set_inv_mass after xrt_start must keep the pinned vertices (inverse mass 0)");
      return XRT_ERR_INVALID_ARGUMENT;
    }
  cudaSetDevice(c.device);
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  std::vector<float4> x(c.nv);
  for (DBuf<float4>* b : {&c.x, &c.x_alt}) {
    XRT_CUDA(&c, cudaMemcpy(x.data(), b->p, sizeof(float4) * c.nv, cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < c.nv; ++i) x[i].w = w[i];
    XRT_CUDA(&c, cudaMemcpy(b->p, x.data(), sizeof(float4) * c.nv, cudaMemcpyHostToDevice));
  }
  c.h_w.assign(w, w + n);
  return XRT_OK;
}

// Constraint arrays sorted by color (stable within a color).
static xrt_status upload_constraints(Context& c) {
  std::vector<int4> scon(c.ne);
  for (uint32_t j = 0; j < c.ne; ++j) {
    const uint32_t o = c.s_perm[j];
    int4 v;
    const bool tiled = c.s_tiles.on;
    v.x = (int)(tiled ? c.s_local[2 * j] : c.h_edges[2 * o]);
    v.y = (int)(tiled ? c.s_local[2 * j + 1] : c.h_edges[2 * o + 1]);
    std::memcpy(&v.z, &c.h_rest[o], 4);
    std::memcpy(&v.w, &c.h_scomp[o], 4);
    scon[j] = v;
  }
  std::vector<int4> bidx(c.nb);
  std::vector<float2> btc(c.nb);
  for (uint32_t j = 0; j < c.nb; ++j) {
    const uint32_t o = c.b_perm[j];
    if (c.b_tiles.on)
      bidx[j] = make_int4((int)c.b_local[4 * j], (int)c.b_local[4 * j + 1], (int)c.b_local[4 * j + 2],
                          (int)c.b_local[4 * j + 3]);
    else
      bidx[j] = make_int4((int)c.h_bends[4 * o], (int)c.h_bends[4 * o + 1],
                          (int)c.h_bends[4 * o + 2], (int)c.h_bends[4 * o + 3]);
    btc[j] = make_float2(c.h_theta[o], c.h_bcomp[o]);
  }
  XRT_CUDA(&c, upload(c.s_con, scon, c.stream));
  XRT_CUDA(&c, upload(c.b_idx, bidx, c.stream));
  XRT_CUDA(&c, upload(c.b_tc, btc, c.stream));
  // the forward tile kernels' per-tile record blocks (TiledSet::rec); footprint-local ids fit
  // 16 bits
  static_assert(xrt::kTileMaxFootprint <= 65536, "16-bit footprint-local vertex ids");
  const float dt = xrt::frame_const(c).dt;  // the compliance terms are evaluated for this dt
  c.rec_dt = dt;
  for (int kind = 0; kind < 2; ++kind) {
    xrt::TiledSet& T = kind == 0 ? c.s_tiles : c.b_tiles;
    if (!T.on) continue;
    const int arity = kind == 0 ? 2 : 4;
    const std::vector<uint32_t>& local = kind == 0 ? c.s_local : c.b_local;
    const std::vector<int4>& meta = c.h_tile_meta[kind];
    std::vector<uint4> rec;
    std::vector<uint32_t> ofs(meta.size() + 1);
    // one segment per tile (stretch) or per local color of a tile (bend): slots [c0, c0 + nc)
    auto segment = [&](uint32_t c0, uint32_t nc) {
      const uint32_t n16 = xrt::color_seg16(nc, arity), ids16 = (2 * arity * nc + 15) / 16;
      const size_t at = rec.size();
      rec.resize(rec.size() + n16, make_uint4(0, 0, 0, 0));
      uint16_t* ids = reinterpret_cast<uint16_t*>(rec.data() + at);
      float2* vals = reinterpret_cast<float2*>(rec.data() + at + ids16);
      for (uint32_t j = 0; j < nc; ++j) {
        const uint32_t slot = c0 + j;
        for (int a = 0; a < arity; ++a) ids[arity * j + a] = (uint16_t)local[arity * slot + a];
        vals[j] = kind == 0 ? make_float2(c.h_rest[c.s_perm[slot]],
                                          xrt::stretch_alpha(c.h_scomp[c.s_perm[slot]], dt))
                            : make_float2(btc[slot].x, xrt::bend_alpha(btc[slot].y, dt));
      }
    };
    const std::vector<uint32_t>& lofs = c.h_tile_lofs[kind];
    const uint32_t L = T.num_local;
    for (size_t t = 0; t < meta.size(); ++t) {
      const uint32_t c0 = (uint32_t)meta[t].z, nc = (uint32_t)meta[t].w;
      ofs[t] = (uint32_t)rec.size();
      for (uint32_t l = 0; l < L; ++l)
        segment(c0 + lofs[t * (L + 1) + l], lofs[t * (L + 1) + l + 1] - lofs[t * (L + 1) + l]);
      (void)nc;
    }
    ofs[meta.size()] = (uint32_t)rec.size();  // the end of the last tile's block
    if (rec.size() >= (1ull << 32)) {
      c.set_error("tile record blocks exceed 2^32 x 16 bytes");
      return XRT_ERR_EDGE_CAPACITY;
    }
    XRT_CUDA(&c, upload(T.rec, rec, c.stream));
    XRT_CUDA(&c, upload(T.rec_ofs, ofs, c.stream));
  }
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  return XRT_OK;
}

static void sort_by_color(const std::vector<uint32_t>& col, uint32_t ncolors,
                          std::vector<uint32_t>& perm, std::vector<ColorRange>& ranges) {
  perm.resize(col.size());
  std::iota(perm.begin(), perm.end(), 0u);
  std::stable_sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) { return col[a] < col[b]; });
  ranges.assign(ncolors, ColorRange{0, 0});
  uint32_t j = 0;
  for (uint32_t k = 0; k < ncolors; ++k) {
    ranges[k].begin = j;
    while (j < perm.size() && col[perm[j]] == k) ++j;
    ranges[k].end = j;
  }
}

// One constraint kind's schedule, filled by schedule_kind.
struct KindSchedule {
  std::vector<uint32_t>& color;       // per constraint (input order)
  uint32_t& ncolors;                  // colors (tile colors x local colors when tiled)
  xrt::TiledSet& tiles;               // on when the tile-local schedule applies
  std::vector<uint32_t>& perm;        // execution slot -> constraint
  std::vector<uint32_t>& local;       // tiled: per slot and arity, footprint-local vertex index
  std::vector<ColorRange>& ranges;    // per color (untiled)
  std::vector<int4>& meta;            // tiled: host copy of the tile records
  std::vector<uint32_t>& lofs;        // tiled: host copy of the local-color offsets
};

// The caller's coloring (validated), else the tile-local Gauss-Seidel schedule (tiles halved
// until every footprint fits a block), else a greedy coloring.
static xrt_status schedule_kind(Context& c, const std::vector<uint32_t>& idx, int arity,
                                const std::vector<uint32_t>& pending,
                                const std::vector<uint32_t>& segments, KindSchedule K) {
  if (!pending.empty()) {
    std::string why;
    if (!xrt::setup::coloring_valid(idx, arity, pending, c.nv, why)) {
      c.set_error("invalid coloring: " + why);
      return XRT_ERR_COLORING;
    }
    K.color = pending;
    K.ncolors = 0;
    for (uint32_t v : K.color) K.ncolors = std::max(K.ncolors, v + 1);
    sort_by_color(K.color, K.ncolors, K.perm, K.ranges);
    return XRT_OK;
  }
  bool tiled = false;
  if (c.tile_vertices > 0 && !idx.empty()) {
    uint32_t tv = c.tile_vertices;
    c.tmp_schedule = xrt::setup::build_tiles(idx, arity, c.nv, tv, segments);
    while (c.tmp_schedule.max_footprint > xrt::kTileMaxFootprint && tv > 32) {
      tv /= 2;
      c.tmp_schedule = xrt::setup::build_tiles(idx, arity, c.nv, tv, segments);
    }
    tiled = c.tmp_schedule.num_tile_colors > 0 &&
            c.tmp_schedule.max_footprint <= xrt::kTileMaxFootprint;
  }
  if (!tiled) {
    K.color = xrt::setup::greedy_color(idx, arity, c.nv, K.ncolors);
    sort_by_color(K.color, K.ncolors, K.perm, K.ranges);
    return XRT_OK;
  }
  // tile-local Gauss-Seidel schedule (a coloring; see setup::TileSchedule)
  xrt::TiledSet& T = K.tiles;
  const xrt::setup::TileSchedule& S = c.tmp_schedule;
  K.color = S.color;
  K.ncolors = S.num_tile_colors * S.num_local;
  T.on = true;
  T.num_local = S.num_local;
  T.max_foot = S.max_footprint;
  T.max_cons = 0;
  T.max_step = 0;
  for (size_t tt = 0; tt + 1 < S.foot_ptr.size(); ++tt)
    T.max_cons = std::max(T.max_cons, S.lc_ptr[(tt + 1) * S.num_local] - S.lc_ptr[tt * S.num_local]);
  for (size_t k = 0; k + 1 < S.lc_ptr.size(); ++k)
    T.max_step = std::max(T.max_step, S.lc_ptr[k + 1] - S.lc_ptr[k]);
  T.tile_colors.clear();
  T.tile_color_cons.clear();
  for (uint32_t k = 0; k < S.num_tile_colors; ++k) {
    T.tile_colors.push_back(ColorRange{S.tile_color_ptr[k], S.tile_color_ptr[k + 1]});
    T.tile_color_cons.push_back(S.lc_ptr[S.tile_color_ptr[k + 1] * S.num_local] -
                                S.lc_ptr[S.tile_color_ptr[k] * S.num_local]);
  }
  K.meta.clear();
  K.lofs.clear();
  for (size_t tt = 0; tt + 1 < S.foot_ptr.size(); ++tt) {
    const uint32_t c0 = S.lc_ptr[tt * S.num_local], c1 = S.lc_ptr[(tt + 1) * S.num_local];
    K.meta.push_back(make_int4((int)S.foot_ptr[tt], (int)(S.foot_ptr[tt + 1] - S.foot_ptr[tt]),
                               (int)c0, (int)(c1 - c0)));
    for (uint32_t l = 0; l <= S.num_local; ++l) K.lofs.push_back(S.lc_ptr[tt * S.num_local + l] - c0);
  }
  T.max_seg16 = 0;  // the largest local color's segment and tile block of segments
  T.max_tile16 = 0;
  for (size_t tt = 0; tt + 1 < S.foot_ptr.size(); ++tt) {
    uint32_t sum = 0;
    for (uint32_t l = 0; l < S.num_local; ++l) {
      const size_t k = tt * S.num_local + l;
      const uint32_t seg = xrt::color_seg16(S.lc_ptr[k + 1] - S.lc_ptr[k], (uint32_t)arity);
      T.max_seg16 = std::max(T.max_seg16, seg);
      sum += seg;
    }
    T.max_tile16 = std::max(T.max_tile16, sum);
  }
  XRT_CUDA(&c, upload(T.foot, S.foot, c.stream));
  XRT_CUDA(&c, upload(T.meta, K.meta, c.stream));
  XRT_CUDA(&c, upload(T.lofs, K.lofs, c.stream));
  K.perm = S.order;
  K.local = S.local_slot;
  return XRT_OK;
}

xrt_status xrt_start(xrt_ctx* h) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (c.started) {
    c.set_error("xrt_start called twice");
    return XRT_ERR_STATE;
  }
  if (c.h_w.empty()) {
    c.set_error("no cloth added");
    return XRT_ERR_STATE;
  }
  cudaSetDevice(c.device);
  c.nv = (uint32_t)c.h_w.size();
  c.ne = (uint32_t)c.h_rest.size();
  c.nf = (uint32_t)(c.h_tri.size() / 3);
  c.nb = (uint32_t)c.h_theta.size();
  c.nl = (uint32_t)c.h_lra_rest.size();
  c.nbind = (uint32_t)c.h_bind.size();
  c.onv = (uint32_t)(c.h_ox0.size() / 3);
  c.onf = (uint32_t)(c.h_otri.size() / 3);
  for (const auto& b : c.h_bind)
    if (c.onv == 0 || b.iu >= c.onv || b.iv >= c.onv || b.iw >= c.onv) {
      c.set_error("binding refers to a missing obstacle vertex");
      return XRT_ERR_INVALID_MESH;
    }
  if (c.instanced && (c.params.pbd_repulsion || c.params.impact_zone || c.params.imminent_repulsion)) {
    c.set_error("pbd_repulsion, imminent_repulsion and impact_zone (Quality-mode self contact) are "
                "not available in a batched context");
    return XRT_ERR_INVALID_ARGUMENT;
  }
  // instances: merged mode is one instance holding every cloth and obstacle
  if (!c.instanced)
    c.instances.assign(1, Context::HostInstance{0, c.nv, 0, c.onv, 0, c.onf, c.particle_diameter});
  std::vector<uint32_t> segments;  // first cloth vertex of each instance
  {
    c.h_inst.clear();
    uint32_t tb = 0;
    for (const auto& I : c.instances) {
      xrt::InstanceRec r{};
      r.diameter = I.diameter;
      r.spacing = I.diameter * c.params.hash_cell_size;  // SpatialHashGPU: diameter x cell size
      r.spacing2 = r.spacing * r.spacing;
      r.d2 = I.diameter * I.diameter;
      r.table_base = tb;
      r.table_size = 2 * I.num_vertices;                  // table of 2V (SpatialHashGPU.cu:166)
      tb += r.table_size;
      r.vertex_base = I.vertex_base;
      r.num_vertices = I.num_vertices;
      c.h_inst.push_back(r);
      segments.push_back(I.vertex_base);
    }
    if (c.h_inst.size() > 1) {
      XRT_CUDA(&c, upload(c.inst, c.h_inst, c.stream));
      std::vector<uint32_t> vi(c.nv);
      for (uint32_t s = 0; s < (uint32_t)c.instances.size(); ++s)
        std::fill(vi.begin() + c.instances[s].vertex_base,
                  vi.begin() + c.instances[s].vertex_base + c.instances[s].num_vertices, s);
      XRT_CUDA(&c, upload(c.vinst, vi, c.stream));
    } else {
      segments.clear();
    }
  }
  // coloring
  for (int kind = 0; kind < 2; ++kind) {
    const std::vector<uint32_t>& idx = kind == 0 ? c.h_edges : c.h_bends;
    KindSchedule K{kind == 0 ? c.h_scolor : c.h_bcolor, kind == 0 ? c.n_scolors : c.n_bcolors,
                   kind == 0 ? c.s_tiles : c.b_tiles, kind == 0 ? c.s_perm : c.b_perm,
                   kind == 0 ? c.s_local : c.b_local, kind == 0 ? c.s_ranges : c.b_ranges,
                   c.h_tile_meta[kind], c.h_tile_lofs[kind]};
    xrt_status st = schedule_kind(c, idx, kind == 0 ? 2 : 4, c.pending_colors[kind], segments, K);
    if (st != XRT_OK) return st;
  }
  if (c.fem.on) {  // the FEM fabric's strain (faces) and isometric bending (bend elements)
    for (int kind = 0; kind < 2; ++kind) {
      xrt::FemKind& F = kind == 0 ? c.fem.strain : c.fem.bend;
      KindSchedule K{F.color, F.ncolors, F.tiles, F.perm, F.local, F.ranges, F.meta, F.lofs};
      xrt_status st = schedule_kind(c, kind == 0 ? c.h_tri : c.h_bends, kind == 0 ? 3 : 4,
                                    c.pending_colors[2 + kind], segments, K);
      if (st != XRT_OK) return st;
    }
  }
  if (c.s_tiles.on || c.b_tiles.on) {
    const size_t smem = std::max(
        std::max(xrt::tile_smem_bytes(c.s_tiles, sizeof(int4) + sizeof(float)),
                 xrt::tile_smem_bytes(c.b_tiles, sizeof(int4) + sizeof(float2))),
        std::max(std::max(xrt::tile_smem_fwd(c.s_tiles, true, true),
                          xrt::tile_smem_fwd(c.s_tiles, true, false)),
                 std::max(xrt::tile_smem_fwd(c.b_tiles, false, true),
                          xrt::tile_smem_fwd(c.b_tiles, false, false))));
    if (smem > 200 * 1024) {
      c.set_error("tile schedule needs more shared memory than a block has");
      return XRT_ERR_INVALID_MESH;
    }
    XRT_CUDA(&c, xrt::configure_tile_kernels(std::max<size_t>(smem, 16)));
    if (c.s_tiles.on) XRT_CUDA(&c, xrt::choose_tile_block(c.s_tiles, false));
    if (c.b_tiles.on) XRT_CUDA(&c, xrt::choose_tile_block(c.b_tiles, true));
  }
  if (c.fem.on) {
    for (const xrt::FemKind* K : {&c.fem.strain, &c.fem.bend})
      if (K->tiles.on && xrt::tile_smem_bytes(K->tiles, sizeof(int4) + sizeof(float)) > 200 * 1024) {
        c.set_error("FEM tile schedule needs more shared memory than a block has");
        return XRT_ERR_INVALID_MESH;
      }
    XRT_CUDA(&c, xrt::fem_configure(c));
    XRT_CUDA(&c, xrt::fem_upload(c));
  }
  xrt_status st = upload_constraints(c);
  if (st != XRT_OK) return st;
  XRT_CUDA(&c, c.s_lambda.reserve(std::max(c.ne, 1u)));
  XRT_CUDA(&c, cudaMemsetAsync(c.s_lambda.p, 0, sizeof(float) * std::max(c.ne, 1u), c.stream));
  // state
  const std::vector<float4> x0 = to_f4(c.h_x0, &c.h_w);
  std::vector<float4> x0_plain = to_f4(c.h_x0, nullptr);
  XRT_CUDA(&c, upload(c.x, x0, c.stream));
  XRT_CUDA(&c, upload(c.x_alt, x0, c.stream));
  XRT_CUDA(&c, upload(c.x0, x0_plain, c.stream));
  XRT_CUDA(&c, upload(c.x_init, x0_plain, c.stream));  // SpatialHashGPU::SetInitialPositions
  XRT_CUDA(&c, c.v.reserve(c.nv));
  XRT_CUDA(&c, cudaMemsetAsync(c.v.p, 0, sizeof(float4) * c.nv, c.stream));
  XRT_CUDA(&c, c.n.reserve(c.nv));
  // topology
  std::vector<int4> tri(c.nf);
  for (uint32_t f = 0; f < c.nf; ++f)
    tri[f] = make_int4((int)c.h_tri[3 * f], (int)c.h_tri[3 * f + 1], (int)c.h_tri[3 * f + 2], 0);
  XRT_CUDA(&c, upload(c.tri, tri, c.stream));
  std::vector<uint32_t> ptr, list;
  xrt::setup::build_vf(c.h_tri, c.nv, ptr, list);
  XRT_CUDA(&c, upload(c.vf_ptr, ptr, c.stream));
  XRT_CUDA(&c, upload(c.vf_list, list, c.stream));
  std::vector<uint2> edge(c.ne);
  for (uint32_t e = 0; e < c.ne; ++e) edge[e] = make_uint2(c.h_edges[2 * e], c.h_edges[2 * e + 1]);
  XRT_CUDA(&c, upload(c.edge, edge, c.stream));
  xrt::setup::build_ve(c.h_edges, c.nv, ptr, list);
  XRT_CUDA(&c, upload(c.ve_ptr, ptr, c.stream));
  XRT_CUDA(&c, upload(c.ve_list, list, c.stream));
  xrt::launch_vertex_normals(c.x0.p, c.tri.p, c.vf_ptr.p, c.vf_list.p, c.n.p, c.nv, c.stream);
  // LRA: by target when every slot vertex is pinned, else slot-major blocks
  {
    c.lra_by_target = true;
    for (uint32_t k = 0; k < c.nl; ++k)
      if (c.h_w[c.h_lra_src[k]] > 0.0f) c.lra_by_target = false;
    std::vector<uint32_t> lptr(c.nv + 1, 0), lsrc(c.nl);
    std::vector<float> lrest(c.nl);
    for (uint32_t k = 0; k < c.nl; ++k) lptr[c.h_lra_tgt[k] + 1]++;
    for (uint32_t i = 0; i < c.nv; ++i) lptr[i + 1] += lptr[i];
    std::vector<uint32_t> fill(lptr.begin(), lptr.end() - 1);
    for (uint32_t k = 0; k < c.nl; ++k) {
      const uint32_t pos = fill[c.h_lra_tgt[k]]++;
      lsrc[pos] = c.h_lra_src[k];
      lrest[pos] = c.h_lra_rest[k];
    }
    XRT_CUDA(&c, upload(c.lra_ptr, lptr, c.stream));
    XRT_CUDA(&c, upload(c.lra_src, lsrc, c.stream));
    XRT_CUDA(&c, upload(c.lra_rest, lrest, c.stream));
    c.lra_blocks.clear();
    if (!c.lra_by_target) {
      XRT_CUDA(&c, upload(c.lra_l_src, c.h_lra_src, c.stream));
      XRT_CUDA(&c, upload(c.lra_l_tgt, c.h_lra_tgt, c.stream));
      XRT_CUDA(&c, upload(c.lra_l_rest, c.h_lra_rest, c.stream));
      uint32_t k = 0;
      while (k < c.nl) {  // maximal runs of one source slot, in list order
        uint32_t e = k;
        while (e < c.nl && c.h_lra_src[e] == c.h_lra_src[k]) ++e;
        c.lra_blocks.push_back(ColorRange{k, e});
        k = e;
      }
    }
  }
  // contacts
  XRT_CUDA(&c, c.vf_idx.reserve(c.nv));
  XRT_CUDA(&c, c.rt_idx.reserve(c.nv));
  XRT_CUDA(&c, c.vf_qs.reserve(c.nv));
  XRT_CUDA(&c, c.rt_qc.reserve(c.nv));
  XRT_CUDA(&c, c.ee_a.reserve(std::max(c.ne, 1u)));
  XRT_CUDA(&c, c.ee_b.reserve(std::max(c.ne, 1u)));
  XRT_CUDA(&c, c.ee_c.reserve(std::max(c.ne, 1u)));
  XRT_CUDA(&c, c.ee_vflag.reserve(std::max(c.nv, 1u)));
  XRT_CUDA(&c, cudaMemsetAsync(c.ee_vflag.p, 0, std::max(c.nv, 1u), c.stream));
  XRT_CUDA(&c, cudaMemsetAsync(c.vf_idx.p, 0xFF, sizeof(int) * c.nv, c.stream));
  XRT_CUDA(&c, cudaMemsetAsync(c.rt_idx.p, 0xFF, sizeof(int) * c.nv, c.stream));
  XRT_CUDA(&c, cudaMemsetAsync(c.vf_qs.p, 0, sizeof(float4) * c.nv, c.stream));
  XRT_CUDA(&c, cudaMemsetAsync(c.rt_qc.p, 0, sizeof(float4) * c.nv, c.stream));
  {
    std::vector<float4> ea(std::max(c.ne, 1u), make_float4(xrt::kScalarMaxHost, 0, 0, 0));
    std::vector<float4> zero(std::max(c.ne, 1u), make_float4(0, 0, 0, 0));
    XRT_CUDA(&c, upload(c.ee_a, ea, c.stream));
    XRT_CUDA(&c, upload(c.ee_b, zero, c.stream));
    XRT_CUDA(&c, upload(c.ee_c, zero, c.stream));
  }
  // particle hash
  {
    const uint32_t table = 2 * c.nv;
    const size_t nbs = (size_t)c.nv * (size_t)c.params.max_neighbor_size;
    XRT_CUDA(&c, c.hash_key.reserve(c.nv));
    XRT_CUDA(&c, c.hash_val.reserve(c.nv));
    XRT_CUDA(&c, c.cell_start.reserve(table));
    XRT_CUDA(&c, c.cell_end.reserve(table));
    XRT_CUDA(&c, c.neighbors.reserve(nbs));
    XRT_CUDA(&c, cudaMemsetAsync(c.cell_end.p, 0, sizeof(uint32_t) * table, c.stream));
    XRT_CUDA(&c, cudaMemsetAsync(c.neighbors.p, 0, sizeof(uint32_t) * nbs, c.stream));
    XRT_CUDA(&c, c.hash_sorter.reserve(c.nv));
  }
  // bindings: GenerateBinding_Kernel (BindingConstraint.cu:20-44) rest lengths from x0
  {
    std::vector<uint32_t> bptr(c.nv + 1, 0);
    for (auto& b : c.h_bind) {
      if (b.L < 1e-6f) {
        const float* po = c.h_ox0.data();
        auto P = [&](uint32_t i) { return xrt::setup::V3{po[3 * i], po[3 * i + 1], po[3 * i + 2]}; };
        const xrt::setup::V3 pu = P(b.iu), pv = P(b.iv), pw = P(b.iw);
        const xrt::setup::V3 pb{(b.u * pu.x + b.v * pv.x) + b.w * pw.x,
                                (b.u * pu.y + b.v * pv.y) + b.w * pw.y,
                                (b.u * pu.z + b.v * pv.z) + b.w * pw.z};
        const xrt::setup::V3 pc{c.h_x0[3 * b.cloth], c.h_x0[3 * b.cloth + 1], c.h_x0[3 * b.cloth + 2]};
        b.L = xrt::setup::length(xrt::setup::sub(pc, pb));
      }
      bptr[b.cloth + 1]++;
    }
    for (uint32_t i = 0; i < c.nv; ++i) bptr[i + 1] += bptr[i];
    std::vector<uint32_t> fill(bptr.begin(), bptr.end() - 1);
    std::vector<float4> ba(std::max<size_t>(c.nbind, 1));
    std::vector<int4> bb(std::max<size_t>(c.nbind, 1));
    for (const auto& b : c.h_bind) {
      const uint32_t pos = fill[b.cloth]++;
      ba[pos] = make_float4(b.u, b.v, b.w, b.L);
      int sbits;
      std::memcpy(&sbits, &b.stiffness, 4);
      bb[pos] = make_int4((int)b.iu, (int)b.iv, (int)b.iw, sbits);
    }
    XRT_CUDA(&c, upload(c.bind_ptr, bptr, c.stream));
    XRT_CUDA(&c, upload(c.bind_a, ba, c.stream));
    XRT_CUDA(&c, upload(c.bind_b, bb, c.stream));
  }
  // obstacle
  if (c.onv > 0) {
    const std::vector<float4> ox = to_f4(c.h_ox0, nullptr);
    XRT_CUDA(&c, upload(c.ox0, ox, c.stream));
    XRT_CUDA(&c, upload(c.ox, ox, c.stream));
    XRT_CUDA(&c, upload(c.ox1, ox, c.stream));
    XRT_CUDA(&c, c.on.reserve(c.onv));
    XRT_CUDA(&c, c.on1.reserve(c.onv));
    c.h_ortri = xrt::setup::build_rtri(c.h_otri, c.onv);
    std::vector<int4> ot(std::max(c.onf, 1u));
    for (uint32_t f = 0; f < c.onf; ++f)
      ot[f] = make_int4((int)c.h_otri[3 * f], (int)c.h_otri[3 * f + 1], (int)c.h_otri[3 * f + 2],
                        (int)c.h_ortri[f]);
    XRT_CUDA(&c, upload(c.otri, ot, c.stream));
    xrt::setup::build_vf(c.h_otri, c.onv, ptr, list);
    XRT_CUDA(&c, upload(c.ovf_ptr, ptr, c.stream));
    XRT_CUDA(&c, upload(c.ovf_list, list, c.stream));
    xrt::launch_vertex_normals(c.ox0.p, c.otri.p, c.ovf_ptr.p, c.ovf_list.p, c.on.p, c.onv, c.stream);
    XRT_CUDA(&c, cudaMemcpyAsync(c.on1.p, c.on.p, sizeof(float4) * c.onv, cudaMemcpyDeviceToDevice,
                                 c.stream));
    if (c.onf > 0) {
      if (c.instanced) {  // one tree per instance (a forest over the instances' triangles)
        std::vector<uint32_t> counts;
        for (const auto& I : c.instances) counts.push_back(I.num_ofaces);
        XRT_CUDA(&c, c.bvh.set_segments(counts, c.stream));
      }
      XRT_CUDA(&c, c.bvh.reserve(c.onf));
      c.bvh.n = c.onf;
      xrt::launch_prims_obstacle(c, 0.0f);  // ClothSolverUniversal::Start: UpdateData(0) + Construct
      c.bvh.construct(0.0f, c.stream, c.err.p);
    }
  }
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  XRT_CUDA(&c, cudaGetLastError());
  c.started = true;
  c.graph_dirty = true;
  return XRT_OK;
}

xrt_status xrt_set_obstacle_targets(xrt_ctx* h, const float* pos) {
  if (!h || !pos) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (require_started(c) != XRT_OK) return XRT_ERR_STATE;
  if (c.onv == 0) {
    c.set_error("no obstacle");
    return XRT_ERR_STATE;
  }
  if (c.skin.on) {
    c.set_error("obstacle skinning is on: its targets come from the joint transforms");
    return XRT_ERR_STATE;
  }
  cudaSetDevice(c.device);
  // one copy of the caller's packed xyz, unpacked on the device; the call returns once the
  // caller's buffer has been read
  XRT_CUDA(&c, c.stage3.reserve(3 * (size_t)c.onv));
  XRT_CUDA(&c, cudaMemcpyAsync(c.stage3.p, pos, 3 * sizeof(float) * (size_t)c.onv,
                               cudaMemcpyHostToDevice, c.stream));
  xrt::launch_unpack_xyz(c.stage3.p, c.ox.p, c.onv, 0.0f, c.stream);
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  return XRT_OK;
}

xrt_status xrt_set_obstacle_skinning(xrt_ctx* h, const float* rest, const uint32_t* outer,
                                     const uint32_t* joints, const float* weights,
                                     uint32_t num_joints) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (require_started(c) != XRT_OK) return XRT_ERR_STATE;
  cudaSetDevice(c.device);
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  if (!rest) {  // off: targets come from xrt_set_obstacle_targets again
    c.skin.on = false;
    return XRT_OK;
  }
  if (!outer || !joints || !weights || num_joints == 0) return XRT_ERR_INVALID_ARGUMENT;
  if (c.onv == 0) {
    c.set_error("no obstacle");
    return XRT_ERR_STATE;
  }
  const uint32_t n = c.onv;
  if (outer[0] != 0) {
    c.set_error("skinning weights: outer[0] must be 0");
    return XRT_ERR_INVALID_ARGUMENT;
  }
  for (uint32_t i = 0; i < n; ++i)
    if (outer[i + 1] < outer[i]) {
      c.set_error("skinning weights: outer offsets must not decrease");
      return XRT_ERR_INVALID_ARGUMENT;
    }
  const uint32_t nnz = outer[n];
  for (uint32_t k = 0; k < nnz; ++k)
    if (joints[k] >= num_joints || !std::isfinite(weights[k])) {
      c.set_error("skinning weights: joint index out of range or weight not finite");
      return XRT_ERR_INVALID_ARGUMENT;
    }
  std::vector<float4> r(n);
  for (uint32_t i = 0; i < n; ++i)
    r[i] = make_float4(rest[3 * i], rest[3 * i + 1], rest[3 * i + 2], 0.0f);
  XRT_CUDA(&c, upload(c.skin.rest, r, c.stream));
  XRT_CUDA(&c, upload(c.skin.outer, std::vector<uint32_t>(outer, outer + n + 1), c.stream));
  XRT_CUDA(&c, upload(c.skin.joint, std::vector<uint32_t>(joints, joints + nnz), c.stream));
  XRT_CUDA(&c, upload(c.skin.weight, std::vector<float>(weights, weights + nnz), c.stream));
  // identity transforms until the first xrt_set_joint_transforms
  std::vector<float> eye((size_t)12 * num_joints, 0.0f);
  for (uint32_t j = 0; j < num_joints; ++j) eye[12 * j] = eye[12 * j + 5] = eye[12 * j + 10] = 1.0f;
  XRT_CUDA(&c, upload(c.skin.transforms, eye, c.stream));
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  c.skin.num_joints = num_joints;
  c.skin.on = true;
  return XRT_OK;
}

xrt_status xrt_set_joint_transforms(xrt_ctx* h, const float* transforms) {
  if (!h || !transforms) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (!c.skin.on) {
    c.set_error("call xrt_set_obstacle_skinning first");
    return XRT_ERR_STATE;
  }
  cudaSetDevice(c.device);
  XRT_CUDA(&c, cudaMemcpyAsync(c.skin.transforms.p, transforms,
                               sizeof(float) * 12 * c.skin.num_joints, cudaMemcpyHostToDevice,
                               c.stream));
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  return XRT_OK;
}

xrt_status xrt_set_joint_transforms_device(xrt_ctx* h, const float* d_transforms) {
  if (!h || !d_transforms) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (!c.skin.on) {
    c.set_error("call xrt_set_obstacle_skinning first");
    return XRT_ERR_STATE;
  }
  cudaSetDevice(c.device);
  XRT_CUDA(&c, cudaMemcpyAsync(c.skin.transforms.p, d_transforms,
                               sizeof(float) * 12 * c.skin.num_joints, cudaMemcpyDeviceToDevice,
                               c.stream));
  return XRT_OK;
}

xrt_status xrt_set_obstacle_targets_device(xrt_ctx* h, const float* d_pos) {
  if (!h || !d_pos) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (require_started(c) != XRT_OK) return XRT_ERR_STATE;
  if (c.skin.on) {
    c.set_error("obstacle skinning is on: its targets come from the joint transforms");
    return XRT_ERR_STATE;
  }
  cudaSetDevice(c.device);
  // 3 floats -> float4 with a strided 2D copy (pitch 12 B in, 16 B out)
  XRT_CUDA(&c, cudaMemcpy2DAsync(c.ox.p, sizeof(float4), d_pos, 3 * sizeof(float), 3 * sizeof(float),
                                 c.onv, cudaMemcpyDeviceToDevice, c.stream));
  return XRT_OK;
}

xrt_status xrt_step_frame(xrt_ctx* h) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (require_started(c) != XRT_OK) return XRT_ERR_STATE;
  cudaSetDevice(c.device);
  const bool eager = c.params.pbd_repulsion || c.params.impact_zone ||  // host reads in the frame
                     c.params.imminent_repulsion;
  if (eager) {
    xrt_status st = xrt::prox_prepare(c);
    if (st != XRT_OK) return st;
  }
  xrt::launch_skin(c);  // obstacle targets from the joint transforms, when skinning is on
  if (c.diff.active) xrt::diff_checkpoint(c);  // state at the frame start, for xrt_backward
  xrt_status st = xrt::frame_core(c, eager);
  if (st != XRT_OK) return st;
  XRT_CUDA(&c, xrt::cache_frame(c));  // when recording: this frame into the frame cache
  c.frame_index++;
  return XRT_OK;
}

}  // extern "C"

// The frame's launches on the current state: a profiled frame, the replayed frame graph or an
// eager frame.  Also the adjoint's plain recomputation of the frames between checkpoints.
xrt_status xrt::frame_core(Context& c, bool eager) {
  c.frame_status = XRT_OK;
  if (c.profiling == 2 && !eager) {
    xrt_status st = profile_frame_graph(c);
    if (st != XRT_OK) return st;
  } else if (c.profiling) {
    record_frame(c);
    XRT_CUDA(&c, cudaGetLastError());
    collect_profile(c);
  } else if (c.graph_enabled && !eager) {
    if (c.graph_dirty || !c.graph_exec) {
      xrt_status st = capture_frame(c);
      if (st != XRT_OK) return st;
    }
    XRT_CUDA(&c, cudaGraphLaunch(c.graph_exec, c.stream));
  } else {
    record_frame(c);
    XRT_CUDA(&c, cudaGetLastError());
  }
  return c.frame_status;
}

extern "C" {

xrt_status xrt_step_frames(xrt_ctx* h, int32_t n) {
  for (int32_t i = 0; i < n; ++i) {
    xrt_status st = xrt_step_frame(h);
    if (st != XRT_OK) return st;
  }
  return XRT_OK;
}

xrt_status xrt_synchronize(xrt_ctx* h) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  cudaSetDevice(c.device);
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  uint32_t err = 0;
  XRT_CUDA(&c, cudaMemcpy(&err, c.err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  if (err) {
    c.set_error("device error word 0x" + std::to_string(err) +
                " (1: traversal bound, 2: tree-walk bound, 4: index range, 8: impact zone size, "
                "16: line-search bound)");
    return XRT_ERR_DEVICE_FLAG;
  }
  return XRT_OK;
}

xrt_status xrt_set_graph_mode(xrt_ctx* h, int32_t enabled) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  h->c.graph_enabled = enabled != 0;
  h->c.graph_dirty = true;
  return XRT_OK;
}

xrt_status xrt_set_dependent_launch(xrt_ctx* h, int32_t enabled) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  h->c.pdl = enabled != 0;
  h->c.graph_dirty = true;
  return XRT_OK;
}

xrt_status xrt_set_vertex_block(xrt_ctx* h, uint32_t threads) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (threads < 64 || threads > 512 || threads % 32 != 0) {
    c.set_error("vertex block must be 64 to 512 threads, a multiple of 32");
    return XRT_ERR_INVALID_ARGUMENT;
  }
  c.vertex_block = threads;
  c.graph_dirty = true;
  return XRT_OK;
}

xrt_status xrt_set_tile_vertices(xrt_ctx* h, uint32_t tile_vertices) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (c.started) {
    c.set_error("xrt_set_tile_vertices must precede xrt_start");
    return XRT_ERR_STATE;
  }
  if (tile_vertices != 0 && (tile_vertices < 32 || tile_vertices > (1u << 20))) {
    c.set_error("tile_vertices must be 0 or in [32, 1048576]");
    return XRT_ERR_INVALID_ARGUMENT;
  }
  c.tile_vertices = tile_vertices;
  return XRT_OK;
}

xrt_status xrt_set_profiling(xrt_ctx* h, int32_t enabled) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  cudaSetDevice(c.device);
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  if (enabled < 0 || enabled > 2) return XRT_ERR_INVALID_ARGUMENT;
  c.profiling = enabled;
  c.prof_used = 0;
  c.prof_frames = 0;
  for (int i = 0; i < 16; ++i) {
    c.prof_ms[i] = 0.0;
    c.prof_launches[i] = 0;
    c.prof_units[i] = 0;
  }
  return XRT_OK;
}

xrt_status xrt_get_profile(xrt_ctx* h, xrt_profile* out) {
  if (!h || !out) return XRT_ERR_INVALID_ARGUMENT;
  const Context& c = h->c;
  std::memset(out, 0, sizeof(*out));
  for (int i = 0; i < 16; ++i) {
    out->ms[i] = c.prof_ms[i];
    out->launches[i] = c.prof_launches[i];
    out->units[i] = c.prof_units[i];
  }
  out->frames = c.prof_frames;
  return XRT_OK;
}

const char* xrt_phase_name(int32_t phase) {
  return (phase >= 0 && phase < XRT_NUM_PHASES) ? kPhaseNames[phase] : "";
}

xrt_status xrt_get_sizes(const xrt_ctx* h, xrt_sizes* out) {
  if (!h || !out) return XRT_ERR_INVALID_ARGUMENT;
  const Context& c = h->c;
  std::memset(out, 0, sizeof(*out));
  out->num_vertices = (uint32_t)c.h_w.size();
  out->num_edges = (uint32_t)c.h_rest.size();
  out->num_triangles = (uint32_t)(c.h_tri.size() / 3);
  out->num_bends = (uint32_t)c.h_theta.size();
  out->num_lra = (uint32_t)c.h_lra_rest.size();
  out->num_bindings = (uint32_t)c.h_bind.size();
  out->num_obstacle_vertices = (uint32_t)(c.h_ox0.size() / 3);
  out->num_obstacle_triangles = (uint32_t)(c.h_otri.size() / 3);
  out->num_stretch_colors = c.n_scolors;
  out->num_bend_colors = c.n_bcolors;
  out->launches_per_frame = c.launches_per_frame;
  out->frame_index = c.frame_index;
  out->particle_diameter = c.h_inst.empty() ? c.particle_diameter : c.h_inst[0].diameter;
  out->num_instances = c.h_inst.empty() ? 1u : (uint32_t)c.h_inst.size();
  out->num_obstacle_bvh_nodes = c.bvh.active ? c.bvh.nodes : 0u;
  uint32_t* tile_colors[2] = {&out->num_stretch_tile_colors, &out->num_bend_tile_colors};
  uint32_t* footprint[2] = {&out->stretch_footprint_vertices, &out->bend_footprint_vertices};
  for (int kind = 0; kind < 2; ++kind) {  // the kinds the frame runs
    const xrt::FemKind& F = kind == 0 ? c.fem.strain : c.fem.bend;
    const xrt::TiledSet& T = c.fem.on ? F.tiles : (kind == 0 ? c.s_tiles : c.b_tiles);
    if (!T.on) continue;
    *tile_colors[kind] = (uint32_t)T.tile_colors.size();
    uint64_t f = 0;
    for (const int4& m : (c.fem.on ? F.meta : c.h_tile_meta[kind])) f += (uint32_t)m.y;
    *footprint[kind] = (uint32_t)f;
  }
  return XRT_OK;
}

xrt_status xrt_get_positions(xrt_ctx* h, float* out) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  if (require_started(h->c) != XRT_OK) return XRT_ERR_STATE;
  cudaSetDevice(h->c.device);
  return read_f4(h->c, h->c.x0, h->c.nv, out);
}
xrt_status xrt_get_velocities(xrt_ctx* h, float* out) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  if (require_started(h->c) != XRT_OK) return XRT_ERR_STATE;
  cudaSetDevice(h->c.device);
  return read_f4(h->c, h->c.v, h->c.nv, out);
}
xrt_status xrt_get_normals(xrt_ctx* h, float* out) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  if (require_started(h->c) != XRT_OK) return XRT_ERR_STATE;
  cudaSetDevice(h->c.device);
  return read_f4(h->c, h->c.n, h->c.nv, out);
}
xrt_status xrt_get_obstacle_positions(xrt_ctx* h, float* out) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  if (require_started(h->c) != XRT_OK) return XRT_ERR_STATE;
  cudaSetDevice(h->c.device);
  return read_f4(h->c, h->c.ox0, h->c.onv, out);
}
xrt_status xrt_get_obstacle_normals(xrt_ctx* h, float* out) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  if (require_started(h->c) != XRT_OK) return XRT_ERR_STATE;
  cudaSetDevice(h->c.device);
  return read_f4(h->c, h->c.on, h->c.onv, out);
}

xrt_status xrt_set_state(xrt_ctx* h, const float* pos, const float* vel) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (require_started(c) != XRT_OK) return XRT_ERR_STATE;
  cudaSetDevice(c.device);
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  if (pos) {
    std::vector<float> p(pos, pos + 3 * (size_t)c.nv);
    const std::vector<float4> a = to_f4(p, &c.h_w), b = to_f4(p, nullptr);
    XRT_CUDA(&c, cudaMemcpy(c.x.p, a.data(), sizeof(float4) * c.nv, cudaMemcpyHostToDevice));
    XRT_CUDA(&c, cudaMemcpy(c.x_alt.p, a.data(), sizeof(float4) * c.nv, cudaMemcpyHostToDevice));
    XRT_CUDA(&c, cudaMemcpy(c.x0.p, b.data(), sizeof(float4) * c.nv, cudaMemcpyHostToDevice));
  }
  if (vel) {
    std::vector<float> p(vel, vel + 3 * (size_t)c.nv);
    const std::vector<float4> b = to_f4(p, nullptr);
    XRT_CUDA(&c, cudaMemcpy(c.v.p, b.data(), sizeof(float4) * c.nv, cudaMemcpyHostToDevice));
  }
  return XRT_OK;
}

xrt_status xrt_get_device_state(xrt_ctx* h, void** dx, void** dv, void** stream) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  if (require_started(h->c) != XRT_OK) return XRT_ERR_STATE;
  if (dx) *dx = h->c.x0.p;
  if (dv) *dv = h->c.v.p;
  if (stream) *stream = (void*)h->c.stream;
  return XRT_OK;
}

xrt_status xrt_get_edges(const xrt_ctx* h, uint32_t* out2, float* rest) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  if (out2) std::copy(h->c.h_edges.begin(), h->c.h_edges.end(), out2);
  if (rest) std::copy(h->c.h_rest.begin(), h->c.h_rest.end(), rest);
  return XRT_OK;
}
xrt_status xrt_get_bends(const xrt_ctx* h, uint32_t* out4, float* th) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  if (out4) std::copy(h->c.h_bends.begin(), h->c.h_bends.end(), out4);
  if (th) std::copy(h->c.h_theta.begin(), h->c.h_theta.end(), th);
  return XRT_OK;
}
xrt_status xrt_get_coloring(const xrt_ctx* h, int32_t kind, uint32_t* colors) {
  if (!h || !colors || kind < 0 || kind > 3) return XRT_ERR_INVALID_ARGUMENT;
  const auto& col = kind == 0   ? h->c.h_scolor
                    : kind == 1 ? h->c.h_bcolor
                    : kind == 2 ? h->c.fem.strain.color
                                : h->c.fem.bend.color;
  std::copy(col.begin(), col.end(), colors);
  return XRT_OK;
}
xrt_status xrt_get_lra(const xrt_ctx* h, uint32_t* src, uint32_t* tgt, float* rest) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  if (src) std::copy(h->c.h_lra_src.begin(), h->c.h_lra_src.end(), src);
  if (tgt) std::copy(h->c.h_lra_tgt.begin(), h->c.h_lra_tgt.end(), tgt);
  if (rest) std::copy(h->c.h_lra_rest.begin(), h->c.h_lra_rest.end(), rest);
  return XRT_OK;
}
xrt_status xrt_get_obstacle_rtri(const xrt_ctx* h, uint32_t* masks) {
  if (!h || !masks) return XRT_ERR_INVALID_ARGUMENT;
  std::copy(h->c.h_ortri.begin(), h->c.h_ortri.end(), masks);
  return XRT_OK;
}
xrt_status xrt_get_inv_mass(const xrt_ctx* h, float* out) {
  if (!h || !out) return XRT_ERR_INVALID_ARGUMENT;
  std::copy(h->c.h_w.begin(), h->c.h_w.end(), out);
  return XRT_OK;
}

}  // extern "C"

xrt_status xrt::export_lbvh(xrt::Lbvh& b, cudaStream_t s, std::string& err, uint32_t* morton,
                              uint32_t* objs, uint32_t* nodes, float* aabbs, int32_t* iesc,
                              int32_t* eesc, int32_t* unique) {
  const uint32_t n = b.n;
  if (!b.active || n == 0) {
    err = "LBVH not built";
    return XRT_ERR_STATE;
  }
  const uint32_t nn = b.nodes;  // 2n - 1 for a single tree
  auto fail = [&](cudaError_t e) {
    err = cudaGetErrorString(e);
    return XRT_ERR_CUDA;
  };
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(e);
  if (morton && (e = cudaMemcpy(morton, b.sorted_morton, 4 * n, cudaMemcpyDeviceToHost))) return fail(e);
  if (objs && (e = cudaMemcpy(objs, b.sorted_index, 4 * n, cudaMemcpyDeviceToHost))) return fail(e);
  if (nodes && (e = cudaMemcpy(nodes, b.node.p, 16 * (size_t)nn, cudaMemcpyDeviceToHost))) return fail(e);
  if (aabbs) {
    std::vector<float4> lo(nn), hi(nn);
    if ((e = cudaMemcpy(lo.data(), b.lo.p, 16 * (size_t)nn, cudaMemcpyDeviceToHost))) return fail(e);
    if ((e = cudaMemcpy(hi.data(), b.hi.p, 16 * (size_t)nn, cudaMemcpyDeviceToHost))) return fail(e);
    for (uint32_t k = 0; k < nn; ++k) {
      float* a = aabbs + 6 * (size_t)k;
      a[0] = lo[k].x; a[1] = lo[k].y; a[2] = lo[k].z;
      a[3] = hi[k].x; a[4] = hi[k].y; a[5] = hi[k].z;
    }
  }
  if (iesc && b.internal > 0 &&
      (e = cudaMemcpy(iesc, b.iesc.p, 4 * (size_t)b.internal, cudaMemcpyDeviceToHost)))
    return fail(e);
  if (eesc && (e = cudaMemcpy(eesc, b.eesc.p, 4 * n, cudaMemcpyDeviceToHost))) return fail(e);
  if (unique) {
    uint32_t dup = 0;
    if ((e = cudaMemcpy(&dup, b.dup.p, 4, cudaMemcpyDeviceToHost))) return fail(e);
    *unique = dup == 0 ? 1 : 0;
  }
  return XRT_OK;
}

extern "C" {

xrt_status xrt_export_obstacle_bvh(xrt_ctx* h, uint32_t* morton, uint32_t* objs, uint32_t* nodes,
                                   float* aabbs, int32_t* iesc, int32_t* eesc) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  cudaSetDevice(h->c.device);
  std::string err;
  xrt_status st = export_lbvh(h->c.bvh, h->c.stream, err, morton, objs, nodes, aabbs, iesc, eesc, nullptr);
  if (st != XRT_OK) h->c.set_error(err);
  return st;
}

xrt_status xrt_export_contacts(xrt_ctx* h, int32_t* vf_index, float* vf_qs, int32_t* rt_index,
                               float* rt_qc, float* ee) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (require_started(c) != XRT_OK) return XRT_ERR_STATE;
  cudaSetDevice(c.device);
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  if (vf_index) XRT_CUDA(&c, cudaMemcpy(vf_index, c.vf_idx.p, 4 * c.nv, cudaMemcpyDeviceToHost));
  if (rt_index) XRT_CUDA(&c, cudaMemcpy(rt_index, c.rt_idx.p, 4 * c.nv, cudaMemcpyDeviceToHost));
  if (vf_qs && read_f4(c, c.vf_qs, c.nv, vf_qs) != XRT_OK) return XRT_ERR_CUDA;
  if (rt_qc && read_f4(c, c.rt_qc, c.nv, rt_qc) != XRT_OK) return XRT_ERR_CUDA;
  if (ee && c.ne) {
    std::vector<float4> a(c.ne), b(c.ne), d(c.ne);
    XRT_CUDA(&c, cudaMemcpy(a.data(), c.ee_a.p, 16 * (size_t)c.ne, cudaMemcpyDeviceToHost));
    XRT_CUDA(&c, cudaMemcpy(b.data(), c.ee_b.p, 16 * (size_t)c.ne, cudaMemcpyDeviceToHost));
    XRT_CUDA(&c, cudaMemcpy(d.data(), c.ee_c.p, 16 * (size_t)c.ne, cudaMemcpyDeviceToHost));
    for (uint32_t e = 0; e < c.ne; ++e) {
      float* r = ee + 12 * (size_t)e;
      r[0] = a[e].x; r[1] = a[e].y; r[2] = a[e].z; r[3] = a[e].w;
      r[4] = b[e].x; r[5] = b[e].y; r[6] = b[e].z;
      r[7] = b[e].w; r[8] = d[e].w;
      r[9] = d[e].x; r[10] = d[e].y; r[11] = d[e].z;
    }
  }
  return XRT_OK;
}

xrt_status xrt_export_neighbors(xrt_ctx* h, uint32_t* out) {
  if (!h || !out) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (require_started(c) != XRT_OK) return XRT_ERR_STATE;
  cudaSetDevice(c.device);
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  XRT_CUDA(&c, cudaMemcpy(out, c.neighbors.p, 4 * (size_t)c.nv * c.params.max_neighbor_size,
                          cudaMemcpyDeviceToHost));
  return XRT_OK;
}

// ---- standalone LBVH ---------------------------------------------------------------------------

xrt_status xrt_lbvh_create(xrt_lbvh** out, int32_t device) {
  if (!out) return XRT_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  std::string why;
  xrt_status st = check_device(device, why);
  if (st != XRT_OK) return st;
  xrt_lbvh* b = new xrt_lbvh();
  b->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      b->err.reserve(1) != cudaSuccess || cudaMemset(b->err.p, 0, 4) != cudaSuccess) {
    delete b;
    return XRT_ERR_CUDA;
  }
  *out = b;
  return XRT_OK;
}

xrt_status xrt_lbvh_destroy(xrt_lbvh* b) {
  if (!b) return XRT_OK;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  b->b.release();
  b->staging.release();
  b->err.release();
  cudaStreamDestroy(b->stream);
  delete b;
  return XRT_OK;
}

xrt_status xrt_lbvh_build_device(xrt_lbvh* b, const float* d_prims, const float* d_pred, uint32_t n,
                                 float scr, void* stream) {
  if (!b || (n && !d_prims)) return XRT_ERR_INVALID_ARGUMENT;
  cudaSetDevice(b->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
  if (b->b.reserve(n) != cudaSuccess) return XRT_ERR_CUDA;
  b->b.n = n;
  xrt::launch_float9_to_float4(d_prims, b->b.v.p, n, s);
  xrt::launch_float9_to_float4(d_pred ? d_pred : d_prims, b->b.pred.p, n, s);
  b->b.construct(scr, s, b->err.p);
  return cudaGetLastError() == cudaSuccess ? XRT_OK : XRT_ERR_CUDA;
}

xrt_status xrt_lbvh_build(xrt_lbvh* b, const float* prims, const float* pred, uint32_t n, float scr) {
  if (!b || (n && !prims)) return XRT_ERR_INVALID_ARGUMENT;
  cudaSetDevice(b->device);
  if (b->staging.reserve(18 * (size_t)std::max(n, 1u)) != cudaSuccess) return XRT_ERR_CUDA;
  if (n) {
    if (cudaMemcpy(b->staging.p, prims, 36 * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess)
      return XRT_ERR_CUDA;
    if (pred && cudaMemcpy(b->staging.p + 9 * (size_t)n, pred, 36 * (size_t)n,
                           cudaMemcpyHostToDevice) != cudaSuccess)
      return XRT_ERR_CUDA;
  }
  xrt_status st = xrt_lbvh_build_device(b, b->staging.p, pred ? b->staging.p + 9 * (size_t)n : nullptr,
                                        n, scr, nullptr);
  if (st != XRT_OK) return st;
  return cudaStreamSynchronize(b->stream) == cudaSuccess ? XRT_OK : XRT_ERR_CUDA;
}

xrt_status xrt_lbvh_refit_device(xrt_lbvh* b, const float* d_pred, uint32_t n, void* stream) {
  if (!b || !d_pred || n != b->b.n) return XRT_ERR_INVALID_ARGUMENT;
  cudaSetDevice(b->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
  xrt::launch_float9_to_float4(d_pred, b->b.pred.p, n, s);
  b->b.refit_from_pred(s, b->err.p);
  return cudaGetLastError() == cudaSuccess ? XRT_OK : XRT_ERR_CUDA;
}

xrt_status xrt_lbvh_refit(xrt_lbvh* b, const float* pred, uint32_t n) {
  if (!b || !pred || n != b->b.n) return XRT_ERR_INVALID_ARGUMENT;
  cudaSetDevice(b->device);
  if (b->staging.reserve(9 * (size_t)std::max(n, 1u)) != cudaSuccess) return XRT_ERR_CUDA;
  if (cudaMemcpy(b->staging.p, pred, 36 * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess)
    return XRT_ERR_CUDA;
  xrt_status st = xrt_lbvh_refit_device(b, b->staging.p, n, nullptr);
  if (st != XRT_OK) return st;
  return cudaStreamSynchronize(b->stream) == cudaSuccess ? XRT_OK : XRT_ERR_CUDA;
}

xrt_status xrt_lbvh_export(xrt_lbvh* b, uint32_t* morton, uint32_t* objs, uint32_t* nodes, float* aabbs,
                           int32_t* iesc, int32_t* eesc, int32_t* unique) {
  if (!b) return XRT_ERR_INVALID_ARGUMENT;
  cudaSetDevice(b->device);
  return export_lbvh(b->b, b->stream, b->last_error, morton, objs, nodes, aabbs, iesc, eesc, unique);
}

xrt_status xrt_lbvh_query(xrt_lbvh* b, int32_t kind, const float* q, uint32_t nq, uint32_t* counts,
                          uint32_t* cands) {
  if (!b || (nq && (!q || !counts || !cands)) || kind < 0 || kind > 2) return XRT_ERR_INVALID_ARGUMENT;
  cudaSetDevice(b->device);
  if (nq == 0) return XRT_OK;
  if (!b->b.active) return XRT_ERR_STATE;
  const size_t per = kind == 0 ? 3 : 6;
  DBuf<float> dq;
  DBuf<uint32_t> dcount, dcand;
  if (dq.reserve(per * nq) || dcount.reserve(nq) || dcand.reserve((size_t)nq * xrt::kMaxCandidatesHost))
    return XRT_ERR_CUDA;
  xrt_status st = XRT_OK;
  if (cudaMemcpy(dq.p, q, per * 4 * nq, cudaMemcpyHostToDevice) != cudaSuccess) st = XRT_ERR_CUDA;
  if (st == XRT_OK) {
    xrt::launch_lbvh_query(b->b, kind, dq.p, nq, dcount.p, dcand.p, b->stream, b->err.p);
    if (cudaStreamSynchronize(b->stream) != cudaSuccess ||
        cudaMemcpy(counts, dcount.p, 4 * (size_t)nq, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(cands, dcand.p, 4 * (size_t)nq * xrt::kMaxCandidatesHost, cudaMemcpyDeviceToHost) !=
            cudaSuccess)
      st = XRT_ERR_CUDA;
  }
  dq.release();
  dcount.release();
  dcand.release();
  return st;
}

xrt_status xrt_lbvh_sizes(const xrt_lbvh* b, uint32_t* n) {
  if (!b || !n) return XRT_ERR_INVALID_ARGUMENT;
  *n = b->b.n;
  return XRT_OK;
}

}  // extern "C"
