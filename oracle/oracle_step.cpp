// oracle_step.cpp — TEST INFRASTRUCTURE ONLY: CPU restatement (C++17 + OpenMP) of the
// reference's Swift-mode cloth frame.  It is the checker for the CUDA library and the timed CPU
// baseline; nothing in the product links or calls it.  Every function names the reference
// file:line it restates.  Loops that the reference runs as one GPU thread per element are
// OpenMP-parallel only where the elements write disjoint data; scatter loops (float atomics in
// the reference) run sequentially in element order, which is the order the CUDA library's
// gathers reproduce.
//
// Frame:              ClothSolverBase::SimulateSwift          src/pipeline/base/ClothSolverBase.cpp:171-261
// predict/finalize:   PredictPositions_Kernel / Finalize_Kernel src/physics/ClothSolverHelper.cu:125-236
// stretch/bend:       SolveStretch_Kernel / SolveBend_Kernel   src/physics/dynamics/BasicSolverHelper.cu:8-138
// LRA:                SolveGeodesicLRA_Kernel                   src/physics/dynamics/LongRangeAttachments.cu:5-26
// binding:            GenerateBinding_Kernel/SolveBinding_Kernel src/physics/dynamics/BindingConstraint.cu:20-99
// obstacle contacts:  Generate*/Solve* kernels                  src/physics/pbd_collision/PBDCollision.cu:17-298
// particle contacts:  SpatialHashGPU + CollideParticles         src/physics/broad_phase/spatial_hash/SpatialHashGPU.cu:9-198,
//                                                               src/physics/ClothSolverHelper.cu:139-219
// normals/interp:     PhysicsMeshHelper.cu:196-310, PhysicsMesh.cu:604-620
// setup:              ClothSolverHelper.cpp:4-109, Geodesic.cpp:6-79, RTriangle.cu:19-84,
//                     universal/ClothSolver.cpp:46-350, PhysicsMeshHelper.cu:131-150
#include <algorithm>
#include <cstring>
#include <map>
#include <queue>
#include <set>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/xrt.h"
#include "../include/xrt_fem.h"
#include "oracle_lbvh.h"

using namespace orc;

namespace {

struct EEContact {
  float dist;
  V3 p2, q2;
  float s, t;
  V3 fn;
};

struct Binding {
  uint32_t cloth;
  float u, v, w;
  uint32_t iu, iv, iw;
  float L, stiffness;
};

struct Cloth {
  std::vector<V3> mesh_pos;
  std::vector<uint32_t> tri;  // local indices
  std::vector<uint32_t> fixed, attached;
  uint32_t offset = 0;
};

struct Oracle {
  xrt_swift_params p{};
  // cloth state
  std::vector<V3> x0, x, v, n, x_init;
  std::vector<float> w;
  std::vector<uint32_t> tri;
  std::vector<Cloth> cloths;
  std::vector<uint32_t> edges;  // 2E, global indices
  std::vector<float> rest, s_comp, s_lambda;
  std::vector<uint32_t> s_color;
  std::vector<uint32_t> bends;  // 4B
  std::vector<float> theta, b_comp;
  std::vector<uint32_t> b_color;
  uint32_t n_s_colors = 0, n_b_colors = 0;
  std::vector<uint32_t> lra_src, lra_tgt;
  std::vector<float> lra_rest;
  std::vector<Binding> bindings;
  std::vector<uint32_t> vf_prefix, vf_list;  // cloth vertex -> faces (ascending)
  float particle_diameter = 0.0f;
  // obstacle
  std::vector<V3> ox0, ox, ox1, on, on1;
  std::vector<uint32_t> otri, ortri, ovf_prefix, ovf_list;
  Lbvh bvh;
  // contacts
  std::vector<int32_t> vf_idx, rt_idx;
  std::vector<V3> vf_qs, rt_qc;
  std::vector<EEContact> ee;
  std::vector<V3> deltas;
  std::vector<int32_t> delta_counts;
  // particle hash
  std::vector<uint32_t> neighbors;
  std::vector<uint32_t> cell_start, cell_end;
  bool started = false;
  uint32_t frame_index = 0;
  std::vector<uint32_t> pending_colors[4];  // stretch, bend, FEM strain, FEM bending
  // FEM fabric (FEMHelper.cu): strain per cloth face, isometric bending per bend element
  bool fem_on = false;
  xrt_fem_material fem{};
  std::vector<float> fem_area, fem_inv;     // per face: area, inverse material matrix (glm order)
  std::vector<float> fem_q, fem_lambda;     // per bend element: row-major Hessian, multiplier
  std::vector<uint32_t> fem_color[2];
  uint32_t fem_ncolors[2] = {0, 0};
  // Quality-mode proximity repulsion / CCD impacts.  Unified numbering: cloth nodes, faces and
  // edges first, then the obstacle's (the reference addresses both through Node*/Face*/Edge*).
  std::vector<uint8_t> cfree;             // Node::is_free of cloth nodes (false when pinned)
  std::vector<V3> cmesh_pos, omesh_pos;   // registration-time positions (Face::n is set from them)
  std::vector<uint32_t> cface_edges, oface_edges;  // 3 per face: edge of (v_i, v_{i+1})
  std::vector<int32_t> cedge_adj, oedge_adj;       // 4 per edge: adjacent faces, -1 = none
  std::vector<uint32_t> crtri;
  std::vector<V3> cface_n0, oface_n0;
  std::vector<uint32_t> oedges;
  Lbvh cloth_bvh;
  std::vector<uint32_t> pairs;            // 2 per face pair (unified face ids)
  std::vector<V3> rep_deltas;
  std::vector<int32_t> rep_counts;
  struct Impact {
    float t;
    float w[4];
    V3 n;
    uint32_t nodes[4];
    int32_t is_vf;
  };
  std::vector<Impact> impacts;
  struct Quad {  // imminent-repulsion quadrature
    uint32_t nodes[4];
    float bary[4];
  };
  std::vector<Quad> quads;
  std::vector<V3> ov;  // obstacle Node::v: 0 until a collision step sets (x - x0) / dt
};

// ---------------------------------------------------------------------------------------------
// setup

// Edge list (our order): first appearance scanning faces, local edges (0,1),(1,2),(2,0), oriented
// as in that first face.  The reference takes vcglib's edge order, which is not reproducible
// without vcglib; both sides of every parity test use this rule.
void build_edges(const std::vector<uint32_t>& tri, uint32_t nv, std::vector<uint32_t>& e,
                 std::vector<std::vector<uint32_t>>& ef) {
  std::map<std::pair<uint32_t, uint32_t>, uint32_t> key;
  const uint32_t nf = (uint32_t)tri.size() / 3;
  for (uint32_t f = 0; f < nf; ++f) {
    for (int k = 0; k < 3; ++k) {
      uint32_t a = tri[f * 3 + k], b = tri[f * 3 + (k + 1) % 3];
      auto kk = std::make_pair(std::min(a, b), std::max(a, b));
      auto it = key.find(kk);
      if (it == key.end()) {
        uint32_t id = (uint32_t)(e.size() / 2);
        key.emplace(kk, id);
        e.push_back(a);
        e.push_back(b);
        ef.push_back({f});
      } else {
        ef[it->second].push_back(f);
      }
    }
  }
  (void)nv;
}

// GenerateBendingElements (ClothSolverHelper.cpp:4-88), including its string test for the
// winding of f1 (":find" of "idx1,idx2" in "a,b,c,a,b,c"), kept with its false positives.
void build_bends(const std::vector<V3>& pos, const std::vector<uint32_t>& tri,
                 const std::vector<uint32_t>& e, const std::vector<std::vector<uint32_t>>& ef,
                 uint32_t offset, std::vector<uint32_t>& out, std::vector<float>& angles) {
  const uint32_t ne = (uint32_t)e.size() / 2;
  for (uint32_t ei = 0; ei < ne; ++ei) {
    const auto& faces = ef[ei];
    if (faces.size() < 2) continue;  // border edge (IsB)
    uint32_t idx1 = e[ei * 2], idx2 = e[ei * 2 + 1];
    for (size_t i = 0; i < faces.size(); ++i) {
      for (size_t j = i + 1; j < faces.size(); ++j) {
        uint32_t f1 = faces[i], f2 = faces[j];
        auto opposite = [&](uint32_t f) {
          for (int k = 0; k < 3; ++k) {
            uint32_t vtx = tri[f * 3 + k];
            if (vtx != e[ei * 2] && vtx != e[ei * 2 + 1]) return vtx;
          }
          return tri[f * 3];
        };
        uint32_t idx3 = opposite(f1), idx4 = opposite(f2);
        std::string s = std::to_string(tri[f1 * 3 + 0]) + "," + std::to_string(tri[f1 * 3 + 1]) +
                        "," + std::to_string(tri[f1 * 3 + 2]);
        s += "," + s;
        const std::string common = std::to_string(idx1) + "," + std::to_string(idx2);
        const bool right_order = s.find(common) != std::string::npos;
        if (!right_order) std::swap(idx1, idx2);
        V3 v1 = pos[idx1], v2 = pos[idx2], v3 = pos[idx3], v4 = pos[idx4];
        V3 n1 = normalize(cross(v1 - v3, v2 - v3));
        V3 n2 = normalize(cross(v2 - v4, v1 - v4));
        float d = dot(n1, n2);
        if (d < -1) d = -1;
        else if (d > 1) d = 1;
        float th = std::acos(d);
        out.push_back(idx1 + offset);
        out.push_back(idx2 + offset);
        out.push_back(idx3 + offset);
        out.push_back(idx4 + offset);
        angles.push_back(th);
      }
    }
  }
}

// Geodesic::ComputeGeodesicDistance (src/utils/Geodesic.cpp:6-79): Dijkstra on the edge graph
// with float path lengths.
std::vector<float> geodesic(const std::vector<V3>& pos, const std::vector<std::vector<uint32_t>>& adj,
                            uint32_t src) {
  std::vector<float> dist(pos.size(), FLT_MAX);
  typedef std::pair<float, uint32_t> FP;
  std::priority_queue<FP, std::vector<FP>, std::greater<FP>> pq;
  dist[src] = 0;
  pq.push(FP(0.0f, src));
  while (!pq.empty()) {
    uint32_t cur = pq.top().second;
    pq.pop();
    for (uint32_t nb : adj[cur]) {
      float wgt = length(pos[nb] - pos[cur]);
      if (dist[nb] > dist[cur] + wgt) {
        dist[nb] = dist[cur] + wgt;
        pq.push(FP(dist[nb], nb));
      }
    }
  }
  return dist;
}

// Greedy coloring in constraint order (our deterministic stand-in for GraphColoring::Paint,
// src/physics/graph_coloring/Base.cu:163-317): smallest color unused by any earlier constraint
// sharing a vertex.
std::vector<uint32_t> greedy_color(const std::vector<uint32_t>& idx, int arity, uint32_t nv,
                                   uint32_t& ncolors) {
  const size_t n = idx.size() / arity;
  std::vector<uint32_t> col(n);
  std::vector<std::vector<uint32_t>> used(nv);
  ncolors = 0;
  for (size_t c = 0; c < n; ++c) {
    uint32_t k = 0;
    for (;; ++k) {
      bool clash = false;
      for (int a = 0; a < arity && !clash; ++a) {
        const auto& u = used[idx[c * arity + a]];
        clash = std::find(u.begin(), u.end(), k) != u.end();
      }
      if (!clash) break;
    }
    col[c] = k;
    for (int a = 0; a < arity; ++a) used[idx[c * arity + a]].push_back(k);
    ncolors = std::max(ncolors, k + 1);
  }
  return col;
}

bool coloring_valid(const std::vector<uint32_t>& idx, int arity, const std::vector<uint32_t>& col,
                    uint32_t nv) {
  std::vector<std::set<uint32_t>> used(nv);
  const size_t n = idx.size() / arity;
  for (size_t c = 0; c < n; ++c)
    for (int a = 0; a < arity; ++a)
      if (!used[idx[c * arity + a]].insert(col[c]).second) return false;
  return true;
}

// RTriBuild_Kernel (RTriangle.cu:19-84) over sorted VF adjacency lists.
std::vector<uint32_t> build_rtri(const std::vector<uint32_t>& tri, const std::vector<uint32_t>& pre,
                                 const std::vector<uint32_t>& list) {
  const uint32_t nf = (uint32_t)tri.size() / 3;
  std::vector<uint32_t> out(nf);
  for (uint32_t fid = 0; fid < nf; ++fid) {
    uint32_t fv[3] = {tri[fid * 3], tri[fid * 3 + 1], tri[fid * 3 + 2]};
    uint32_t info = 0, j_start = pre[fv[0]], j_end = pre[fv[0] + 1];
    for (uint32_t iv = 0; iv < 3; ++iv) {
      uint32_t off = j_start, i_end = j_end;
      uint32_t i_f = list[off++];
      if (i_f == fid) info |= (1u << iv);
      uint32_t jv = (iv + 1) % 3;
      j_start = pre[fv[jv]];
      j_end = pre[fv[jv] + 1];
      uint32_t of = 0xffffffffu;
      for (uint32_t jno = j_start; jno < j_end; ++jno) {
        if (list[jno] == i_f && fid != i_f) {
          of = i_f;
          break;
        }
      }
      for (; off < i_end && of == 0xffffffffu; ++off) {
        i_f = list[off];
        for (uint32_t jno = j_start; jno < j_end; ++jno) {
          if (list[jno] == i_f && fid != i_f) {
            of = i_f;
            break;
          }
        }
      }
      if (fid < of) info |= (1u << (iv + 3));
    }
    out[fid] = info;
  }
  return out;
}

void build_vf(const std::vector<uint32_t>& tri, uint32_t nv, std::vector<uint32_t>& pre,
              std::vector<uint32_t>& list) {
  std::vector<std::vector<uint32_t>> vf(nv);
  for (uint32_t f = 0; f < tri.size() / 3; ++f)
    for (int k = 0; k < 3; ++k) vf[tri[f * 3 + k]].push_back(f);
  pre.assign(nv + 1, 0);
  list.clear();
  for (uint32_t i = 0; i < nv; ++i) {
    std::sort(vf[i].begin(), vf[i].end());
    vf[i].erase(std::unique(vf[i].begin(), vf[i].end()), vf[i].end());
    list.insert(list.end(), vf[i].begin(), vf[i].end());
    pre[i + 1] = (uint32_t)list.size();
  }
}

// UpdateNodeNormals (PhysicsMeshHelper.cu:196-210, 282-295): area-weighted by 1/(|e0|^2|e1|^2),
// summed per vertex in ascending face order, then normalized.
void vertex_normals(const std::vector<V3>& pos, const std::vector<uint32_t>& tri,
                    const std::vector<uint32_t>& pre, const std::vector<uint32_t>& list,
                    std::vector<V3>& out) {
  const long nv = (long)pos.size();
  out.assign(nv, V3{0, 0, 0});
#pragma omp parallel for schedule(static)
  for (long i = 0; i < nv; ++i) {
    V3 acc{0, 0, 0};
    for (uint32_t k = pre[i]; k < pre[i + 1]; ++k) {
      uint32_t f = list[k];
      int j = 0;
      while (tri[f * 3 + j] != (uint32_t)i) ++j;
      V3 xi = pos[i];
      V3 e0 = pos[tri[f * 3 + (j + 1) % 3]] - xi;
      V3 e1 = pos[tri[f * 3 + (j + 2) % 3]] - xi;
      V3 c = cross(e0, e1) / (dot(e0, e0) * dot(e1, e1));
      acc.x += c.x;
      acc.y += c.y;
      acc.z += c.z;
    }
    out[i] = normalize(acc);
  }
}

// ---------------------------------------------------------------------------------------------
// particle hash (SpatialHashGPU.cu)

inline int int_coord(float value, float spacing) { return (int)std::floor(value / spacing); }
inline int hash_coords(int x, int y, int z, int table) {
  int32_t h = (int32_t)(((uint32_t)x * 92837111u) ^ ((uint32_t)y * 689287499u) ^
                        ((uint32_t)z * 283923481u));
  int32_t r = h % table;
  return r < 0 ? -r : r;
}

void hash_particles(Oracle& o) {
  const uint32_t nv = (uint32_t)o.x.size();
  const float spacing = o.particle_diameter * o.p.hash_cell_size;
  const float spacing2 = spacing * spacing;
  const float d2 = o.particle_diameter * o.particle_diameter;
  const int table = (int)(2 * nv);
  const uint32_t maxnb = (uint32_t)o.p.max_neighbor_size;
  std::vector<uint32_t> hash(nv), index(nv);
  for (uint32_t i = 0; i < nv; ++i) {
    V3 q = o.x[i];
    hash[i] = (uint32_t)hash_coords(int_coord(q.x, spacing), int_coord(q.y, spacing),
                                    int_coord(q.z, spacing), table);
    index[i] = i;
  }
  // cub::DeviceRadixSort::SortPairs is stable (SpatialHashGPU.cu:102-119)
  std::stable_sort(index.begin(), index.end(),
                   [&](uint32_t a, uint32_t b) { return hash[a] < hash[b]; });
  std::vector<uint32_t> sorted_hash(nv);
  for (uint32_t i = 0; i < nv; ++i) sorted_hash[i] = hash[index[i]];
  o.cell_start.assign(table, 0xffffffffu);
  if (o.cell_end.size() != (size_t)table) o.cell_end.assign(table, 0u);
  for (uint32_t id = 0; id < nv; ++id) {  // FindCellStart_Kernel
    uint32_t h = sorted_hash[id];
    if (id == 0 || h != sorted_hash[id - 1]) {
      o.cell_start[h] = id;
      if (id > 0) o.cell_end[sorted_hash[id - 1]] = id;
    }
    if (id == nv - 1) o.cell_end[h] = id + 1;
  }
  // thrust::device_vector::resize value-initialises the table (SpatialHashGPU.cu:173)
  if (o.neighbors.size() != (size_t)nv * maxnb) o.neighbors.assign((size_t)nv * maxnb, 0u);
#pragma omp parallel for schedule(dynamic, 256)
  for (long tid = 0; tid < (long)nv; ++tid) {  // CacheNeighbors_Kernel
    const uint32_t id = index[tid];
    const V3 pos = o.x[id];
    const V3 orig = o.x_init[id];
    const int ix = int_coord(pos.x, spacing), iy = int_coord(pos.y, spacing),
              iz = int_coord(pos.z, spacing);
    uint64_t ni = id;
    const uint64_t limit = (uint64_t)nv * maxnb;
    bool full = false;
    for (int xx = ix - 1; xx <= ix + 1 && !full; ++xx)
      for (int yy = iy - 1; yy <= iy + 1 && !full; ++yy)
        for (int zz = iz - 1; zz <= iz + 1 && !full; ++zz) {
          int h = hash_coords(xx, yy, zz, table);
          uint32_t start = o.cell_start[h];
          if (start == 0xffffffffu) continue;
          uint32_t end = std::min(o.cell_end[h], start + maxnb);
          for (uint32_t i = start; i < end; ++i) {
            uint32_t nb = index[i];
            V3 dp = pos - o.x[nb];
            V3 d0 = orig - o.x_init[nb];
            if (nb != id && dot(dp, dp) < spacing2 && dot(d0, d0) > d2) {
              o.neighbors[ni] = nb;
              ni += nv;
              if (ni >= limit) {
                full = true;
                break;
              }
            }
          }
        }
    if (!full && ni < limit) o.neighbors[ni] = 0xffffffffu;
  }
}

// ComputeFriction (ClothSolverHelper.cu:156-169)
inline V3 friction_of(float mu, V3 correction, V3 rel_vel) {
  V3 fr{0, 0, 0};
  float cl = length(correction);
  if (mu > 0.0f && cl > 0.0f) {
    V3 nrm = correction / cl;
    V3 tan_vel = rel_vel - nrm * dot(rel_vel, nrm);
    float tl = length(tan_vel);
    float max_tl = cl * mu;
    fr = -tan_vel * mmin(max_tl / tl, 1.0f);
  }
  return fr;
}

// ApplyDeltas_Kernel (ClothSolverHelper.cu:139-148)
void apply_deltas(Oracle& o) {
  const long nv = (long)o.x.size();
#pragma omp parallel for schedule(static)
  for (long i = 0; i < nv; ++i) {
    float count = (float)o.delta_counts[i];
    if (count > 0.0f) {
      o.x[i] += o.deltas[i] / count * o.p.relaxation_factor;
      o.deltas[i] = V3{0, 0, 0};
      o.delta_counts[i] = 0;
    }
  }
}

// CollideParticles_Kernel (ClothSolverHelper.cu:171-219) followed by ApplyDeltas.
void collide_particles(Oracle& o) {
  const uint32_t nv = (uint32_t)o.x.size();
  const uint64_t limit = (uint64_t)nv * (uint64_t)o.p.max_neighbor_size;
  const float dia = o.particle_diameter;
#pragma omp parallel for schedule(static)
  for (long id = 0; id < (long)nv; ++id) {
    V3 pd{0, 0, 0};
    int cnt = 0;
    V3 pred_i = o.x[id];
    V3 vel_i = pred_i - o.x0[id];
    float w_i = o.w[id];
    for (uint64_t k = (uint64_t)id; k < limit; k += nv) {
      uint32_t j = o.neighbors[k];
      if (j >= nv) break;  // reference: j > num_particles; j == nv never occurs
      float w_j = o.w[j];
      float denom = w_i + w_j;
      if (denom <= 0) continue;
      V3 pred_j = o.x[j];
      V3 diff = pred_i - pred_j;
      float distance = length(diff);
      if (distance >= dia) continue;
      V3 gradient = diff / (distance + kEps);
      float lambda = (distance - dia) / denom;
      V3 common = lambda * gradient;
      cnt++;
      pd -= w_i * common;
      V3 rel = vel_i - (pred_j - o.x0[j]);
      V3 fr = friction_of(o.p.friction, common, rel);
      pd += w_i * fr;
    }
    o.deltas[id] = pd;
    o.delta_counts[id] = cnt;
  }
  apply_deltas(o);
}

// ---------------------------------------------------------------------------------------------
// constraints

// SolveStretch_Kernel (BasicSolverHelper.cu:80-132)
void solve_stretch(Oracle& o, uint32_t color, float dt, int iter) {
  const long ne = (long)o.rest.size();
#pragma omp parallel for schedule(static)
  for (long id = 0; id < ne; ++id) {
    if (o.s_color[id] != color) continue;
    if (iter == 0) o.s_lambda[id] = 0.0f;
    uint32_t i1 = o.edges[id * 2], i2 = o.edges[id * 2 + 1];
    float expected = o.rest[id];
    V3 diff = o.x[i1] - o.x[i2];
    float distance = std::sqrt(fdot(diff, diff));
    float w1 = o.w[i1], w2 = o.w[i2];
    if (distance != expected && w1 + w2 > 0.0f) {
      V3 gradient = diff * (1.0f / (distance + kEps));
      float alpha_tilde = o.s_comp[id] / (dt * dt);
      float constraint = distance - expected;
      float dl = fma1(-alpha_tilde, o.s_lambda[id], -constraint) / (w1 + w2 + alpha_tilde);
      V3 corr = dl * gradient;
      o.s_lambda[id] = o.s_lambda[id] + dl;
      o.x[i1] = fmad(corr, w1, o.x[i1]);
      o.x[i2] = fmad(-corr, w2, o.x[i2]);
    }
  }
}

// SolveBend_Kernel (BasicSolverHelper.cu:8-72)
void solve_bend(Oracle& o, uint32_t color, float dt) {
  const long nb = (long)o.theta.size();
#pragma omp parallel for schedule(static)
  for (long id = 0; id < nb; ++id) {
    if (o.b_color[id] != color) continue;
    uint32_t i1 = o.bends[id * 4], i2 = o.bends[id * 4 + 1], i3 = o.bends[id * 4 + 2],
             i4 = o.bends[id * 4 + 3];
    float expected = o.theta[id];
    float w1 = o.w[i1], w2 = o.w[i2], w3 = o.w[i3], w4 = o.w[i4];
    V3 p1 = o.x[i1];
    V3 p2 = o.x[i2] - p1;
    V3 p3 = o.x[i3] - p1;
    V3 p4 = o.x[i4] - p1;
    V3 c23 = fcross(p2, p3), c24 = fcross(p2, p4);
    float l23 = std::sqrt(fdot(c23, c23)), l24 = std::sqrt(fdot(c24, c24));
    V3 n1 = c23 * (1.0f / l23);  // normalize
    V3 n2 = c24 * (1.0f / l24);
    float d = clampf(fdot(n1, n2), 0.0f, 1.0f);
    float angle = acos_as(d);  // the reference calls acos; see oracle_math.h
    if (angle < kEps || std::isnan(d)) continue;
    float r3 = 1.0f / (l23 + kEps);
    float r4 = 1.0f / (l24 + kEps);
    V3 q3 = fmad(fcross(n1, p2), d, fcross(p2, n2)) * r3;
    V3 q4 = fmad(fcross(n2, p2), d, fcross(p2, n1)) * r4;
    V3 q2 = -(fmad(fcross(n1, p3), d, fcross(p3, n2)) * r3) -
            fmad(fcross(n2, p4), d, fcross(p4, n1)) * r4;
    V3 q1 = -q2 - q3 - q4;
    float xpbd_bend = o.b_comp[id] / dt / dt;
    float denom = xpbd_bend + fma1(w4, fdot(q4, q4),
                                   fma1(w3, fdot(q3, q3), fma1(w2, fdot(q2, q2), w1 * fdot(q1, q1))));
    if (denom < kEps) continue;
    float lambda = std::sqrt(fma1(-d, d, 1.0f)) * (angle - expected) / denom;
    float scaling = 1.0f;
    o.x[i1] = fmad(q1, scaling * w1 * lambda, o.x[i1]);
    o.x[i2] = fmad(q2, scaling * w2 * lambda, o.x[i2]);
    o.x[i3] = fmad(q3, scaling * w3 * lambda, o.x[i3]);
    o.x[i4] = fmad(q4, scaling * w4 * lambda, o.x[i4]);
  }
}

// ---- FEM fabric ---------------------------------------------------------------------------
// ComputeStrainMeta (FEMHelper.cu:10-39) per cloth face and ComputeHessianEnergy
// (FEMHelper.cu:209-233) per bend element, from the initial world positions.  glm's matrices are
// column-major: P[c][r]; the inverse of a 2x2 is [m11, -m01; -m10, m00] / det in that layout.
void fem_setup(Oracle& o) {
  const size_t nf = o.tri.size() / 3, nb = o.bends.size() / 4;
  o.fem_area.assign(nf, 0.0f);
  o.fem_inv.assign(4 * nf, 0.0f);
  for (size_t f = 0; f < nf; ++f) {
    const V3 p0 = o.x0[o.tri[3 * f]], p1 = o.x0[o.tri[3 * f + 1]], p2 = o.x0[o.tri[3 * f + 2]];
    const V3 normal0 = cross(p1 - p0, p2 - p0);
    o.fem_area[f] = 0.5f * length(normal0);
    const V3 axis0_1 = normalize(p1 - p0);
    const V3 axis0_2 = normalize(cross(normal0, axis0_1));
    const float a0 = dot(p0, axis0_2), b0 = dot(p0, axis0_1);
    const float a1 = dot(p1, axis0_2), b1 = dot(p1, axis0_1);
    const float a2 = dot(p2, axis0_2), b2 = dot(p2, axis0_1);
    const float P00 = a0 - a2, P10 = b0 - b2, P01 = a1 - a2, P11 = b1 - b2;
    const float det = P00 * P11 - P10 * P01;
    float* inv = &o.fem_inv[4 * f];
    if (std::fabs(det) > kEps) {
      const float r = 1.0f / det;
      inv[0] = P11 * r;
      inv[1] = (-P01) * r;
      inv[2] = (-P10) * r;
      inv[3] = P00 * r;
    } else {
      inv[0] = inv[3] = 1.0f;
    }
  }
  o.fem_q.assign(16 * nb, 0.0f);
  o.fem_lambda.assign(nb, 0.0f);
  auto cot = [](V3 v, V3 w) { return dot(v, w) / length(cross(v, w)); };  // MathFunctions::CotTheta
  for (size_t b = 0; b < nb; ++b) {
    const V3 p0 = o.x0[o.bends[4 * b]], p1 = o.x0[o.bends[4 * b + 1]],
             p2 = o.x0[o.bends[4 * b + 2]], p3 = o.x0[o.bends[4 * b + 3]];
    const V3 e0 = p1 - p0, e1 = p2 - p0, e2 = p3 - p0, e3 = p2 - p1, e4 = p3 - p1;
    const float c01 = cot(e0, e1), c02 = cot(e0, e2), c03 = cot(-e0, e3), c04 = cot(-e0, e4);
    const float A0 = 0.5f * length(cross(p1 - p0, p2 - p0));
    const float A1 = 0.5f * length(cross(p0 - p1, p3 - p1));
    const float coeff = 3.0f / (A0 + A1);
    const float K[4] = {c03 + c04, c01 + c02, -c01 - c03, -c02 - c04};
    for (int j = 0; j < 4; ++j)
      for (int i = 0; i < 4; ++i) o.fem_q[16 * b + 4 * j + i] = coeff * (K[i] * K[j]);
  }
}

// SolveStrain_Kernel + ComputeStrainCorrection (FEMHelper.cu:96-207).
void solve_fem_strain(Oracle& o, uint32_t color) {
  const xrt_fem_material& m = o.fem;
  const float d = 1.0f - m.xy_poisson_ratio * m.yx_poisson_ratio;
  const float C00 = m.xx_stiffness / d, C01 = m.xx_stiffness * m.yx_poisson_ratio / d;
  const float C11 = m.yy_stiffness / d, C10 = m.yy_stiffness * m.xy_poisson_ratio / d;
  const float C22 = m.xy_stiffness;
  const long nf = (long)o.tri.size() / 3;
#pragma omp parallel for schedule(static)
  for (long f = 0; f < nf; ++f) {
    if (o.fem_color[0][f] != color) continue;
    const uint32_t i0 = o.tri[3 * f], i1 = o.tri[3 * f + 1], i2 = o.tri[3 * f + 2];
    const V3 p13 = o.x[i0] - o.x[i2], p23 = o.x[i1] - o.x[i2];
    const float* inv = &o.fem_inv[4 * f];
    const float F[3][2] = {{p13.x * inv[0] + p23.x * inv[2], p13.x * inv[1] + p23.x * inv[3]},
                           {p13.y * inv[0] + p23.y * inv[2], p13.y * inv[1] + p23.y * inv[3]},
                           {p13.z * inv[0] + p23.z * inv[2], p13.z * inv[1] + p23.z * inv[3]}};
    const float E00 = 0.5f * (F[0][0] * F[0][0] + F[1][0] * F[1][0] + F[2][0] * F[2][0] - 1.0f);
    const float E11 = 0.5f * (F[0][1] * F[0][1] + F[1][1] * F[1][1] + F[2][1] * F[2][1] - 1.0f);
    const float E01 = 0.5f * (F[0][0] * F[0][1] + F[1][0] * F[1][1] + F[2][0] * F[2][1]);
    const float S00 = C00 * E00 + C01 * E11, S11 = C10 * E00 + C11 * E11, S01 = C22 * E01;
    float Pk[3][2];
    for (int c = 0; c < 3; ++c) {
      Pk[c][0] = S00 * F[c][0] + S01 * F[c][1];
      Pk[c][1] = S01 * F[c][0] + S11 * F[c][1];
    }
    const float psi = 0.5f * (((E00 * S00 + E01 * S01) + E01 * S01) + E11 * S11);
    const float area = o.fem_area[f];
    const float energy = area * psi;
    V3 g0, g1;
    for (int c = 0; c < 3; ++c) {
      set(g0, c, (inv[0] * Pk[c][0] + inv[1] * Pk[c][1]) * area);
      set(g1, c, (inv[2] * Pk[c][0] + inv[3] * Pk[c][1]) * area);
    }
    const V3 g2 = -g0 - g1;
    const float w0 = o.w[i0], w1 = o.w[i1], w2 = o.w[i2];
    float sum = w0 * dot(g0, g0);
    sum = sum + w1 * dot(g1, g1);
    sum = sum + w2 * dot(g2, g2);
    if (!(std::fabs(sum) > kEps)) continue;
    const float s = energy / sum;
    if (w0 > kEps) o.x[i0] = o.x[i0] + (-(s * w0)) * g0;
    if (w1 > kEps) o.x[i1] = o.x[i1] + (-(s * w1)) * g1;
    if (w2 > kEps) o.x[i2] = o.x[i2] + (-(s * w2)) * g2;
  }
}

// SolveIsometricBending_Kernel (FEMHelper.cu:325-388).
void solve_iso_bend(Oracle& o, uint32_t color, float dt, int iter) {
  const float alpha = 1.0f / (o.fem.bending_stiffness * dt * dt);
  const long nb = (long)o.bends.size() / 4;
#pragma omp parallel for schedule(static)
  for (long b = 0; b < nb; ++b) {
    if (o.fem_color[1][b] != color) continue;
    if (iter == 0) o.fem_lambda[b] = 0.0f;
    const uint32_t id[4] = {o.bends[4 * b], o.bends[4 * b + 1], o.bends[4 * b + 2],
                            o.bends[4 * b + 3]};
    const float* Q = &o.fem_q[16 * b];
    const V3 x[4] = {o.x[id[0]], o.x[id[1]], o.x[id[2]], o.x[id[3]]};
    float energy = 0.0f;
    for (int k = 0; k < 4; ++k)
      for (int j = 0; j < 4; ++j) energy = energy + Q[4 * j + k] * dot(x[k], x[j]);
    energy = energy * 0.5f;
    if (std::fabs(energy) < kEps) continue;
    V3 d[4] = {};
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) d[j] = d[j] + Q[4 * j + i] * x[i];
    const float w[4] = {o.w[id[0]], o.w[id[1]], o.w[id[2]], o.w[id[3]]};
    const float coeff = (w[0] * dot(d[0], d[0]) + w[1] * dot(d[1], d[1])) +
                        (w[2] * dot(d[2], d[2]) + w[3] * dot(d[3], d[3]));
    const float dl = (-energy - alpha * o.fem_lambda[b]) / (coeff + alpha);
    for (int i = 0; i < 4; ++i) o.x[id[i]] = x[i] + (dl * w[i]) * d[i];
    o.fem_lambda[b] = o.fem_lambda[b] + dl;
  }
}

// SolveGeodesicLRA_Kernel (LongRangeAttachments.cu:5-26).  Constraints are applied in list order
// (slot-major); the reference's concurrent "+=" of several slots on one vertex is a race whose
// sequential order we fix.
void solve_lra(Oracle& o) {
  const size_t n = o.lra_rest.size();
  const float s = o.p.long_range_stretchiness;
  for (size_t c = 0; c < n; ++c) {
    uint32_t src = o.lra_src[c], tgt = o.lra_tgt[c];
    float target = o.lra_rest[c] * s;
    if (o.w[tgt] < kEps && target > 0) continue;
    V3 diff = o.x[tgt] - o.x[src];
    float dist = length(diff);
    if (dist > target) o.x[tgt] += -diff + diff / dist * target;
  }
}

// SolveBinding_Kernel (BindingConstraint.cu:56-92)
void solve_binding(Oracle& o) {
  for (const Binding& b : o.bindings) {
    V3 pc = o.x[b.cloth];
    float im = o.w[b.cloth];
    if (im < kEps) continue;
    V3 pu = o.ox[b.iu], pv = o.ox[b.iv], pw = o.ox[b.iw];
    V3 pob = b.u * pu + b.v * pv + b.w * pw;
    float C = length(pc - pob) - b.L;
    V3 nn = normalize(pc - pob);
    float s = im;
    s = C / s;
    if (C < 0.0f) continue;
    s *= b.stiffness;
    V3 dc = -s * im * nn;
    o.x[b.cloth] += dc;
  }
}

// ---------------------------------------------------------------------------------------------
// obstacle

// BVH::UpdateData (BVH.cu:382-421, 565-573) with ccd=false, then Construct(scr=0).
void rebuild_obstacle_bvh(Oracle& o, float tol) {
  const uint32_t nf = (uint32_t)o.otri.size() / 3;
  o.bvh.objects.resize(nf);
  for (uint32_t f = 0; f < nf; ++f) {
    uint32_t a = o.otri[f * 3], b = o.otri[f * 3 + 1], c = o.otri[f * 3 + 2];
    Prim& pr = o.bvh.objects[f];
    pr.idx1 = a;
    pr.idx2 = b;
    pr.idx3 = c;
    pr.v1 = o.ox0[a] + tol * o.on[a];
    pr.v2 = o.ox0[b] + tol * o.on[b];
    pr.v3 = o.ox0[c] + tol * o.on[c];
    pr.pred1 = pr.v1;
    pr.pred2 = pr.v2;
    pr.pred3 = pr.v3;
  }
  o.bvh.construct(0.0f);
}

// PhysicsMesh::Interpolate (PhysicsMesh.cu:610-620), UpdateMidstepNormals
// (PhysicsMeshHelper.cu:212-225, 297-310), BVH::RefitMidstep (BVH.cu:770-818).
void obstacle_pass(Oracle& o, int step, int num_steps) {
  const long nv = (long)o.ox.size();
  float alpha = ((float)step + 1.0f) / (float)num_steps;
  for (long i = 0; i < nv; ++i) o.ox1[i] = (1.0f - alpha) * o.ox0[i] + alpha * o.ox[i];
  vertex_normals(o.ox1, o.otri, o.ovf_prefix, o.ovf_list, o.on1);
  if (!o.bvh.active) return;
  const uint32_t n = o.bvh.num_objects(), ni = n - 1;
  const float tol = o.p.bvh_tolerance;
  for (uint32_t i = 0; i < n; ++i) {
    uint32_t k = ni + i;
    uint32_t obj = o.bvh.nodes[k].object;
    Prim& pr = o.bvh.objects[obj];
    uint32_t a = o.otri[obj * 3], b = o.otri[obj * 3 + 1], c = o.otri[obj * 3 + 2];
    pr.pred1 = o.ox1[a] + tol * o.on1[a];
    pr.pred2 = o.ox1[b] + tol * o.on1[b];
    pr.pred3 = o.ox1[c] + tol * o.on1[c];
    Box& bx = o.bvh.aabbs[k];
    bx = box_merge_point(bx, pr.pred1);
    bx = box_merge_point(bx, pr.pred2);
    bx = box_merge_point(bx, pr.pred3);
  }
  o.bvh.merge_internal_cas();
}

// GenerateVF_DCD_Kernel, GenerateVFCCD_Kernel, GenerateEE_DCD_Kernel (PBDCollision.cu)
void generate_contacts(Oracle& o) {
  const long nv = (long)o.x.size();
  const long ne = (long)o.rest.size();
  const Lbvh& bvh = o.bvh;
#pragma omp parallel for schedule(dynamic, 128)
  for (long i = 0; i < nv; ++i) {
    uint32_t buf[kMaxBuffer];
    // VF DCD
    {
      V3 pred = o.x[i];
      uint32_t nf = bvh.query_point(pred, buf);
      float hit = kScalarMax;
      int hit_idx = -1;
      V3 hit_qs{0, 0, 0};
      for (uint32_t k = 0; k < nf; ++k) {
        const Prim& pr = bvh.objects[buf[k]];
        V3 qs;
        float u, v, ww;
        float dist = nearest_point(pred, pr.pred1, pr.pred2, pr.pred3, qs, u, v, ww);
        if (dist < hit) {
          hit = dist;
          hit_qs = qs;
          hit_idx = (int)buf[k];
        }
      }
      o.vf_idx[i] = hit_idx;
      o.vf_qs[i] = hit_qs;
    }
    // VF CCD
    {
      o.rt_idx[i] = -1;
      o.rt_qc[i] = V3{0, 0, 0};
      V3 p1 = o.x0[i], p2 = o.x[i];
      V3 d = p2 - p1;
      const float len = length(d);
      if (!(len < kEps)) {
        d = d / len;
        uint32_t nf = bvh.query_segment(p1, p2, buf);
        float hit = kScalarMax;
        int hit_idx = -1;
        V3 qc{0, 0, 0};
        for (uint32_t k = 0; k < nf; ++k) {
          const Prim& pr = bvh.objects[buf[k]];
          float dist = ray_intersect(p1, d, len, pr.pred1, pr.pred2, pr.pred3);
          if (dist < hit) {
            qc = p1 + dist * d;
            hit = dist;
            hit_idx = (int)buf[k];
          }
        }
        o.rt_idx[i] = hit_idx;
        o.rt_qc[i] = qc;
      }
    }
  }
#pragma omp parallel for schedule(dynamic, 128)
  for (long e = 0; e < ne; ++e) {
    uint32_t buf[kMaxBuffer];
    uint32_t i1 = o.edges[e * 2], i2 = o.edges[e * 2 + 1];
    V3 pc = o.x[i1], qc = o.x[i2];
    uint32_t nf = bvh.query_segment(pc, qc, buf);
    float s = 0, t = 0;
    V3 p2{0, 0, 0}, q2{0, 0, 0}, fn{0, 0, 0};
    float min_dist = kScalarMax;
    for (uint32_t k = 0; k < nf; ++k) {
      uint32_t f = buf[k];
      const Prim& pr = bvh.objects[f];
      uint32_t info = o.ortri[f];
      V3 ov[3] = {pr.pred1, pr.pred2, pr.pred3};
      for (uint32_t a = 0; a < 3; ++a) {
        if ((info >> (a + 3u)) & 1u) {
          float _s, _t;
          V3 c1, c2;
          uint32_t b = (a + 1) % 3;
          if (closest_pt_segment_segment(pc, qc, ov[a], ov[b], _s, _t, c1, c2) != 0.0f) {
            V3 dd = c1 - c2;
            float dist = length(dd);
            if (dist < min_dist) {
              min_dist = dist;
              p2 = ov[a];
              q2 = ov[b];
              s = _s;
              t = _t;
              fn = face_normal(ov[0], ov[1], ov[2]);
            }
          }
        }
      }
    }
    o.ee[e] = EEContact{min_dist, p2, q2, s, t, fn};
  }
}

// SolveVFCCD_Kernel (PBDCollision.cu:279-298), SolveVFDCD_Kernel (:57-80),
// SolveEEDCD_Kernel (:163-212), ApplyDeltas.
void solve_contacts(Oracle& o) {
  const long nv = (long)o.x.size();
  const long ne = (long)o.rest.size();
#pragma omp parallel for schedule(static)
  for (long i = 0; i < nv; ++i) {
    if (o.rt_idx[i] == -1) continue;
    const Prim& pr = o.bvh.objects[o.rt_idx[i]];
    V3 nc = face_normal(pr.pred1, pr.pred2, pr.pred3);
    float lambda = dot(nc, o.x[i] - o.rt_qc[i]);
    if (lambda < 0) {
      V3 corr = -lambda * nc;
      o.x[i] += corr;
    }
  }
#pragma omp parallel for schedule(static)
  for (long i = 0; i < nv; ++i) {
    if (o.vf_idx[i] == -1) continue;
    const Prim& pr = o.bvh.objects[o.vf_idx[i]];
    V3 ns = face_normal(pr.pred1, pr.pred2, pr.pred3);
    float lambda = dot(ns, o.x[i] - o.vf_qs[i]) - 1e-3f;
    if (lambda < 0) {
      V3 corr = -lambda * ns;
      o.x[i] += corr;
    }
  }
  for (long e = 0; e < ne; ++e) {
    const EEContact& c = o.ee[e];
    if (c.dist > 1e6f) continue;
    uint32_t i1 = o.edges[e * 2], i2 = o.edges[e * 2 + 1];
    V3 p1 = o.x[i1], q1 = o.x[i2];
    float s = c.s, t = c.t;
    V3 c1 = (1 - s) * p1 + s * q1;
    V3 c2 = (1 - t) * c.p2 + t * c.q2;
    V3 d = c1 - c2;
    float len = length(d);
    if (len < kEps) continue;
    float proj = dot(d, c.fn) - 1e-3f;
    float lambda = proj;
    if (lambda > 0) continue;
    V3 corr1 = -(1 - s) * lambda * c.fn;
    V3 corr2 = -(s)*lambda * c.fn;
    o.deltas[i1] += corr1;
    o.deltas[i2] += corr2;
    o.delta_counts[i1] += 1;
    o.delta_counts[i2] += 1;
  }
  apply_deltas(o);
}

// ---------------------------------------------------------------------------------------------
// Quality-mode proximity repulsion and CCD impacts
//   UpdatePairs / Traverse ........ src/physics/repulsion/PBDRepulsion.cu:22-32,
//                                   src/physics/broad_phase/lbvh/BVH.cu:1149-1227, 1315-1340
//   BVH::Update(ccd) .............. BVH.cu:820-852
//   EvaluateRep / ApplyPBDImpulse . PBDRepulsion.cu:264-313, 329-515
//   Proximity ctor ................ src/physics/repulsion/Proximity.cu:10-37
//   signed distances / InEdge ..... src/math/BasicPrimitiveTests.cu:286-301, 369-436
//   CheckImpact(s) ................ src/physics/impact_zone/ImpactHelper.cu:34-177

struct UNodes {  // unified node view: cloth then obstacle
  const Oracle& o;
  uint32_t V;
  explicit UNodes(const Oracle& oo) : o(oo), V((uint32_t)oo.x.size()) {}
  V3 x(uint32_t i) const { return i < V ? o.x[i] : o.ox[i - V]; }
  V3 x0(uint32_t i) const { return i < V ? o.x0[i] : o.ox0[i - V]; }
  float w(uint32_t i) const { return i < V ? o.w[i] : 1.0f / 1e3f; }  // PhysicsMeshHelper.cu:148
  bool free_(uint32_t i) const { return i < V ? o.cfree[i] != 0 : false; }
  uint32_t F() const { return (uint32_t)o.tri.size() / 3; }
  uint32_t E() const { return (uint32_t)o.edges.size() / 2; }
  uint32_t fnode(uint32_t f, int k) const {
    return f < F() ? o.tri[f * 3 + k] : V + o.otri[(f - F()) * 3 + k];
  }
  uint32_t fedge(uint32_t f, int k) const {
    return f < F() ? o.cface_edges[f * 3 + k] : E() + o.oface_edges[(f - F()) * 3 + k];
  }
  uint32_t frtri(uint32_t f) const { return f < F() ? o.crtri[f] : o.ortri[f - F()]; }
  V3 fn0(uint32_t f) const { return f < F() ? o.cface_n0[f] : o.oface_n0[f - F()]; }
  bool ffree(uint32_t f) const { return free_(fnode(f, 0)) && free_(fnode(f, 1)) && free_(fnode(f, 2)); }
  uint32_t enode(uint32_t e, int k) const {
    return e < E() ? o.edges[e * 2 + k] : V + o.oedges[(e - E()) * 2 + k];
  }
  int32_t eadj(uint32_t e, int k) const {
    if (e < E()) return o.cedge_adj[e * 4 + k];
    int32_t a = o.oedge_adj[(e - E()) * 4 + k];
    return a < 0 ? -1 : (int32_t)(F() + (uint32_t)a);
  }
  bool efree(uint32_t e) const { return free_(enode(e, 0)) && free_(enode(e, 1)); }
};

inline float mixed(V3 a, V3 b, V3 c) { return dot(a, cross(b, c)); }

// SignedVertexFaceDistance (BasicPrimitiveTests.cu:369-386).  On a degenerate face the reference
// returns before writing w; here w stays at the caller's zeros.
float signed_vf_distance(V3 x, V3 y0, V3 y1, V3 y2, V3& n, float* w) {
  n = cross(normalize(y1 - y0), normalize(y2 - y0));
  if (dot(n, n) < 1e-6f) return std::numeric_limits<float>::infinity();
  n = normalize(n);
  float h = dot(x - y0, n);
  float b0 = mixed(y1 - x, y2 - x, n);
  float b1 = mixed(y2 - x, y0 - x, n);
  float b2 = mixed(y0 - x, y1 - x, n);
  w[0] = 1.0f;
  w[1] = -b0 / (b0 + b1 + b2);
  w[2] = -b1 / (b0 + b1 + b2);
  w[3] = -b2 / (b0 + b1 + b2);
  return h;
}

// SignedEdgeEdgeDistance (BasicPrimitiveTests.cu:420-436); its glm::normalize(n) result is
// discarded in the reference, so n stays unnormalized.
float signed_ee_distance(V3 x0, V3 x1, V3 y0, V3 y1, V3& n, float* w) {
  n = cross(normalize(x1 - x0), normalize(y1 - y0));
  if (dot(n, n) < 1e-6f) return std::numeric_limits<float>::infinity();
  float h = dot(x0 - y0, n);
  float a0 = mixed(y1 - x1, y0 - x1, n);
  float a1 = mixed(y0 - x0, y1 - x0, n);
  float b0 = mixed(x0 - y1, x1 - y1, n);
  float b1 = mixed(x1 - y0, x0 - y0, n);
  w[0] = a0 / (a0 + a1);
  w[1] = a1 / (a0 + a1);
  w[2] = -b0 / (b0 + b1);
  w[3] = -b1 / (b0 + b1);
  return h;
}

// InEdge (BasicPrimitiveTests.cu:286-301): Face::n is the normal set at registration.
bool in_edge(const UNodes& u, float wt, uint32_t e0, uint32_t e1) {
  V3 xx = (1 - wt) * u.x(u.enode(e0, 0)) + wt * u.x(u.enode(e0, 1));
  bool in = true;
  for (int k = 0; k < 4; ++k) {
    int32_t f = u.eadj(e1, k);
    if (f < 0) continue;
    V3 e = u.x(u.enode(e1, 1)) - u.x(u.enode(e1, 0));
    V3 nn = u.fn0((uint32_t)f);
    V3 r = xx - u.x(u.enode(e1, 0));
    in &= (mixed(e, nn, r) >= 0);
  }
  return in;
}

// Edge::ComputeNormal (src/memory/Edge.cu:42-59)
V3 edge_normal(const UNodes& u, uint32_t e) {
  V3 ans{0, 0, 0};
  int cnt = 0;
  for (int k = 0; k < 4; ++k) {
    int32_t f = u.eadj(e, k);
    if (f < 0) break;
    ans += face_normal(u.x(u.fnode(f, 0)), u.x(u.fnode(f, 1)), u.x(u.fnode(f, 2)));
    cnt++;
  }
  if (cnt == 0) return ans;
  return ans / (float)cnt;
}

struct Impulse {
  uint32_t nodes[4];
  V3 corr[4];
};

// EvaluateVFProximity (PBDRepulsion.cu:329-409) with the Proximity(node, face) normal rule.
bool evaluate_vf(const UNodes& u, uint32_t node, uint32_t face, float h, Impulse& imp) {
  const uint32_t f0 = u.fnode(face, 0), f1 = u.fnode(face, 1), f2 = u.fnode(face, 2);
  if (node == f0 || node == f1 || node == f2) return false;
  const uint32_t nd[4] = {node, f0, f1, f2};
  V3 pn;
  float pw[4] = {0, 0, 0, 0};
  float d0 = signed_vf_distance(u.x0(nd[0]), u.x0(nd[1]), u.x0(nd[2]), u.x0(nd[3]), pn, pw);
  if (d0 < 0.0f && u.ffree(face)) pn = -pn;
  V3 fn;
  float w[4] = {0, 0, 0, 0};
  signed_vf_distance(u.x(nd[0]), u.x(nd[1]), u.x(nd[2]), u.x(nd[3]), fn, w);
  bool inside = mmin(-w[1], mmin(-w[2], -w[3])) >= 1e-6f;
  if (!inside) return false;
  V3 n = face_normal(u.x(nd[1]), u.x(nd[2]), u.x(nd[3]));
  float side = dot(n, pn) > 0.0f ? 1.0f : -1.0f;
  V3 q = u.x(nd[0]), p1 = u.x(nd[1]), p2 = u.x(nd[2]), p3 = u.x(nd[3]);
  q = q - p1;
  p2 = p2 - p1;
  p3 = p3 - p1;
  n = side * cross(p2, p3);
  float c23 = length(n);
  n = normalize(n);
  float C = dot(q, n) - h;
  if (C > 0) return false;
  V3 dcq = n;
  V3 dcp2 = (cross(p3, q) + cross(n, p3) * dot(n, q)) / c23;
  V3 dcp3 = -(cross(p2, q) + cross(n, p2) * dot(n, q)) / c23;
  V3 dcp1 = -dcq - dcp2 - dcp3;
  float denom = u.w(nd[0]) * dot(dcq, dcq) + u.w(nd[1]) * dot(dcp1, dcp1) +
                u.w(nd[2]) * dot(dcp2, dcp2) + u.w(nd[3]) * dot(dcp3, dcp3);
  if (denom < kEps) return false;
  float s = C / denom;
  imp.corr[0] = -u.w(nd[0]) * s * dcq;
  imp.corr[1] = -u.w(nd[1]) * s * dcp1;
  imp.corr[2] = -u.w(nd[2]) * s * dcp2;
  imp.corr[3] = -u.w(nd[3]) * s * dcp3;
  for (int k = 0; k < 4; ++k) imp.nodes[k] = nd[k];
  return true;
}

// EvaluateEEProximity (PBDRepulsion.cu:411-468) with the Proximity(edge, edge) normal rule.
bool evaluate_ee(const UNodes& u, uint32_t e0, uint32_t e1, float h, Impulse& imp) {
  const uint32_t nd[4] = {u.enode(e0, 0), u.enode(e0, 1), u.enode(e1, 0), u.enode(e1, 1)};
  if (nd[0] == nd[2] || nd[0] == nd[3] || nd[1] == nd[2] || nd[1] == nd[3]) return false;
  V3 pn;
  float pw[4] = {0, 0, 0, 0};
  float d0 = signed_ee_distance(u.x0(nd[0]), u.x0(nd[1]), u.x0(nd[2]), u.x0(nd[3]), pn, pw);
  if (!u.efree(e1)) {
    pn = edge_normal(u, e1);
  } else if (d0 < 0.0f) {
    pn = -pn;
  }
  V3 ln;
  float b[4] = {0, 0, 0, 0};
  signed_ee_distance(u.x(nd[0]), u.x(nd[1]), u.x(nd[2]), u.x(nd[3]), ln, b);
  bool inside = mmin(mmin(b[0], b[1]), mmin(-b[2], -b[3])) >= 1e-6f && in_edge(u, b[1], e0, e1) &&
                in_edge(u, -b[3], e1, e0);
  if (!inside) return false;
  V3 d{0, 0, 0};
  for (int k = 0; k < 4; ++k) d += b[k] * u.x(nd[k]);
  V3 n = pn;
  float C = dot(d, n) - h;
  if (C > 0) return false;
  b[2] *= -1;
  b[3] *= -1;
  V3 grads[4] = {b[0] * n, b[1] * n, -b[2] * n, -b[3] * n};
  float denom = 0;
  for (int k = 0; k < 4; ++k) denom += u.w(nd[k]) * b[k] * b[k];
  if (denom < kEps) return false;
  float s = C / denom;
  for (int k = 0; k < 4; ++k) {
    imp.nodes[k] = nd[k];
    imp.corr[k] = -s * u.w(nd[k]) * grads[k];
  }
  return true;
}

// BVH::UpdateData(faces, 0, false) + Construct() of the cloth (ClothSolverBase.cpp:277-278).
void build_cloth_bvh(Oracle& o) {
  const uint32_t nf = (uint32_t)o.tri.size() / 3;
  o.cloth_bvh.objects.resize(nf);
  for (uint32_t f = 0; f < nf; ++f) {
    Prim& pr = o.cloth_bvh.objects[f];
    uint32_t a = o.tri[f * 3], b = o.tri[f * 3 + 1], c = o.tri[f * 3 + 2];
    pr.idx1 = a; pr.idx2 = b; pr.idx3 = c;
    pr.v1 = o.x0[a] + 0.0f * o.n[a];
    pr.v2 = o.x0[b] + 0.0f * o.n[b];
    pr.v3 = o.x0[c] + 0.0f * o.n[c];
    pr.pred1 = pr.v1; pr.pred2 = pr.v2; pr.pred3 = pr.v3;
  }
  o.cloth_bvh.construct(0.0f);
}

// BVH::Update(faces, ccd = true) (BVH.cu:820-852): pred = x, leaves grow by the x/x0 bounds of
// their face, internal boxes become the union of their leaves.
void update_bvh_ccd(Lbvh& b, const std::vector<V3>& x, const std::vector<V3>& x0,
                    const std::vector<uint32_t>& tri) {
  if (!b.active) return;
  const uint32_t n = b.num_objects(), ni = n - 1;
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t k = ni + i, obj = b.nodes[k].object;
    const uint32_t id[3] = {tri[obj * 3], tri[obj * 3 + 1], tri[obj * 3 + 2]};
    Prim& pr = b.objects[obj];
    pr.pred1 = x[id[0]];
    pr.pred2 = x[id[1]];
    pr.pred3 = x[id[2]];
    Box fb;  // Face::ComputeBounds(true)
    for (int c = 0; c < 3; ++c) {
      fb = box_merge_point(fb, x[id[c]]);
      fb = box_merge_point(fb, x0[id[c]]);
    }
    b.aabbs[k] = box_merge(b.aabbs[k], fb);
  }
  b.merge_internal_cas();
}

// CountPairs_Kernel + inclusive scan + FindPairs_Kernel (BVH.cu:1149-1227, 1315-1340): pairs of
// one query are written back to front.
void traverse_pairs(const Lbvh& lhs, const Lbvh& rhs, uint32_t lhs_face_base,
                    uint32_t rhs_face_base, float thickness, std::vector<uint32_t>& out) {
  if (!lhs.active || !rhs.active) return;
  const uint32_t nq = lhs.num_objects(), nil = nq - 1, nir = rhs.num_objects() - 1;
  std::vector<std::vector<uint32_t>> hits(nq);
  for (uint32_t id = 0; id < nq; ++id) {
    Box q = lhs.aabbs[nil + id];
    for (int i = 0; i < 3; ++i) {  // Bounds::Dilate
      set(q.lo, i, get(q.lo, i) - thickness);
      set(q.hi, i, get(q.hi, i) + thickness);
    }
    int node = 0;
    while (node != -1) {
      const BVNode& nd = rhs.nodes[node];
      if (box_overlap_box(rhs.aabbs[node], q)) {
        if (nd.object != kNone) {
          hits[id].push_back(nd.object);
          node = rhs.eesc[node - nir];
        } else {
          node = (int)nd.left;
        }
      } else {
        node = nd.object != kNone ? rhs.eesc[node - nir] : rhs.iesc[node];
      }
    }
  }
  for (uint32_t id = 0; id < nq; ++id) {
    const uint32_t obj = lhs.nodes[nil + id].object;
    for (size_t k = hits[id].size(); k-- > 0;) {
      out.push_back(lhs_face_base + obj);
      out.push_back(rhs_face_base + hits[id][k]);
    }
  }
}

// PBDRepulsionSolver::UpdatePairs (PBDRepulsion.cu:22-32)
void update_pairs(Oracle& o, float thickness) {
  update_bvh_ccd(o.cloth_bvh, o.x, o.x0, o.tri);
  o.pairs.clear();
  const uint32_t F = (uint32_t)o.tri.size() / 3;
  traverse_pairs(o.cloth_bvh, o.bvh, 0, F, thickness, o.pairs);
  traverse_pairs(o.cloth_bvh, o.cloth_bvh, 0, 0, thickness, o.pairs);
}

// EvaluateRep_Kernel + ApplyPBDImpulse_Kernel (PBDRepulsion.cu:470-515, 299-313); the deltas
// are summed in pair order (float atomics in the reference).
void solve_repulsion(Oracle& o, float h, float relaxation) {
  UNodes u(o);
  const uint32_t V = u.V;
  o.rep_deltas.assign(V, V3{0, 0, 0});
  o.rep_counts.assign(V, 0);
  auto accumulate = [&](const Impulse& imp) {
    for (int k = 0; k < 4; ++k) {
      if (length(imp.corr[k]) < kEps) continue;
      if (!u.free_(imp.nodes[k])) continue;
      o.rep_deltas[imp.nodes[k]] += imp.corr[k];
      o.rep_counts[imp.nodes[k]] += 1;
    }
  };
  const size_t np = o.pairs.size() / 2;
  for (size_t p = 0; p < np; ++p) {
    const uint32_t f0 = o.pairs[2 * p], f1 = o.pairs[2 * p + 1];
    const uint32_t r0 = u.frtri(f0), r1 = u.frtri(f1);
    for (int i = 0; i < 3; ++i) {
      if (!((r0 >> i) & 1u)) continue;
      Impulse imp;
      if (evaluate_vf(u, u.fnode(f0, i), f1, h, imp)) accumulate(imp);
    }
    for (int i = 0; i < 3; ++i) {
      if (!((r0 >> (i + 3)) & 1u)) continue;
      for (int j = 0; j < 3; ++j) {
        if (!((r1 >> (j + 3)) & 1u)) continue;
        Impulse imp;
        if (evaluate_ee(u, u.fedge(f0, i), u.fedge(f1, j), h, imp)) accumulate(imp);
      }
    }
  }
  for (uint32_t i = 0; i < V; ++i) {
    float count = (float)o.rep_counts[i];
    if (count <= kEps) continue;
    V3 dx = o.rep_deltas[i] / count * relaxation;
    o.x[i] = o.x[i] + dx;
  }
}

// ImminentRepulsion::UpdateProximity + Generate (ImminentRepulsion.cu:21-102,
// ImminentRepulsionHelper.cu:10-66): pairs cloth x cloth then cloth x obstacle (thickness 1e-6),
// edge-edge quadratures of every pair, then vertex-face ones, at x0.
void imminent_generate(Oracle& o) {
  UNodes u(o);
  std::vector<uint32_t> pairs;
  traverse_pairs(o.cloth_bvh, o.cloth_bvh, 0, 0, 1e-6f, pairs);
  traverse_pairs(o.cloth_bvh, o.bvh, 0, u.F(), 1e-6f, pairs);
  o.quads.clear();
  const size_t np = pairs.size() / 2;
  for (int pass = 0; pass < 2; ++pass) {
    for (size_t p = 0; p < np; ++p) {
      const uint32_t f0 = pairs[2 * p], f1 = pairs[2 * p + 1];
      if (f0 == f1) continue;
      const uint32_t r0 = u.frtri(f0), r1 = u.frtri(f1);
      if (pass == 0) {  // CheckImminentEEQuadrature
        for (int i = 0; i < 3; ++i) {
          if (!((r0 >> (i + 3)) & 1u)) continue;
          for (int j = 0; j < 3; ++j) {
            if (!((r1 >> (j + 3)) & 1u)) continue;
            const uint32_t e0 = u.fedge(f0, i), e1 = u.fedge(f1, j);
            const uint32_t nd[4] = {u.enode(e0, 0), u.enode(e0, 1), u.enode(e1, 0), u.enode(e1, 1)};
            if (nd[0] == nd[2] || nd[0] == nd[3] || nd[1] == nd[2] || nd[1] == nd[3]) continue;
            V3 fn;
            float w[4] = {0, 0, 0, 0};
            signed_ee_distance(u.x0(nd[0]), u.x0(nd[1]), u.x0(nd[2]), u.x0(nd[3]), fn, w);
            if (!(mmin(mmin(w[0], w[1]), mmin(-w[2], -w[3])) >= 1e-6f && in_edge(u, w[1], e0, e1) &&
                  in_edge(u, -w[3], e1, e0)))
              continue;
            o.quads.push_back(Oracle::Quad{{nd[0], nd[1], nd[2], nd[3]}, {w[0], w[1], w[2], w[3]}});
          }
        }
      } else {  // CheckImminentVFQuadrature
        for (int i = 0; i < 3; ++i) {
          if (!((r0 >> i) & 1u)) continue;
          const uint32_t node = u.fnode(f0, i);
          const uint32_t a = u.fnode(f1, 0), b = u.fnode(f1, 1), c = u.fnode(f1, 2);
          if (node == a || node == b || node == c) continue;
          V3 fn;
          float w[4] = {0, 0, 0, 0};
          signed_vf_distance(u.x0(node), u.x0(a), u.x0(b), u.x0(c), fn, w);
          if (!(mmin(-w[1], mmin(-w[2], -w[3])) >= 1e-6f)) continue;
          o.quads.push_back(Oracle::Quad{{a, b, c, node}, {w[1], w[2], w[3], w[0]}});
        }
      }
    }
  }
}

// ImminentRepulsion::Solve (ImminentRepulsion.cu:104-169) with add_repulsion = true: cloth
// velocities (x - x0) / dt, EvaluateImminentImpulse of every quadrature, deltas summed in
// quadrature order, ApplyImminentImpulse.
void imminent_solve(Oracle& o, float h, float relaxation, float dt) {
  UNodes u(o);
  const uint32_t V = u.V;
  if (o.ov.size() != o.ox.size()) o.ov.assign(o.ox.size(), V3{0, 0, 0});
  for (uint32_t i = 0; i < V; ++i) o.v[i] = (o.x[i] - o.x0[i]) / dt;
  o.rep_deltas.assign(V, V3{0, 0, 0});
  o.rep_counts.assign(V, 0);
  for (const Oracle::Quad& q : o.quads) {
    V3 pr{0, 0, 0}, vr{0, 0, 0};
    for (int i = 0; i < 4; ++i) {
      pr = pr + q.bary[i] * u.x0(q.nodes[i]);
      vr = vr + q.bary[i] * (q.nodes[i] < V ? o.v[q.nodes[i]] : o.ov[q.nodes[i] - V]);
    }
    const float npr = length(pr);
    if (npr > h || npr < 1e-5f) continue;
    pr = normalize(pr);
    const float vr_nrm = dot(vr, pr);
    if (vr_nrm > (h - npr) * 0.1f) continue;
    V3 I = (vr_nrm * dt) * pr;
    const V3 vr_tan = vr - vr_nrm * pr;
    if (length(vr_tan) > h * 0.01f) {  // friction coefficient 0
      const float imp_norm = length(I), coeff = 0.0f;
      const V3 dir = normalize(vr_tan);
      const V3 friction = imp_norm * coeff > length(vr_tan) ? -vr_tan : (-dir * imp_norm) * coeff;
      I = I + friction * 1.0f;
    }
    float inv_cm = 0.0f;
    for (int i = 0; i < 4; ++i) inv_cm += (q.bary[i] * q.bary[i]) * u.w(q.nodes[i]);
    if (inv_cm < 1e-5f) continue;
    for (int i = 0; i < 4; ++i) {  // AccumulateImpulses
      const V3 corr = I * ((-u.w(q.nodes[i]) * q.bary[i]) / inv_cm);
      if (length(corr) < kEps || !u.free_(q.nodes[i])) continue;
      o.rep_deltas[q.nodes[i]] += corr;
      o.rep_counts[q.nodes[i]] += 1;
    }
  }
  for (uint32_t i = 0; i < V; ++i) {
    float count = (float)o.rep_counts[i];
    if (count <= kEps) continue;
    o.x[i] = o.x[i] + o.rep_deltas[i] / count * relaxation;
  }
}

// CheckImpact (ImpactHelper.cu:34-87)
bool check_impact(const UNodes& u, bool vf, const uint32_t* nd, Oracle::Impact& im) {
  for (int k = 0; k < 4; ++k) im.nodes[k] = nd[k];
  V3 x0 = u.x0(nd[0]);
  V3 v0 = u.x(nd[0]) - x0;
  V3 x1 = u.x0(nd[1]) - x0, x2 = u.x0(nd[2]) - x0, x3 = u.x0(nd[3]) - x0;
  V3 v1 = (u.x(nd[1]) - u.x0(nd[1])) - v0;
  V3 v2 = (u.x(nd[2]) - u.x0(nd[2])) - v0;
  V3 v3 = (u.x(nd[3]) - u.x0(nd[3])) - v0;
  float a0 = mixed(x1, x2, x3);
  float a1 = mixed(v1, x2, x3) + mixed(x1, v2, x3) + mixed(x1, x2, v3);
  float a2 = mixed(x1, v2, v3) + mixed(v1, x2, v3) + mixed(v1, v2, x3);
  float a3 = mixed(v1, v2, v3);
  float t[3];
  int ns = solve_cubic(a3, a2, a1, a0, t);
  for (int i = 0; i < ns; ++i) {
    if (t[i] < 0 || t[i] > 1) continue;
    im.t = t[i];
    auto pos = [&](uint32_t id) { return u.x0(id) + t[i] * (u.x(id) - u.x0(id)); };
    V3 p0 = pos(nd[0]), p1 = pos(nd[1]), p2 = pos(nd[2]), p3 = pos(nd[3]);
    float d;
    bool inside;
    if (vf) {
      d = signed_vf_distance(p0, p1, p2, p3, im.n, im.w);
      inside = mmin(-im.w[1], mmin(-im.w[2], -im.w[3])) >= -1e-6f;
    } else {
      d = signed_ee_distance(p0, p1, p2, p3, im.n, im.w);
      inside = mmin(mmin(im.w[0], im.w[1]), mmin(-im.w[2], -im.w[3])) >= -1e-6f;
    }
    if (dot(im.n, im.w[1] * v1 + im.w[2] * v2 + im.w[3] * v3) > 0) im.n = -im.n;
    if (mabs(d) < 1e-6f && inside) return true;
  }
  return false;
}

Box node_bounds(const UNodes& u, const uint32_t* ids, int count) {  // ComputeBounds(ccd = true)
  Box b;
  for (int k = 0; k < count; ++k) {
    b = box_merge_point(b, u.x(ids[k]));
    b = box_merge_point(b, u.x0(ids[k]));
  }
  return b;
}

bool overlap_dilated(const Box& a, const Box& b, float thickness) {  // Bounds::Overlap(b, h)
  Box d = b;
  for (int i = 0; i < 3; ++i) {
    set(d.lo, i, get(d.lo, i) - thickness);
    set(d.hi, i, get(d.hi, i) + thickness);
  }
  return box_overlap_box(a, d);
}

// CheckImpacts_Kernel (ImpactHelper.cu:116-171): 6 vertex-face and 9 edge-edge tests per pair.
void check_impacts(Oracle& o, float thickness) {
  UNodes u(o);
  const size_t np = o.pairs.size() / 2;
  o.impacts.assign(np * 15, Oracle::Impact{});
  for (size_t p = 0; p < np; ++p) {
    const uint32_t fa = o.pairs[2 * p], fb = o.pairs[2 * p + 1];
    size_t index = 15 * p;
    for (int side = 0; side < 2; ++side) {
      const uint32_t f0 = side == 0 ? fa : fb, f1 = side == 0 ? fb : fa;
      for (int i = 0; i < 3; ++i) {
        Oracle::Impact& im = o.impacts[index++];
        im.is_vf = 1;
        const uint32_t nd[4] = {u.fnode(f0, i), u.fnode(f1, 0), u.fnode(f1, 1), u.fnode(f1, 2)};
        for (int k = 0; k < 4; ++k) {
          im.nodes[k] = nd[k];
          im.w[k] = 0;
        }
        bool ok = false;
        if (!(nd[0] == nd[1] || nd[0] == nd[2] || nd[0] == nd[3])) {
          const uint32_t fn3[3] = {nd[1], nd[2], nd[3]};
          if (overlap_dilated(node_bounds(u, nd, 1), node_bounds(u, fn3, 3), thickness))
            ok = check_impact(u, true, nd, im);
        }
        if (!ok) im.t = -1;
      }
    }
    for (int i = 0; i < 3; ++i) {
      for (int j = 0; j < 3; ++j) {
        Oracle::Impact& im = o.impacts[index++];
        im.is_vf = 0;
        const uint32_t ea = u.fedge(fa, i), eb = u.fedge(fb, j);
        const uint32_t nd[4] = {u.enode(ea, 0), u.enode(ea, 1), u.enode(eb, 0), u.enode(eb, 1)};
        for (int k = 0; k < 4; ++k) {
          im.nodes[k] = nd[k];
          im.w[k] = 0;
        }
        bool ok = false;
        if (!(nd[0] == nd[2] || nd[0] == nd[3] || nd[1] == nd[2] || nd[1] == nd[3])) {
          if (overlap_dilated(node_bounds(u, nd, 2), node_bounds(u, nd + 2, 2), thickness))
            ok = check_impact(u, false, nd, im);
        }
        if (!ok) im.t = -1;
      }
    }
  }
}

// Face edges, edge adjacency and registration-time face normals (Face::SetEdge, Face::Update,
// PhysicsMeshHelper.cu:118-123) of a triangle list.
void face_topology(const std::vector<uint32_t>& tri, const std::vector<uint32_t>& edges,
                   const std::vector<V3>& reg_pos, std::vector<uint32_t>& face_edges,
                   std::vector<int32_t>& edge_adj, std::vector<V3>& face_n0) {
  std::map<std::pair<uint32_t, uint32_t>, uint32_t> key;
  for (uint32_t e = 0; e < edges.size() / 2; ++e)
    key[std::make_pair(std::min(edges[2 * e], edges[2 * e + 1]),
                       std::max(edges[2 * e], edges[2 * e + 1]))] = e;
  const uint32_t nf = (uint32_t)tri.size() / 3;
  face_edges.assign(3 * (size_t)nf, 0);
  edge_adj.assign(2 * edges.size(), -1);
  std::vector<int> fill(edges.size() / 2, 0);
  face_n0.resize(nf);
  for (uint32_t f = 0; f < nf; ++f) {
    for (int k = 0; k < 3; ++k) {
      uint32_t a = tri[f * 3 + k], b = tri[f * 3 + (k + 1) % 3];
      uint32_t e = key[std::make_pair(std::min(a, b), std::max(a, b))];
      face_edges[f * 3 + k] = e;
      if (fill[e] < 4) edge_adj[e * 4 + fill[e]++] = (int32_t)f;
    }
    V3 d1 = reg_pos[tri[f * 3 + 1]] - reg_pos[tri[f * 3]];
    V3 d2 = reg_pos[tri[f * 3 + 2]] - reg_pos[tri[f * 3]];
    face_n0[f] = normalize(cross(d1, d2));
  }
}

// ---------------------------------------------------------------------------------------------
// frame — ClothSolverBase::SimulateSwift (ClothSolverBase.cpp:171-261)

// ---------------------------------------------------------------------------------------------
// impact-zone collision step — ImpactZoneOptimization::CollisionStep (impact_zone/Entry.cu:140-256)

// The reference's reduction of a zone quantity (ReduceBaselineLocal/Global_Kernel,
// ParallelOptimizer.cu:335-428): 256-element blocks summed by the stride tree
// s[t] += s[t + d] (t % 2d == 0, d = 1 .. 128), then the block sums by the same tree.
float blocked_sum(std::vector<float> v) {
  do {
    const size_t nb = std::max<size_t>(1, (v.size() + 255) / 256);
    std::vector<float> next(nb);
    for (size_t b = 0; b < nb; ++b) {
      float s[256];
      for (int t = 0; t < 256; ++t) s[t] = b * 256 + t < v.size() ? v[b * 256 + t] : 0.0f;
      for (int d = 1; d < 256; d *= 2)
        for (int t = 0; t < 256; t += 2 * d) s[t] += s[t + d];
      next[b] = s[0];
    }
    v.swap(next);
  } while (v.size() > 1);
  return v[0];
}

struct IZone {
  std::vector<uint32_t> impacts;  // ids into the step's impact list
  std::set<uint32_t> nodes;
  bool active = true, enabled = true;
};

struct IZStep {
  Oracle& o;
  int deform = 0;
  float obstacle_mass = 1e3f, thickness = 1e-4f;
  std::vector<Oracle::Impact> store;
  std::vector<IZone> zones;
  uint32_t V() const { return (uint32_t)o.x.size(); }
  bool is_cloth(uint32_t v) const { return v < V(); }
  bool is_free(uint32_t v) const { return is_cloth(v) && o.cfree[v] != 0; }
  bool deformable(uint32_t v) const { return deform == 1 || is_free(v); }
  // moved by the optimizer: free cloth nodes, and obstacle nodes at deform 1 (a pinned cloth node
  // would enter with mass 1 / 0)
  bool optimized(uint32_t v) const { return is_free(v) || (deform == 1 && !is_cloth(v)); }
  V3 pos(uint32_t v) const { return is_cloth(v) ? o.x[v] : o.ox[v - V()]; }
  void set_pos(uint32_t v, V3 p) {
    if (is_cloth(v)) o.x[v] = p; else o.ox[v - V()] = p;
  }
};

// independentImpacts (Entry.cu:25-63): impacts sorted by t; rounds of
// InitializeImpactNodes / CollectRelativeImpacts / SetImpactMinIndices / CheckIndependentImpacts
// (ImpactHelper.cu:234-343) until no impact is added.
std::vector<Oracle::Impact> independent_impacts(IZStep& z, std::vector<Oracle::Impact> imp) {
  std::stable_sort(imp.begin(), imp.end(),
                   [](const Oracle::Impact& a, const Oracle::Impact& b) { return a.t < b.t; });
  const int n = (int)imp.size();
  std::map<uint32_t, bool> removed;
  std::map<uint32_t, int> min_index;
  for (const auto& im : imp)
    for (uint32_t v : im.nodes)
      if (z.deformable(v)) {
        removed[v] = false;
        min_index[v] = n;
      }
  std::vector<int> ans(n, 0);
  int num, new_num = n;
  do {
    num = new_num;
    std::map<uint32_t, int> mins;
    for (int i = 0; i < n; ++i) {
      bool flag = true;
      for (uint32_t v : imp[i].nodes)
        if (z.deformable(v) && removed[v]) flag = false;
      if (!flag) continue;
      for (uint32_t v : imp[i].nodes) {
        if (!z.deformable(v)) continue;
        auto it = mins.find(v);
        if (it == mins.end() || i < it->second) mins[v] = i;
      }
    }
    for (const auto& kv : mins) min_index[kv.first] = kv.second;
    for (int i = 0; i < n; ++i) {
      bool flag = true;
      for (uint32_t v : imp[i].nodes)
        if (z.deformable(v) && (removed[v] || min_index[v] != i)) flag = false;
      if (!flag) continue;
      ans[i] = 1;
      for (uint32_t v : imp[i].nodes)
        if (z.deformable(v)) removed[v] = true;
    }
    new_num = n - (int)std::count(ans.begin(), ans.end(), 1);
  } while (num > new_num);
  std::vector<Oracle::Impact> out;
  for (int i = 0; i < n; ++i)
    if (ans[i]) out.push_back(imp[i]);
  return out;
}

// IsolateImpacts (ImpactZoneHelper.cu:214-304): FloodFillColoring_Kernel from the first uncolored
// impact, WriteBackNodeColor_Kernel, repeated.  An impact that no fill reaches (every node a
// pinned cloth node) is dropped.
std::vector<IZone> isolate(IZStep& z, const std::vector<uint32_t>& ids) {
  const int kOutside = -2, kInside = -1;
  std::map<uint32_t, int> color;
  auto col = [&](uint32_t v) {
    auto it = color.find(v);
    return it == color.end() ? kOutside : it->second;
  };
  for (uint32_t id : ids)
    for (uint32_t v : z.store[id].nodes) color[v] = kInside;
  std::vector<int> icol(ids.size(), -1);
  std::vector<IZone> out;
  for (int c = 0;; ++c) {
    size_t first = 0;
    while (first < ids.size() && icol[first] != -1) ++first;
    if (first == ids.size()) break;
    std::vector<uint32_t> stack(std::begin(z.store[ids[first]].nodes),
                                std::end(z.store[ids[first]].nodes));
    while (!stack.empty()) {
      uint32_t v = stack.back();
      stack.pop_back();
      const bool cloth = z.is_cloth(v);
      if (cloth && !z.is_free(v)) continue;
      const uint32_t lv = cloth ? v : v - z.V();
      const auto& pre = cloth ? z.o.vf_prefix : z.o.ovf_prefix;
      const auto& lst = cloth ? z.o.vf_list : z.o.ovf_list;
      const auto& tri = cloth ? z.o.tri : z.o.otri;
      for (uint32_t q = pre[lv]; q < pre[lv + 1]; ++q)
        for (int k = 0; k < 3; ++k) {
          uint32_t u = (cloth ? 0 : z.V()) + tri[lst[q] * 3 + k];
          if (col(u) == kInside) {
            color[u] = c;
            stack.push_back(u);
          }
        }
    }
    IZone zone;
    for (size_t m = 0; m < ids.size(); ++m) {
      if (icol[m] != -1) continue;
      for (uint32_t v : z.store[ids[m]].nodes)
        if (col(v) >= 0) {
          icol[m] = c;
          zone.impacts.push_back(ids[m]);
          break;
        }
    }
    if (icol[first] == -1) icol[first] = -2;
    if (!zone.impacts.empty()) {
      for (uint32_t id : zone.impacts)
        for (uint32_t v : z.store[id].nodes) zone.nodes.insert(v);
      out.push_back(zone);
    }
  }
  return out;
}

bool share_node(const IZone& a, const IZone& b) {  // ImpactZone::Intersects
  for (uint32_t v : b.nodes)
    if (a.nodes.count(v)) return true;
  return false;
}

void merge_into(IZone& a, IZone& b) {  // ImpactZone::Merge
  a.impacts.insert(a.impacts.end(), b.impacts.begin(), b.impacts.end());
  a.nodes.insert(b.nodes.begin(), b.nodes.end());
  a.active = a.enabled = true;
  b.enabled = false;
}

// AddImpacts (ImpactZoneHelper.cu:325-367), the merge pass repeated until no two zones share a
// node, a disabled zone absorbing nothing.
void add_impacts(IZStep& z, std::vector<IZone> fresh) {
  const size_t n0 = z.zones.size();
  for (auto& q : z.zones) q.active = false;
  for (size_t i = 0; i < n0; ++i)
    for (auto& f : fresh)
      if (f.enabled && share_node(z.zones[i], f)) merge_into(z.zones[i], f);
  for (auto& f : fresh)
    if (f.enabled) z.zones.push_back(f);
  for (bool changed = true; changed;) {
    changed = false;
    for (size_t i = 0; i < z.zones.size(); ++i)
      for (size_t j = i + 1; j < z.zones.size(); ++j)
        if (z.zones[i].enabled && z.zones[j].enabled && share_node(z.zones[i], z.zones[j])) {
          merge_into(z.zones[i], z.zones[j]);
          changed = true;
        }
  }
  std::vector<IZone> keep;
  for (auto& q : z.zones)
    if (q.enabled) keep.push_back(q);
  z.zones.swap(keep);
}

// ParallelImpactZoneOptimizer + ParallelOptimizer::Solve over the active zones
// (ParallelImpactZoneOptimizer.cu:13-528, ParallelOptimizer.cu:513-880).
void solve_zones(IZStep& z, const std::vector<V3>& cx1, const std::vector<V3>& ox1) {
  const float mu = 1e3f, eps_s = 1e-12f, eps_f = 1e-10f, alpha = 0.5f;
  struct Work {
    std::vector<uint32_t> nodes, entries;
    std::vector<int> loc;  // 4 per entry
    std::vector<V3> X, Xt;
    int conv;
  };
  std::vector<Work> ws;
  std::vector<float> inv_all;
  for (const IZone& q : z.zones) {
    if (!q.active) continue;
    Work w;
    for (uint32_t v : q.nodes)
      if (z.optimized(v)) w.nodes.push_back(v);
    w.entries = q.impacts;
    for (uint32_t id : w.entries)
      for (uint32_t v : z.store[id].nodes) {
        auto it = std::lower_bound(w.nodes.begin(), w.nodes.end(), v);
        w.loc.push_back(it != w.nodes.end() && *it == v ? (int)(it - w.nodes.begin()) : -1);
      }
    for (uint32_t v : w.nodes)  // CollisionInv_Kernel
      inv_all.push_back(z.is_cloth(v) ? z.o.w[v] : 1.0f / z.obstacle_mass);
    ws.push_back(w);
  }
  if (ws.empty()) return;
  const float inv = inv_all.empty() ? 0.0f : blocked_sum(inv_all) / (float)inv_all.size();
  auto x1 = [&](uint32_t v) { return z.is_cloth(v) ? cx1[v] : ox1[v - z.V()]; };
  auto mass = [&](uint32_t v) { return z.is_cloth(v) ? 1.0f / z.o.w[v] : z.obstacle_mass; };
  for (Work& w : ws) {
    const size_t nn = w.nodes.size(), ni = w.entries.size();
    for (uint32_t v : w.nodes) w.X.push_back(z.pos(v));
    w.Xt = w.X;
    std::vector<float> lambda(ni, 0.0f), cc(ni);
    auto constraint = [&](size_t e, const std::vector<V3>& Xs) {
      const Oracle::Impact& im = z.store[w.entries[e]];
      float c = -z.thickness;
      for (int j = 0; j < 4; ++j) {
        const int k = w.loc[4 * e + j];
        c += im.w[j] * dot(im.n, k > -1 ? Xs[k] : z.pos(im.nodes[j]));
      }
      return c;
    };
    float s = 1e-3f * (float)nn;
    w.conv = 100;
    std::vector<V3> grad(nn);
    std::vector<std::vector<uint32_t>> slots(nn);  // per node: 4 entry + j, ascending
    for (size_t q = 0; q < w.loc.size(); ++q)
      if (w.loc[q] > -1) slots[w.loc[q]].push_back((uint32_t)q);
    for (int it = 0; it < 100; ++it) {
      std::vector<float> c2(ni), l2(ni);
      for (size_t e = 0; e < ni; ++e) {
        const float q = constraint(e, w.X) + lambda[e] / mu;
        cc[e] = q < 0.0f ? q : 0.0f;  // ClampViolation, sign 1
        c2[e] = cc[e] * cc[e];
        l2[e] = lambda[e] * lambda[e];
      }
      const float C2 = blocked_sum(c2), L2 = blocked_sum(l2);
      std::vector<float> g2(nn), ob(nn);
      for (size_t k = 0; k < nn; ++k) {  // ObjectiveGradient, then the constraint terms
        const uint32_t v = w.nodes[k];
        V3 g = (inv * mass(v)) * (w.X[k] - x1(v));
        bool first = true;
        V3 acc{0, 0, 0};
        for (uint32_t q : slots[k]) {  // reduce_by_key over the slots of the node
          const size_t e = q / 4;
          const int j = (int)(q % 4);
          const Oracle::Impact& im = z.store[w.entries[e]];
          V3 t = ((mu * cc[e]) * im.w[j]) * im.n;
          acc = first ? t : acc + t;
          first = false;
        }
        g = g + acc;
        grad[k] = g;
        g2[k] = dot(g, g);
        V3 d = w.X[k] - x1(v);
        ob[k] = mass(v) * dot(d, d);
      }
      const float G2 = blocked_sum(g2), O = blocked_sum(ob);
      const float f = (0.5f * inv) * O + (0.5f * mu) * C2 - (0.5f * L2) / mu;
      s = s / 0.7f;
      for (int ls = 0;; ++ls) {
        s = s * 0.7f;
        std::vector<float> ot(nn), ct(ni);
        for (size_t k = 0; k < nn; ++k) {
          w.Xt[k] = w.X[k] - s * grad[k];
          V3 d = w.Xt[k] - x1(w.nodes[k]);
          ot[k] = mass(w.nodes[k]) * dot(d, d);
        }
        for (size_t e = 0; e < ni; ++e) {
          float q = constraint(e, w.Xt) + lambda[e] / mu;
          q = q < 0.0f ? q : 0.0f;
          ct[e] = q * q;
        }
        const float Ot = blocked_sum(ot), C2t = blocked_sum(ct);
        const float ft = (0.5f * inv) * Ot + (0.5f * mu) * C2t - (0.5f * L2) / mu;
        if (s < eps_s || ft < f - (alpha * s) * G2 || mabs(f - ft) < eps_f) break;
        if (ls + 1 >= 1024) {
          s = 0.0f;
          break;
        }
      }
      if (s < eps_s) {
        w.conv = it;
        break;
      }
      w.X = w.Xt;
      for (size_t e = 0; e < ni; ++e) {  // UpdateMultiplier
        const float q = lambda[e] + mu * constraint(e, w.X);
        lambda[e] = q < 0.0f ? q : 0.0f;
      }
    }
  }
  int K = -1;
  for (const Work& w : ws) K = std::max(K, w.conv);
  for (const Work& w : ws) {  // Finalize: the last zones to converge keep X
    const bool keep = w.conv == K && K < 100;
    for (size_t k = 0; k < w.nodes.size(); ++k) z.set_pos(w.nodes[k], keep ? w.X[k] : w.Xt[k]);
  }
}

// CollisionStep; stats8 in the layout of xrt_collision_stats.
void collision_step(Oracle& o, float obstacle_mass, float thickness, int32_t* stats8) {
  int32_t st[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const uint32_t F = (uint32_t)o.tri.size() / 3, OF = (uint32_t)o.otri.size() / 3;
  if (F == 0) {
    st[0] = 1;
    if (stats8) std::copy(st, st + 8, stats8);
    return;
  }
  const std::vector<V3> cx1 = o.x, ox1 = o.ox;  // SetupNode / SetupObstacleNode: x1 = x
  const float dt = o.p.frame_time / (float)o.p.num_substeps;
  o.ov.assign(o.ox.size(), V3{0, 0, 0});
  for (size_t i = 0; i < o.ox.size(); ++i) o.ov[i] = (o.ox[i] - o.ox0[i]) / dt;
  auto ccd_tree = [](Lbvh& b, const std::vector<V3>& x, const std::vector<V3>& x0,
                     const std::vector<V3>& n, const std::vector<uint32_t>& tri) {
    b = Lbvh();
    b.objects.resize(tri.size() / 3);
    for (size_t f = 0; f < tri.size() / 3; ++f) {  // UpdateObjects_Kernel, ccd = true
      Prim& pr = b.objects[f];
      const uint32_t a = tri[3 * f], bb = tri[3 * f + 1], c = tri[3 * f + 2];
      pr.idx1 = a; pr.idx2 = bb; pr.idx3 = c;
      pr.v1 = x0[a] + 0.0f * n[a]; pr.v2 = x0[bb] + 0.0f * n[bb]; pr.v3 = x0[c] + 0.0f * n[c];
      pr.pred1 = x[a] + 0.0f * n[a]; pr.pred2 = x[bb] + 0.0f * n[bb]; pr.pred3 = x[c] + 0.0f * n[c];
    }
    b.construct(0.0f);
  };
  Lbvh cbvh, obvh;
  ccd_tree(cbvh, o.x, o.x0, o.n, o.tri);
  if (OF) ccd_tree(obvh, o.ox, o.ox0, o.on, o.otri);
  IZStep z{o};
  z.obstacle_mass = obstacle_mass;
  z.thickness = thickness;
  bool success = false;
  for (int deform = 0; deform < 2 && !success; ++deform) {
    z.deform = deform;
    z.store.clear();
    z.zones.clear();
    st[1] = deform;
    st[2] = 0;
    for (int pass = 0; pass < 100; ++pass) {
      st[2] = pass + 1;
      o.pairs.clear();  // FindImpacts: Traverse(cloth, obstacle), Traverse(cloth, cloth), CheckImpacts
      traverse_pairs(cbvh, obvh, 0, F, thickness, o.pairs);
      traverse_pairs(cbvh, cbvh, 0, 0, thickness, o.pairs);
      check_impacts(o, thickness);
      std::vector<Oracle::Impact> found;
      for (const auto& im : o.impacts)
        if (!(im.t < 0.0f)) found.push_back(im);
      if (found.empty()) {
        success = true;
        break;
      }
      std::vector<Oracle::Impact> indep = independent_impacts(z, found);
      std::vector<uint32_t> ids;
      for (const auto& im : indep) {
        ids.push_back((uint32_t)z.store.size());
        z.store.push_back(im);
      }
      st[3] += (int32_t)indep.size();
      add_impacts(z, isolate(z, ids));
      for (const auto& q : z.zones) st[5] += q.active ? 1 : 0;
      solve_zones(z, cx1, ox1);
      update_bvh_ccd(cbvh, o.x, o.x0, o.tri);
      if (deform == 1) {
        if (OF) update_bvh_ccd(obvh, o.ox, o.ox0, o.otri);
        z.obstacle_mass *= 0.5f;
      }
    }
    st[4] = (int32_t)z.zones.size();
  }
  st[0] = success ? 1 : 0;
  if (stats8) std::copy(st, st + 8, stats8);
}

void step_frame(Oracle& o) {
  const xrt_swift_params& p = o.p;
  const float substep_time = p.frame_time / (float)p.num_substeps;
  const long nv = (long)o.x.size();
  const bool obstacle_updated = p.update_obstacle_animation && !o.otri.empty();
  if (obstacle_updated) rebuild_obstacle_bvh(o, 0.0f);
  const bool has_obstacle = o.bvh.active;
  const bool repulsion = p.pbd_repulsion != 0;
  const bool imminent = p.imminent_repulsion != 0;
  if (repulsion || imminent) {  // SimulateQuality (ClothSolverBase.cpp:276-293)
    build_cloth_bvh(o);
    if (imminent) imminent_generate(o);
    if (!o.otri.empty()) update_bvh_ccd(o.bvh, o.ox, o.ox0, o.otri);
  }
  const int frequency = (p.num_substeps * p.num_iterations) / p.num_collision_passes;
  int cnt = 0;
  for (int substep = 0; substep < p.num_substeps; ++substep) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < nv; ++i) {  // PredictPositions_Kernel
      if (o.w[i] > kEps) o.v[i] += V3{p.gravity[0], p.gravity[1], p.gravity[2]} * substep_time;
      o.x[i] = o.x0[i] + o.v[i] * substep_time;
    }
    if (p.enable_self_collision && substep % p.inter_leaved_hash == 0) hash_particles(o);
    for (int it = 0; it < p.num_iterations; ++it) {
      if (imminent)  // ClothSolverBase.cpp:296-301
        imminent_solve(o, p.imminent_thickness, p.repulsion_relaxation, substep_time);
      if (repulsion) {  // ClothSolverBase.cpp:303-313
        if (it % 10 == 0) update_pairs(o, 1e-6f);
        solve_repulsion(o, p.pbd_thickness, p.repulsion_relaxation);
      }
      if (p.enable_self_collision) collide_particles(o);
      int current = substep * p.num_iterations + it;
      if (current % frequency == 0) {
        if (obstacle_updated) obstacle_pass(o, cnt, p.num_collision_passes);
        if (has_obstacle) generate_contacts(o);
        cnt++;
      }
      if (o.fem_on) {  // SimulateQuality's fabric (ClothSolverBase.cpp:315-323)
        for (uint32_t c = 0; c < o.fem_ncolors[0]; ++c) solve_fem_strain(o, c);
        if (o.fem.solve_bending && !o.bends.empty())
          for (uint32_t c = 0; c < o.fem_ncolors[1]; ++c) solve_iso_bend(o, c, substep_time, it);
      } else {
        for (uint32_t c = 0; c < o.n_s_colors; ++c) solve_stretch(o, c, substep_time, it);
        if (p.solve_bending)
          for (uint32_t c = 0; c < o.n_b_colors; ++c) solve_bend(o, c, substep_time);
      }
      if (p.geodesic_lra) solve_lra(o);
      if (has_obstacle) {
        solve_contacts(o);
      } else {
        apply_deltas(o);
      }
      if (!o.otri.empty()) solve_binding(o);
    }
    if (p.impact_zone)  // SimulateQuality's CollisionStep (ClothSolverBase.cpp:329-336)
      collision_step(o, p.impact_zone_obstacle_mass, p.impact_zone_thickness, nullptr);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < nv; ++i) {  // Finalize_Kernel
      V3 np = o.x[i];
      V3 raw = (np - o.x0[i]) / substep_time;
      o.v[i] = raw * (1 - p.damping * substep_time);
      o.x0[i] = np;
    }
  }
  if (!o.otri.empty()) {
    o.ox0 = o.ox;  // PredictedToPositions
    vertex_normals(o.ox0, o.otri, o.ovf_prefix, o.ovf_list, o.on);
  }
  vertex_normals(o.x0, o.tri, o.vf_prefix, o.vf_list, o.n);
  o.frame_index++;
}

void start(Oracle& o) {
  const uint32_t nv = (uint32_t)o.x0.size();
  // coloring
  for (int kind = 0; kind < 2; ++kind) {
    const std::vector<uint32_t>& idx = kind == 0 ? o.edges : o.bends;
    const int arity = kind == 0 ? 2 : 4;
    std::vector<uint32_t>& col = kind == 0 ? o.s_color : o.b_color;
    uint32_t& nc = kind == 0 ? o.n_s_colors : o.n_b_colors;
    if (!o.pending_colors[kind].empty()) {
      col = o.pending_colors[kind];
      nc = 0;
      for (uint32_t c : col) nc = std::max(nc, c + 1);
    } else {
      col = greedy_color(idx, arity, nv, nc);
    }
  }
  if (o.fem_on) {  // FEM fabric: strain over the faces (kind 2), bending over the bends (kind 3)
    for (int kind = 0; kind < 2; ++kind) {
      const std::vector<uint32_t>& idx = kind == 0 ? o.tri : o.bends;
      std::vector<uint32_t>& col = o.fem_color[kind];
      uint32_t& nc = o.fem_ncolors[kind];
      if (!o.pending_colors[2 + kind].empty()) {
        col = o.pending_colors[2 + kind];
        nc = 0;
        for (uint32_t c : col) nc = std::max(nc, c + 1);
      } else {
        col = greedy_color(idx, kind == 0 ? 3 : 4, nv, nc);
      }
    }
    fem_setup(o);
  }
  o.s_lambda.assign(o.rest.size(), 0.0f);
  build_vf(o.tri, nv, o.vf_prefix, o.vf_list);
  vertex_normals(o.x0, o.tri, o.vf_prefix, o.vf_list, o.n);
  o.x_init = o.x0;  // SpatialHashGPU::SetInitialPositions (universal/ClothSolver.cpp:88)
  o.deltas.assign(nv, V3{0, 0, 0});
  o.delta_counts.assign(nv, 0);
  o.vf_idx.assign(nv, -1);
  o.rt_idx.assign(nv, -1);
  o.vf_qs.assign(nv, V3{0, 0, 0});
  o.rt_qc.assign(nv, V3{0, 0, 0});
  o.ee.assign(o.rest.size(), EEContact{kScalarMax, {0, 0, 0}, {0, 0, 0}, 0, 0, {0, 0, 0}});
  if (!o.otri.empty()) {
    const uint32_t onv = (uint32_t)o.ox0.size();
    build_vf(o.otri, onv, o.ovf_prefix, o.ovf_list);
    vertex_normals(o.ox0, o.otri, o.ovf_prefix, o.ovf_list, o.on);
    o.on1 = o.on;
    o.ox1 = o.ox0;
    rebuild_obstacle_bvh(o, 0.0f);  // ClothSolverUniversal::Start (ClothSolver.cpp:60-61)
    o.ortri = build_rtri(o.otri, o.ovf_prefix, o.ovf_list);
  }
  // proximity topology: face edges, edge adjacency, registration normals, cloth R-triangles
  face_topology(o.tri, o.edges, o.cmesh_pos, o.cface_edges, o.cedge_adj, o.cface_n0);
  o.crtri = build_rtri(o.tri, o.vf_prefix, o.vf_list);
  if (!o.otri.empty()) {
    std::vector<std::vector<uint32_t>> oef;
    o.oedges.clear();
    build_edges(o.otri, (uint32_t)o.ox0.size(), o.oedges, oef);
    face_topology(o.otri, o.oedges, o.omesh_pos, o.oface_edges, o.oedge_adj, o.oface_n0);
  }
  // bindings: GenerateBinding_Kernel (BindingConstraint.cu:20-44) from x0 of both meshes
  for (Binding& b : o.bindings) {
    V3 pcl = o.x0[b.cloth];
    V3 pb = b.u * o.ox0[b.iu] + b.v * o.ox0[b.iv] + b.w * o.ox0[b.iw];
    if (b.L < kEps) b.L = length(pcl - pb);
  }
  o.started = true;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// C API of the oracle (test infrastructure)

extern "C" {

// The reference's effective Swift-mode defaults, restated field by field so that a CPU-only run
// needs nothing from the CUDA library:
//   SolverSettings (config/Base.hpp:91-97): 1 substep, 200 iterations, max speed 1e6,
//     gravity (0, -9.8, 0), damping 0.98;
//   BasicFabricSettings (config/Base.hpp:38-45): stretch 0, bend 1e2, relaxation 0.25,
//     long-range stretchiness 1.1, solve bending; GEODESIC_LRA is parsed but never applied, the
//     solver always runs the geodesic form (LongRangeAttachments.cu:5-26);
//   SwiftModeCollisionSettings (config/Base.hpp:128-133): 10 passes, SDF margin 1e-2, BVH
//     tolerance 0.003; ParticleCollisionSettings (config/Base.hpp:59-66): friction 0.1, 64
//     neighbors, hash every 3 substeps, self collision on, diameter 1.3 x first edge, cell 1.5;
//   frame time 1/60 (utils/Timer.hpp:177), obstacle animation on (core/Common.hpp:81);
//   RepulsionSettings (config/Base.hpp:108-114) and ImpactZoneSettings (:116-119) for the
//     Quality stages, which are off in the Swift frame.
void orc_default_params(xrt_swift_params* p) {
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
  p->pbd_thickness = 1e-4f;
  p->repulsion_relaxation = 0.25f;
  p->impact_zone = 0;
  p->impact_zone_obstacle_mass = 1e3f;
  p->impact_zone_thickness = 1e-4f;
  p->imminent_repulsion = 0;
  p->imminent_thickness = 1e-3f;
}

// FEMFabricSettings (config/Base.hpp:47-57).
void orc_default_fem_material(xrt_fem_material* m) {
  std::memset(m, 0, sizeof(*m));
  m->xx_stiffness = m->yy_stiffness = m->xy_stiffness = 1.0f;
  m->xy_poisson_ratio = m->yx_poisson_ratio = 0.3f;
  m->bending_stiffness = 1.0f;
  m->solve_bending = 1;
}

void* orc_create() { return new Oracle(); }
void orc_destroy(void* h) { delete static_cast<Oracle*>(h); }
int orc_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

void orc_set_params(void* h, const xrt_swift_params* p) { static_cast<Oracle*>(h)->p = *p; }

int orc_add_cloth(void* h, const xrt_cloth_desc* d) {
  Oracle& o = *static_cast<Oracle*>(h);
  Cloth c;
  c.offset = (uint32_t)o.x0.size();
  c.mesh_pos.resize(d->num_vertices);
  for (uint32_t i = 0; i < d->num_vertices; ++i)
    c.mesh_pos[i] = V3{d->positions[i * 3], d->positions[i * 3 + 1], d->positions[i * 3 + 2]};
  c.tri.assign(d->triangles, d->triangles + 3 * (size_t)d->num_triangles);
  for (uint32_t i = 0; i < d->num_vertices; ++i) {
    V3 q = c.mesh_pos[i];
    if (d->model_matrix) q = transform_point(d->model_matrix, q);
    o.x0.push_back(q);
    o.x.push_back(c.mesh_pos[i]);
    o.v.push_back(V3{0, 0, 0});
    o.w.push_back(1.0f);
  }
  for (uint32_t k = 0; k < 3 * d->num_triangles; ++k) o.tri.push_back(d->triangles[k] + c.offset);
  o.cfree.resize(o.x0.size(), 1);
  for (uint32_t i = 0; i < d->num_fixed; ++i) {
    o.w[c.offset + d->fixed_indices[i]] = 0.0f;  // SetInvMass(0) + SetFree(false)
    o.cfree[c.offset + d->fixed_indices[i]] = 0;
  }
  o.cmesh_pos.insert(o.cmesh_pos.end(), c.mesh_pos.begin(), c.mesh_pos.end());
  // edges / stretch (PrepareBasicStretchData, ClothSolverHelper.cpp:90-109)
  std::vector<uint32_t> e;
  std::vector<std::vector<uint32_t>> ef;
  build_edges(c.tri, d->num_vertices, e, ef);
  for (size_t k = 0; k < e.size() / 2; ++k) {
    o.edges.push_back(e[k * 2] + c.offset);
    o.edges.push_back(e[k * 2 + 1] + c.offset);
    o.rest.push_back(length(c.mesh_pos[e[k * 2]] - c.mesh_pos[e[k * 2 + 1]]));
    o.s_comp.push_back(o.p.stretch_compliance);
  }
  if (o.p.solve_bending) {
    std::vector<uint32_t> b;
    std::vector<float> th;
    build_bends(c.mesh_pos, c.tri, e, ef, c.offset, b, th);
    o.bends.insert(o.bends.end(), b.begin(), b.end());
    o.theta.insert(o.theta.end(), th.begin(), th.end());
    o.b_comp.insert(o.b_comp.end(), th.size(), o.p.bend_compliance);
  }
  // geodesic LRA (ClothObjectBase.cpp:79-93)
  if (d->num_attached > 0 && o.p.geodesic_lra) {
    std::vector<std::vector<uint32_t>> adj(d->num_vertices);
    for (size_t k = 0; k < e.size() / 2; ++k) {
      adj[e[k * 2]].push_back(e[k * 2 + 1]);
      adj[e[k * 2 + 1]].push_back(e[k * 2]);
    }
    for (auto& a : adj) std::sort(a.begin(), a.end());
    for (uint32_t s = 0; s < d->num_attached; ++s) {
      uint32_t slot = d->attached_indices[s];
      std::vector<float> dist = geodesic(c.mesh_pos, adj, slot);
      for (uint32_t vtx = 0; vtx < d->num_vertices; ++vtx) {
        o.lra_src.push_back(slot + c.offset);
        o.lra_tgt.push_back(vtx + c.offset);
        o.lra_rest.push_back(dist[vtx]);
      }
    }
  }
  for (uint32_t i = 0; i < d->num_binded; ++i) {
    Binding b;
    b.cloth = d->binded_indices[i] + c.offset;
    b.iu = d->bind_obstacle_tri[i * 3];
    b.iv = d->bind_obstacle_tri[i * 3 + 1];
    b.iw = d->bind_obstacle_tri[i * 3 + 2];
    b.u = d->bind_barycentric[i * 3];
    b.v = d->bind_barycentric[i * 3 + 1];
    b.w = d->bind_barycentric[i * 3 + 2];
    b.L = d->bind_distances ? d->bind_distances[i] : 0.0f;
    b.stiffness = d->bind_stiffnesses ? d->bind_stiffnesses[i] : 1.0f;
    o.bindings.push_back(b);
  }
  // particle diameter (universal/ClothObject.hpp:36-37): the last cloth added wins
  if (d->particle_diameter > 0.0f) {
    o.particle_diameter = d->particle_diameter;
  } else {
    o.particle_diameter =
        length(c.mesh_pos[c.tri[0]] - c.mesh_pos[c.tri[1]]) * o.p.particle_diameter;
  }
  o.cloths.push_back(std::move(c));
  return (int)o.cloths.back().offset;
}

int orc_add_obstacle(void* h, const xrt_obstacle_desc* d) {
  Oracle& o = *static_cast<Oracle*>(h);
  uint32_t off = (uint32_t)o.ox0.size();
  for (uint32_t i = 0; i < d->num_vertices; ++i) {
    V3 q{d->positions[i * 3], d->positions[i * 3 + 1], d->positions[i * 3 + 2]};
    o.omesh_pos.push_back(q);
    if (d->model_matrix) q = transform_point(d->model_matrix, q);
    o.ox0.push_back(q);
    o.ox.push_back(q);
  }
  for (uint32_t k = 0; k < 3 * d->num_triangles; ++k) o.otri.push_back(d->triangles[k] + off);
  return (int)off;
}

void orc_set_coloring(void* h, int kind, const uint32_t* colors, uint32_t n) {
  Oracle& o = *static_cast<Oracle*>(h);
  o.pending_colors[kind & 3].assign(colors, colors + n);
}
void orc_set_fem_material(void* h, const xrt_fem_material* m) {
  Oracle& o = *static_cast<Oracle*>(h);
  o.fem_on = m != nullptr;
  if (m) o.fem = *m;
}
void orc_set_compliance(void* h, int kind, const float* c, uint32_t n) {
  Oracle& o = *static_cast<Oracle*>(h);
  (kind == 0 ? o.s_comp : o.b_comp).assign(c, c + n);
}
void orc_set_inv_mass(void* h, const float* w, uint32_t n) {
  static_cast<Oracle*>(h)->w.assign(w, w + n);
}
void orc_start(void* h) { start(*static_cast<Oracle*>(h)); }
void orc_set_obstacle_targets(void* h, const float* pos) {
  Oracle& o = *static_cast<Oracle*>(h);
  for (size_t i = 0; i < o.ox.size(); ++i) o.ox[i] = V3{pos[i * 3], pos[i * 3 + 1], pos[i * 3 + 2]};
}
void orc_step_frame(void* h) { step_frame(*static_cast<Oracle*>(h)); }

static void put3(const std::vector<V3>& v, float* out) {
  for (size_t i = 0; i < v.size(); ++i) {
    out[i * 3] = v[i].x;
    out[i * 3 + 1] = v[i].y;
    out[i * 3 + 2] = v[i].z;
  }
}
void orc_get_sizes(void* h, uint32_t* out8) {
  Oracle& o = *static_cast<Oracle*>(h);
  out8[0] = (uint32_t)o.x0.size();
  out8[1] = (uint32_t)o.rest.size();
  out8[2] = (uint32_t)o.tri.size() / 3;
  out8[3] = (uint32_t)o.theta.size();
  out8[4] = (uint32_t)o.lra_rest.size();
  out8[5] = (uint32_t)o.ox0.size();
  out8[6] = (uint32_t)o.otri.size() / 3;
  out8[7] = o.n_s_colors | (o.n_b_colors << 16);
}
void orc_get_positions(void* h, float* out) { put3(static_cast<Oracle*>(h)->x0, out); }
void orc_get_velocities(void* h, float* out) { put3(static_cast<Oracle*>(h)->v, out); }
void orc_get_normals(void* h, float* out) { put3(static_cast<Oracle*>(h)->n, out); }
void orc_get_obstacle_positions(void* h, float* out) { put3(static_cast<Oracle*>(h)->ox0, out); }
float orc_particle_diameter(void* h) { return static_cast<Oracle*>(h)->particle_diameter; }
void orc_get_edges(void* h, uint32_t* e, float* rest) {
  Oracle& o = *static_cast<Oracle*>(h);
  std::copy(o.edges.begin(), o.edges.end(), e);
  std::copy(o.rest.begin(), o.rest.end(), rest);
}
void orc_get_bends(void* h, uint32_t* b, float* th) {
  Oracle& o = *static_cast<Oracle*>(h);
  std::copy(o.bends.begin(), o.bends.end(), b);
  std::copy(o.theta.begin(), o.theta.end(), th);
}
void orc_get_coloring(void* h, int kind, uint32_t* out) {
  Oracle& o = *static_cast<Oracle*>(h);
  const auto& c = kind == 0 ? o.s_color : o.b_color;
  std::copy(c.begin(), c.end(), out);
}
int orc_coloring_valid(void* h, int kind) {
  Oracle& o = *static_cast<Oracle*>(h);
  return kind == 0 ? coloring_valid(o.edges, 2, o.s_color, (uint32_t)o.x0.size())
                   : coloring_valid(o.bends, 4, o.b_color, (uint32_t)o.x0.size());
}
void orc_get_lra(void* h, uint32_t* src, uint32_t* tgt, float* rest) {
  Oracle& o = *static_cast<Oracle*>(h);
  std::copy(o.lra_src.begin(), o.lra_src.end(), src);
  std::copy(o.lra_tgt.begin(), o.lra_tgt.end(), tgt);
  std::copy(o.lra_rest.begin(), o.lra_rest.end(), rest);
}
void orc_get_rtri(void* h, uint32_t* out) {
  Oracle& o = *static_cast<Oracle*>(h);
  std::copy(o.ortri.begin(), o.ortri.end(), out);
}
static void export_bvh(const Lbvh& b, uint32_t* morton, uint32_t* objs, uint32_t* nodes,
                       float* aabbs, int32_t* iesc, int32_t* eesc) {
  const size_t n = b.num_objects();
  if (morton) std::copy(b.sorted_morton.begin(), b.sorted_morton.end(), morton);
  if (objs) std::copy(b.sorted_objects.begin(), b.sorted_objects.end(), objs);
  for (size_t k = 0; k < b.nodes.size(); ++k) {
    if (nodes) {
      nodes[k * 4] = b.nodes[k].parent;
      nodes[k * 4 + 1] = b.nodes[k].left;
      nodes[k * 4 + 2] = b.nodes[k].right;
      nodes[k * 4 + 3] = b.nodes[k].object;
    }
    if (aabbs) {
      const Box& bx = b.aabbs[k];
      float* a = aabbs + k * 6;
      a[0] = bx.lo.x; a[1] = bx.lo.y; a[2] = bx.lo.z;
      a[3] = bx.hi.x; a[4] = bx.hi.y; a[5] = bx.hi.z;
    }
  }
  if (iesc && n > 1) std::copy(b.iesc.begin(), b.iesc.begin() + (n - 1), iesc);
  if (eesc) std::copy(b.eesc.begin(), b.eesc.end(), eesc);
}
void orc_export_obstacle_bvh(void* h, uint32_t* morton, uint32_t* objs, uint32_t* nodes,
                             float* aabbs, int32_t* iesc, int32_t* eesc) {
  export_bvh(static_cast<Oracle*>(h)->bvh, morton, objs, nodes, aabbs, iesc, eesc);
}
void orc_export_contacts(void* h, int32_t* vf_index, float* vf_qs, int32_t* rt_index, float* rt_qc,
                         float* ee) {
  Oracle& o = *static_cast<Oracle*>(h);
  if (vf_index) std::copy(o.vf_idx.begin(), o.vf_idx.end(), vf_index);
  if (vf_qs) put3(o.vf_qs, vf_qs);
  if (rt_index) std::copy(o.rt_idx.begin(), o.rt_idx.end(), rt_index);
  if (rt_qc) put3(o.rt_qc, rt_qc);
  if (ee) {
    for (size_t k = 0; k < o.ee.size(); ++k) {
      const EEContact& c = o.ee[k];
      float* r = ee + k * 12;
      r[0] = c.dist;
      r[1] = c.p2.x; r[2] = c.p2.y; r[3] = c.p2.z;
      r[4] = c.q2.x; r[5] = c.q2.y; r[6] = c.q2.z;
      r[7] = c.s; r[8] = c.t;
      r[9] = c.fn.x; r[10] = c.fn.y; r[11] = c.fn.z;
    }
  }
}
void orc_export_neighbors(void* h, uint32_t* out) {
  Oracle& o = *static_cast<Oracle*>(h);
  std::copy(o.neighbors.begin(), o.neighbors.end(), out);
}
void orc_hash_now(void* h) {  // run SpatialHashGPU::Hash on the current predicted positions
  Oracle& o = *static_cast<Oracle*>(h);
  hash_particles(o);
}

// ---- Quality-mode proximity repulsion and CCD impacts ------------------------------------------
void orc_cloth_bvh_build(void* h) { build_cloth_bvh(*static_cast<Oracle*>(h)); }
void orc_obstacle_bvh_update_ccd(void* h) {
  Oracle& o = *static_cast<Oracle*>(h);
  update_bvh_ccd(o.bvh, o.ox, o.ox0, o.otri);
}
uint32_t orc_update_pairs(void* h, float thickness) {
  Oracle& o = *static_cast<Oracle*>(h);
  update_pairs(o, thickness);
  return (uint32_t)(o.pairs.size() / 2);
}
void orc_solve_repulsion(void* h, float thickness, float relaxation) {
  solve_repulsion(*static_cast<Oracle*>(h), thickness, relaxation);
}
void orc_check_impacts(void* h, float thickness) { check_impacts(*static_cast<Oracle*>(h), thickness); }
uint32_t orc_imminent_generate(void* h) {
  Oracle& o = *static_cast<Oracle*>(h);
  imminent_generate(o);
  return (uint32_t)o.quads.size();
}
void orc_get_quads(void* h, uint32_t* nodes, float* bary) {
  const Oracle& o = *static_cast<Oracle*>(h);
  for (size_t q = 0; q < o.quads.size(); ++q)
    for (int k = 0; k < 4; ++k) {
      nodes[4 * q + k] = o.quads[q].nodes[k];
      bary[4 * q + k] = o.quads[q].bary[k];
    }
}
void orc_imminent_solve(void* h, float thickness, float relaxation, float dt) {
  imminent_solve(*static_cast<Oracle*>(h), thickness, relaxation, dt);
}
void orc_collision_step(void* h, float obstacle_mass, float thickness, int32_t* stats8) {
  collision_step(*static_cast<Oracle*>(h), obstacle_mass, thickness, stats8);
}
uint32_t orc_get_pairs(void* h, uint32_t* out) {
  Oracle& o = *static_cast<Oracle*>(h);
  if (out) std::copy(o.pairs.begin(), o.pairs.end(), out);
  return (uint32_t)(o.pairs.size() / 2);
}
void orc_get_impacts(void* h, float* t, float* w, float* n, uint32_t* nodes, int32_t* is_vf) {
  Oracle& o = *static_cast<Oracle*>(h);
  for (size_t k = 0; k < o.impacts.size(); ++k) {
    const Oracle::Impact& im = o.impacts[k];
    if (t) t[k] = im.t;
    for (int j = 0; j < 4; ++j) {
      if (w) w[k * 4 + j] = im.w[j];
      if (nodes) nodes[k * 4 + j] = im.nodes[j];
    }
    if (n) {
      n[k * 3] = im.n.x;
      n[k * 3 + 1] = im.n.y;
      n[k * 3 + 2] = im.n.z;
    }
    if (is_vf) is_vf[k] = im.is_vf;
  }
}
void orc_set_positions_predicted(void* h, const float* x) {  // cloth x (predicted) only
  Oracle& o = *static_cast<Oracle*>(h);
  for (size_t i = 0; i < o.x.size(); ++i) o.x[i] = V3{x[i * 3], x[i * 3 + 1], x[i * 3 + 2]};
}
void orc_get_positions_predicted(void* h, float* out) { put3(static_cast<Oracle*>(h)->x, out); }
void orc_export_cloth_bvh(void* h, uint32_t* morton, uint32_t* objs, uint32_t* nodes, float* aabbs,
                          int32_t* iesc, int32_t* eesc) {
  export_bvh(static_cast<Oracle*>(h)->cloth_bvh, morton, objs, nodes, aabbs, iesc, eesc);
}

// ---- standalone LBVH -------------------------------------------------------------------------
void* orc_lbvh_create() { return new Lbvh(); }
void orc_lbvh_destroy(void* h) { delete static_cast<Lbvh*>(h); }
void orc_lbvh_build(void* h, const float* prims, const float* pred, uint32_t n, float scr) {
  Lbvh& b = *static_cast<Lbvh*>(h);
  b.objects.resize(n);
  for (uint32_t i = 0; i < n; ++i) {
    const float* q = prims + (size_t)i * 9;
    const float* r = pred ? pred + (size_t)i * 9 : q;
    Prim& pr = b.objects[i];
    pr.v1 = V3{q[0], q[1], q[2]};
    pr.v2 = V3{q[3], q[4], q[5]};
    pr.v3 = V3{q[6], q[7], q[8]};
    pr.pred1 = V3{r[0], r[1], r[2]};
    pr.pred2 = V3{r[3], r[4], r[5]};
    pr.pred3 = V3{r[6], r[7], r[8]};
    pr.idx1 = i * 3;
    pr.idx2 = i * 3 + 1;
    pr.idx3 = i * 3 + 2;
  }
  b.construct(scr);
}
void orc_lbvh_refit(void* h, const float* pred, uint32_t n) {
  Lbvh& b = *static_cast<Lbvh*>(h);
  std::vector<V3> p3((size_t)n * 3);
  for (size_t k = 0; k < (size_t)n * 3; ++k) p3[k] = V3{pred[k * 3], pred[k * 3 + 1], pred[k * 3 + 2]};
  b.refit_pred(p3);
}
void orc_lbvh_export(void* h, uint32_t* morton, uint32_t* objs, uint32_t* nodes, float* aabbs,
                     int32_t* iesc, int32_t* eesc, int32_t* unique) {
  Lbvh& b = *static_cast<Lbvh*>(h);
  export_bvh(b, morton, objs, nodes, aabbs, iesc, eesc);
  if (unique) *unique = b.morton_unique ? 1 : 0;
}
void orc_lbvh_query(void* h, int kind, const float* q, uint32_t n, uint32_t* counts,
                    uint32_t* cands) {
  Lbvh& b = *static_cast<Lbvh*>(h);
#pragma omp parallel for schedule(dynamic, 64)
  for (long i = 0; i < (long)n; ++i) {
    uint32_t* out = cands + (size_t)i * kMaxBuffer;
    uint32_t c = 0;
    if (kind == 0) {
      c = b.query_point(V3{q[i * 3], q[i * 3 + 1], q[i * 3 + 2]}, out);
    } else if (kind == 1) {
      const float* s = q + (size_t)i * 6;
      c = b.query_segment(V3{s[0], s[1], s[2]}, V3{s[3], s[4], s[5]}, out);
    } else {
      const float* s = q + (size_t)i * 6;
      Box bx;
      bx.lo = V3{s[0], s[1], s[2]};
      bx.hi = V3{s[3], s[4], s[5]};
      c = b.query_box(bx, out);
    }
    counts[i] = c;
  }
}

// ---- primitive KATs ----------------------------------------------------------------------------
uint32_t orc_expand_bits(uint32_t v) { return expand_bits(v); }
uint32_t orc_morton_code(const float* p) { return morton_code(V3{p[0], p[1], p[2]}); }
float orc_nearest_point(const float* p, const float* tri, float* qs, float* uvw) {
  V3 q;
  float u, v, w;
  float d = nearest_point(V3{p[0], p[1], p[2]}, V3{tri[0], tri[1], tri[2]},
                          V3{tri[3], tri[4], tri[5]}, V3{tri[6], tri[7], tri[8]}, q, u, v, w);
  qs[0] = q.x; qs[1] = q.y; qs[2] = q.z;
  uvw[0] = u; uvw[1] = v; uvw[2] = w;
  return d;
}
float orc_ray_intersect(const float* o, const float* d, float len, const float* tri) {
  return ray_intersect(V3{o[0], o[1], o[2]}, V3{d[0], d[1], d[2]}, len, V3{tri[0], tri[1], tri[2]},
                       V3{tri[3], tri[4], tri[5]}, V3{tri[6], tri[7], tri[8]});
}
float orc_closest_seg_seg(const float* p1, const float* q1, const float* p2, const float* q2,
                          float* st, float* c1c2) {
  V3 c1, c2;
  float s, t;
  float d = closest_pt_segment_segment(V3{p1[0], p1[1], p1[2]}, V3{q1[0], q1[1], q1[2]},
                                       V3{p2[0], p2[1], p2[2]}, V3{q2[0], q2[1], q2[2]}, s, t, c1,
                                       c2);
  st[0] = s; st[1] = t;
  c1c2[0] = c1.x; c1c2[1] = c1.y; c1c2[2] = c1.z;
  c1c2[3] = c2.x; c1c2[4] = c2.y; c1c2[5] = c2.z;
  return d;
}
int orc_solve_cubic(float a, float b, float c, float d, float* x) { return solve_cubic(a, b, c, d, x); }
float orc_acos_as(float x) { return acos_as(x); }

}  // extern "C"
