// api_contact.cpp — C ABI of the Quality-mode self-contact operators (include/xrt_contact.h) and
// the host setup of their topology.
//
// Topology follows the reference's mesh records: Face::SetEdge (edge i joins nodes i and i+1,
// src/memory/Face.cu:9-21), Face::n set once at registration from the mesh positions
// (PhysicsMeshHelper.cu:118-123, Face::Update), Edge::adjacents (up to MAX_EF_ADJACENTS = 4
// faces, here in ascending face order), Node::is_free (false for pinned cloth vertices and for
// every obstacle vertex), R-triangle masks of both meshes (ClothSolverBase.cpp:489-525).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <string>
#include <vector>

#include "../../include/xrt_contact.h"
#include "context.h"
#include "setup.h"

using xrt::Context;

namespace {

template <typename T>
cudaError_t put(xrt::DBuf<T>& d, const std::vector<T>& h, cudaStream_t s) {
  cudaError_t e = d.reserve(h.empty() ? 1 : h.size());
  if (e != cudaSuccess || h.empty()) return e;
  return cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

void face_topology(const std::vector<uint32_t>& tri, const std::vector<uint32_t>& edges,
                   const std::vector<float>& reg, uint32_t node_off, uint32_t edge_off,
                   uint32_t face_off, const std::vector<uint32_t>& rtri, std::vector<int4>& face,
                   std::vector<int4>& fedge, std::vector<float4>& fn0, std::vector<uint2>& uedge,
                   std::vector<int4>& eadj) {
  std::map<uint64_t, uint32_t> key;
  const uint32_t ne = (uint32_t)(edges.size() / 2);
  for (uint32_t e = 0; e < ne; ++e) {
    const uint32_t a = edges[2 * e], b = edges[2 * e + 1];
    key[((uint64_t)std::min(a, b) << 32) | std::max(a, b)] = e;
    uedge.push_back(make_uint2(a + node_off, b + node_off));
  }
  std::vector<int4> adj(ne, make_int4(-1, -1, -1, -1));
  std::vector<int> fill(ne, 0);
  const uint32_t nf = (uint32_t)(tri.size() / 3);
  for (uint32_t f = 0; f < nf; ++f) {
    int ed[3];
    for (int k = 0; k < 3; ++k) {
      const uint32_t a = tri[3 * f + k], b = tri[3 * f + (k + 1) % 3];
      const uint32_t e = key[((uint64_t)std::min(a, b) << 32) | std::max(a, b)];
      ed[k] = (int)(e + edge_off);
      int* slot = fill[e] == 0 ? &adj[e].x : fill[e] == 1 ? &adj[e].y : fill[e] == 2 ? &adj[e].z
                                                                                     : &adj[e].w;
      if (fill[e] < 4) {
        *slot = (int)(f + face_off);
        fill[e]++;
      }
    }
    face.push_back(make_int4((int)(tri[3 * f] + node_off), (int)(tri[3 * f + 1] + node_off),
                             (int)(tri[3 * f + 2] + node_off), (int)rtri[f]));
    fedge.push_back(make_int4(ed[0], ed[1], ed[2], 0));
    auto P = [&](uint32_t i) { return xrt::setup::V3{reg[3 * i], reg[3 * i + 1], reg[3 * i + 2]}; };
    const xrt::setup::V3 p0 = P(tri[3 * f]), p1 = P(tri[3 * f + 1]), p2 = P(tri[3 * f + 2]);
    const xrt::setup::V3 d1 = xrt::setup::sub(p1, p0), d2 = xrt::setup::sub(p2, p0);
    const float cx = d1.y * d2.z - d2.y * d1.z, cy = d1.z * d2.x - d2.z * d1.x,
                cz = d1.x * d2.y - d2.x * d1.y;
    const float inv = 1.0f / std::sqrt((cx * cx + cy * cy) + cz * cz);
    fn0.push_back(make_float4(cx * inv, cy * inv, cz * inv, 0.0f));
  }
  eadj.insert(eadj.end(), adj.begin(), adj.end());
}

}  // namespace

xrt_status xrt::prox_prepare(Context& c) {
  if (c.prox.ready) return XRT_OK;
  if (!c.started) {
    c.set_error("call xrt_start first");
    return XRT_ERR_STATE;
  }
  if (c.instanced) {  // the obstacle LBVH of a batched context is a forest, one tree per instance
    c.set_error("Quality-mode self contact is available in merged contexts only");
    return XRT_ERR_STATE;
  }
  std::vector<int4> face, fedge, eadj;
  std::vector<float4> fn0;
  std::vector<uint2> uedge;
  std::vector<float> creg;
  for (const auto& cl : c.cloths) creg.insert(creg.end(), cl.mesh_pos.begin(), cl.mesh_pos.end());
  std::vector<uint32_t> cptr, clist;
  const std::vector<uint32_t> crtri = xrt::setup::build_rtri(c.h_tri, c.nv);
  face_topology(c.h_tri, c.h_edges, creg, 0, 0, 0, crtri, face, fedge, fn0, uedge, eadj);
  if (c.onf > 0) {
    std::vector<uint32_t> oedges;
    std::vector<std::vector<uint32_t>> oef;
    xrt::setup::build_edges(c.h_otri, oedges, oef);
    face_topology(c.h_otri, oedges, c.h_omesh, c.nv, c.ne, c.nf, c.h_ortri, face, fedge, fn0,
                  uedge, eadj);
  }
  cudaStream_t s = c.stream;
  XRT_CUDA(&c, put(c.prox.face, face, s));
  XRT_CUDA(&c, put(c.prox.fedge, fedge, s));
  XRT_CUDA(&c, put(c.prox.fn0, fn0, s));
  XRT_CUDA(&c, put(c.prox.edge, uedge, s));
  XRT_CUDA(&c, put(c.prox.eadj, eadj, s));
  XRT_CUDA(&c, put(c.prox.cfree, c.h_cfree, s));
  XRT_CUDA(&c, c.prox.ov.reserve(std::max(c.onv, 1u)));  // obstacle Node::v starts at 0
  XRT_CUDA(&c, cudaMemsetAsync(c.prox.ov.p, 0, sizeof(float4) * std::max(c.onv, 1u), s));
  XRT_CUDA(&c, c.prox.counts.reserve(std::max(c.nf, 1u)));
  XRT_CUDA(&c, c.prox.incl.reserve(2 * (size_t)std::max(c.nf, 1u)));
  XRT_CUDA(&c, c.prox.total.reserve(2));
  XRT_CUDA(&c, c.prox.deltas.reserve(3 * (size_t)c.nv));
  XRT_CUDA(&c, c.prox.rcounts.reserve(c.nv));
  XRT_CUDA(&c, cudaMemsetAsync(c.prox.deltas.p, 0, sizeof(float) * 3 * c.nv, s));
  XRT_CUDA(&c, cudaMemsetAsync(c.prox.rcounts.p, 0, sizeof(int) * c.nv, s));
  XRT_CUDA(&c, c.prox.cbvh.reserve(c.nf));
  XRT_CUDA(&c, cudaStreamSynchronize(s));
  c.prox.ready = true;
  return XRT_OK;
}

using xrt::prox_prepare;

extern "C" {

xrt_status xrt_cloth_bvh_build(xrt_ctx* h) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  cudaSetDevice(c.device);
  xrt_status st = prox_prepare(c);
  if (st != XRT_OK) return st;
  xrt::launch_cloth_bvh_build(c);
  XRT_CUDA(&c, cudaGetLastError());
  return XRT_OK;
}

xrt_status xrt_obstacle_bvh_update_ccd(xrt_ctx* h) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  cudaSetDevice(c.device);
  xrt_status st = prox_prepare(c);
  if (st != XRT_OK) return st;
  xrt::launch_update_ccd(c.bvh, c.ox.p, c.ox0.p, c.otri.p, c.stream, c.err.p);
  XRT_CUDA(&c, cudaGetLastError());
  return XRT_OK;
}

xrt_status xrt_proximity_update_pairs(xrt_ctx* h, float thickness, uint32_t* out_n) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  cudaSetDevice(c.device);
  xrt_status st = prox_prepare(c);
  if (st != XRT_OK) return st;
  if (!c.prox.cbvh.active) {
    c.set_error("build the cloth LBVH first (xrt_cloth_bvh_build)");
    return XRT_ERR_STATE;
  }
  XRT_CUDA(&c, xrt::prox_update_pairs(c, thickness));
  if (out_n) *out_n = c.prox.npairs;
  return XRT_OK;
}

xrt_status xrt_proximity_solve(xrt_ctx* h, float thickness, float relaxation) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  cudaSetDevice(c.device);
  xrt_status st = prox_prepare(c);
  if (st != XRT_OK) return st;
  xrt::prox_solve(c, thickness, relaxation);
  XRT_CUDA(&c, cudaGetLastError());
  return XRT_OK;
}

xrt_status xrt_impacts_check(xrt_ctx* h, float thickness, uint32_t* out_n) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  cudaSetDevice(c.device);
  xrt_status st = prox_prepare(c);
  if (st != XRT_OK) return st;
  XRT_CUDA(&c, xrt::prox_check_impacts(c, thickness));
  if (out_n) *out_n = c.prox.nimpacts;
  return XRT_OK;
}

xrt_status xrt_imminent_generate(xrt_ctx* h, uint32_t* out_n) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  cudaSetDevice(c.device);
  xrt_status st = prox_prepare(c);
  if (st != XRT_OK) return st;
  if (!c.prox.cbvh.active) {
    c.set_error("build the cloth LBVH first (xrt_cloth_bvh_build)");
    return XRT_ERR_STATE;
  }
  XRT_CUDA(&c, xrt::prox_imminent_generate(c));
  std::vector<uint4> q(c.prox.nquads);
  if (!q.empty())
    XRT_CUDA(&c, cudaMemcpyAsync(q.data(), c.prox.qnodes.p, sizeof(uint4) * q.size(),
                                 cudaMemcpyDeviceToHost, c.stream));
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  uint32_t n = 0;
  for (const uint4& v : q) n += v.x != 0xFFFFFFFFu;
  if (out_n) *out_n = n;
  return XRT_OK;
}

// Slots are 12 per pair (9 edge-edge, then 3 vertex-face); exported compacted in Generate's
// order: the edge-edge quadratures of every pair, then the vertex-face ones.
xrt_status xrt_export_quads(xrt_ctx* h, uint32_t* nodes, float* bary) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  cudaSetDevice(c.device);
  const size_t ns = c.prox.nquads;
  std::vector<uint4> q(ns);
  std::vector<float4> b(ns);
  if (ns) {
    XRT_CUDA(&c, cudaMemcpyAsync(q.data(), c.prox.qnodes.p, sizeof(uint4) * ns,
                                 cudaMemcpyDeviceToHost, c.stream));
    XRT_CUDA(&c, cudaMemcpyAsync(b.data(), c.prox.qbary.p, sizeof(float4) * ns,
                                 cudaMemcpyDeviceToHost, c.stream));
  }
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  size_t o = 0;
  for (int vf = 0; vf < 2; ++vf)
    for (size_t s = 0; s < ns; ++s) {
      if (q[s].x == 0xFFFFFFFFu || ((s % 12) >= 9) != (vf == 1)) continue;
      const uint32_t qn[4] = {q[s].x, q[s].y, q[s].z, q[s].w};
      const float qb[4] = {b[s].x, b[s].y, b[s].z, b[s].w};
      for (int k = 0; k < 4; ++k) {
        if (nodes) nodes[4 * o + k] = qn[k];
        if (bary) bary[4 * o + k] = qb[k];
      }
      ++o;
    }
  return XRT_OK;
}

xrt_status xrt_imminent_solve(xrt_ctx* h, float thickness, float relaxation, float dt) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  cudaSetDevice(c.device);
  xrt_status st = prox_prepare(c);
  if (st != XRT_OK) return st;
  xrt::prox_imminent_solve(c, thickness, relaxation, dt);
  XRT_CUDA(&c, cudaGetLastError());
  return XRT_OK;
}

xrt_status xrt_export_pairs(xrt_ctx* h, uint32_t* pairs) {
  if (!h || !pairs) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  cudaSetDevice(c.device);
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  if (c.prox.npairs)
    XRT_CUDA(&c, cudaMemcpy(pairs, c.prox.pairs.p, 8 * (size_t)c.prox.npairs, cudaMemcpyDeviceToHost));
  return XRT_OK;
}

xrt_status xrt_export_impacts(xrt_ctx* h, float* t, float* w, float* n, uint32_t* nodes,
                              int32_t* is_vf) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  cudaSetDevice(c.device);
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  const size_t ni = c.prox.nimpacts;
  if (ni == 0) return XRT_OK;
  if (t) XRT_CUDA(&c, cudaMemcpy(t, c.prox.imp_t.p, 4 * ni, cudaMemcpyDeviceToHost));
  if (w) XRT_CUDA(&c, cudaMemcpy(w, c.prox.imp_w.p, 16 * ni, cudaMemcpyDeviceToHost));
  if (nodes) XRT_CUDA(&c, cudaMemcpy(nodes, c.prox.imp_nodes.p, 16 * ni, cudaMemcpyDeviceToHost));
  if (n || is_vf) {
    std::vector<float4> hn(ni);
    XRT_CUDA(&c, cudaMemcpy(hn.data(), c.prox.imp_n.p, 16 * ni, cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < ni; ++k) {
      if (n) {
        n[3 * k] = hn[k].x;
        n[3 * k + 1] = hn[k].y;
        n[3 * k + 2] = hn[k].z;
      }
      if (is_vf) is_vf[k] = hn[k].w != 0.0f ? 1 : 0;
    }
  }
  return XRT_OK;
}

xrt_status xrt_export_cloth_bvh(xrt_ctx* h, uint32_t* morton, uint32_t* objs, uint32_t* nodes,
                                float* aabbs, int32_t* iesc, int32_t* eesc) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  cudaSetDevice(c.device);
  std::string err;
  xrt_status st = xrt::export_lbvh(c.prox.cbvh, c.stream, err, morton, objs, nodes, aabbs, iesc,
                                   eesc, nullptr);
  if (st != XRT_OK) c.set_error(err);
  return st;
}

xrt_status xrt_get_predicted(xrt_ctx* h, float* out) {
  if (!h || !out) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (!c.started) return XRT_ERR_STATE;
  cudaSetDevice(c.device);
  std::vector<float4> x(c.nv);
  XRT_CUDA(&c, cudaMemcpyAsync(x.data(), c.x.p, 16 * (size_t)c.nv, cudaMemcpyDeviceToHost, c.stream));
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  for (uint32_t i = 0; i < c.nv; ++i) {
    out[3 * i] = x[i].x;
    out[3 * i + 1] = x[i].y;
    out[3 * i + 2] = x[i].z;
  }
  return XRT_OK;
}

xrt_status xrt_set_predicted(xrt_ctx* h, const float* pos) {
  if (!h || !pos) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (!c.started) return XRT_ERR_STATE;
  cudaSetDevice(c.device);
  std::vector<float4> x(c.nv);
  for (uint32_t i = 0; i < c.nv; ++i)
    x[i] = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], c.h_w[i]);
  XRT_CUDA(&c, cudaMemcpyAsync(c.x.p, x.data(), 16 * (size_t)c.nv, cudaMemcpyHostToDevice, c.stream));
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  return XRT_OK;
}

}  // extern "C"
