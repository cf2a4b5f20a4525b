// setup.cpp — host-side setup of the cloth step (runs once per xrt_start / xrt_add_cloth).
//
// Rest data follow the reference's setup code with glm's float evaluation order (this file is
// compiled without FMA contraction):
//   stretch rest lengths ....... PrepareBasicStretchData (src/physics/ClothSolverHelper.cpp:90-109)
//   bend elements / rest angles  GenerateBendingElements (ClothSolverHelper.cpp:4-88), including the
//                                string test for the winding of the first face
//   geodesic LRA lengths ....... Geodesic::ComputeGeodesicDistance (src/utils/Geodesic.cpp:6-79)
//   representative triangles ... RTriBuild_Kernel (src/physics/representative_triangle/RTriangle.cu:19-84)
// The reference takes edge order from vcglib; here edges are numbered by first appearance over
// the faces, and the graph coloring (randomized in the reference, GraphColoring::Paint,
// src/physics/graph_coloring/Base.cu:163-317) is a deterministic greedy coloring unless the
// caller supplies one.
#include "setup.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <map>
#include <queue>
#include <set>

namespace xrt {
namespace setup {

static inline V3 add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 mul(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
static inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
float length(V3 a) { return std::sqrt(dot(a, a)); }
static inline V3 normalize(V3 a) { return mul(a, 1.0f / std::sqrt(dot(a, a))); }

V3 transform_point(const float* m, V3 p) {
  float r[3];
  for (int k = 0; k < 3; ++k) {
    const float a0 = m[0 + k] * p.x, a1 = m[4 + k] * p.y, a2 = m[8 + k] * p.z, a3 = m[12 + k] * 1.0f;
    r[k] = (a0 + a1) + (a2 + a3);
  }
  return V3{r[0], r[1], r[2]};
}

void build_edges(const std::vector<uint32_t>& tri, std::vector<uint32_t>& e,
                 std::vector<std::vector<uint32_t>>& ef) {
  std::map<uint64_t, uint32_t> seen;
  const uint32_t nf = (uint32_t)(tri.size() / 3);
  for (uint32_t f = 0; f < nf; ++f) {
    for (int k = 0; k < 3; ++k) {
      const uint32_t a = tri[f * 3 + k], b = tri[f * 3 + (k + 1) % 3];
      const uint64_t key = ((uint64_t)std::min(a, b) << 32) | std::max(a, b);
      auto it = seen.find(key);
      if (it == seen.end()) {
        seen.emplace(key, (uint32_t)(e.size() / 2));
        e.push_back(a);
        e.push_back(b);
        ef.push_back(std::vector<uint32_t>{f});
      } else {
        ef[it->second].push_back(f);
      }
    }
  }
}

void build_bends(const std::vector<V3>& pos, const std::vector<uint32_t>& tri,
                 const std::vector<uint32_t>& e, const std::vector<std::vector<uint32_t>>& ef,
                 uint32_t offset, std::vector<uint32_t>& out, std::vector<float>& angles) {
  const size_t ne = e.size() / 2;
  for (size_t ei = 0; ei < ne; ++ei) {
    const std::vector<uint32_t>& faces = ef[ei];
    if (faces.size() < 2) continue;
    const uint32_t ea = e[ei * 2], eb = e[ei * 2 + 1];
    uint32_t idx1 = ea, idx2 = eb;
    for (size_t i = 0; i < faces.size(); ++i) {
      for (size_t j = i + 1; j < faces.size(); ++j) {
        const uint32_t f1 = faces[i], f2 = faces[j];
        auto opposite = [&](uint32_t f) {
          for (int k = 0; k < 3; ++k) {
            const uint32_t q = tri[f * 3 + k];
            if (q != ea && q != eb) return q;
          }
          return tri[f * 3];
        };
        const uint32_t idx3 = opposite(f1), idx4 = opposite(f2);
        std::string f1s = std::to_string(tri[f1 * 3]) + "," + std::to_string(tri[f1 * 3 + 1]) + "," +
                          std::to_string(tri[f1 * 3 + 2]);
        f1s += "," + f1s;
        const std::string common = std::to_string(idx1) + "," + std::to_string(idx2);
        if (f1s.find(common) == std::string::npos) std::swap(idx1, idx2);
        const V3 v1 = pos[idx1], v2 = pos[idx2], v3 = pos[idx3], v4 = pos[idx4];
        const V3 n1 = normalize(cross(sub(v1, v3), sub(v2, v3)));
        const V3 n2 = normalize(cross(sub(v2, v4), sub(v1, v4)));
        float d = dot(n1, n2);
        if (d < -1) d = -1;
        else if (d > 1) d = 1;
        out.push_back(idx1 + offset);
        out.push_back(idx2 + offset);
        out.push_back(idx3 + offset);
        out.push_back(idx4 + offset);
        angles.push_back(std::acos(d));
      }
    }
  }
}

std::vector<float> geodesic(const std::vector<V3>& pos,
                            const std::vector<std::vector<uint32_t>>& adj, uint32_t src) {
  std::vector<float> dist(pos.size(), FLT_MAX);
  typedef std::pair<float, uint32_t> Item;
  std::priority_queue<Item, std::vector<Item>, std::greater<Item>> pq;
  dist[src] = 0.0f;
  pq.push(Item(0.0f, src));
  while (!pq.empty()) {
    const uint32_t cur = pq.top().second;
    pq.pop();
    for (uint32_t nb : adj[cur]) {
      const float w = length(sub(pos[nb], pos[cur]));
      if (dist[nb] > dist[cur] + w) {
        dist[nb] = dist[cur] + w;
        pq.push(Item(dist[nb], nb));
      }
    }
  }
  return dist;
}

std::vector<uint32_t> greedy_color(const std::vector<uint32_t>& idx, int arity, uint32_t nv,
                                   uint32_t& ncolors) {
  const size_t n = idx.size() / arity;
  std::vector<uint32_t> col(n);
  // per vertex: bit mask of the first 64 colors, overflow list beyond
  std::vector<uint64_t> mask(nv, 0);
  std::vector<std::vector<uint32_t>> over(nv);
  ncolors = 0;
  for (size_t c = 0; c < n; ++c) {
    uint64_t used = 0;
    for (int a = 0; a < arity; ++a) used |= mask[idx[c * arity + a]];
    uint32_t k;
    if (~used) {
      k = (uint32_t)__builtin_ctzll(~used);
    } else {
      k = 64;
      for (;; ++k) {
        bool clash = false;
        for (int a = 0; a < arity && !clash; ++a) {
          const auto& o = over[idx[c * arity + a]];
          clash = std::find(o.begin(), o.end(), k) != o.end();
        }
        if (!clash) break;
      }
    }
    col[c] = k;
    for (int a = 0; a < arity; ++a) {
      if (k < 64) mask[idx[c * arity + a]] |= (1ull << k);
      else over[idx[c * arity + a]].push_back(k);
    }
    ncolors = std::max(ncolors, k + 1);
  }
  return col;
}

bool coloring_valid(const std::vector<uint32_t>& idx, int arity, const std::vector<uint32_t>& col,
                    uint32_t nv, std::string& why) {
  const size_t n = idx.size() / arity;
  if (col.size() != n) {
    why = "coloring has " + std::to_string(col.size()) + " entries, expected " + std::to_string(n);
    return false;
  }
  std::vector<std::set<uint32_t>> used(nv);
  for (size_t c = 0; c < n; ++c)
    for (int a = 0; a < arity; ++a)
      if (!used[idx[c * arity + a]].insert(col[c]).second) {
        why = "constraints sharing vertex " + std::to_string(idx[c * arity + a]) + " have color " +
              std::to_string(col[c]);
        return false;
      }
  return true;
}

void build_vf(const std::vector<uint32_t>& tri, uint32_t nv, std::vector<uint32_t>& ptr,
              std::vector<uint32_t>& list) {
  ptr.assign(nv + 1, 0);
  const uint32_t nf = (uint32_t)(tri.size() / 3);
  for (uint32_t f = 0; f < nf; ++f)
    for (int k = 0; k < 3; ++k) ptr[tri[f * 3 + k] + 1]++;
  for (uint32_t i = 0; i < nv; ++i) ptr[i + 1] += ptr[i];
  list.assign(ptr[nv], 0);
  std::vector<uint32_t> fill(ptr.begin(), ptr.end() - 1);
  for (uint32_t f = 0; f < nf; ++f)  // ascending f keeps every list sorted
    for (uint32_t k = 0; k < 3; ++k) list[fill[tri[f * 3 + k]]++] = (f << 2) | k;
}

void build_ve(const std::vector<uint32_t>& edges, uint32_t nv, std::vector<uint32_t>& ptr,
              std::vector<uint32_t>& list) {
  ptr.assign(nv + 1, 0);
  const uint32_t ne = (uint32_t)(edges.size() / 2);
  for (uint32_t e = 0; e < ne; ++e) {
    ptr[edges[2 * e] + 1]++;
    ptr[edges[2 * e + 1] + 1]++;
  }
  for (uint32_t i = 0; i < nv; ++i) ptr[i + 1] += ptr[i];
  list.assign(ptr[nv], 0);
  std::vector<uint32_t> fill(ptr.begin(), ptr.end() - 1);
  for (uint32_t e = 0; e < ne; ++e) {
    list[fill[edges[2 * e]]++] = (e << 1) | 0u;
    list[fill[edges[2 * e + 1]]++] = (e << 1) | 1u;
  }
}

std::vector<uint32_t> build_rtri(const std::vector<uint32_t>& tri, uint32_t nv) {
  // sorted, de-duplicated vertex -> face lists (the reference's std::set per vertex)
  std::vector<std::vector<uint32_t>> vf(nv);
  const uint32_t nf = (uint32_t)(tri.size() / 3);
  for (uint32_t f = 0; f < nf; ++f)
    for (int k = 0; k < 3; ++k) vf[tri[f * 3 + k]].push_back(f);
  std::vector<uint32_t> pre(nv + 1, 0), lst;
  for (uint32_t i = 0; i < nv; ++i) {
    auto& l = vf[i];
    std::sort(l.begin(), l.end());
    l.erase(std::unique(l.begin(), l.end()), l.end());
    lst.insert(lst.end(), l.begin(), l.end());
    pre[i + 1] = (uint32_t)lst.size();
  }
  std::vector<uint32_t> out(nf, 0);
  for (uint32_t fid = 0; fid < nf; ++fid) {
    const uint32_t fv[3] = {tri[fid * 3], tri[fid * 3 + 1], tri[fid * 3 + 2]};
    uint32_t info = 0;
    uint32_t j_start = pre[fv[0]], j_end = pre[fv[0] + 1];
    for (uint32_t iv = 0; iv < 3; ++iv) {
      uint32_t off = j_start;
      const uint32_t i_end = j_end;
      uint32_t i_f = lst[off++];
      if (i_f == fid) info |= 1u << iv;
      const uint32_t jv = (iv + 1) % 3;
      j_start = pre[fv[jv]];
      j_end = pre[fv[jv] + 1];
      uint32_t of = 0xFFFFFFFFu;
      for (uint32_t jno = j_start; jno < j_end; ++jno)
        if (lst[jno] == i_f && fid != i_f) {
          of = i_f;
          break;
        }
      for (; off < i_end && of == 0xFFFFFFFFu; ++off) {
        i_f = lst[off];
        for (uint32_t jno = j_start; jno < j_end; ++jno)
          if (lst[jno] == i_f && fid != i_f) {
            of = i_f;
            break;
          }
      }
      if (fid < of) info |= 1u << (iv + 3);
    }
    out[fid] = info;
  }
  return out;
}

TileSchedule build_tiles(const std::vector<uint32_t>& idx, int arity, uint32_t nv,
                         uint32_t tile_vertices, const std::vector<uint32_t>& segments) {
  TileSchedule S;
  const size_t n = idx.size() / arity;
  // vertex -> tile: tiles are cut inside each segment from its first vertex
  std::vector<uint32_t> seg = segments.empty() ? std::vector<uint32_t>{0u} : segments;
  seg.push_back(nv);
  std::vector<uint32_t> seg_tile(seg.size(), 0);
  for (size_t s = 0; s + 1 < seg.size(); ++s)
    seg_tile[s + 1] = seg_tile[s] + std::max(1u, (seg[s + 1] - seg[s] + tile_vertices - 1) / tile_vertices);
  const uint32_t ntiles = seg_tile.back();
  auto tile_of = [&](uint32_t v) {
    const size_t s = (size_t)(std::upper_bound(seg.begin(), seg.end() - 1, v) - seg.begin()) - 1;
    return seg_tile[s] + (v - seg[s]) / tile_vertices;
  };
  // constraint -> tile of its smallest vertex
  std::vector<std::vector<uint32_t>> members(ntiles);
  std::vector<uint32_t> ctile(n);
  for (size_t c = 0; c < n; ++c) {
    uint32_t m = idx[c * arity];
    for (int a = 1; a < arity; ++a) m = std::min(m, idx[c * arity + a]);
    ctile[c] = tile_of(m);
    members[ctile[c]].push_back((uint32_t)c);
  }
  // footprints
  std::vector<std::vector<uint32_t>> foot(ntiles);
  for (uint32_t t = 0; t < ntiles; ++t) {
    auto& f = foot[t];
    for (uint32_t c : members[t])
      for (int a = 0; a < arity; ++a) f.push_back(idx[c * arity + a]);
    std::sort(f.begin(), f.end());
    f.erase(std::unique(f.begin(), f.end()), f.end());
  }
  // tile colors: greedy over tiles in order; conflict = shared footprint vertex
  std::vector<uint32_t> tcolor(ntiles, 0);
  std::vector<uint64_t> vmask(nv, 0);  // tile colors (< 64) already touching a vertex
  for (uint32_t t = 0; t < ntiles; ++t) {
    uint64_t used = 0;
    for (uint32_t v : foot[t]) used |= vmask[v];
    if (~used == 0) return TileSchedule{};  // more than 64 tile colors: caller falls back
    const uint32_t k = (uint32_t)__builtin_ctzll(~used);
    tcolor[t] = k;
    for (uint32_t v : foot[t]) vmask[v] |= 1ull << k;
    S.num_tile_colors = std::max(S.num_tile_colors, k + 1);
  }
  // local colors inside each tile (constraint order)
  std::vector<uint32_t> lcolor(n, 0);
  std::vector<std::vector<uint32_t>> by_local(ntiles);
  for (uint32_t t = 0; t < ntiles; ++t) {
    std::vector<uint32_t> sub;
    sub.reserve(members[t].size() * arity);
    for (uint32_t c : members[t])
      for (int a = 0; a < arity; ++a) sub.push_back(idx[c * arity + a]);
    // greedy on the tile's constraints with vertex masks keyed by footprint position
    std::vector<uint64_t> m(foot[t].size(), 0);
    for (size_t j = 0; j < members[t].size(); ++j) {
      uint64_t used = 0;
      uint32_t slot[4];
      for (int a = 0; a < arity; ++a) {
        slot[a] = (uint32_t)(std::lower_bound(foot[t].begin(), foot[t].end(), sub[j * arity + a]) -
                             foot[t].begin());
        used |= m[slot[a]];
      }
      if (~used == 0) return TileSchedule{};  // more than 64 local colors
      const uint32_t k = (uint32_t)__builtin_ctzll(~used);
      lcolor[members[t][j]] = k;
      for (int a = 0; a < arity; ++a) m[slot[a]] |= 1ull << k;
      S.num_local = std::max(S.num_local, k + 1);
    }
  }
  S.color.resize(n);
  for (size_t c = 0; c < n; ++c) S.color[c] = tcolor[ctile[c]] * S.num_local + lcolor[c];
  // execution order: tile color, tile, local color, constraint order
  S.tile_color_ptr.assign(1, 0);
  S.foot_ptr.assign(1, 0);
  S.lc_ptr.clear();
  for (uint32_t k = 0; k < S.num_tile_colors; ++k) {
    for (uint32_t t = 0; t < ntiles; ++t) {
      if (tcolor[t] != k || members[t].empty()) continue;
      S.tiles.push_back(t);
      S.foot.insert(S.foot.end(), foot[t].begin(), foot[t].end());
      S.foot_ptr.push_back((uint32_t)S.foot.size());
      S.max_footprint = std::max(S.max_footprint, (uint32_t)foot[t].size());
      for (uint32_t l = 0; l < S.num_local; ++l) {
        S.lc_ptr.push_back((uint32_t)S.order.size());
        for (uint32_t c : members[t]) {
          if (lcolor[c] != l) continue;
          S.order.push_back(c);
          for (int a = 0; a < arity; ++a)
            S.local_slot.push_back((uint32_t)(std::lower_bound(foot[t].begin(), foot[t].end(),
                                                               idx[c * arity + a]) -
                                              foot[t].begin()));
        }
      }
    }
    S.tile_color_ptr.push_back((uint32_t)S.tiles.size());
  }
  S.lc_ptr.push_back((uint32_t)S.order.size());
  return S;
}

void fem_strain_rest(const std::vector<float>& x, const std::vector<uint32_t>& tri,
                     std::vector<float>& area, std::vector<float>& inv) {
  const size_t nf = tri.size() / 3;
  area.assign(nf, 0.0f);
  inv.assign(4 * nf, 0.0f);
  auto P = [&](uint32_t v) { return V3{x[3 * v], x[3 * v + 1], x[3 * v + 2]}; };
  for (size_t f = 0; f < nf; ++f) {
    const V3 p0 = P(tri[3 * f]), p1 = P(tri[3 * f + 1]), p2 = P(tri[3 * f + 2]);
    const V3 normal0 = cross(sub(p1, p0), sub(p2, p0));
    area[f] = 0.5f * length(normal0);
    const V3 axis0_1 = normalize(sub(p1, p0));
    const V3 axis0_2 = normalize(cross(normal0, axis0_1));
    // material coordinates (dot with axis0_2, dot with axis0_1); P[c][r] in glm's order
    const float q0x = dot(p0, axis0_2), q0y = dot(p0, axis0_1);
    const float q1x = dot(p1, axis0_2), q1y = dot(p1, axis0_1);
    const float q2x = dot(p2, axis0_2), q2y = dot(p2, axis0_1);
    const float m00 = q0x - q2x, m10 = q0y - q2y, m01 = q1x - q2x, m11 = q1y - q2y;
    const float det = m00 * m11 - m10 * m01;
    float* o = &inv[4 * f];
    if (std::fabs(det) > 1e-6f) {
      const float r = 1.0f / det;
      o[0] = m11 * r;      // inv[0][0]
      o[1] = (-m01) * r;   // inv[0][1]
      o[2] = (-m10) * r;   // inv[1][0]
      o[3] = m00 * r;      // inv[1][1]
    } else {  // degenerate rest triangle: area ~0, its projection never moves anything
      o[0] = o[3] = 1.0f;
    }
  }
}

static inline float cot_theta(V3 v, V3 w) { return dot(v, w) / length(cross(v, w)); }

void iso_bend_hessian(const std::vector<float>& x, const std::vector<uint32_t>& bends,
                      std::vector<float>& q) {
  const size_t nb = bends.size() / 4;
  q.assign(16 * nb, 0.0f);
  auto P = [&](uint32_t v) { return V3{x[3 * v], x[3 * v + 1], x[3 * v + 2]}; };
  for (size_t b = 0; b < nb; ++b) {
    const V3 p0 = P(bends[4 * b]), p1 = P(bends[4 * b + 1]), p2 = P(bends[4 * b + 2]),
             p3 = P(bends[4 * b + 3]);
    const V3 e0 = sub(p1, p0), e1 = sub(p2, p0), e2 = sub(p3, p0), e3 = sub(p2, p1),
             e4 = sub(p3, p1);
    const V3 ne0 = V3{-e0.x, -e0.y, -e0.z};
    const float c01 = cot_theta(e0, e1), c02 = cot_theta(e0, e2);
    const float c03 = cot_theta(ne0, e3), c04 = cot_theta(ne0, e4);
    const float A0 = 0.5f * length(cross(sub(p1, p0), sub(p2, p0)));  // TriangleArea(p0, p1, p2)
    const float A1 = 0.5f * length(cross(sub(p0, p1), sub(p3, p1)));  // TriangleArea(p1, p0, p3)
    const float coeff = 3.0f / (A0 + A1);
    const float K[4] = {c03 + c04, c01 + c02, -c01 - c03, -c02 - c04};
    float* o = &q[16 * b];
    for (int j = 0; j < 4; ++j)
      for (int i = 0; i < 4; ++i) o[4 * j + i] = coeff * (K[i] * K[j]);  // Q[j][i]
  }
}

}  // namespace setup
}  // namespace xrt
