// setup.h — host-side setup of the cloth step: topology, rest state, coloring, adjacency.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

namespace xrt {
namespace setup {

struct V3 {
  float x, y, z;
};

V3 transform_point(const float* m, V3 p);

// Edges in order of first appearance over the faces, oriented as in that face; ef[e] lists the
// faces of edge e in ascending order.
void build_edges(const std::vector<uint32_t>& tri, std::vector<uint32_t>& e,
                 std::vector<std::vector<uint32_t>>& ef);

// GenerateBendingElements (src/physics/ClothSolverHelper.cpp:4-88).
void build_bends(const std::vector<V3>& pos, const std::vector<uint32_t>& tri,
                 const std::vector<uint32_t>& e, const std::vector<std::vector<uint32_t>>& ef,
                 uint32_t offset, std::vector<uint32_t>& out, std::vector<float>& angles);

// Geodesic::ComputeGeodesicDistance (src/utils/Geodesic.cpp:6-79).
std::vector<float> geodesic(const std::vector<V3>& pos,
                            const std::vector<std::vector<uint32_t>>& adj, uint32_t src);

// Greedy coloring of constraints (each `arity` vertex indices) in constraint order.
std::vector<uint32_t> greedy_color(const std::vector<uint32_t>& idx, int arity, uint32_t nv,
                                   uint32_t& ncolors);
bool coloring_valid(const std::vector<uint32_t>& idx, int arity, const std::vector<uint32_t>& col,
                    uint32_t nv, std::string& why);

// vertex -> (face << 2 | corner), ascending faces
void build_vf(const std::vector<uint32_t>& tri, uint32_t nv, std::vector<uint32_t>& ptr,
              std::vector<uint32_t>& list);
// vertex -> (edge << 1 | side), ascending edges
void build_ve(const std::vector<uint32_t>& edges, uint32_t nv, std::vector<uint32_t>& ptr,
              std::vector<uint32_t>& list);
// RTriBuild_Kernel (src/physics/representative_triangle/RTriangle.cu:19-84)
std::vector<uint32_t> build_rtri(const std::vector<uint32_t>& tri, uint32_t nv);

float length(V3 a);
V3 sub(V3 a, V3 b);

}  // namespace setup
}  // namespace xrt
