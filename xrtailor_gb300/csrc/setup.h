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

// Tile schedule of a constraint set for tile-local Gauss-Seidel.  Vertices are cut into
// contiguous tiles; a constraint belongs to the tile of its smallest vertex; tiles whose
// footprints (vertices their constraints touch) intersect get different tile colors; inside a
// tile the constraints get local colors.  Processing tile color by tile color, local color by
// local color, is a coloring of the whole set: global color = tile_color * num_local + local.
struct TileSchedule {
  uint32_t num_tile_colors = 0, num_local = 0;
  std::vector<uint32_t> color;          // global color per constraint (input order)
  std::vector<uint32_t> order;          // constraints in execution order
  std::vector<uint32_t> local_slot;     // per execution slot and arity: footprint-local index
  std::vector<uint32_t> tiles;          // tiles in execution order (grouped by tile color)
  std::vector<uint32_t> tile_color_ptr; // num_tile_colors + 1 offsets into `tiles`
  std::vector<uint32_t> foot_ptr;       // per executed tile: footprint range into `foot`
  std::vector<uint32_t> foot;           // footprint vertices (ascending)
  std::vector<uint32_t> lc_ptr;         // per executed tile: num_local + 1 offsets into `order`
  uint32_t max_footprint = 0;
};
// `segments`: ascending first vertex of each independent mesh (instance); tiles never cross a
// segment and are numbered inside it exactly as for that mesh alone, so a batch of meshes gets
// the schedule every mesh would get on its own.  Empty = one segment.
// FEM fabric rest state from the initial world positions x (3 per vertex).
// ComputeStrainMeta (FEMHelper.cu:10-39) per face of `tri`: area and the inverse 2x2 material
// matrix in glm's column-major order (4 floats per face; identity for a degenerate face).
void fem_strain_rest(const std::vector<float>& x, const std::vector<uint32_t>& tri,
                     std::vector<float>& area, std::vector<float>& inv);
// ComputeHessianEnergy (FEMHelper.cu:209-233) per bend element (4 ids): the 4x4 Hessian
// 3 / (A0 + A1) K K^T with the cotangent weights K, row-major (16 floats per element).
void iso_bend_hessian(const std::vector<float>& x, const std::vector<uint32_t>& bends,
                      std::vector<float>& q);

TileSchedule build_tiles(const std::vector<uint32_t>& idx, int arity, uint32_t nv,
                         uint32_t tile_vertices, const std::vector<uint32_t>& segments = {});

}  // namespace setup
}  // namespace xrt
