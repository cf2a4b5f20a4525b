// oracle_lbvh.h — TEST INFRASTRUCTURE: CPU restatement of the reference LBVH, its stackless
// queries and the primitive tests used by the Swift contact kernels.  Only tests/, the smoke
// check and bench.py's CPU baseline may use it; the product path never does.
//
//   LBVH build ............ xrtailor/src/physics/broad_phase/lbvh/BVH.cu:22-329, 382-722
//   refit .................. BVH.cu:515-538 (AssignAABBCAS), 770-818 (RefitMidstep)
//   stackless queries ...... BVH.cu:957-1055, Bounds.cu:115-191
//   primitive tests ........ xrtailor/src/math/BasicPrimitiveTests.cu:6-361
#pragma once
#include <vector>
#include <cstdint>
#include <limits>
#include "oracle_math.h"

namespace orc {

static const uint32_t kNone = 0xFFFFFFFFu;
static const uint32_t kMaxBuffer = 256;  // LBVH_MAX_BUFFER_SIZE, core/Common.cuh:23

struct Prim {
  V3 v1, v2, v3, pred1, pred2, pred3;
  uint32_t idx1, idx2, idx3;
};

struct Box {
  V3 lo{std::numeric_limits<float>::infinity(), std::numeric_limits<float>::infinity(),
        std::numeric_limits<float>::infinity()};
  V3 hi{-std::numeric_limits<float>::infinity(), -std::numeric_limits<float>::infinity(),
        -std::numeric_limits<float>::infinity()};
};

struct BVNode {
  uint32_t parent = kNone, left = kNone, right = kNone, object = kNone;
};

// Bounds::Merge(const Bounds&) (Bounds.cu:193-202): per-axis ternary min / max.
static inline Box box_merge(const Box& a, const Box& b) {
  Box r;
  for (int i = 0; i < 3; ++i) {
    set(r.lo, i, mmin(get(a.lo, i), get(b.lo, i)));
    set(r.hi, i, mmax(get(a.hi, i), get(b.hi, i)));
  }
  return r;
}
// Bounds::Merge(const Vector3&) (Bounds.cu:204-213) and operator+=(Vector3) (Bounds.cu:80-83).
static inline Box box_merge_point(const Box& a, V3 p) {
  Box r;
  for (int i = 0; i < 3; ++i) {
    set(r.lo, i, mmin(get(a.lo, i), get(p, i)));
    set(r.hi, i, mmax(get(a.hi, i), get(p, i)));
  }
  return r;
}
// Merge() used by AssignAABBCAS (BVH.cu:503-513): fminf / fmaxf.
static inline Box box_merge_f(const Box& a, const Box& b) {
  Box r;
  r.hi = V3{std::fmax(a.hi.x, b.hi.x), std::fmax(a.hi.y, b.hi.y), std::fmax(a.hi.z, b.hi.z)};
  r.lo = V3{std::fmin(a.lo.x, b.lo.x), std::fmin(a.lo.y, b.lo.y), std::fmin(a.lo.z, b.lo.z)};
  return r;
}
static inline V3 box_center(const Box& b) { return 0.5f * (b.lo + b.hi); }  // Bounds::Center

// Bounds::Overlap(point), strict (Bounds.cu:130-136)
static inline bool box_overlap_point(const Box& b, V3 p) {
  return p.x > b.lo.x && p.x < b.hi.x && p.y > b.lo.y && p.y < b.hi.y && p.z > b.lo.z &&
         p.z < b.hi.z;
}
// Bounds::Overlap(box) (Bounds.cu:115-124)
static inline bool box_overlap_box(const Box& a, const Box& b) {
  for (int i = 0; i < 3; ++i) {
    if (get(a.lo, i) > get(b.hi, i)) return false;
    if (get(a.hi, i) < get(b.lo, i)) return false;
  }
  return true;
}
bool box_overlap_segment(const Box& b, V3 p1, V3 p2);  // Bounds.cu:138-191

// Morton code (BVH.cu:22-46) and its normalisation (ComputeMortons_Kernel, BVH.cu:465-479).
uint32_t expand_bits(uint32_t v);
uint32_t morton_code(V3 p);
uint32_t morton_of_box(const Box& leaf, const Box& whole);

struct Lbvh {
  std::vector<Prim> objects;          // original primitive order
  std::vector<Box> aabbs;             // 2N-1, leaves at N-1+i in sorted order
  std::vector<BVNode> nodes;          // 2N-1, root at 0
  std::vector<int32_t> iesc, eesc;    // escape index tables
  std::vector<uint32_t> sorted_morton, sorted_objects;
  bool morton_unique = true;
  bool active = false;
  uint32_t num_objects() const { return (uint32_t)objects.size(); }

  void construct(float scr);                              // BVH::Construct
  void refit_pred(const std::vector<V3>& pred3);          // leaves += pred, CAS-merge internals
  void merge_internal_cas();                              // AssignAABBCAS_Kernel semantics
  // QueryDeviceStackless; returns the number of candidates written (<= 256), in traversal order.
  uint32_t query_point(V3 p, uint32_t* out) const;
  uint32_t query_segment(V3 p0, V3 p1, uint32_t* out) const;
  uint32_t query_box(const Box& q, uint32_t* out) const;
};

// Bounds(const Primitive&, scr) / InitAABBs_Kernel (BVH.cu:423-462)
Box init_leaf_box(const Prim& f, float scr);

// BasicPrimitiveTests (src/math/BasicPrimitiveTests.cu)
float nearest_point(V3 p, V3 a, V3 b, V3 c, V3& qs, float& u, float& v, float& w);
float ray_intersect(V3 o, V3 d, float ray_length, V3 a, V3 b, V3 c);
float closest_pt_segment_segment(V3 p1, V3 q1, V3 p2, V3 q2, float& s, float& t, V3& c1, V3& c2);
// MathFunctions::SolveCubic (src/math/MathFunctions.cu:91-150)
int solve_cubic(float a, float b, float c, float d, float x[3]);

}  // namespace orc
