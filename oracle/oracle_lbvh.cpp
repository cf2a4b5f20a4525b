// oracle_lbvh.cpp — TEST INFRASTRUCTURE: CPU restatement of the reference LBVH and primitive
// tests (see oracle_lbvh.h for the reference anchors of each function).
#include "oracle_lbvh.h"

#include <algorithm>
#include <numeric>

namespace orc {

// GetIntersection / InBox / Bounds::Overlap(p1, p2, hit) — Bounds.cu:138-191
static inline int get_intersection(float d1, float d2, V3 p1, V3 p2, V3& hit) {
  if ((d1 * d2) >= 0.0f) return 0;
  if (d1 == d2) return 0;
  hit = p1 + (p2 - p1) * (-d1 / (d2 - d1));
  return 1;
}
static inline int in_box(V3 hit, V3 lo, V3 hi, int axis) {
  if (axis == 1 && hit.z > lo.z && hit.z < hi.z && hit.y > lo.y && hit.y < hi.y) return 1;
  if (axis == 2 && hit.z > lo.z && hit.z < hi.z && hit.x > lo.x && hit.x < hi.x) return 1;
  if (axis == 3 && hit.x > lo.x && hit.x < hi.x && hit.y > lo.y && hit.y < hi.y) return 1;
  return 0;
}
bool box_overlap_segment(const Box& b, V3 p1, V3 p2) {
  const V3 lo = b.lo, hi = b.hi;
  if (p2.x < lo.x && p1.x < lo.x) return false;
  if (p2.x > hi.x && p1.x > hi.x) return false;
  if (p2.y < lo.y && p1.y < lo.y) return false;
  if (p2.y > hi.y && p1.y > hi.y) return false;
  if (p2.z < lo.z && p1.z < lo.z) return false;
  if (p2.z > hi.z && p1.z > hi.z) return false;
  if (p1.x > lo.x && p1.x < hi.x && p1.y > lo.y && p1.y < hi.y && p1.z > lo.z && p1.z < hi.z)
    return true;
  V3 hit{0, 0, 0};
  if ((get_intersection(p1.x - lo.x, p2.x - lo.x, p1, p2, hit) && in_box(hit, lo, hi, 1)) ||
      (get_intersection(p1.y - lo.y, p2.y - lo.y, p1, p2, hit) && in_box(hit, lo, hi, 2)) ||
      (get_intersection(p1.z - lo.z, p2.z - lo.z, p1, p2, hit) && in_box(hit, lo, hi, 3)) ||
      (get_intersection(p1.x - hi.x, p2.x - hi.x, p1, p2, hit) && in_box(hit, lo, hi, 1)) ||
      (get_intersection(p1.y - hi.y, p2.y - hi.y, p1, p2, hit) && in_box(hit, lo, hi, 2)) ||
      (get_intersection(p1.z - hi.z, p2.z - hi.z, p1, p2, hit) && in_box(hit, lo, hi, 3)))
    return true;
  return false;
}

// expand_bits / morton_code — BVH.cu:22-46
uint32_t expand_bits(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}
uint32_t morton_code(V3 p) {
  const float res = 1024.0f;
  float x = mmin(mmax(p.x * res, 0.0f), res - 1.0f);
  float y = mmin(mmax(p.y * res, 0.0f), res - 1.0f);
  float z = mmin(mmax(p.z * res, 0.0f), res - 1.0f);
  const uint32_t xx = expand_bits((uint32_t)x);
  const uint32_t yy = expand_bits((uint32_t)y);
  const uint32_t zz = expand_bits((uint32_t)z);
  return xx * 4 + yy * 2 + zz;
}
uint32_t morton_of_box(const Box& leaf, const Box& whole) {
  V3 p = box_center(leaf);
  p.x -= whole.lo.x;
  p.y -= whole.lo.y;
  p.z -= whole.lo.z;
  p.x /= (whole.hi.x - whole.lo.x);
  p.y /= (whole.hi.y - whole.lo.y);
  p.z /= (whole.hi.z - whole.lo.z);
  return morton_code(p);
}

Box init_leaf_box(const Prim& f, float scr) {
  Box b;
  b.lo = V3{mmin(mmin3(f.v1.x, f.v2.x, f.v3.x), mmin3(f.pred1.x, f.pred2.x, f.pred3.x)),
            mmin(mmin3(f.v1.y, f.v2.y, f.v3.y), mmin3(f.pred1.y, f.pred2.y, f.pred3.y)),
            mmin(mmin3(f.v1.z, f.v2.z, f.v3.z), mmin3(f.pred1.z, f.pred2.z, f.pred3.z))};
  b.hi = V3{mmax(mmax3(f.v1.x, f.v2.x, f.v3.x), mmax3(f.pred1.x, f.pred2.x, f.pred3.x)),
            mmax(mmax3(f.v1.y, f.v2.y, f.v3.y), mmax3(f.pred1.y, f.pred2.y, f.pred3.y)),
            mmax(mmax3(f.v1.z, f.v2.z, f.v3.z), mmax3(f.pred1.z, f.pred2.z, f.pred3.z))};
  V3 center = (b.lo + b.hi) * 0.5f;
  V3 n1 = normalize(b.lo - center);
  V3 n2 = normalize(b.hi - center);
  b.lo += scr * n1;
  b.hi += scr * n2;
  return b;
}

static inline int clz32(uint32_t x) { return x == 0 ? 32 : __builtin_clz(x); }
static inline int clz64(uint64_t x) { return x == 0 ? 64 : __builtin_clzll(x); }
static inline int common_upper_bits(uint32_t a, uint32_t b) { return clz32(a ^ b); }
static inline int common_upper_bits(uint64_t a, uint64_t b) { return clz64(a ^ b); }

// determine_range — BVH.cu:57-102 (32-bit) / 104-148 (64-bit)
template <typename K>
static void determine_range(const K* code, uint32_t num_leaves, uint32_t idx, uint32_t& first,
                            uint32_t& last) {
  if (idx == 0) {
    first = 0;
    last = num_leaves - 1;
    return;
  }
  const K self = code[idx];
  const int L_delta = common_upper_bits(self, code[idx - 1]);
  const int R_delta = common_upper_bits(self, code[idx + 1]);
  const int d = (R_delta > L_delta) ? 1 : -1;
  const int delta_min = std::min(L_delta, R_delta);
  int l_max = 2;
  int delta = -1;
  int i_tmp = (int)idx + d * l_max;
  if (0 <= i_tmp && i_tmp < (int)num_leaves) delta = common_upper_bits(self, code[i_tmp]);
  while (delta > delta_min) {
    l_max <<= 1;
    i_tmp = (int)idx + d * l_max;
    delta = -1;
    if (0 <= i_tmp && i_tmp < (int)num_leaves) delta = common_upper_bits(self, code[i_tmp]);
  }
  int l = 0;
  int t = l_max >> 1;
  while (t > 0) {
    i_tmp = (int)idx + (l + t) * d;
    delta = -1;
    if (0 <= i_tmp && i_tmp < (int)num_leaves) delta = common_upper_bits(self, code[i_tmp]);
    if (delta > delta_min) l += t;
    t >>= 1;
  }
  uint32_t jdx = (uint32_t)((int)idx + l * d);
  if (d < 0) std::swap(idx, jdx);
  first = idx;
  last = jdx;
}

// find_split — BVH.cu:150-210
template <typename K>
static uint32_t find_split(const K* code, uint32_t first, uint32_t last) {
  const K first_code = code[first];
  const K last_code = code[last];
  if (first_code == last_code) return (first + last) >> 1;
  const int delta_node = common_upper_bits(first_code, last_code);
  int split = (int)first;
  int stride = (int)(last - first);
  do {
    stride = (stride + 1) >> 1;
    const int middle = split + stride;
    if (middle < (int)last) {
      const int delta = common_upper_bits(first_code, code[middle]);
      if (delta > delta_node) split = middle;
    }
  } while (stride > 1);
  return (uint32_t)split;
}

// ConstructInternalNodes{32,64}Bits_Kernel — BVH.cu:275-329
template <typename K>
static void construct_internal(std::vector<BVNode>& nodes, const K* code, uint32_t n) {
  for (uint32_t idx = 0; idx + 1 < n; ++idx) {
    nodes[idx].object = kNone;
    uint32_t a, b;
    determine_range(code, n, idx, a, b);
    const uint32_t gamma = find_split(code, a, b);
    nodes[idx].left = gamma;
    nodes[idx].right = gamma + 1;
    if (std::min(a, b) == gamma) nodes[idx].left += n - 1;
    if (std::max(a, b) == gamma + 1) nodes[idx].right += n - 1;
    nodes[nodes[idx].left].parent = idx;
    nodes[nodes[idx].right].parent = idx;
  }
}

void Lbvh::construct(float scr) {
  const uint32_t n = num_objects();
  active = false;
  aabbs.clear();
  nodes.clear();
  iesc.clear();
  eesc.clear();
  sorted_morton.clear();
  sorted_objects.clear();
  if (n == 0) return;
  const uint32_t ni = n - 1, nn = 2 * n - 1;
  aabbs.assign(nn, Box());
  for (uint32_t i = 0; i < n; ++i) aabbs[ni + i] = init_leaf_box(objects[i], scr);
  Box whole;
  for (uint32_t i = 0; i < n; ++i) whole = box_merge(whole, aabbs[ni + i]);
  std::vector<uint32_t> morton(n), idx(n);
  for (uint32_t i = 0; i < n; ++i) morton[i] = morton_of_box(aabbs[ni + i], whole);
  std::iota(idx.begin(), idx.end(), 0u);
  // thrust::stable_sort_by_key(morton, zip(leaf aabbs, indices)) — BVH.cu:666-668
  std::stable_sort(idx.begin(), idx.end(),
                   [&](uint32_t a, uint32_t b) { return morton[a] < morton[b]; });
  std::vector<Box> leaves(n);
  sorted_morton.resize(n);
  for (uint32_t i = 0; i < n; ++i) {
    leaves[i] = aabbs[ni + idx[i]];
    sorted_morton[i] = morton[idx[i]];
  }
  for (uint32_t i = 0; i < n; ++i) aabbs[ni + i] = leaves[i];
  sorted_objects = idx;
  morton_unique = true;
  for (uint32_t i = 1; i < n; ++i)
    if (sorted_morton[i] == sorted_morton[i - 1]) morton_unique = false;

  nodes.assign(nn, BVNode());
  for (uint32_t i = 0; i < n; ++i) nodes[ni + i].object = idx[i];
  if (morton_unique) {
    construct_internal(nodes, sorted_morton.data(), n);
  } else {
    std::vector<uint64_t> m64(n);
    for (uint32_t i = 0; i < n; ++i) m64[i] = ((uint64_t)sorted_morton[i] << 32) | idx[i];
    construct_internal(nodes, m64.data(), n);
  }
  // AssignAABBAtomic_Kernel (BVH.cu:540-557): every internal box becomes the union of its leaves.
  // Internal nodes are numbered so that a parent precedes neither child in any fixed order, so
  // the union is taken by an explicit post-order walk.
  if (n > 1) {
    std::vector<uint32_t> order;
    order.reserve(nn);
    std::vector<uint32_t> stack{0u};
    while (!stack.empty()) {
      uint32_t k = stack.back();
      stack.pop_back();
      order.push_back(k);
      if (nodes[k].object == kNone) {
        stack.push_back(nodes[k].left);
        stack.push_back(nodes[k].right);
      }
    }
    for (auto it = order.rbegin(); it != order.rend(); ++it) {
      uint32_t k = *it;
      if (nodes[k].object == kNone)
        aabbs[k] = box_merge(aabbs[nodes[k].left], aabbs[nodes[k].right]);
    }
  }
  // BuildInternal/ExternalEscapeIndexTable_Kernel — BVH.cu:212-273
  iesc.assign(n, -1);
  eesc.assign(n, -1);
  for (uint32_t k = 0; k < ni; ++k) {
    uint32_t parent = nodes[k].parent;
    if (parent == kNone) {
      iesc[k] = -1;
      continue;
    }
    if (k == nodes[parent].left) {
      iesc[k] = (int32_t)nodes[parent].right;
    } else {
      uint32_t cur = parent;
      while (cur != kNone) {
        const BVNode& cn = nodes[cur];
        if (cn.parent == kNone) {
          iesc[k] = -1;
          break;
        }
        if (cur == nodes[cn.parent].right) {
          cur = cn.parent;
        } else {
          iesc[k] = (int32_t)nodes[cn.parent].right;
          break;
        }
      }
    }
  }
  for (uint32_t i = 0; i < n; ++i) {
    uint32_t k = ni + i;
    uint32_t parent = nodes[k].parent;
    if (parent == kNone) {  // single-object tree: the reference reads nodes[0xFFFFFFFF] here
      eesc[i] = -1;
      continue;
    }
    if (k == nodes[parent].left)
      eesc[i] = (int32_t)nodes[parent].right;
    else
      eesc[i] = iesc[parent];
  }
  active = true;
}

void Lbvh::merge_internal_cas() {
  // AssignAABBCAS_Kernel (BVH.cu:515-538): the second child to arrive merges both children;
  // every internal node is recomputed from its children, bottom-up.
  const uint32_t n = num_objects();
  if (n <= 1) return;
  std::vector<uint32_t> order;
  std::vector<uint32_t> stack{0u};
  while (!stack.empty()) {
    uint32_t k = stack.back();
    stack.pop_back();
    order.push_back(k);
    if (nodes[k].object == kNone) {
      stack.push_back(nodes[k].left);
      stack.push_back(nodes[k].right);
    }
  }
  for (auto it = order.rbegin(); it != order.rend(); ++it) {
    uint32_t k = *it;
    if (nodes[k].object == kNone)
      aabbs[k] = box_merge_f(aabbs[nodes[k].left], aabbs[nodes[k].right]);
  }
}

void Lbvh::refit_pred(const std::vector<V3>& pred3) {
  // RefitExternalNode_Kernel(self, predicted, ...) (BVH.cu:854-877) with per-primitive pred
  // triples, then AssignAABBCAS.
  const uint32_t n = num_objects();
  const uint32_t ni = n - 1;
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t k = ni + i;
    const uint32_t obj = nodes[k].object;
    Prim& p = objects[obj];
    p.pred1 = pred3[obj * 3 + 0];
    p.pred2 = pred3[obj * 3 + 1];
    p.pred3 = pred3[obj * 3 + 2];
    Box b = aabbs[k];
    b = box_merge_point(b, p.pred1);
    b = box_merge_point(b, p.pred2);
    b = box_merge_point(b, p.pred3);
    aabbs[k] = b;
  }
  merge_internal_cas();
}

uint32_t Lbvh::query_point(V3 p, uint32_t* out) const {
  int node = 0;
  uint32_t found = 0;
  const uint32_t ni = num_objects() - 1;
  while (node != -1) {
    if (found >= kMaxBuffer) break;
    const BVNode& nd = nodes[node];
    if (box_overlap_point(aabbs[node], p)) {
      if (nd.object != kNone) {
        out[found++] = nd.object;
        node = eesc[node - ni];
      } else {
        node = (int)nd.left;
      }
    } else {
      node = (nd.object != kNone) ? eesc[node - ni] : iesc[node];
    }
  }
  return found;
}

uint32_t Lbvh::query_segment(V3 p0, V3 p1, uint32_t* out) const {
  int node = 0;
  uint32_t found = 0;
  const uint32_t ni = num_objects() - 1;
  while (node != -1) {
    if (found >= kMaxBuffer) break;
    const BVNode& nd = nodes[node];
    if (box_overlap_segment(aabbs[node], p0, p1)) {
      if (nd.object != kNone) {
        out[found++] = nd.object;
        node = eesc[node - ni];
      } else {
        node = (int)nd.left;
      }
    } else {
      node = (nd.object != kNone) ? eesc[node - ni] : iesc[node];
    }
  }
  return found;
}

uint32_t Lbvh::query_box(const Box& q, uint32_t* out) const {
  int node = 0;
  uint32_t found = 0;
  const uint32_t ni = num_objects() - 1;
  while (node != -1) {
    if (found >= kMaxBuffer) break;
    const BVNode& nd = nodes[node];
    if (box_overlap_box(aabbs[node], q)) {
      if (nd.object != kNone) {
        out[found++] = nd.object;
        node = eesc[node - ni];
      } else {
        node = (int)nd.left;
      }
    } else {
      node = (nd.object != kNone) ? eesc[node - ni] : iesc[node];
    }
  }
  return found;
}

// NearestPoint — BasicPrimitiveTests.cu:6-100
float nearest_point(V3 p, V3 a, V3 b, V3 c, V3& qs, float& _u, float& _v, float& _w) {
  V3 e1 = b - a;
  V3 e2 = c - a;
  V3 e3 = c - b;
  V3 v1 = p - a;
  float d1 = dot(e1, v1), d2 = dot(e2, v1);
  if (d1 <= 0 && d2 <= 0) {
    qs = a;
    _u = 1; _v = 0; _w = 0;
    return length(p - qs);
  }
  V3 v2 = p - b;
  float d3 = dot(e1, v2), d4 = dot(e2, v2);
  if (d3 >= 0 && d4 <= d3) {
    qs = b;
    _u = 0; _v = 1; _w = 0;
    return length(p - qs);
  }
  float vc = d1 * d4 - d3 * d2;
  if (vc <= 0 && d1 >= 0 && d3 <= 0) {
    float v = d1 / (d1 - d3);
    qs = a + v * e1;
    _u = 1 - v; _v = v; _w = 0;
    return length(p - qs);
  }
  V3 v3 = p - c;
  float d5 = dot(e1, v3), d6 = dot(e2, v3);
  if (d6 >= 0 && d5 <= d6) {
    qs = c;
    _u = 0; _v = 0; _w = 1;
    return length(p - qs);
  }
  float vb = d5 * d2 - d1 * d6;
  if (vb <= 0 && d2 >= 0 && d6 <= 0) {
    float w = d2 / (d2 - d6);
    qs = a + w * e2;
    _u = 1 - w; _v = 0; _w = w;
    return length(p - qs);
  }
  float va = d3 * d6 - d5 * d4;
  if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
    float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    qs = b + w * e3;
    _u = 0; _v = 1 - w; _w = w;
    return length(p - qs);
  }
  float d = 1 / (va + vb + vc);
  float v = vb * d;
  float w = vc * d;
  qs = a + e1 * v + e2 * w;
  _u = 1 - v - w; _v = v; _w = w;
  return length(p - qs);
}

// RayIntersect(o, d, ray_length, Primitive) — BasicPrimitiveTests.cu:242-284
float ray_intersect(V3 o, V3 d, float ray_length, V3 a, V3 b, V3 c) {
  V3 e1 = b - a;
  V3 e2 = c - a;
  V3 n = cross(d, e2);
  float det = dot(e1, n);
  if (mabs(det) < kEps) return kScalarMax;
  float inv_det = 1 / det;
  V3 t = o - a;
  float u = dot(t, n) * inv_det;
  if (u < 0 || u > 1) return kScalarMax;
  V3 q = cross(t, e1);
  float v = dot(d, q) * inv_det;
  if (v < 0 || v + u > 1) return kScalarMax;
  float s = dot(e2, q) * inv_det;
  if (s > 0 && s < ray_length) return s;
  return std::numeric_limits<float>::infinity();
}

// ClosestPtSegmentSegment — BasicPrimitiveTests.cu:303-361
float closest_pt_segment_segment(V3 p1, V3 q1, V3 p2, V3 q2, float& s, float& t, V3& c1, V3& c2) {
  V3 d1 = q1 - p1;
  V3 d2 = q2 - p2;
  V3 r = p1 - p2;
  float a = dot(d1, d1);
  float e = dot(d2, d2);
  float f = dot(d2, r);
  if (a <= kEps && e <= kEps) {
    s = t = 0;
    c1 = p1;
    c2 = p2;
    return length(c1 - c2);
  }
  if (a <= kEps) {
    s = 0;
    t = f / e;
    t = clampf(t, 0.0f, 1.0f);
  } else {
    float c = dot(d1, r);
    if (e <= kEps) {
      t = 0;
      s = clampf(-c / a, 0.0f, 1.0f);
    } else {
      float b = dot(d1, d2);
      float denom = a * e - b * b;
      if (denom > kEps)
        s = clampf((b * f - c * e) / denom, 0.0f, 1.0f);
      else
        s = 0;
      t = (b * s + f) / e;
      if (t < kEps) {
        t = 0;
        s = clampf(-c / a, 0.0f, 1.0f);
      } else if (t > 1) {
        t = 1;
        s = clampf((b - c) / a, 0.0f, 1.0f);
      }
    }
  }
  c1 = p1 + d1 * s;
  c2 = p2 + d2 * t;
  return length(c1 - c2);
}

// NewtonsMethod / SolveQuadratic / SolveCubic — MathFunctions.cu:91-150
static float newtons_method(float a, float b, float c, float d, float x0, int dir) {
  if (dir != 0) {
    float y0 = d + x0 * (c + x0 * (b + x0 * a));
    float ddy0 = 2.0f * b + x0 * (6.0f * a);
    x0 += dir * std::sqrt(mabs(2.0f * y0 / ddy0));
  }
  for (int iter = 0; iter < 100; iter++) {
    float y = d + x0 * (c + x0 * (b + x0 * a));
    float dy = c + x0 * (2.0f * b + 3.0f * x0 * a);
    if (dy == 0) return x0;
    float x1 = x0 - y / dy;
    if (mabs(x0 - x1) < 1e-6f) return x0;
    x0 = x1;
  }
  return x0;
}
static int solve_quadratic(float a, float b, float c, float x[2]) {
  float d = b * b - 4.0f * a * c;
  if (d < 0) {
    x[0] = -b / (2.0f * a);
    return 0;
  }
  float q = -(b + (b < 0.0f ? -1 : 1) * std::sqrt(d)) * 0.5f;
  int i = 0;
  if (mabs(a) > 1e-12f * mabs(q)) x[i++] = q / a;
  if (mabs(q) > 1e-12f * mabs(c)) x[i++] = c / q;
  if (i == 2 && x[0] > x[1]) std::swap(x[0], x[1]);
  return i;
}
// xc[0] starts at 0: the reference leaves it uninitialized when SolveQuadratic accepts no root
// with a non-negative discriminant (a = b = 0), and starts Newton's method from it.
int solve_cubic(float a, float b, float c, float d, float x[3]) {
  float xc[2] = {0.0f, 0.0f};
  int n = solve_quadratic(3.0f * a, 2.0f * b, c, xc);
  if (n == 0) {
    x[0] = newtons_method(a, b, c, d, xc[0], 0);
    return 1;
  } else if (n == 1) {
    return solve_quadratic(b, c, d, x);
  } else {
    float yc[2] = {d + xc[0] * (c + xc[0] * (b + xc[0] * a)),
                   d + xc[1] * (c + xc[1] * (b + xc[1] * a))};
    int i = 0;
    if (yc[0] * a >= 0) x[i++] = newtons_method(a, b, c, d, xc[0], -1);
    if (yc[0] * yc[1] <= 0) {
      int closer = mabs(yc[0]) < mabs(yc[1]) ? 0 : 1;
      x[i++] = newtons_method(a, b, c, d, xc[closer], closer == 0 ? 1 : -1);
    }
    if (yc[1] * a <= 0) x[i++] = newtons_method(a, b, c, d, xc[1], 1);
    return i;
  }
}

}  // namespace orc
