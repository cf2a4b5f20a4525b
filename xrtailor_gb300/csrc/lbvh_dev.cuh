// lbvh_dev.cuh — device-side LBVH box tests and the stackless traversal shared by the query,
// contact-generation and self-contact kernels.
//
// Box tests restate Bounds::Overlap (xrtailor/src/physics/broad_phase/Bounds.cu:115-191);
// the traversal restates QueryDeviceStackless (xrtailor/src/physics/broad_phase/lbvh/BVH.cu:957-1055):
// left-first, escape indices instead of a stack, at most LBVH_MAX_BUFFER_SIZE (256) hits.
// Candidates are handed to a visitor in traversal order instead of a 1 KB per-thread buffer, so
// the narrow phase runs inline with identical first-minimum semantics.
#pragma once
#include "common.cuh"
#include "context.h"

namespace xrt {

__device__ __forceinline__ bool overlap_point(float4 l, float4 h, f3 p) {
  return p.x > l.x && p.x < h.x && p.y > l.y && p.y < h.y && p.z > l.z && p.z < h.z;
}

__device__ __forceinline__ int seg_intersection(float d1, float d2, f3 p1, f3 p2, f3& hit) {
  if ((d1 * d2) >= 0.0f) return 0;
  if (d1 == d2) return 0;
  hit = p1 + (p2 - p1) * (-d1 / (d2 - d1));
  return 1;
}
__device__ __forceinline__ int seg_in_box(f3 q, float4 l, float4 h, int axis) {
  if (axis == 1 && q.z > l.z && q.z < h.z && q.y > l.y && q.y < h.y) return 1;
  if (axis == 2 && q.z > l.z && q.z < h.z && q.x > l.x && q.x < h.x) return 1;
  if (axis == 3 && q.x > l.x && q.x < h.x && q.y > l.y && q.y < h.y) return 1;
  return 0;
}

__device__ __forceinline__ bool overlap_segment(float4 l, float4 h, f3 p1, f3 p2) {
  if (p2.x < l.x && p1.x < l.x) return false;
  if (p2.x > h.x && p1.x > h.x) return false;
  if (p2.y < l.y && p1.y < l.y) return false;
  if (p2.y > h.y && p1.y > h.y) return false;
  if (p2.z < l.z && p1.z < l.z) return false;
  if (p2.z > h.z && p1.z > h.z) return false;
  if (p1.x > l.x && p1.x < h.x && p1.y > l.y && p1.y < h.y && p1.z > l.z && p1.z < h.z) return true;
  f3 hit = mk3(0, 0, 0);
  if ((seg_intersection(p1.x - l.x, p2.x - l.x, p1, p2, hit) && seg_in_box(hit, l, h, 1)) ||
      (seg_intersection(p1.y - l.y, p2.y - l.y, p1, p2, hit) && seg_in_box(hit, l, h, 2)) ||
      (seg_intersection(p1.z - l.z, p2.z - l.z, p1, p2, hit) && seg_in_box(hit, l, h, 3)) ||
      (seg_intersection(p1.x - h.x, p2.x - h.x, p1, p2, hit) && seg_in_box(hit, l, h, 1)) ||
      (seg_intersection(p1.y - h.y, p2.y - h.y, p1, p2, hit) && seg_in_box(hit, l, h, 2)) ||
      (seg_intersection(p1.z - h.z, p2.z - h.z, p1, p2, hit) && seg_in_box(hit, l, h, 3)))
    return true;
  return false;
}

__device__ __forceinline__ bool overlap_box(float4 l, float4 h, f3 qlo, f3 qhi) {
  return !(l.x > qhi.x || h.x < qlo.x || l.y > qhi.y || h.y < qlo.y || l.z > qhi.z || h.z < qlo.z);
}

// Bottom-up merge (AssignAABBCAS_Kernel, BVH.cu:515-538).  Each leaf walks towards the root; at
// every internal node the first arrival stops and the second merges both children.  The arrival
// counters are never reset: every walk adds exactly two arrivals per internal node, so the parity
// of the counter tells first from second.  Walks are bounded by the tree height (<= n).
__device__ __forceinline__ void lbvh_merge_upwards(uint32_t leaf_node, uint32_t n, float4* lo,
                                                   float4* hi, const int4* node, uint32_t* flags,
                                                   uint32_t* err) {
  int parent = node[leaf_node].x;
  uint32_t steps = 0;
  while (parent >= 0) {
    if (++steps > n) {
      raise_error(err, kErrTreeWalk);
      return;
    }
    // acq_rel: releases this thread's box stores with the arrival; the second arrival acquires
    // the first's (one ordered atomic instead of two device-wide fences around a relaxed one)
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;"
                 : "=r"(old)
                 : "l"(flags + parent)
                 : "memory");
    if ((old & 1u) == 0u) return;  // first arrival
    const int4 nd = node[parent];
    const float4 la = __ldcg(&lo[nd.y]), ha = __ldcg(&hi[nd.y]);
    const float4 lb = __ldcg(&lo[nd.z]), hb = __ldcg(&hi[nd.z]);
    const float4 ol = __ldcg(&lo[parent]), oh = __ldcg(&hi[parent]);
    __stcg(&lo[parent], make_float4(fminf(la.x, lb.x), fminf(la.y, lb.y), fminf(la.z, lb.z), ol.w));
    __stcg(&hi[parent], make_float4(fmaxf(ha.x, hb.x), fmaxf(ha.y, hb.y), fmaxf(ha.z, hb.z), oh.w));
    parent = nd.x;
  }
}

// ---- instances (InstView) ----------------------------------------------------------------------
__device__ __forceinline__ uint32_t inst_index(const InstView& I, uint32_t v) {
  return I.count == 1 ? 0u : __ldg(&I.of_vertex[v]);
}
__device__ __forceinline__ InstanceRec inst_rec(const InstView& I, uint32_t s) {
  return I.count == 1 ? I.one : I.rec[s];
}

// ---- forests (LbvhForest) ----------------------------------------------------------------------
__device__ __forceinline__ int4 forest_rec(const LbvhForest& F, uint32_t s) {
  return F.nseg == 1 ? F.one : F.seg[s];
}

// Segment owning element i of a forest-wide range: field 0 = primitive / sorted leaf position,
// 2 = node, 3 = internal node.  The last segment whose base is <= i: empty segments share their
// base with the next one, so the segment found always owns i.
__device__ __forceinline__ uint32_t forest_find(const LbvhForest& F, uint32_t i, int field) {
  if (F.nseg == 1) return 0;
  uint32_t lo = 0, hi = F.nseg;  // base(lo) <= i < base(hi)
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    const int4 r = F.seg[mid];
    const uint32_t b = (uint32_t)(field == 0 ? r.x : (field == 2 ? r.z : r.w));
    if (b <= i) lo = mid;
    else hi = mid;
  }
  return lo;
}

// The tree of segment s with local links; objects are local, global = rec.x + object.
__device__ __forceinline__ LbvhView forest_view(const LbvhForest& F, uint32_t s) {
  const int4 r = forest_rec(F, s);
  return LbvhView{(uint32_t)r.y, F.all.pred + 3 * (size_t)r.x, F.all.lo + r.z, F.all.hi + r.z};
}

// Stackless traversal state; one node visit per lbvh_step.
struct TraverseState {
  int node;        // next node, -1 = done
  uint32_t found;  // leaves visited (capped at kMaxCandidates)
  uint32_t guard;  // node visits (bounded by 2n + 2)
};

__device__ __forceinline__ TraverseState lbvh_begin(const LbvhView& b) {
  return TraverseState{b.n == 0 ? -1 : 0, 0u, 0u};
}

// One node visit; returns false once the traversal has ended (no visit made).
template <class Overlap, class Visit>
__device__ __forceinline__ bool lbvh_step(const LbvhView& b, TraverseState& st, Overlap ov,
                                          Visit visit, uint32_t* err) {
  if (st.node == -1 || st.found >= kMaxCandidates) return false;
  if (++st.guard > 2 * b.n + 2) {
    raise_error(err, kErrTraversal);
    st.node = -1;
    return false;
  }
  const float4 l = b.lo[st.node], h = b.hi[st.node];
  if (ov(l, h)) {
    if ((uint32_t)st.node >= b.n - 1) {
      visit((uint32_t)__float_as_int(l.w));
      ++st.found;
      st.node = __float_as_int(h.w);
    } else {
      st.node = __float_as_int(l.w);
    }
  } else {
    st.node = __float_as_int(h.w);
  }
  return true;
}

// Stackless traversal; `ov(lo, hi)` tests a node box, `visit(object)` receives each hit.
template <class Overlap, class Visit>
__device__ __forceinline__ uint32_t lbvh_traverse(const LbvhView& b, Overlap ov, Visit visit,
                                                  uint32_t* err) {
  TraverseState st = lbvh_begin(b);
  while (lbvh_step(b, st, ov, visit, err)) {
  }
  return st.found;
}

// Persistent query loop with dynamic work fetch: every lane works on one query at a time and
// takes a new one from `counter` when its query is done, so a warp's lanes stay busy while the
// traversal lengths of neighbouring queries differ by orders of magnitude.  Lanes refill together
// (one atomic per warp) once at least `kRefill` of them are idle.  A query is still processed by
// exactly one lane, in the same order, so its result is that of a plain per-thread traversal.
//   start(q)  -> bool:  set up query q, false = nothing to traverse (finish(q) still runs)
//   step()    -> bool:  one traversal step of the lane's query, false = done
//   finish(q):          write the result of query q
template <class Start, class Step, class Finish>
__device__ __forceinline__ void work_queue(uint32_t* counter, uint32_t nq, Start start, Step step,
                                           Finish finish) {
  constexpr unsigned kAll = 0xFFFFFFFFu;
  constexpr int kRefill = 8;
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t q = kNone;
  bool drained = false;  // the counter has passed nq
  for (;;) {
    const unsigned idle = __ballot_sync(kAll, q == kNone);
    if (!drained && (idle == kAll || __popc(idle) >= kRefill)) {
      const int leader = __ffs(idle) - 1;
      uint32_t base = 0;
      if ((int)lane == leader) base = atomicAdd(counter, (uint32_t)__popc(idle));
      base = __shfl_sync(kAll, base, leader);
      if (base + (uint32_t)__popc(idle) >= nq) drained = true;
      if (q == kNone) {
        const uint32_t cand = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
        if (cand < nq) {
          q = cand;
          if (!start(q)) {
            finish(q);
            q = kNone;
          }
        }
      }
    }
    if (__all_sync(kAll, q == kNone) && drained) break;
    if (q != kNone && !step()) {
      finish(q);
      q = kNone;
    }
  }
}

}  // namespace xrt
