// contact.cu — obstacle motion within a frame and Swift obstacle-contact generation.
//
//   Interpolate_Kernel .............. xrtailor/src/physics/PhysicsMesh.cu:610-620
//   UpdateNodeMidstepNormals ........ xrtailor/src/physics/PhysicsMeshHelper.cu:212-225, 297-310
//   GenerateVF_DCD_Kernel ........... xrtailor/src/physics/pbd_collision/PBDCollision.cu:17-46
//   GenerateVFCCD_Kernel ............ PBDCollision.cu:236-267
//   GenerateEE_DCD_Kernel ........... PBDCollision.cu:100-151 (R-triangle edge filter RTriangle.cu:12-17)
//   PredictedToPositions/UpdateNormals PhysicsMesh.cu:604-608, PhysicsMeshHelper.cu:196-210
//
// Vertex normals are gathered per vertex over its faces in ascending face order (the reference
// scatters them with float atomics); the interpolated midstep position x1 of a neighbor is
// recomputed from x0 and x inside the gather, so interpolation and normals are one kernel.
#include <algorithm>

#include "common.cuh"
#include "context.h"
#include "lbvh_dev.cuh"
#include "prim_tests.cuh"

namespace xrt {
namespace {

__device__ __forceinline__ f3 lerp_pos(const float4* __restrict__ x0, const float4* __restrict__ x,
                                       int i, float alpha) {
  return (1.0f - alpha) * mk3(x0[i]) + alpha * mk3(x[i]);
}

__global__ void k_obstacle_pass(const float4* __restrict__ x0, const float4* __restrict__ x,
                                float4* __restrict__ x1, float4* __restrict__ n1,
                                const int4* __restrict__ tri, const uint32_t* __restrict__ ptr,
                                const uint32_t* __restrict__ list, uint32_t nv, float alpha) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const f3 xi = lerp_pos(x0, x, i, alpha);
  f3 acc = mk3(0, 0, 0);
  for (uint32_t k = ptr[i]; k < ptr[i + 1]; ++k) {
    const uint32_t fc = list[k];
    const int4 t = tri[fc >> 2];
    const int id[3] = {t.x, t.y, t.z};
    const int j = (int)(fc & 3u);
    const f3 e0 = lerp_pos(x0, x, id[(j + 1) % 3], alpha) - xi;
    const f3 e1 = lerp_pos(x0, x, id[(j + 2) % 3], alpha) - xi;
    acc = acc + cross(e0, e1) / (dot(e0, e0) * dot(e1, e1));
  }
  x1[i] = mk4(xi, 0.0f);
  n1[i] = mk4(normalize(acc), 0.0f);
}

__global__ void k_vertex_normals(const float4* __restrict__ x, const int4* __restrict__ tri,
                                 const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ list,
                                 float4* __restrict__ out, uint32_t nv) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const f3 xi = mk3(x[i]);
  f3 acc = mk3(0, 0, 0);
  for (uint32_t k = ptr[i]; k < ptr[i + 1]; ++k) {
    const uint32_t fc = list[k];
    const int4 t = tri[fc >> 2];
    const int id[3] = {t.x, t.y, t.z};
    const int j = (int)(fc & 3u);
    const f3 e0 = mk3(x[id[(j + 1) % 3]]) - xi;
    const f3 e1 = mk3(x[id[(j + 2) % 3]]) - xi;
    acc = acc + cross(e0, e1) / (dot(e0, e0) * dot(e1, e1));
  }
  out[i] = mk4(normalize(acc), 0.0f);
}

// Frame end: x0 = x, then normals of the new x0 (computed from x, which is the same data).
__global__ void k_obstacle_commit(const float4* __restrict__ x, float4* __restrict__ x0,
                                  float4* __restrict__ nrm, const int4* __restrict__ tri,
                                  const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ list,
                                  uint32_t nv) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const f3 xi = mk3(x[i]);
  f3 acc = mk3(0, 0, 0);
  for (uint32_t k = ptr[i]; k < ptr[i + 1]; ++k) {
    const uint32_t fc = list[k];
    const int4 t = tri[fc >> 2];
    const int id[3] = {t.x, t.y, t.z};
    const int j = (int)(fc & 3u);
    const f3 e0 = mk3(x[id[(j + 1) % 3]]) - xi;
    const f3 e1 = mk3(x[id[(j + 2) % 3]]) - xi;
    acc = acc + cross(e0, e1) / (dot(e0, e0) * dot(e1, e1));
  }
  x0[i] = mk4(xi, 0.0f);
  nrm[i] = mk4(normalize(acc), 0.0f);
}

// The generation kernels run at four blocks per SM (at most 64 registers): more queries in flight
// for the latency-bound traversals (the 512-garment batch: 83 ms of generation per frame, against
// 114 ms with the edge queries at 94 registers and 88 ms with every kernel at 40 registers).
// Contact generation, one query per cloth vertex (VF) or edge (EE) against the tree of its
// instance, run as persistent work queues (work_queue, lbvh_dev.cuh): traversal lengths differ by
// orders of magnitude between cloth near the obstacle and cloth away from it, and a plain
// one-thread-per-query launch left ~2 of 32 lanes of a warp busy.  Contacts record global
// triangle ids.

// VF-DCD (nearest obstacle point of the predicted vertex) and VF-CCD (first obstacle hit of the
// segment x0 -> x) of one vertex, in one walk of its instance's tree.  Each query keeps the state
// of its own stackless traversal: where its box test fails at an internal node that the other
// query enters, it stays off until the walk reaches that node's escape index (the first node
// after the subtree), and it stops after its own 256th leaf.  So each query tests the same nodes
// in the same order as alone, visits the same leaves in the same order and ends at the same cap:
// both results are those of the two separate traversals (GenerateVF_DCD_Kernel,
// GenerateVFCCD_Kernel), with the nodes they share fetched once.
__global__ void __launch_bounds__(kBlock, 4) k_generate_vf(LbvhForest F, InstView I,
                                                        const float4* __restrict__ x,
                                                        const float4* __restrict__ x0,
                                                        uint32_t nv, int* __restrict__ vf_idx,
                                                        float4* __restrict__ vf_qs,
                                                        int* __restrict__ rt_idx,
                                                        float4* __restrict__ rt_qc, uint32_t* err,
                                                        uint32_t* counter) {
  constexpr int kOn = -1, kDone = -2;  // a query's state; >= 0: off until the walk reaches it
  LbvhView b{};
  int node = -1, base = 0;
  uint32_t guard = 0;
  // DCD
  f3 pred{}, dqs{};
  float dhit = kScalarMax;
  int didx = -1, dstate = kDone;
  uint32_t dfound = 0;
  // CCD
  f3 p1{}, dir{}, cqc{};
  float len = 0, chit = kScalarMax;
  int cidx = -1, cstate = kDone;
  uint32_t cfound = 0;
  auto visit_dcd = [&](uint32_t f) {
    f3 qs;
    const float dist = nearest_point(pred, mk3(b.pred[3 * f]), mk3(b.pred[3 * f + 1]),
                                     mk3(b.pred[3 * f + 2]), qs);
    if (dist < dhit) {
      dhit = dist;
      dqs = qs;
      didx = base + (int)f;
    }
  };
  auto visit_ccd = [&](uint32_t f) {
    const float dist = ray_intersect(p1, dir, len, mk3(b.pred[3 * f]), mk3(b.pred[3 * f + 1]),
                                     mk3(b.pred[3 * f + 2]));
    if (dist < chit) {
      cqc = p1 + dist * dir;
      chit = dist;
      cidx = base + (int)f;
    }
  };
  work_queue(
      counter, nv,
      [&](uint32_t i) {
        const uint32_t sg = inst_index(I, i);
        b = forest_view(F, sg);
        base = forest_rec(F, sg).x;
        pred = mk3(x[i]);
        dhit = kScalarMax;
        didx = -1;
        dqs = mk3(0, 0, 0);
        dfound = 0;
        p1 = mk3(x0[i]);
        dir = pred - p1;
        len = length(dir);
        chit = kScalarMax;
        cidx = -1;
        cqc = mk3(0, 0, 0);
        cfound = 0;
        node = lbvh_begin(b).node;
        guard = 0;
        dstate = node != -1 ? kOn : kDone;
        cstate = node != -1 && !(len < kEps) ? kOn : kDone;  // a still vertex casts no ray
        if (cstate == kOn) dir = dir / len;
        return node != -1;
      },
      [&]() {
        if (node == -1) return false;
        if (dstate == node) dstate = kOn;  // the walk left the subtree the query skipped
        if (cstate == node) cstate = kOn;
        if (++guard > 2 * b.n + 2) {
          raise_error(err, kErrTraversal);
          node = -1;
          return false;
        }
        const bool don = dstate == kOn, con = cstate == kOn;
        const float4 l = b.lo[node], h = b.hi[node];
        const bool od = don && overlap_point(l, h, pred);
        const bool oc = con && overlap_segment(l, h, p1, pred);
        const int esc = __float_as_int(h.w);
        if ((uint32_t)node >= b.n - 1) {
          const uint32_t f = (uint32_t)__float_as_int(l.w);
          if (od) {
            visit_dcd(f);
            if (++dfound >= kMaxCandidates) dstate = kDone;
          }
          if (oc) {
            visit_ccd(f);
            if (++cfound >= kMaxCandidates) cstate = kDone;
          }
          node = esc;
        } else if (od || oc) {
          // off for the subtree (an escape of -1: for the rest of the walk)
          if (don && !od) dstate = esc >= 0 ? esc : kDone;
          if (con && !oc) cstate = esc >= 0 ? esc : kDone;
          node = __float_as_int(l.w);
        } else {
          node = esc;
        }
        if (dstate == kDone && cstate == kDone) node = -1;
        return node != -1;
      },
      [&](uint32_t i) {
        vf_idx[i] = didx;
        vf_qs[i] = mk4(dqs, 0.0f);
        rt_idx[i] = cidx;
        rt_qc[i] = mk4(cqc, 0.0f);
      });
}

// EE-DCD: closest R-triangle-owned obstacle edge to each cloth edge.
__global__ void __launch_bounds__(kBlock, 4) k_generate_ee(LbvhForest F, InstView I,
                                                        const float4* __restrict__ x,
                                                        const uint2* __restrict__ edge, uint32_t ne,
                                                        const int4* __restrict__ otri_all,
                                                        float4* __restrict__ ee_a,
                                                        float4* __restrict__ ee_b,
                                                        float4* __restrict__ ee_c,
                                                        uint8_t* __restrict__ vflag, uint32_t* err,
                                                        uint32_t* counter) {
  LbvhView b{};
  TraverseState st{};
  const int4* otri = nullptr;
  f3 pc{}, qc{}, p2{}, q2{}, fn{};
  float s = 0, t = 0, min_dist = kScalarMax;
  auto overlap = [&](float4 l, float4 h) { return overlap_segment(l, h, pc, qc); };
  auto visit = [&](uint32_t f) {
    const uint32_t info = (uint32_t)otri[f].w;
    const f3 ov[3] = {mk3(b.pred[3 * f]), mk3(b.pred[3 * f + 1]), mk3(b.pred[3 * f + 2])};
#pragma unroll
    for (uint32_t a = 0; a < 3; ++a) {
      if ((info >> (a + 3u)) & 1u) {
        float _s, _t;
        f3 c1, c2;
        const uint32_t bb = (a + 1u) % 3u;
        if (closest_seg_seg(pc, qc, ov[a], ov[bb], _s, _t, c1, c2) != 0.0f) {
          const float dist = length(c1 - c2);
          if (dist < min_dist) {
            min_dist = dist;
            p2 = ov[a];
            q2 = ov[bb];
            s = _s;
            t = _t;
            fn = face_normal(ov[0], ov[1], ov[2]);
          }
        }
      }
    }
  };
  work_queue(
      counter, ne,
      [&](uint32_t e) {
        const uint2 ed = edge[e];
        const uint32_t sg = inst_index(I, ed.x);
        b = forest_view(F, sg);
        otri = otri_all + forest_rec(F, sg).x;
        pc = mk3(x[ed.x]);
        qc = mk3(x[ed.y]);
        s = 0;
        t = 0;
        p2 = mk3(0, 0, 0);
        q2 = mk3(0, 0, 0);
        fn = mk3(0, 0, 0);
        min_dist = kScalarMax;
        st = lbvh_begin(b);
        return st.node != -1;
      },
      [&]() { return lbvh_step(b, st, overlap, visit, err); },
      [&](uint32_t e) {
        ee_a[e] = make_float4(min_dist, p2.x, p2.y, p2.z);
        ee_b[e] = make_float4(q2.x, q2.y, q2.z, s);
        ee_c[e] = make_float4(fn.x, fn.y, fn.z, t);
        if (min_dist <= 1e6f) {  // a contact (the EE solve's test): flag both endpoints
          const uint2 ed = edge[e];
          vflag[ed.x] = 1;
          vflag[ed.y] = 1;
        }
      });
}

}  // namespace

void launch_obstacle_pass(Context& c, int step, int num_steps) {
  if (c.onv == 0) return;
  const float alpha = ((float)step + 1.0f) / (float)num_steps;
  k_obstacle_pass<<<grid_for(c.onv), kBlock, 0, c.stream>>>(c.ox0.p, c.ox.p, c.ox1.p, c.on1.p,
                                                            c.otri.p, c.ovf_ptr.p, c.ovf_list.p,
                                                            c.onv, alpha);
  launch_refit_midstep(c.bvh, c.ox1.p, c.on1.p, c.otri.p, c.params.bvh_tolerance, c.stream, c.err.p);
}

void launch_generate_contacts(Context& c) {
  if (!c.bvh.active) return;
  const LbvhForest F = c.bvh.forest();
  const InstView I = c.inst_view();
  // persistent work queues: a few resident waves of blocks fetch queries until the counters
  // pass the end
  const unsigned cap = (unsigned)c.num_sms * 8u;
  cudaMemsetAsync(c.gen_counter.p, 0, sizeof(uint32_t) * 3, c.stream);
  cudaMemsetAsync(c.ee_vflag.p, 0, c.nv, c.stream);  // this pass's contacts set it
  k_generate_vf<<<std::min(grid_for(c.nv), cap), kBlock, 0, c.stream>>>(
      F, I, c.x.p, c.x0.p, c.nv, c.vf_idx.p, c.vf_qs.p, c.rt_idx.p, c.rt_qc.p, c.err.p,
      c.gen_counter.p);
  k_generate_ee<<<std::min(grid_for(c.ne), cap), kBlock, 0, c.stream>>>(
      F, I, c.x.p, c.edge.p, c.ne, c.otri.p, c.ee_a.p, c.ee_b.p, c.ee_c.p, c.ee_vflag.p, c.err.p,
      c.gen_counter.p + 2);
}

void launch_obstacle_commit(Context& c) {
  if (c.onv == 0) return;
  k_obstacle_commit<<<grid_for(c.onv), kBlock, 0, c.stream>>>(c.ox.p, c.ox0.p, c.on.p, c.otri.p,
                                                              c.ovf_ptr.p, c.ovf_list.p, c.onv);
}

void launch_vertex_normals(const float4* x, const int4* tri, const uint32_t* ptr,
                           const uint32_t* list, float4* out, uint32_t nv, cudaStream_t s) {
  if (nv == 0) return;
  k_vertex_normals<<<grid_for(nv), kBlock, 0, s>>>(x, tri, ptr, list, out, nv);
}

void launch_prims_obstacle(Context& c, float tol) {
  launch_prims_from_mesh(c.bvh, c.ox0.p, c.on.p, c.otri.p, c.onf, tol, c.stream);
}

}  // namespace xrt
