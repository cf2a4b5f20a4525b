// proximity.cu — cloth self-contact of XRTailor's Quality mode on the GB300: face-pair broad
// phase over the cloth and obstacle LBVHs, vertex-face / edge-edge proximity repulsion, and the
// CCD narrow phase (coplanarity cubic) over the same face pairs.
//
//   BVH::Update(faces, ccd) ........ xrtailor/src/physics/broad_phase/lbvh/BVH.cu:820-852
//   CountPairs/FindPairs/Traverse .. BVH.cu:1149-1227, 1315-1340 (count, scan, fill back to front)
//   UpdatePairs .................... xrtailor/src/physics/repulsion/PBDRepulsion.cu:22-32
//   EvaluateRep / ApplyPBDImpulse .. PBDRepulsion.cu:264-313, 329-515; Proximity.cu:10-37
//   signed distances, InEdge ....... xrtailor/src/math/BasicPrimitiveTests.cu:286-301, 369-436
//   CheckImpact(s) ................. xrtailor/src/physics/impact_zone/ImpactHelper.cu:34-177,
//                                    SolveCubic xrtailor/src/math/MathFunctions.cu:91-150
//
// Nodes, faces and edges of the cloth and of the obstacle share one numbering (cloth first), the
// device counterpart of the reference's Node*/Face*/Edge* pointers.  Repulsion deltas are summed
// with float atomics in launch order, as in the reference; every other output is deterministic.
#include <algorithm>

#include "common.cuh"
#include "context.h"
#include "lbvh_dev.cuh"

namespace xrt {
namespace {

struct PNodes {
  const float4* cx;   // cloth x, w = inverse mass
  const float4* cx0;
  const float4* ox;
  const float4* ox0;
  const uint8_t* cfree;
  uint32_t V;
  __device__ __forceinline__ f3 x(uint32_t i) const { return i < V ? mk3(cx[i]) : mk3(ox[i - V]); }
  __device__ __forceinline__ f3 x0(uint32_t i) const { return i < V ? mk3(cx0[i]) : mk3(ox0[i - V]); }
  __device__ __forceinline__ float w(uint32_t i) const { return i < V ? cx[i].w : 1.0f / 1e3f; }
  __device__ __forceinline__ bool free_(uint32_t i) const { return i < V && cfree[i] != 0; }
};

struct PTopo {
  const int4* face;    // n0, n1, n2 (unified), r-triangle mask
  const int4* fedge;   // unified edge of (v_i, v_i+1)
  const float4* fn0;   // registration-time face normal
  const uint2* edge;   // unified nodes
  const int4* eadj;    // adjacent unified faces, -1 = none
};

__device__ __forceinline__ float mixed(f3 a, f3 b, f3 c) { return dot(a, cross(b, c)); }

__device__ float signed_vf_distance(f3 x, f3 y0, f3 y1, f3 y2, f3& n, float* w) {
  n = cross(normalize(y1 - y0), normalize(y2 - y0));
  if (dot(n, n) < 1e-6f) return __int_as_float(0x7f800000);
  n = normalize(n);
  const float h = dot(x - y0, n);
  const float b0 = mixed(y1 - x, y2 - x, n);
  const float b1 = mixed(y2 - x, y0 - x, n);
  const float b2 = mixed(y0 - x, y1 - x, n);
  w[0] = 1.0f;
  w[1] = -b0 / (b0 + b1 + b2);
  w[2] = -b1 / (b0 + b1 + b2);
  w[3] = -b2 / (b0 + b1 + b2);
  return h;
}

__device__ float signed_ee_distance(f3 x0, f3 x1, f3 y0, f3 y1, f3& n, float* w) {
  n = cross(normalize(x1 - x0), normalize(y1 - y0));
  if (dot(n, n) < 1e-6f) return __int_as_float(0x7f800000);
  const float h = dot(x0 - y0, n);  // the reference discards normalize(n)
  const float a0 = mixed(y1 - x1, y0 - x1, n);
  const float a1 = mixed(y0 - x0, y1 - x0, n);
  const float b0 = mixed(x0 - y1, x1 - y1, n);
  const float b1 = mixed(x1 - y0, x0 - y0, n);
  w[0] = a0 / (a0 + a1);
  w[1] = a1 / (a0 + a1);
  w[2] = -b0 / (b0 + b1);
  w[3] = -b1 / (b0 + b1);
  return h;
}

__device__ bool in_edge(const PNodes& u, const PTopo& t, float wt, uint32_t e0, uint32_t e1) {
  const uint2 a = t.edge[e0], b = t.edge[e1];
  const f3 xx = (1 - wt) * u.x(a.x) + wt * u.x(a.y);
  const int4 adj = t.eadj[e1];
  const int fs[4] = {adj.x, adj.y, adj.z, adj.w};
  bool in = true;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (fs[k] < 0) continue;
    const f3 e = u.x(b.y) - u.x(b.x);
    const f3 nn = mk3(t.fn0[fs[k]]);
    const f3 r = xx - u.x(b.x);
    in &= (mixed(e, nn, r) >= 0);
  }
  return in;
}

__device__ f3 edge_normal(const PNodes& u, const PTopo& t, uint32_t e) {
  f3 ans = mk3(0, 0, 0);
  int cnt = 0;
  const int4 adj = t.eadj[e];
  const int fs[4] = {adj.x, adj.y, adj.z, adj.w};
  for (int k = 0; k < 4; ++k) {
    if (fs[k] < 0) break;
    const int4 f = t.face[fs[k]];
    ans = ans + face_normal(u.x(f.x), u.x(f.y), u.x(f.z));
    cnt++;
  }
  if (cnt == 0) return ans;
  return ans / (float)cnt;
}

struct Impulse {
  uint32_t nodes[4];
  f3 corr[4];
};

__device__ bool evaluate_vf(const PNodes& u, const PTopo& t, uint32_t node, uint32_t face, float h,
                            Impulse& imp) {
  const int4 fc = t.face[face];
  const uint32_t f0 = fc.x, f1 = fc.y, f2 = fc.z;
  if (node == f0 || node == f1 || node == f2) return false;
  const uint32_t nd[4] = {node, f0, f1, f2};
  f3 pn;
  float pw[4] = {0, 0, 0, 0};
  const float d0 = signed_vf_distance(u.x0(nd[0]), u.x0(nd[1]), u.x0(nd[2]), u.x0(nd[3]), pn, pw);
  const bool face_free = u.free_(f0) && u.free_(f1) && u.free_(f2);
  if (d0 < 0.0f && face_free) pn = -pn;
  f3 fn;
  float w[4] = {0, 0, 0, 0};
  signed_vf_distance(u.x(nd[0]), u.x(nd[1]), u.x(nd[2]), u.x(nd[3]), fn, w);
  const bool inside = tmin(-w[1], tmin(-w[2], -w[3])) >= 1e-6f;
  if (!inside) return false;
  f3 n = face_normal(u.x(nd[1]), u.x(nd[2]), u.x(nd[3]));
  const float side = dot(n, pn) > 0.0f ? 1.0f : -1.0f;
  f3 q = u.x(nd[0]), p1 = u.x(nd[1]), p2 = u.x(nd[2]), p3 = u.x(nd[3]);
  q = q - p1;
  p2 = p2 - p1;
  p3 = p3 - p1;
  n = side * cross(p2, p3);
  const float c23 = length(n);
  n = normalize(n);
  const float C = dot(q, n) - h;
  if (C > 0) return false;
  const f3 dcq = n;
  const f3 dcp2 = (cross(p3, q) + cross(n, p3) * dot(n, q)) / c23;
  const f3 dcp3 = -(cross(p2, q) + cross(n, p2) * dot(n, q)) / c23;
  const f3 dcp1 = -dcq - dcp2 - dcp3;
  const float denom = u.w(nd[0]) * dot(dcq, dcq) + u.w(nd[1]) * dot(dcp1, dcp1) +
                      u.w(nd[2]) * dot(dcp2, dcp2) + u.w(nd[3]) * dot(dcp3, dcp3);
  if (denom < kEps) return false;
  const float s = C / denom;
  imp.corr[0] = -u.w(nd[0]) * s * dcq;
  imp.corr[1] = -u.w(nd[1]) * s * dcp1;
  imp.corr[2] = -u.w(nd[2]) * s * dcp2;
  imp.corr[3] = -u.w(nd[3]) * s * dcp3;
#pragma unroll
  for (int k = 0; k < 4; ++k) imp.nodes[k] = nd[k];
  return true;
}

__device__ bool evaluate_ee(const PNodes& u, const PTopo& t, uint32_t e0, uint32_t e1, float h,
                            Impulse& imp) {
  const uint2 a = t.edge[e0], b = t.edge[e1];
  const uint32_t nd[4] = {a.x, a.y, b.x, b.y};
  if (nd[0] == nd[2] || nd[0] == nd[3] || nd[1] == nd[2] || nd[1] == nd[3]) return false;
  f3 pn;
  float pw[4] = {0, 0, 0, 0};
  const float d0 = signed_ee_distance(u.x0(nd[0]), u.x0(nd[1]), u.x0(nd[2]), u.x0(nd[3]), pn, pw);
  const bool e1_free = u.free_(b.x) && u.free_(b.y);
  if (!e1_free) pn = edge_normal(u, t, e1);
  else if (d0 < 0.0f) pn = -pn;
  f3 ln;
  float bb[4] = {0, 0, 0, 0};
  signed_ee_distance(u.x(nd[0]), u.x(nd[1]), u.x(nd[2]), u.x(nd[3]), ln, bb);
  const bool inside = tmin(tmin(bb[0], bb[1]), tmin(-bb[2], -bb[3])) >= 1e-6f &&
                      in_edge(u, t, bb[1], e0, e1) && in_edge(u, t, -bb[3], e1, e0);
  if (!inside) return false;
  f3 d = mk3(0, 0, 0);
#pragma unroll
  for (int k = 0; k < 4; ++k) d = d + bb[k] * u.x(nd[k]);
  const f3 n = pn;
  const float C = dot(d, n) - h;
  if (C > 0) return false;
  bb[2] *= -1;
  bb[3] *= -1;
  const f3 grads[4] = {bb[0] * n, bb[1] * n, -bb[2] * n, -bb[3] * n};
  float denom = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) denom += u.w(nd[k]) * bb[k] * bb[k];
  if (denom < kEps) return false;
  const float s = C / denom;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    imp.nodes[k] = nd[k];
    imp.corr[k] = -s * u.w(nd[k]) * grads[k];
  }
  return true;
}

__device__ __forceinline__ void accumulate(const PNodes& u, const Impulse& imp, float* deltas,
                                           int* counts) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (length(imp.corr[k]) < kEps) continue;
    if (!u.free_(imp.nodes[k])) continue;
    const uint32_t i = imp.nodes[k];
    atomicAdd(&deltas[3 * i], imp.corr[k].x);
    atomicAdd(&deltas[3 * i + 1], imp.corr[k].y);
    atomicAdd(&deltas[3 * i + 2], imp.corr[k].z);
    atomicAdd(&counts[i], 1);
  }
}

// Update(faces, ccd = true): pred = x of the face, leaf box grows by the x / x0 bounds, then the
// bottom-up merge.  `node_base` offsets face node ids (0 for the cloth, V for the obstacle) into
// the positions arrays passed here.
__global__ void k_update_ccd(uint32_t n, const float4* __restrict__ x, const float4* __restrict__ x0,
                             const int4* __restrict__ tri, float4* pred, float4* lo, float4* hi,
                             const int4* node, uint32_t* flags, uint32_t* err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = n - 1 + i;
  float4 l = lo[k], hh = hi[k];
  const uint32_t obj = (uint32_t)__float_as_int(l.w);
  const int4 t = tri[obj];
  const int id[3] = {t.x, t.y, t.z};
  float fl[3] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000)};
  float fh[3] = {-fl[0], -fl[1], -fl[2]};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const f3 a = mk3(x[id[c]]), b = mk3(x0[id[c]]);
    pred[3 * obj + c] = mk4(a, 0.0f);
    fl[0] = tmin(fl[0], a.x); fl[1] = tmin(fl[1], a.y); fl[2] = tmin(fl[2], a.z);
    fh[0] = tmax(fh[0], a.x); fh[1] = tmax(fh[1], a.y); fh[2] = tmax(fh[2], a.z);
    fl[0] = tmin(fl[0], b.x); fl[1] = tmin(fl[1], b.y); fl[2] = tmin(fl[2], b.z);
    fh[0] = tmax(fh[0], b.x); fh[1] = tmax(fh[1], b.y); fh[2] = tmax(fh[2], b.z);
  }
  l.x = tmin(l.x, fl[0]); l.y = tmin(l.y, fl[1]); l.z = tmin(l.z, fl[2]);
  hh.x = tmax(hh.x, fh[0]); hh.y = tmax(hh.y, fh[1]); hh.z = tmax(hh.z, fh[2]);
  __stcg(&lo[k], l);
  __stcg(&hi[k], hh);
  lbvh_merge_upwards(k, n, lo, hi, node, flags, err);
}

// CountPairs_Kernel (no candidate limit): queries are the leaves of `lhs` in sorted order.
template <bool FILL>
__global__ void k_pairs(LbvhView lhs, LbvhView rhs, float thickness, uint32_t* __restrict__ counts,
                        const uint32_t* __restrict__ incl, uint32_t lhs_base, uint32_t rhs_base,
                        uint32_t out_base, uint2* __restrict__ pairs, uint32_t* err) {
  const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= lhs.n) return;
  const uint32_t k = lhs.n - 1 + id;
  const float4 ql = lhs.lo[k], qh = lhs.hi[k];
  const f3 qlo = mk3(ql.x - thickness, ql.y - thickness, ql.z - thickness);
  const f3 qhi = mk3(qh.x + thickness, qh.y + thickness, qh.z + thickness);
  const uint32_t obj_l = (uint32_t)__float_as_int(ql.w);
  const uint32_t nir = rhs.n - 1;
  int nodei = 0;
  uint32_t found = 0, guard = 0;
  int index = FILL ? (int)(out_base + incl[id]) - 1 : 0;
  while (nodei != -1) {
    if (++guard > 2 * rhs.n + 2) {
      raise_error(err, kErrTraversal);
      break;
    }
    const float4 l = rhs.lo[nodei], h = rhs.hi[nodei];
    if (overlap_box(l, h, qlo, qhi)) {
      if ((uint32_t)nodei >= nir) {
        if (FILL) pairs[index--] = make_uint2(lhs_base + obj_l, rhs_base + (uint32_t)__float_as_int(l.w));
        ++found;
        nodei = __float_as_int(h.w);
      } else {
        nodei = __float_as_int(l.w);
      }
    } else {
      nodei = __float_as_int(h.w);
    }
  }
  if (!FILL) counts[id] = found;
}

// Inclusive scan of a 1024-element tile by one block: warp shuffles, then the warp totals.
__device__ uint32_t block_scan1024(uint32_t v, uint32_t* sw /* 32 */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t o = __shfl_up_sync(0xFFFFFFFFu, v, d);
    if (lane >= d) v += o;
  }
  if (lane == 31) sw[warp] = v;
  __syncthreads();
  if (warp == 0) {
    uint32_t t = sw[lane];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t o = __shfl_up_sync(0xFFFFFFFFu, t, d);
      if (lane >= d) t += o;
    }
    sw[lane] = t;
  }
  __syncthreads();
  return v + (warp ? sw[warp - 1] : 0u);
}

// Phase 1 of the multi-block scan: the sum of each 1024-element tile.
__global__ void __launch_bounds__(1024) k_tile_sums(const uint32_t* __restrict__ in, uint32_t n,
                                                    uint32_t* __restrict__ sums) {
  __shared__ uint32_t sw[32];
  const uint32_t i = blockIdx.x * 1024u + threadIdx.x;
  const uint32_t v = block_scan1024(i < n ? in[i] : 0u, sw);
  if (threadIdx.x == 1023) sums[blockIdx.x] = v;
}

// Phase 3: each tile scanned, plus the inclusive scan of the tile sums before it.
__global__ void __launch_bounds__(1024) k_tile_scan(const uint32_t* __restrict__ in, uint32_t n,
                                                    const uint32_t* __restrict__ sums,
                                                    const uint32_t* __restrict__ sums_incl,
                                                    uint32_t* __restrict__ out) {
  __shared__ uint32_t sw[32];
  const uint32_t i = blockIdx.x * 1024u + threadIdx.x;
  const uint32_t base = sums_incl[blockIdx.x] - sums[blockIdx.x];
  const uint32_t v = block_scan1024(i < n ? in[i] : 0u, sw);
  if (i < n) out[i] = base + v;
}

// Inclusive scan of `n` counts by one block of 1024 threads; total[0] = sum.
__global__ void __launch_bounds__(1024) k_scan_inclusive(const uint32_t* __restrict__ in,
                                                         uint32_t* __restrict__ out, uint32_t n,
                                                         uint32_t* __restrict__ total) {
  __shared__ uint32_t s[1024];
  const uint32_t per = (n + 1023) / 1024;
  const uint32_t b = threadIdx.x * per, e = min(b + per, n);
  uint32_t sum = 0;
  for (uint32_t i = b; i < e; ++i) sum += in[i];
  s[threadIdx.x] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const uint32_t v = threadIdx.x >= (unsigned)off ? s[threadIdx.x - off] : 0u;
    __syncthreads();
    s[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = s[threadIdx.x] - sum;
  for (uint32_t i = b; i < e; ++i) {
    run += in[i];
    out[i] = run;
  }
  if (threadIdx.x == 1023) *total = s[1023];
}

__global__ void k_evaluate_rep(PNodes u, PTopo t, const uint2* __restrict__ pairs, uint32_t np,
                               float h, float* deltas, int* counts) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const uint2 pr = pairs[p];
  const int4 fa = t.face[pr.x], fb = t.face[pr.y];
  const uint32_t r0 = (uint32_t)fa.w, r1 = (uint32_t)fb.w;
  const uint32_t fan[3] = {(uint32_t)fa.x, (uint32_t)fa.y, (uint32_t)fa.z};
  for (int i = 0; i < 3; ++i) {
    if (!((r0 >> i) & 1u)) continue;
    Impulse imp;
    if (evaluate_vf(u, t, fan[i], pr.y, h, imp)) accumulate(u, imp, deltas, counts);
  }
  const int4 ea = t.fedge[pr.x], eb = t.fedge[pr.y];
  const uint32_t eas[3] = {(uint32_t)ea.x, (uint32_t)ea.y, (uint32_t)ea.z};
  const uint32_t ebs[3] = {(uint32_t)eb.x, (uint32_t)eb.y, (uint32_t)eb.z};
  for (int i = 0; i < 3; ++i) {
    if (!((r0 >> (i + 3)) & 1u)) continue;
    for (int j = 0; j < 3; ++j) {
      if (!((r1 >> (j + 3)) & 1u)) continue;
      Impulse imp;
      if (evaluate_ee(u, t, eas[i], ebs[j], h, imp)) accumulate(u, imp, deltas, counts);
    }
  }
}

__global__ void k_apply_rep(float4* __restrict__ x, float* __restrict__ deltas, int* __restrict__ counts,
                            uint32_t nv, float relaxation) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const float count = (float)counts[i];
  if (count <= kEps) return;
  const f3 d = mk3(deltas[3 * i], deltas[3 * i + 1], deltas[3 * i + 2]);
  const f3 dx = d / count * relaxation;
  const float4 p = x[i];
  x[i] = mk4(mk3(p) + dx, p.w);
  deltas[3 * i] = 0.0f;
  deltas[3 * i + 1] = 0.0f;
  deltas[3 * i + 2] = 0.0f;
  counts[i] = 0;
}

// ---- CCD narrow phase -------------------------------------------------------------------------

__device__ float newtons_method(float a, float b, float c, float d, float x0, int dir) {
  if (dir != 0) {
    const float y0 = d + x0 * (c + x0 * (b + x0 * a));
    const float ddy0 = 2.0f * b + x0 * (6.0f * a);
    x0 += dir * sqrtf(tabs(2.0f * y0 / ddy0));
  }
  for (int iter = 0; iter < 100; iter++) {
    const float y = d + x0 * (c + x0 * (b + x0 * a));
    const float dy = c + x0 * (2.0f * b + 3.0f * x0 * a);
    if (dy == 0) return x0;
    const float x1 = x0 - y / dy;
    if (tabs(x0 - x1) < 1e-6f) return x0;
    x0 = x1;
  }
  return x0;
}

__device__ int solve_quadratic(float a, float b, float c, float x[2]) {
  const float d = b * b - 4.0f * a * c;
  if (d < 0) {
    x[0] = -b / (2.0f * a);
    return 0;
  }
  const float q = -(b + (b < 0.0f ? -1 : 1) * sqrtf(d)) * 0.5f;
  int i = 0;
  if (tabs(a) > 1e-12f * tabs(q)) x[i++] = q / a;
  if (tabs(q) > 1e-12f * tabs(c)) x[i++] = c / q;
  if (i == 2 && x[0] > x[1]) {
    const float tt = x[0];
    x[0] = x[1];
    x[1] = tt;
  }
  return i;
}

// SolveCubic (MathFunctions.cu:128-150).  When the derivative quadratic has a non-negative
// discriminant but no accepted root (a = b = 0: a linear coplanarity polynomial, e.g. parallel
// motion), the reference starts Newton's method from an uninitialized xc[0]; here it starts from 0.
__device__ int solve_cubic(float a, float b, float c, float d, float x[3]) {
  float xc[2] = {0.0f, 0.0f};
  const int n = solve_quadratic(3.0f * a, 2.0f * b, c, xc);
  if (n == 0) {
    x[0] = newtons_method(a, b, c, d, xc[0], 0);
    return 1;
  } else if (n == 1) {
    return solve_quadratic(b, c, d, x);
  }
  const float yc[2] = {d + xc[0] * (c + xc[0] * (b + xc[0] * a)),
                       d + xc[1] * (c + xc[1] * (b + xc[1] * a))};
  int i = 0;
  if (yc[0] * a >= 0) x[i++] = newtons_method(a, b, c, d, xc[0], -1);
  if (yc[0] * yc[1] <= 0) {
    const int closer = tabs(yc[0]) < tabs(yc[1]) ? 0 : 1;
    x[i++] = newtons_method(a, b, c, d, xc[closer], closer == 0 ? 1 : -1);
  }
  if (yc[1] * a <= 0) x[i++] = newtons_method(a, b, c, d, xc[1], 1);
  return i;
}

struct ImpactOut {
  float* t;
  float4* w;
  float4* n;   // xyz = normal, w = 1 for vertex-face
  uint4* nodes;
};

__device__ bool check_impact(const PNodes& u, bool vf, const uint32_t* nd, float& t_out, float* w,
                             f3& n) {
  const f3 x0 = u.x0(nd[0]);
  const f3 v0 = u.x(nd[0]) - x0;
  const f3 x1 = u.x0(nd[1]) - x0, x2 = u.x0(nd[2]) - x0, x3 = u.x0(nd[3]) - x0;
  const f3 v1 = (u.x(nd[1]) - u.x0(nd[1])) - v0;
  const f3 v2 = (u.x(nd[2]) - u.x0(nd[2])) - v0;
  const f3 v3 = (u.x(nd[3]) - u.x0(nd[3])) - v0;
  const float a0 = mixed(x1, x2, x3);
  const float a1 = mixed(v1, x2, x3) + mixed(x1, v2, x3) + mixed(x1, x2, v3);
  const float a2 = mixed(x1, v2, v3) + mixed(v1, x2, v3) + mixed(v1, v2, x3);
  const float a3 = mixed(v1, v2, v3);
  float t[3];
  const int ns = solve_cubic(a3, a2, a1, a0, t);
  for (int i = 0; i < ns; ++i) {
    if (t[i] < 0 || t[i] > 1) continue;
    t_out = t[i];
    f3 p[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) p[k] = u.x0(nd[k]) + t[i] * (u.x(nd[k]) - u.x0(nd[k]));
    float d;
    bool inside;
    if (vf) {
      d = signed_vf_distance(p[0], p[1], p[2], p[3], n, w);
      inside = tmin(-w[1], tmin(-w[2], -w[3])) >= -1e-6f;
    } else {
      d = signed_ee_distance(p[0], p[1], p[2], p[3], n, w);
      inside = tmin(tmin(w[0], w[1]), tmin(-w[2], -w[3])) >= -1e-6f;
    }
    if (dot(n, w[1] * v1 + w[2] * v2 + w[3] * v3) > 0) n = -n;
    if (tabs(d) < 1e-6f && inside) return true;
  }
  return false;
}

__device__ __forceinline__ void grow(float* lo, float* hi, f3 p) {
  lo[0] = tmin(lo[0], p.x); lo[1] = tmin(lo[1], p.y); lo[2] = tmin(lo[2], p.z);
  hi[0] = tmax(hi[0], p.x); hi[1] = tmax(hi[1], p.y); hi[2] = tmax(hi[2], p.z);
}

// ComputeBounds(ccd = true) of `cnt` nodes of `nd` starting at `first`
__device__ void ccd_bounds(const PNodes& u, const uint32_t* nd, int first, int cnt, float* lo,
                           float* hi) {
  lo[0] = lo[1] = lo[2] = __int_as_float(0x7f800000);
  hi[0] = hi[1] = hi[2] = -lo[0];
  for (int k = first; k < first + cnt; ++k) {
    grow(lo, hi, u.x(nd[k]));
    grow(lo, hi, u.x0(nd[k]));
  }
}

__device__ bool overlap_dilated(const float* alo, const float* ahi, const float* blo,
                                const float* bhi, float th) {
  for (int i = 0; i < 3; ++i) {
    if (alo[i] > bhi[i] + th) return false;
    if (ahi[i] < blo[i] - th) return false;
  }
  return true;
}

// One thread per test: test k of pair p writes slot 15 p + k.  k = 3 side + i (side 0: vertex i of
// the first face against the second face, side 1: the reverse), then k = 6 + 3 i + j (edge i of
// the first face against edge j of the second), the reference's order.
__global__ void __launch_bounds__(kBlock, 3) k_check_impacts(PNodes u, PTopo t,
                                                             const uint2* __restrict__ pairs, uint32_t np,
                                float thickness, ImpactOut out) {
  const size_t index = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (index >= 15 * (size_t)np) return;
  const uint32_t p = (uint32_t)(index / 15), k = (uint32_t)(index % 15);
  const uint2 pr = pairs[p];
  const bool vf = k < 6;
  uint32_t nd[4];
  bool distinct;
  if (vf) {
    const uint32_t side = k / 3, i = k % 3;
    const int4 a = t.face[side == 0 ? pr.x : pr.y], b = t.face[side == 0 ? pr.y : pr.x];
    nd[0] = (uint32_t)(i == 0 ? a.x : (i == 1 ? a.y : a.z));
    nd[1] = (uint32_t)b.x;
    nd[2] = (uint32_t)b.y;
    nd[3] = (uint32_t)b.z;
    distinct = !(nd[0] == nd[1] || nd[0] == nd[2] || nd[0] == nd[3]);
  } else {
    const uint32_t i = (k - 6) / 3, j = (k - 6) % 3;
    const int4 ea = t.fedge[pr.x], eb = t.fedge[pr.y];
    const uint2 e0 = t.edge[i == 0 ? ea.x : (i == 1 ? ea.y : ea.z)];
    const uint2 e1 = t.edge[j == 0 ? eb.x : (j == 1 ? eb.y : eb.z)];
    nd[0] = e0.x;
    nd[1] = e0.y;
    nd[2] = e1.x;
    nd[3] = e1.y;
    distinct = !(nd[0] == nd[2] || nd[0] == nd[3] || nd[1] == nd[2] || nd[1] == nd[3]);
  }
  float w[4] = {0, 0, 0, 0};
  f3 n = mk3(0, 0, 0);
  float tt = 0;
  bool ok = false;
  if (distinct) {
    const int na = vf ? 1 : 2;
    float alo[3], ahi[3], blo[3], bhi[3];
    ccd_bounds(u, nd, 0, na, alo, ahi);
    ccd_bounds(u, nd, na, 4 - na, blo, bhi);
    if (overlap_dilated(alo, ahi, blo, bhi, thickness)) ok = check_impact(u, vf, nd, tt, w, n);
  }
  out.t[index] = ok ? tt : -1.0f;
  out.w[index] = make_float4(w[0], w[1], w[2], w[3]);
  out.n[index] = make_float4(n.x, n.y, n.z, vf ? 1.0f : 0.0f);
  out.nodes[index] = make_uint4(nd[0], nd[1], nd[2], nd[3]);
}

// ---- imminent repulsion (ImminentRepulsion.cu, ImminentRepulsionHelper.cu) ---------------------

// CheckImminentVFQuadrature (ImminentRepulsionHelper.cu:10-38): the vertex inside the face at x0;
// nodes (face 0, 1, 2, vertex), weights rotated to match.
__device__ bool imminent_vf(const PNodes& u, uint32_t node, int4 fc, uint4& qn, float4& qb) {
  const uint32_t f0 = (uint32_t)fc.x, f1 = (uint32_t)fc.y, f2 = (uint32_t)fc.z;
  if (node == f0 || node == f1 || node == f2) return false;
  f3 fn;
  float w[4] = {0, 0, 0, 0};
  signed_vf_distance(u.x0(node), u.x0(f0), u.x0(f1), u.x0(f2), fn, w);
  if (!(tmin(-w[1], tmin(-w[2], -w[3])) >= 1e-6f)) return false;
  qn = make_uint4(f0, f1, f2, node);
  qb = make_float4(w[1], w[2], w[3], w[0]);
  return true;
}

// CheckImminentEEQuadrature (ImminentRepulsionHelper.cu:40-66)
__device__ bool imminent_ee(const PNodes& u, const PTopo& t, uint32_t e0, uint32_t e1, uint4& qn,
                            float4& qb) {
  const uint2 a = t.edge[e0], b = t.edge[e1];
  if (a.x == b.x || a.x == b.y || a.y == b.x || a.y == b.y) return false;
  f3 fn;
  float w[4] = {0, 0, 0, 0};
  signed_ee_distance(u.x0(a.x), u.x0(a.y), u.x0(b.x), u.x0(b.y), fn, w);
  if (!(tmin(tmin(w[0], w[1]), tmin(-w[2], -w[3])) >= 1e-6f && in_edge(u, t, w[1], e0, e1) &&
        in_edge(u, t, -w[3], e1, e0)))
    return false;
  qn = make_uint4(a.x, a.y, b.x, b.y);
  qb = make_float4(w[0], w[1], w[2], w[3]);
  return true;
}

// EvaluateEE/VFQuadrature_Kernel: slot 12 p + 3 i + j edge i of the first face against edge j
// of the second (both owned by their r-triangles), slot 12 p + 9 + i vertex i of the first face
// (owned) against the second face; a face paired with itself gives nothing.
__global__ void k_imminent_quads(PNodes u, PTopo t, const uint2* __restrict__ pairs, uint32_t np,
                                 uint4* __restrict__ qnodes, float4* __restrict__ qbary) {
  const size_t slot = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= 12 * (size_t)np) return;
  const uint32_t p = (uint32_t)(slot / 12), k = (uint32_t)(slot % 12);
  const uint2 pr = pairs[p];
  uint4 qn = make_uint4(kNone, kNone, kNone, kNone);
  float4 qb = make_float4(0, 0, 0, 0);
  if (pr.x != pr.y) {
    const int4 fa = t.face[pr.x], fb = t.face[pr.y];
    const uint32_t r0 = (uint32_t)fa.w, r1 = (uint32_t)fb.w;
    if (k < 9) {
      const uint32_t i = k / 3, j = k % 3;
      if (((r0 >> (i + 3)) & 1u) && ((r1 >> (j + 3)) & 1u)) {
        const int4 ea = t.fedge[pr.x], eb = t.fedge[pr.y];
        const uint32_t e0 = (uint32_t)(i == 0 ? ea.x : (i == 1 ? ea.y : ea.z));
        const uint32_t e1 = (uint32_t)(j == 0 ? eb.x : (j == 1 ? eb.y : eb.z));
        if (!imminent_ee(u, t, e0, e1, qn, qb)) qn.x = kNone;
      }
    } else {
      const uint32_t i = k - 9;
      if ((r0 >> i) & 1u) {
        const uint32_t node = (uint32_t)(i == 0 ? fa.x : (i == 1 ? fa.y : fa.z));
        if (!imminent_vf(u, node, fb, qn, qb)) qn.x = kNone;
      }
    }
  }
  qnodes[slot] = qn;
  qbary[slot] = qb;
}

// UpdateVelocity_Kernel (ImminentRepulsion.cu:147-151): v = (x - x0) / dt for the cloth
__global__ void k_imminent_velocity(const float4* __restrict__ x, const float4* __restrict__ x0,
                                    float4* __restrict__ v, uint32_t n, float dt) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  v[i] = mk4((mk3(x[i]) - mk3(x0[i])) / dt, v[i].w);
}

// ComputeImminentImpulse_Kernel + EvaluateImminentImpulse (ImminentRepulsionHelper.cu:68-131)
// with add_repulsion = true; AccumulateImpulses (float atomics, as the reference).
__global__ void k_imminent_impulse(PNodes u, const float4* __restrict__ cv,
                                   const float4* __restrict__ ov, const uint4* __restrict__ qnodes,
                                   const float4* __restrict__ qbary, uint32_t nq, float h, float dt,
                                   float* deltas, int* counts) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const uint4 qn = qnodes[q];
  if (qn.x == kNone) return;
  const float4 qb = qbary[q];
  const uint32_t nd[4] = {qn.x, qn.y, qn.z, qn.w};
  const float b[4] = {qb.x, qb.y, qb.z, qb.w};
  f3 pr = mk3(0.0f, 0.0f, 0.0f), vr = mk3(0.0f, 0.0f, 0.0f);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    pr = pr + b[i] * u.x0(nd[i]);
    vr = vr + b[i] * (nd[i] < u.V ? mk3(cv[nd[i]]) : mk3(ov[nd[i] - u.V]));
  }
  const float npr = length(pr);
  if (npr > h) return;
  if (npr < 1e-5f) return;
  pr = normalize(pr);
  const float vr_nrm = dot(vr, pr);
  const float target = (h - npr) * 0.1f;
  if (vr_nrm > target) return;
  f3 I = (vr_nrm * dt) * pr;
  const f3 vr_tan = vr - vr_nrm * pr;
  if (length(vr_tan) > h * 0.01f) {  // friction coefficient 0: the term adds signed zeros
    const float imp_norm = length(I);
    const f3 dir = normalize(vr_tan);
    const float coeff = 0.0f;
    const f3 friction = imp_norm * coeff > length(vr_tan) ? -vr_tan : (-dir * imp_norm) * coeff;
    I = I + friction * 1.0f;
  }
  float inv_cm = 0.0f;
#pragma unroll
  for (int i = 0; i < 4; ++i) inv_cm += (b[i] * b[i]) * u.w(nd[i]);
  if (inv_cm < 1e-5f) return;
  Impulse imp;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float beta = (-u.w(nd[i]) * b[i]) / inv_cm;
    imp.corr[i] = I * beta;
    imp.nodes[i] = nd[i];
  }
  accumulate(u, imp, deltas, counts);
}

PNodes nodes_of(const Context& c) {
  return PNodes{c.x.p, c.x0.p, c.ox.p, c.ox0.p, c.prox.cfree.p, c.nv};
}
PTopo topo_of(const Context& c) {
  return PTopo{c.prox.face.p, c.prox.fedge.p, c.prox.fn0.p, c.prox.edge.p, c.prox.eadj.p};
}

}  // namespace

// Tiles of 1024 summed, the tile sums scanned by one block, the tiles scanned with their offsets.
cudaError_t scan_inclusive(ScanScratch& w, const uint32_t* in, uint32_t* out, uint32_t n,
                           uint32_t* total, cudaStream_t s) {
  const uint32_t nt = std::max(1u, (n + 1023) / 1024);
  cudaError_t e = w.sums.reserve(nt);
  if (e == cudaSuccess) e = w.incl.reserve(nt);
  if (e != cudaSuccess) return e;
  if (n == 0) return cudaMemsetAsync(total, 0, sizeof(uint32_t), s);
  k_tile_sums<<<nt, 1024, 0, s>>>(in, n, w.sums.p);
  k_scan_inclusive<<<1, 1024, 0, s>>>(w.sums.p, w.incl.p, nt, total);
  k_tile_scan<<<nt, 1024, 0, s>>>(in, n, w.sums.p, w.incl.p, out);
  return cudaGetLastError();
}

void launch_cloth_bvh_build(Context& c) {
  Lbvh& b = c.prox.cbvh;
  b.n = c.nf;
  launch_prims_from_mesh(b, c.x0.p, c.n.p, c.tri.p, c.nf, 0.0f, c.stream);
  b.construct(0.0f, c.stream, c.err.p);
}

void launch_update_ccd(Lbvh& b, const float4* x, const float4* x0, const int4* tri, cudaStream_t s,
                       uint32_t* err) {
  if (!b.active) return;
  k_update_ccd<<<grid_for(b.n), kBlock, 0, s>>>(b.n, x, x0, tri, b.pred.p, b.lo.p, b.hi.p, b.node.p,
                                                b.flags.p, err);
}

// UpdatePairs: cloth BVH Update(ccd), then cloth x obstacle and cloth x cloth pairs.
cudaError_t prox_update_pairs(Context& c, float thickness) {
  launch_update_ccd(c.prox.cbvh, c.x.p, c.x0.p, c.tri.p, c.stream, c.err.p);
  return prox_face_pairs(c, c.prox.cbvh, c.bvh, thickness);
}

// Traverse(cloth, obstacle) followed by Traverse(cloth, cloth) into the pair list.  The pair
// count is read back to size the list (the reference reads num.back() the same way).
cudaError_t prox_face_pairs(Context& c, const Lbvh& cloth, const Lbvh& obstacle, float thickness,
                            bool self_first) {
  ProximityState& P = c.prox;
  P.npairs = 0;
  if (!cloth.active) return cudaGetLastError();
  const LbvhView lhs = cloth.view();
  const uint32_t nq = lhs.n;
  struct Side {
    LbvhView rhs;
    uint32_t base;
    bool on;
  } sides[2] = {{obstacle.view(), c.nf, obstacle.active}, {lhs, 0u, true}};
  if (self_first) std::swap(sides[0], sides[1]);
  uint32_t totals[2] = {0, 0};
  for (int s = 0; s < 2; ++s) {
    if (!sides[s].on) continue;
    k_pairs<false><<<grid_for(nq), kBlock, 0, c.stream>>>(lhs, sides[s].rhs, thickness, P.counts.p,
                                                          nullptr, 0, 0, 0, nullptr, c.err.p);
    const cudaError_t e = scan_inclusive(P.scan, P.counts.p, P.incl.p + (size_t)s * nq, nq,
                                         P.total.p + s, c.stream);
    if (e != cudaSuccess) return e;
  }
  cudaError_t e = cudaMemcpyAsync(totals, P.total.p, sizeof(totals), cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return e;
  for (int s = 0; s < 2; ++s)
    if (!sides[s].on) totals[s] = 0;
  const uint32_t np = totals[0] + totals[1];
  if (np > P.pairs.n) {
    e = P.pairs.reserve((size_t)np + np / 4 + 1024);
    if (e != cudaSuccess) return e;
  }
  uint32_t out_base = 0;
  for (int s = 0; s < 2; ++s) {
    if (!sides[s].on) continue;
    k_pairs<true><<<grid_for(nq), kBlock, 0, c.stream>>>(lhs, sides[s].rhs, thickness, nullptr,
                                                         P.incl.p + (size_t)s * nq, 0,
                                                         sides[s].base, out_base, P.pairs.p, c.err.p);
    out_base += totals[s];
  }
  P.npairs = np;
  return cudaGetLastError();
}

void prox_solve(Context& c, float thickness, float relaxation) {
  ProximityState& P = c.prox;
  if (P.npairs)
    k_evaluate_rep<<<grid_for(P.npairs), kBlock, 0, c.stream>>>(nodes_of(c), topo_of(c), P.pairs.p,
                                                                P.npairs, thickness, P.deltas.p,
                                                                P.rcounts.p);
  k_apply_rep<<<grid_for(c.nv), kBlock, 0, c.stream>>>(c.x.p, P.deltas.p, P.rcounts.p, c.nv,
                                                       relaxation);
}

void launch_node_velocity(const float4* x, const float4* x0, float4* v, uint32_t n, float dt,
                          cudaStream_t s) {
  if (n) k_imminent_velocity<<<grid_for(n), kBlock, 0, s>>>(x, x0, v, n, dt);
}

// UpdateProximity (Traverse cloth x cloth, then cloth x obstacle, thickness 1e-6, on the trees as
// they are) + Generate: the quadrature slots of the frame.
cudaError_t prox_imminent_generate(Context& c) {
  ProximityState& P = c.prox;
  cudaError_t e = prox_face_pairs(c, P.cbvh, c.bvh, 1e-6f, /*self_first=*/true);
  if (e != cudaSuccess) return e;
  const size_t nq = 12 * (size_t)P.npairs;
  if (nq > P.qnodes.n) {
    if ((e = P.qnodes.reserve(nq + nq / 4)) || (e = P.qbary.reserve(nq + nq / 4))) return e;
  }
  P.nquads = (uint32_t)nq;
  if (nq)
    k_imminent_quads<<<grid_for((uint32_t)nq), kBlock, 0, c.stream>>>(nodes_of(c), topo_of(c),
                                                                      P.pairs.p, P.npairs,
                                                                      P.qnodes.p, P.qbary.p);
  return cudaGetLastError();
}

// ImminentRepulsion::Solve: cloth velocities, impulses of every quadrature, ApplyImminentImpulse.
void prox_imminent_solve(Context& c, float thickness, float relaxation, float dt) {
  ProximityState& P = c.prox;
  launch_node_velocity(c.x.p, c.x0.p, c.v.p, c.nv, dt, c.stream);
  if (P.nquads)
    k_imminent_impulse<<<grid_for(P.nquads), kBlock, 0, c.stream>>>(
        nodes_of(c), c.v.p, P.ov.p, P.qnodes.p, P.qbary.p, P.nquads, thickness, dt, P.deltas.p,
        P.rcounts.p);
  k_apply_rep<<<grid_for(c.nv), kBlock, 0, c.stream>>>(c.x.p, P.deltas.p, P.rcounts.p, c.nv,
                                                       relaxation);
}

cudaError_t prox_check_impacts(Context& c, float thickness) {
  ProximityState& P = c.prox;
  const size_t ni = 15 * (size_t)P.npairs;
  cudaError_t e = cudaSuccess;
  if (ni > P.imp_t.n) {
    if ((e = P.imp_t.reserve(ni)) || (e = P.imp_w.reserve(ni)) || (e = P.imp_n.reserve(ni)) ||
        (e = P.imp_nodes.reserve(ni)))
      return e;
  }
  P.nimpacts = (uint32_t)ni;
  if (P.npairs)
    k_check_impacts<<<grid_for((uint32_t)ni), kBlock, 0, c.stream>>>(
        nodes_of(c), topo_of(c), P.pairs.p, P.npairs, thickness,
        ImpactOut{P.imp_t.p, P.imp_w.p, P.imp_n.p, P.imp_nodes.p});
  return cudaGetLastError();
}

}  // namespace xrt
