// lbvh.cu — linear BVH over triangles: Morton codes, stable radix sort, Karras hierarchy,
// bottom-up boxes, escape tables, refit and stackless queries.
//
// Reference: xrtailor/src/physics/broad_phase/lbvh/BVH.cu — expand_bits/morton_code :22-46,
// determine_range/find_split :57-210, escape tables :212-273, Karras nodes :275-329,
// UpdateObjects :382-421, InitAABBs :423-462, ComputeMortons :465-479, AssignAABBCAS :515-538,
// Construct :618-722, RefitMidstep :770-818, QueryDeviceStackless :957-1055; box tests
// xrtailor/src/physics/broad_phase/Bounds.cu.
//
// Layout: node k keeps its box and its traversal links in two float4s (32 B, one sector):
//   lo = {lower.xyz, left child (internal) | object (leaf)}, hi = {upper.xyz, escape index}.
// A leaf is node >= n-1.  Stackless traversal therefore reads 32 contiguous bytes per visit.
// The hierarchy is always built on 64-bit keys (code << 32 | object): for unique codes this gives
// exactly the tree the reference builds on 32-bit codes (every common-prefix length is decided
// in the high word), and for duplicate codes it is the reference's own 64-bit fallback.
#include "common.cuh"
#include "context.h"
#include "lbvh_dev.cuh"

namespace xrt {
namespace {

__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__device__ __forceinline__ uint32_t morton_code(f3 p) {
  const float res = 1024.0f;
  float x = tmin(tmax(p.x * res, 0.0f), res - 1.0f);
  float y = tmin(tmax(p.y * res, 0.0f), res - 1.0f);
  float z = tmin(tmax(p.z * res, 0.0f), res - 1.0f);
  return expand_bits((uint32_t)x) * 4 + expand_bits((uint32_t)y) * 2 + expand_bits((uint32_t)z);
}

// Order-preserving float <-> uint mapping for atomic min / max of the root box.
__device__ __forceinline__ uint32_t f2o(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// Root boxes of every segment: 6 ordered-int extrema each.
__global__ void k_root_init(uint32_t* root, uint32_t nseg, uint32_t* dup) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 6 * nseg) {
    const uint32_t k = t % 6;
    root[t] = k < 3 ? f2o(__int_as_float(0x7f800000)) : f2o(__int_as_float((int)0xff800000));
  }
  if (t == 0) *dup = 0;
}

// InitAABBs_Kernel + the root reduction (thrust::reduce of Bounds::Merge), per segment.  Min /
// max are exact, so the reduction order does not matter: warps whose lanes share one segment
// reduce by shuffles, a warp that straddles a segment boundary commits lane by lane.
__global__ void __launch_bounds__(kBlock) k_leaf_boxes(const float4* __restrict__ v,
                                                       const float4* __restrict__ pred, uint32_t n,
                                                       float scr, float4* __restrict__ leaf_lo,
                                                       float4* __restrict__ leaf_hi,
                                                       uint32_t* __restrict__ root, LbvhForest F) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  float lo[3] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000)};
  float hi[3] = {-lo[0], -lo[1], -lo[2]};
  if (i < n) {
    f3 v1 = mk3(v[3 * i]), v2 = mk3(v[3 * i + 1]), v3 = mk3(v[3 * i + 2]);
    f3 p1 = mk3(pred[3 * i]), p2 = mk3(pred[3 * i + 1]), p3 = mk3(pred[3 * i + 2]);
    f3 bl = mk3(tmin(tmin(v1.x, tmin(v2.x, v3.x)), tmin(p1.x, tmin(p2.x, p3.x))),
                tmin(tmin(v1.y, tmin(v2.y, v3.y)), tmin(p1.y, tmin(p2.y, p3.y))),
                tmin(tmin(v1.z, tmin(v2.z, v3.z)), tmin(p1.z, tmin(p2.z, p3.z))));
    f3 bu = mk3(tmax(tmax(v1.x, tmax(v2.x, v3.x)), tmax(p1.x, tmax(p2.x, p3.x))),
                tmax(tmax(v1.y, tmax(v2.y, v3.y)), tmax(p1.y, tmax(p2.y, p3.y))),
                tmax(tmax(v1.z, tmax(v2.z, v3.z)), tmax(p1.z, tmax(p2.z, p3.z))));
    f3 center = (bl + bu) * 0.5f;
    f3 n1 = normalize(bl - center);
    f3 n2 = normalize(bu - center);
    bl = bl + scr * n1;
    bu = bu + scr * n2;
    leaf_lo[i] = mk4(bl, 0.0f);
    leaf_hi[i] = mk4(bu, 0.0f);
    lo[0] = bl.x; lo[1] = bl.y; lo[2] = bl.z;
    hi[0] = bu.x; hi[1] = bu.y; hi[2] = bu.z;
  }
  const uint32_t seg = i < n ? forest_find(F, i, 0) : 0xFFFFFFFFu;
  const int lane = threadIdx.x & 31;
  if (__match_any_sync(0xFFFFFFFFu, seg) == 0xFFFFFFFFu) {
    if (seg == 0xFFFFFFFFu) return;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float a = lo[k], b = hi[k];
      for (int off = 16; off > 0; off >>= 1) {
        a = fminf(a, __shfl_xor_sync(0xFFFFFFFFu, a, off));
        b = fmaxf(b, __shfl_xor_sync(0xFFFFFFFFu, b, off));
      }
      lo[k] = a;
      hi[k] = b;
    }
    if (lane != 0) return;
  } else if (seg == 0xFFFFFFFFu) {
    return;
  }
  uint32_t* r = root + 6 * (size_t)seg;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    atomicMin(&r[k], f2o(lo[k]));
    atomicMax(&r[3 + k], f2o(hi[k]));
  }
}

// ComputeMortons_Kernel: centre of the leaf box normalised by its segment's root box.
__global__ void k_morton(const float4* __restrict__ leaf_lo, const float4* __restrict__ leaf_hi,
                         const uint32_t* __restrict__ root_all, uint32_t n,
                         uint32_t* __restrict__ morton, uint32_t* __restrict__ index, LbvhForest F) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t* root = root_all + 6 * (size_t)forest_find(F, i, 0);
  const f3 wl = mk3(o2f(root[0]), o2f(root[1]), o2f(root[2]));
  const f3 wu = mk3(o2f(root[3]), o2f(root[4]), o2f(root[5]));
  f3 p = 0.5f * (mk3(leaf_lo[i]) + mk3(leaf_hi[i]));
  p.x = p.x - wl.x;
  p.y = p.y - wl.y;
  p.z = p.z - wl.z;
  p.x = p.x / (wu.x - wl.x);
  p.y = p.y / (wu.y - wl.y);
  p.z = p.z / (wu.z - wl.z);
  morton[i] = morton_code(p);
  index[i] = i;
}

// Segment pass of the sort: after the Morton pass, a stable sort by segment groups each
// segment's primitives in (code, index) order, the order the segment alone would have.
__global__ void k_seg_keys(const uint32_t* __restrict__ sindex, uint32_t n, uint32_t* __restrict__ key,
                           uint32_t* __restrict__ val, LbvhForest F) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  key[i] = forest_find(F, sindex[i], 0);
  val[i] = i;
}
__global__ void k_seg_gather(const uint32_t* __restrict__ perm, const uint32_t* __restrict__ m_in,
                             const uint32_t* __restrict__ i_in, uint32_t n,
                             uint32_t* __restrict__ m_out, uint32_t* __restrict__ i_out) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const uint32_t q = perm[p];
  m_out[p] = m_in[q];
  i_out[p] = i_in[q];
}

// ConstructLeafNodes_Kernel + leaf boxes in sorted order + 64-bit keys + uniqueness count.
// Objects and keys use segment-local primitive ids.
__global__ void k_leaves(const uint32_t* __restrict__ smorton, const uint32_t* __restrict__ sindex,
                         const float4* __restrict__ leaf_lo, const float4* __restrict__ leaf_hi,
                         uint32_t n, float4* __restrict__ lo, float4* __restrict__ hi,
                         int4* __restrict__ node, unsigned long long* __restrict__ key64,
                         uint32_t* __restrict__ dup, LbvhForest F) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int4 r = forest_rec(F, forest_find(F, i, 0));
  const uint32_t li = i - (uint32_t)r.x;
  const uint32_t gobj = sindex[i];
  const uint32_t obj = gobj - (uint32_t)r.x;
  const uint32_t k = (uint32_t)r.z + (uint32_t)r.y - 1 + li;
  const float4 a = leaf_lo[gobj], b = leaf_hi[gobj];
  lo[k] = make_float4(a.x, a.y, a.z, __int_as_float((int)obj));
  hi[k] = make_float4(b.x, b.y, b.z, __int_as_float(-1));
  node[k] = make_int4(-1, -1, -1, (int)obj);
  const uint32_t m = smorton[i];
  key64[i] = ((unsigned long long)m << 32) | obj;
  if (li > 0 && smorton[i - 1] == m) atomicAdd(dup, 1u);
}

__device__ __forceinline__ int cub64(unsigned long long a, unsigned long long b) {
  return __clzll((long long)(a ^ b));
}

// ConstructInternalNodes64Bits_Kernel with determine_range / find_split, one thread per internal
// node of the forest, on its segment's keys with local ids.
__global__ void k_internal(const unsigned long long* __restrict__ code_all, uint32_t n_internal,
                           float4* __restrict__ lo_all, int4* __restrict__ node_all, LbvhForest F) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_internal) return;
  const int4 r = forest_rec(F, forest_find(F, g, 3));
  const uint32_t idx = g - (uint32_t)r.w;
  const uint32_t n = (uint32_t)r.y;
  const unsigned long long* __restrict__ code = code_all + r.x;
  float4* __restrict__ lo = lo_all + r.z;
  int4* __restrict__ node = node_all + r.z;
  uint32_t first, last;
  if (idx == 0) {
    first = 0;
    last = n - 1;
  } else {
    const unsigned long long self = code[idx];
    const int L = cub64(self, code[idx - 1]);
    const int R = cub64(self, code[idx + 1]);
    const int d = (R > L) ? 1 : -1;
    const int dmin = min(L, R);
    int lmax = 2;
    int delta = -1;
    int it = (int)idx + d * lmax;
    if (0 <= it && it < (int)n) delta = cub64(self, code[it]);
    while (delta > dmin) {
      lmax <<= 1;
      it = (int)idx + d * lmax;
      delta = -1;
      if (0 <= it && it < (int)n) delta = cub64(self, code[it]);
    }
    int l = 0;
    for (int t = lmax >> 1; t > 0; t >>= 1) {
      it = (int)idx + (l + t) * d;
      delta = -1;
      if (0 <= it && it < (int)n) delta = cub64(self, code[it]);
      if (delta > dmin) l += t;
    }
    uint32_t j = (uint32_t)((int)idx + l * d);
    first = d < 0 ? j : idx;
    last = d < 0 ? idx : j;
  }
  uint32_t gamma;
  {
    const unsigned long long fc = code[first], lc = code[last];
    if (fc == lc) {
      gamma = (first + last) >> 1;
    } else {
      const int dn = cub64(fc, lc);
      int split = (int)first;
      int stride = (int)(last - first);
      do {
        stride = (stride + 1) >> 1;
        const int middle = split + stride;
        if (middle < (int)last && cub64(fc, code[middle]) > dn) split = middle;
      } while (stride > 1);
      gamma = (uint32_t)split;
    }
  }
  uint32_t left = gamma, right = gamma + 1;
  if (min(first, last) == gamma) left += n - 1;
  if (max(first, last) == gamma + 1) right += n - 1;
  node[idx].y = (int)left;
  node[idx].z = (int)right;
  node[idx].w = -1;
  node[left].x = (int)idx;
  node[right].x = (int)idx;
  if (idx == 0) node[0].x = -1;
  lo[idx].w = __int_as_float((int)left);
}

// Bottom-up merge from the leaf at sorted position i (forest-wide), within its segment.
__device__ __forceinline__ void merge_from_leaf(const LbvhForest& F, uint32_t i, float4* lo,
                                                float4* hi, const int4* node, uint32_t* flags,
                                                uint32_t* err) {
  const int4 r = forest_rec(F, forest_find(F, i, 0));
  const uint32_t n = (uint32_t)r.y;
  if (n < 2) return;
  lbvh_merge_upwards(n - 1 + (i - (uint32_t)r.x), n, lo + r.z, hi + r.z, node + r.z, flags + r.w,
                     err);
}

__global__ void k_build_internal_boxes(uint32_t n, float4* lo, float4* hi, const int4* node,
                                       uint32_t* flags, uint32_t* err, LbvhForest F) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  merge_from_leaf(F, i, lo, hi, node, flags, err);
}

// BuildInternal/ExternalEscapeIndexTable_Kernel, stored in hi.w and in the export tables (internal
// nodes at internal_base, leaves at prim_base of their segment), one thread per forest node.
__global__ void k_escape(uint32_t n_nodes, const int4* __restrict__ node_all,
                         float4* __restrict__ hi_all, int32_t* __restrict__ iesc,
                         int32_t* __restrict__ eesc, uint32_t* err, LbvhForest F) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_nodes) return;
  const int4 r = forest_rec(F, forest_find(F, g, 2));
  const uint32_t n = (uint32_t)r.y;
  const uint32_t k = g - (uint32_t)r.z;
  const int4* __restrict__ node = node_all + r.z;
  const int parent = node[k].x;
  int esc = -1;
  if (parent >= 0) {
    if ((int)k == node[parent].y) {
      esc = node[parent].z;
    } else {
      int cur = parent;
      uint32_t steps = 0;
      while (true) {
        if (++steps > n) {
          raise_error(err, kErrTreeWalk);
          break;
        }
        const int up = node[cur].x;
        if (up < 0) {
          esc = -1;
          break;
        }
        if (cur == node[up].z) {
          cur = up;
        } else {
          esc = node[up].z;
          break;
        }
      }
    }
  }
  hi_all[g].w = __int_as_float(esc);
  if (k + 1 < n) iesc[r.w + k] = esc;
  else eesc[r.x + k - (n - 1)] = esc;
}

__global__ void k_prims_mesh(const float4* __restrict__ x, const float4* __restrict__ nrm,
                             const int4* __restrict__ tri, uint32_t nf, float tol,
                             float4* __restrict__ v, float4* __restrict__ pred) {
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int4 t = tri[f];
  const int id[3] = {t.x, t.y, t.z};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    f3 q = mk3(x[id[k]]) + tol * mk3(nrm[id[k]]);
    v[3 * f + k] = mk4(q, 0.0f);
    pred[3 * f + k] = mk4(q, 0.0f);
  }
}

// UpdateObjects_Kernel with ccd = true (BVH.cu:382-418): v from x0, pred from x.
__global__ void k_prims_ccd(const float4* __restrict__ x, const float4* __restrict__ x0,
                            const float4* __restrict__ nrm, const int4* __restrict__ tri,
                            uint32_t nf, float tol, float4* __restrict__ v,
                            float4* __restrict__ pred) {
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int4 t = tri[f];
  const int id[3] = {t.x, t.y, t.z};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const f3 n = mk3(nrm[id[k]]);
    v[3 * f + k] = mk4(mk3(x0[id[k]]) + tol * n, 0.0f);
    pred[3 * f + k] = mk4(mk3(x[id[k]]) + tol * n, 0.0f);
  }
}

// Forest node of the leaf at sorted position i, and its global primitive (from the leaf's
// local object).
__device__ __forceinline__ uint32_t leaf_node_of(const LbvhForest& F, uint32_t i, uint32_t& base) {
  const int4 r = forest_rec(F, forest_find(F, i, 0));
  base = (uint32_t)r.x;
  return (uint32_t)r.z + (uint32_t)r.y - 1 + (i - (uint32_t)r.x);
}

// RefitExternalNodeMidstep_Kernel + AssignAABBCAS_Kernel, fused.
__global__ void k_refit_midstep(uint32_t n, const float4* __restrict__ x1,
                                const float4* __restrict__ n1, const int4* __restrict__ tri,
                                float tol, float4* pred, float4* lo, float4* hi, const int4* node,
                                uint32_t* flags, uint32_t* err, LbvhForest F) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t base;
  const uint32_t k = leaf_node_of(F, i, base);
  float4 l = lo[k], h = hi[k];
  const uint32_t obj = base + (uint32_t)__float_as_int(l.w);
  const int4 t = tri[obj];
  const int id[3] = {t.x, t.y, t.z};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const f3 q = mk3(x1[id[c]]) + tol * mk3(n1[id[c]]);
    pred[3 * obj + c] = mk4(q, 0.0f);
    l.x = tmin(l.x, q.x); l.y = tmin(l.y, q.y); l.z = tmin(l.z, q.z);
    h.x = tmax(h.x, q.x); h.y = tmax(h.y, q.y); h.z = tmax(h.z, q.z);
  }
  __stcg(&lo[k], l);
  __stcg(&hi[k], h);
  merge_from_leaf(F, i, lo, hi, node, flags, err);
}

// RefitExternalNode_Kernel(predicted) with per-primitive pred already in place.
__global__ void k_refit_pred(uint32_t n, const float4* __restrict__ pred, float4* lo, float4* hi,
                             const int4* node, uint32_t* flags, uint32_t* err, LbvhForest F) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t base;
  const uint32_t k = leaf_node_of(F, i, base);
  float4 l = lo[k], h = hi[k];
  const uint32_t obj = base + (uint32_t)__float_as_int(l.w);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const f3 q = mk3(pred[3 * obj + c]);
    l.x = tmin(l.x, q.x); l.y = tmin(l.y, q.y); l.z = tmin(l.z, q.z);
    h.x = tmax(h.x, q.x); h.y = tmax(h.y, q.y); h.z = tmax(h.z, q.z);
  }
  __stcg(&lo[k], l);
  __stcg(&hi[k], h);
  merge_from_leaf(F, i, lo, hi, node, flags, err);
}

}  // namespace

namespace {

template <int KIND>
__global__ void k_query(LbvhView b, const float* __restrict__ q, uint32_t nq,
                        uint32_t* __restrict__ counts, uint32_t* __restrict__ cands, uint32_t* err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  f3 a, c;
  if (KIND == 0) {
    a = mk3(q[3 * i], q[3 * i + 1], q[3 * i + 2]);
    c = a;
  } else {
    a = mk3(q[6 * i], q[6 * i + 1], q[6 * i + 2]);
    c = mk3(q[6 * i + 3], q[6 * i + 4], q[6 * i + 5]);
  }
  uint32_t* out = cands + (size_t)i * kMaxCandidates;
  uint32_t found = 0;
  auto visit = [&](uint32_t obj) { out[found++] = obj; };
  if (KIND == 0)
    lbvh_traverse(b, [&](float4 l, float4 h) { return overlap_point(l, h, a); }, visit, err);
  else if (KIND == 1)
    lbvh_traverse(b, [&](float4 l, float4 h) { return overlap_segment(l, h, a, c); }, visit, err);
  else
    lbvh_traverse(b, [&](float4 l, float4 h) { return overlap_box(l, h, a, c); }, visit, err);
  counts[i] = found;
}

__global__ void k_float9_to_float4(const float* __restrict__ in, float4* __restrict__ out,
                                   uint32_t n_points) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_points) return;
  out[i] = make_float4(in[3 * i], in[3 * i + 1], in[3 * i + 2], 0.0f);
}

}  // namespace

cudaError_t Lbvh::set_segments(const std::vector<uint32_t>& counts, cudaStream_t s) {
  h_seg.clear();
  if (counts.size() <= 1) return cudaSuccess;
  uint32_t pb = 0, nb = 0, ib = 0;
  for (uint32_t c : counts) {
    h_seg.push_back(make_int4((int)pb, (int)c, (int)nb, (int)ib));
    pb += c;
    nb += c ? 2 * c - 1 : 0;
    ib += c ? c - 1 : 0;
  }
  cudaError_t e = seg.reserve(h_seg.size());
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(seg.p, h_seg.data(), sizeof(int4) * h_seg.size(), cudaMemcpyHostToDevice, s);
  return e;
}

cudaError_t Lbvh::reserve(uint32_t np) {
  const size_t nn = np ? 2 * (size_t)np - 1 : 1;
  cudaError_t e = cudaSuccess;
  if (nseg() > 1) {
    if (e == cudaSuccess) e = skey.reserve(np);
    if (e == cudaSuccess) e = sval.reserve(np);
  }
  if (e == cudaSuccess) e = v.reserve(3 * (size_t)np);
  if (e == cudaSuccess) e = pred.reserve(3 * (size_t)np);
  if (e == cudaSuccess) e = leaf_lo.reserve(np);
  if (e == cudaSuccess) e = leaf_hi.reserve(np);
  if (e == cudaSuccess) e = lo.reserve(nn);
  if (e == cudaSuccess) e = hi.reserve(nn);
  if (e == cudaSuccess) e = node.reserve(nn);
  if (e == cudaSuccess) e = morton.reserve(np);
  if (e == cudaSuccess) e = index.reserve(np);
  if (e == cudaSuccess) e = key64.reserve(np);
  if (e == cudaSuccess) e = flags.reserve(np);
  if (e == cudaSuccess) e = iesc.reserve(np);
  if (e == cudaSuccess) e = eesc.reserve(np);
  if (e == cudaSuccess) e = root.reserve(6 * (size_t)nseg());
  if (e == cudaSuccess) e = dup.reserve(1);
  if (e == cudaSuccess) e = sorter.reserve(np);
  return e;
}

void Lbvh::construct(float scr, cudaStream_t s, uint32_t* d_err) {
  active = n > 0;
  if (n == 0) return;
  const LbvhForest F = forest();
  const uint32_t S = nseg();
  nodes = 0;
  internal = 0;
  if (S == 1) {
    nodes = 2 * n - 1;
    internal = n - 1;
  } else {
    for (const int4& r : h_seg) {
      nodes += r.y ? 2 * (uint32_t)r.y - 1 : 0;
      internal += r.y ? (uint32_t)r.y - 1 : 0;
    }
  }
  uint32_t* rootu = reinterpret_cast<uint32_t*>(root.p);
  k_root_init<<<grid_for(6 * S), kBlock, 0, s>>>(rootu, S, dup.p);
  k_leaf_boxes<<<grid_for(n), kBlock, 0, s>>>(v.p, pred.p, n, scr, leaf_lo.p, leaf_hi.p, rootu, F);
  k_morton<<<grid_for(n), kBlock, 0, s>>>(leaf_lo.p, leaf_hi.p, rootu, n, morton.p, index.p, F);
  // Morton codes have 30 bits: four 8-bit passes leave the result in (morton, index)
  sorter.sort(morton.p, index.p, n, 30, s, &sorted_morton, &sorted_index);
  if (S > 1) {
    int bits = 0;
    while ((1u << bits) < S) ++bits;
    k_seg_keys<<<grid_for(n), kBlock, 0, s>>>(sorted_index, n, skey.p, sval.p, F);
    uint32_t *k2 = nullptr, *perm = nullptr;
    sorter.sort(skey.p, sval.p, n, bits, s, &k2, &perm);
    // gather into whichever key / value pair the segment pass's result does not occupy
    const bool in_own = perm == sval.p;
    uint32_t* m_out = in_own ? sorter.keys_tmp.p : skey.p;
    uint32_t* i_out = in_own ? sorter.vals_tmp.p : sval.p;
    k_seg_gather<<<grid_for(n), kBlock, 0, s>>>(perm, sorted_morton, sorted_index, n, m_out, i_out);
    sorted_morton = m_out;
    sorted_index = i_out;
  }
  k_leaves<<<grid_for(n), kBlock, 0, s>>>(sorted_morton, sorted_index, leaf_lo.p, leaf_hi.p, n, lo.p,
                                          hi.p, node.p, key64.p, dup.p, F);
  if (internal > 0) {
    k_internal<<<grid_for(internal), kBlock, 0, s>>>(key64.p, internal, lo.p, node.p, F);
    cudaMemsetAsync(flags.p, 0, sizeof(uint32_t) * internal, s);
    k_build_internal_boxes<<<grid_for(n), kBlock, 0, s>>>(n, lo.p, hi.p, node.p, flags.p, d_err, F);
  }
  k_escape<<<grid_for(nodes), kBlock, 0, s>>>(nodes, node.p, hi.p, iesc.p, eesc.p, d_err, F);
}

void Lbvh::refit_from_pred(cudaStream_t s, uint32_t* d_err) {
  if (!active) return;
  k_refit_pred<<<grid_for(n), kBlock, 0, s>>>(n, pred.p, lo.p, hi.p, node.p, flags.p, d_err,
                                              forest());
}

void Lbvh::release() {
  v.release(); pred.release(); leaf_lo.release(); leaf_hi.release(); lo.release(); hi.release();
  node.release(); morton.release(); index.release(); key64.release(); flags.release();
  iesc.release(); eesc.release(); root.release(); dup.release(); skey.release(); sval.release();
  seg.release();
  sorter.keys_tmp.release(); sorter.vals_tmp.release(); sorter.hist.release(); sorter.sums.release();
}

void launch_prims_from_mesh(Lbvh& b, const float4* x, const float4* nrm, const int4* tri,
                            uint32_t nf, float tol, cudaStream_t s) {
  if (nf == 0) return;
  k_prims_mesh<<<grid_for(nf), kBlock, 0, s>>>(x, nrm, tri, nf, tol, b.v.p, b.pred.p);
}

void launch_prims_ccd(Lbvh& b, const float4* x, const float4* x0, const float4* nrm,
                      const int4* tri, uint32_t nf, float tol, cudaStream_t s) {
  if (nf == 0) return;
  k_prims_ccd<<<grid_for(nf), kBlock, 0, s>>>(x, x0, nrm, tri, nf, tol, b.v.p, b.pred.p);
}

void launch_refit_midstep(Lbvh& b, const float4* x1, const float4* n1, const int4* tri, float tol,
                          cudaStream_t s, uint32_t* d_err) {
  if (!b.active) return;
  k_refit_midstep<<<grid_for(b.n), kBlock, 0, s>>>(b.n, x1, n1, tri, tol, b.pred.p, b.lo.p, b.hi.p,
                                                   b.node.p, b.flags.p, d_err, b.forest());
}

void launch_lbvh_query(const Lbvh& b, int kind, const float* d_q, uint32_t nq, uint32_t* d_counts,
                       uint32_t* d_cands, cudaStream_t s, uint32_t* d_err) {
  if (nq == 0 || !b.active) return;
  if (kind == 0)
    k_query<0><<<grid_for(nq), kBlock, 0, s>>>(b.view(), d_q, nq, d_counts, d_cands, d_err);
  else if (kind == 1)
    k_query<1><<<grid_for(nq), kBlock, 0, s>>>(b.view(), d_q, nq, d_counts, d_cands, d_err);
  else
    k_query<2><<<grid_for(nq), kBlock, 0, s>>>(b.view(), d_q, nq, d_counts, d_cands, d_err);
}

void launch_float9_to_float4(const float* d_in, float4* d_out, uint32_t n_prims, cudaStream_t s) {
  if (n_prims == 0) return;
  k_float9_to_float4<<<grid_for(3 * n_prims), kBlock, 0, s>>>(d_in, d_out, 3 * n_prims);
}

}  // namespace xrt
