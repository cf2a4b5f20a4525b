// solver.cu — integration and graph-colored XPBD projection of the Swift substep.
//
//   predict / finalize ..... PredictPositions_Kernel, Finalize_Kernel
//                            (xrtailor/src/physics/ClothSolverHelper.cu:125-137, 222-236)
//   stretch ................ SolveStretch_Kernel (xrtailor/src/physics/dynamics/BasicSolverHelper.cu:80-132)
//   bend ................... SolveBend_Kernel (BasicSolverHelper.cu:8-72)
//   long-range attachment .. SolveGeodesicLRA_Kernel (xrtailor/src/physics/dynamics/LongRangeAttachments.cu:5-26)
//   contact response ....... SolveVFCCD/SolveVFDCD/SolveEEDCD_Kernel (xrtailor/src/physics/pbd_collision/PBDCollision.cu),
//                            ApplyDeltas_Kernel (ClothSolverHelper.cu:139-148)
//   binding ................ SolveBinding_Kernel (xrtailor/src/physics/dynamics/BindingConstraint.cu:56-92)
//
// Layout: positions are float4 {x, y, z, inverse mass}; one 16-byte load gives a vertex and its
// weight.  Stretch and bend constraints are stored sorted by color, each color a contiguous
// range, so a color launch touches only its own constraints (the reference launches E threads per
// color and lets the other colors exit) and, because a color is an independent set, writes its
// vertices without atomics.  Contact deltas are gathered per vertex over its incident edges in
// ascending edge order, replacing float atomics with a fixed summation order.
#include "common.cuh"
#include "context.h"

namespace xrt {
namespace {

__global__ void k_predict(float4* __restrict__ x, const float4* __restrict__ x0,
                          float4* __restrict__ v, uint32_t nv, float dt, float gx, float gy,
                          float gz) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const float w = x[i].w;
  f3 vel = mk3(v[i]);
  if (w > kEps) vel = vel + mk3(gx, gy, gz) * dt;
  v[i] = mk4(vel, 0.0f);
  x[i] = mk4(mk3(x0[i]) + vel * dt, w);
}

// Finalize of substep s, optionally fused with PredictPositions of substep s+1 or with the
// frame-end vertex normals (UpdateNodeNormals, PhysicsMeshHelper.cu:196-210, 282-295).
template <bool PREDICT, bool NORMALS>
__global__ void k_finalize(float4* __restrict__ x, float4* __restrict__ x0, float4* __restrict__ v,
                           uint32_t nv, float dt, float damping, float gx, float gy, float gz,
                           const int4* __restrict__ tri, const uint32_t* __restrict__ vf_ptr,
                           const uint32_t* __restrict__ vf_list, float4* __restrict__ nrm) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const float4 p = x[i];
  const f3 np = mk3(p);
  const f3 raw = (np - mk3(x0[i])) / dt;
  f3 vel = raw * (1 - damping * dt);
  x0[i] = mk4(np, 0.0f);
  if (PREDICT) {
    if (p.w > kEps) vel = vel + mk3(gx, gy, gz) * dt;
    x[i] = mk4(np + vel * dt, p.w);
  }
  v[i] = mk4(vel, 0.0f);
  if (NORMALS) {
    f3 acc = mk3(0, 0, 0);
    for (uint32_t k = vf_ptr[i]; k < vf_ptr[i + 1]; ++k) {
      const uint32_t fc = vf_list[k];
      const int4 t = tri[fc >> 2];
      const int id[3] = {t.x, t.y, t.z};
      const int j = (int)(fc & 3u);
      const f3 e0 = mk3(x[id[(j + 1) % 3]]) - np;
      const f3 e1 = mk3(x[id[(j + 2) % 3]]) - np;
      const f3 c = cross(e0, e1) / (dot(e0, e0) * dot(e1, e1));
      acc = acc + c;
    }
    nrm[i] = mk4(normalize(acc), 0.0f);
  }
}

// XPBD distance constraint on two vertices; returns true when it moved them (lam updated).
__device__ __forceinline__ bool stretch_project(float4& a, float4& b, float rest, float compliance,
                                                float dt, float& lam) {
  const f3 diff = mk3(a) - mk3(b);
  const float distance = length(diff);
  const float w1 = a.w, w2 = b.w;
  if (!(distance != rest && w1 + w2 > 0.0f)) return false;
  const f3 gradient = diff / (distance + kEps);
  const float alpha_tilde = compliance / (dt * dt);
  const float constraint = distance - rest;
  const float dl = (-constraint - alpha_tilde * lam) / (w1 + w2 + alpha_tilde);
  const f3 corr = dl * gradient;
  lam = lam + dl;
  const f3 c1 = corr * w1;
  const f3 c2 = -corr * w2;
  a = make_float4(a.x + c1.x, a.y + c1.y, a.z + c1.z, a.w);
  b = make_float4(b.x + c2.x, b.y + c2.y, b.z + c2.z, b.w);
  return true;
}

template <bool RESET>
__global__ void k_stretch(const int4* __restrict__ con, float* __restrict__ lambda,
                          float4* __restrict__ x, uint32_t begin, uint32_t end, float dt) {
  const uint32_t j = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= end) return;
  const int4 c = __ldg(&con[j]);
  float lam = RESET ? 0.0f : lambda[j];
  float4 a = x[c.x], b = x[c.y];
  if (stretch_project(a, b, __int_as_float(c.z), __int_as_float(c.w), dt, lam)) {
    x[c.x] = a;
    x[c.y] = b;
    lambda[j] = lam;
  } else if (RESET) {
    lambda[j] = 0.0f;
  }
}

// Tile-local Gauss-Seidel: block = one tile of the launched tile color.  The tile's footprint is
// staged in shared memory, its local colors run in order with a block barrier between them, and
// the footprint is written back.  Tiles of one tile color have disjoint footprints.
// Shared memory of a tile launch: footprint positions, then the tile's constraint records (and,
// for stretch, the multipliers).  Everything global is read once, up front, in coalesced sweeps,
// so the chain of local colors touches only shared memory.
template <bool RESET>
__global__ void __launch_bounds__(kBlock) k_stretch_tiles(
    const int4* __restrict__ con, float* __restrict__ lambda, float4* __restrict__ x,
    const uint32_t* __restrict__ foot, const uint32_t* __restrict__ foot_ptr,
    const uint32_t* __restrict__ lc_ptr, uint32_t tile_begin, uint32_t num_local,
    uint32_t max_foot, uint32_t max_cons, float dt) {
  extern __shared__ float4 smem[];
  float4* sx = smem;
  int4* sc = reinterpret_cast<int4*>(sx + max_foot);
  float* sl = reinterpret_cast<float*>(sc + max_cons);
  const uint32_t t = tile_begin + blockIdx.x;
  const uint32_t fb = foot_ptr[t], fe = foot_ptr[t + 1];
  const uint32_t* lp = lc_ptr + (size_t)t * num_local;
  const uint32_t c0 = lp[0], c1 = lp[num_local];
  for (uint32_t k = fb + threadIdx.x; k < fe; k += blockDim.x) sx[k - fb] = x[foot[k]];
  for (uint32_t j = c0 + threadIdx.x; j < c1; j += blockDim.x) {
    sc[j - c0] = __ldg(&con[j]);
    sl[j - c0] = RESET ? 0.0f : lambda[j];
  }
  __syncthreads();
  for (uint32_t l = 0; l < num_local; ++l) {
    const uint32_t cb = lp[l] - c0, ce = lp[l + 1] - c0;
    for (uint32_t j = cb + threadIdx.x; j < ce; j += blockDim.x) {
      const int4 c = sc[j];
      float lam = sl[j];
      float4 a = sx[c.x], b = sx[c.y];
      if (stretch_project(a, b, __int_as_float(c.z), __int_as_float(c.w), dt, lam)) {
        sx[c.x] = a;
        sx[c.y] = b;
        sl[j] = lam;
      }
    }
    __syncthreads();
  }
  for (uint32_t k = fb + threadIdx.x; k < fe; k += blockDim.x) x[foot[k]] = sx[k - fb];
  for (uint32_t j = c0 + threadIdx.x; j < c1; j += blockDim.x) lambda[j] = sl[j - c0];
}

// Dihedral bend projection of SolveBend_Kernel on four vertices.
__device__ __forceinline__ void bend_project(float4& a1, float4& a2, float4& a3, float4& a4,
                                             float theta, float compliance, float dt);

__global__ void k_bend(const int4* __restrict__ idx, const float2* __restrict__ tc,
                       float4* __restrict__ x, uint32_t begin, uint32_t end, float dt) {
  const uint32_t j = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= end) return;
  const int4 b = __ldg(&idx[j]);
  const float2 th = __ldg(&tc[j]);
  float4 a1 = x[b.x], a2 = x[b.y], a3 = x[b.z], a4 = x[b.w];
  bend_project(a1, a2, a3, a4, th.x, th.y, dt);
  x[b.x] = a1;  // unchanged values when the constraint is inactive; a color is independent
  x[b.y] = a2;
  x[b.z] = a3;
  x[b.w] = a4;
}

__global__ void __launch_bounds__(kBlock) k_bend_tiles(
    const int4* __restrict__ idx, const float2* __restrict__ tc, float4* __restrict__ x,
    const uint32_t* __restrict__ foot, const uint32_t* __restrict__ foot_ptr,
    const uint32_t* __restrict__ lc_ptr, uint32_t tile_begin, uint32_t num_local,
    uint32_t max_foot, uint32_t max_cons, float dt) {
  extern __shared__ float4 smem[];
  float4* sx = smem;
  int4* sc = reinterpret_cast<int4*>(sx + max_foot);
  float2* st = reinterpret_cast<float2*>(sc + max_cons);
  const uint32_t t = tile_begin + blockIdx.x;
  const uint32_t fb = foot_ptr[t], fe = foot_ptr[t + 1];
  const uint32_t* lp = lc_ptr + (size_t)t * num_local;
  const uint32_t c0 = lp[0], c1 = lp[num_local];
  for (uint32_t k = fb + threadIdx.x; k < fe; k += blockDim.x) sx[k - fb] = x[foot[k]];
  for (uint32_t j = c0 + threadIdx.x; j < c1; j += blockDim.x) {
    sc[j - c0] = __ldg(&idx[j]);
    st[j - c0] = __ldg(&tc[j]);
  }
  __syncthreads();
  for (uint32_t l = 0; l < num_local; ++l) {
    const uint32_t cb = lp[l] - c0, ce = lp[l + 1] - c0;
    for (uint32_t j = cb + threadIdx.x; j < ce; j += blockDim.x) {
      const int4 b = sc[j];
      const float2 th = st[j];
      float4 a1 = sx[b.x], a2 = sx[b.y], a3 = sx[b.z], a4 = sx[b.w];
      bend_project(a1, a2, a3, a4, th.x, th.y, dt);
      sx[b.x] = a1;
      sx[b.y] = a2;
      sx[b.z] = a3;
      sx[b.w] = a4;
    }
    __syncthreads();
  }
  for (uint32_t k = fb + threadIdx.x; k < fe; k += blockDim.x) x[foot[k]] = sx[k - fb];
}

__device__ __forceinline__ void bend_project(float4& a1, float4& a2, float4& a3, float4& a4,
                                             float theta, float compliance, float dt) {
  const float w1 = a1.w, w2 = a2.w, w3 = a3.w, w4 = a4.w;
  const f3 p1 = mk3(a1);
  const f3 p2 = mk3(a2) - p1;
  const f3 p3 = mk3(a3) - p1;
  const f3 p4 = mk3(a4) - p1;
  const f3 n1 = normalize(cross(p2, p3));
  const f3 n2 = normalize(cross(p2, p4));
  const float d = tclamp(dot(n1, n2), 0.0f, 1.0f);
  const float angle = acos_as(d);  // d in [0, 1] (or NaN, rejected below)
  if (angle < kEps || isnan(d)) return;
  const f3 q3 = (cross(p2, n2) + cross(n1, p2) * d) / (length(cross(p2, p3)) + kEps);
  const f3 q4 = (cross(p2, n1) + cross(n2, p2) * d) / (length(cross(p2, p4)) + kEps);
  const f3 q2 = -(cross(p3, n2) + cross(n1, p3) * d) / (length(cross(p2, p3)) + kEps) -
                (cross(p4, n1) + cross(n2, p4) * d) / (length(cross(p2, p4)) + kEps);
  const f3 q1 = -q2 - q3 - q4;
  const float xpbd_bend = compliance / dt / dt;
  const float denom =
      xpbd_bend + (w1 * dot(q1, q1) + w2 * dot(q2, q2) + w3 * dot(q3, q3) + w4 * dot(q4, q4));
  if (denom < kEps) return;
  const float lambda = sqrtf(1.0f - d * d) * (angle - theta) / denom;
  const float scaling = 1.0f;
  const f3 c1 = scaling * w1 * lambda * q1;
  const f3 c2 = scaling * w2 * lambda * q2;
  const f3 c3 = scaling * w3 * lambda * q3;
  const f3 c4 = scaling * w4 * lambda * q4;
  a1 = make_float4(a1.x + c1.x, a1.y + c1.y, a1.z + c1.z, w1);
  a2 = make_float4(a2.x + c2.x, a2.y + c2.y, a2.z + c2.z, w2);
  a3 = make_float4(a3.x + c3.x, a3.y + c3.y, a3.z + c3.z, w3);
  a4 = make_float4(a4.x + c4.x, a4.y + c4.y, a4.z + c4.z, w4);
}

__device__ __forceinline__ f3 lra_project(f3 xt, f3 xs, float w_t, float rest, float stretch) {
  const float target = rest * stretch;
  if (w_t < kEps && target > 0) return xt;
  const f3 diff = xt - xs;
  const float dist = length(diff);
  if (dist > target) xt = xt + (-diff + diff / dist * target);
  return xt;
}

// All slots pinned: per target vertex, its slots in list order (slot sources never move here).
__global__ void k_lra_by_target(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ src,
                                const float* __restrict__ rest, float4* __restrict__ x, uint32_t nv,
                                float stretch) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nv) return;
  const uint32_t b = ptr[t], e = ptr[t + 1];
  if (b == e) return;
  const float4 p = x[t];
  f3 xt = mk3(p);
  for (uint32_t k = b; k < e; ++k) xt = lra_project(xt, mk3(x[src[k]]), p.w, rest[k], stretch);
  if (xt.x != p.x || xt.y != p.y || xt.z != p.z) x[t] = mk4(xt, p.w);
}

// Free slot vertices: one launch per slot over that slot's constraint block (list order).
__global__ void k_lra_block(const uint32_t* __restrict__ tgt, const uint32_t* __restrict__ src,
                            const float* __restrict__ rest, float4* __restrict__ x, uint32_t begin,
                            uint32_t end, float stretch) {
  const uint32_t k = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= end) return;
  const uint32_t t = tgt[k];
  const float4 p = x[t];
  const f3 xt = lra_project(mk3(p), mk3(x[src[k]]), p.w, rest[k], stretch);
  if (xt.x != p.x || xt.y != p.y || xt.z != p.z) x[t] = mk4(xt, p.w);
}

__device__ __forceinline__ f3 prim_normal(const float4* __restrict__ pred, int f) {
  return face_normal(mk3(pred[3 * f]), mk3(pred[3 * f + 1]), mk3(pred[3 * f + 2]));
}

// SolveVFCCD_Kernel then SolveVFDCD_Kernel for one vertex.
__global__ void k_vf_solve(float4* __restrict__ x, const int* __restrict__ rt_idx,
                           const float4* __restrict__ rt_qc, const int* __restrict__ vf_idx,
                           const float4* __restrict__ vf_qs, const float4* __restrict__ pred,
                           uint32_t nv) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const int rc = rt_idx[i], vc = vf_idx[i];
  if (rc == -1 && vc == -1) return;
  float4 p = x[i];
  f3 q = mk3(p);
  if (rc != -1) {
    const f3 nc = prim_normal(pred, rc);
    const float lambda = dot(nc, q - mk3(rt_qc[i]));
    if (lambda < 0) q = q + (-lambda * nc);
  }
  if (vc != -1) {
    const f3 ns = prim_normal(pred, vc);
    const float lambda = dot(ns, q - mk3(vf_qs[i])) - 1e-3f;
    if (lambda < 0) q = q + (-lambda * ns);
  }
  x[i] = mk4(q, p.w);
}

// SolveEEDCD_Kernel + ApplyDeltas_Kernel + SolveBinding_Kernel per vertex (Jacobi: reads x_in,
// writes x_out).
template <bool CONTACTS, bool BINDINGS>
__global__ void k_ee_apply(const float4* __restrict__ x_in, float4* __restrict__ x_out, uint32_t nv,
                           const uint32_t* __restrict__ ve_ptr, const uint32_t* __restrict__ ve_list,
                           const uint2* __restrict__ edge, const float4* __restrict__ ee_a,
                           const float4* __restrict__ ee_b, const float4* __restrict__ ee_c,
                           float relaxation, const uint32_t* __restrict__ bind_ptr,
                           const float4* __restrict__ bind_a, const int4* __restrict__ bind_b,
                           const float4* __restrict__ ox) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const float4 p = x_in[i];
  f3 q = mk3(p);
  if (CONTACTS) {
    f3 delta = mk3(0, 0, 0);
    int count = 0;
    for (uint32_t k = ve_ptr[i]; k < ve_ptr[i + 1]; ++k) {
      const uint32_t code = ve_list[k];
      const uint32_t e = code >> 1;
      const float4 ca = ee_a[e];
      if (ca.x > 1e6f) continue;
      const float4 cb = ee_b[e], cc = ee_c[e];
      const uint2 ed = edge[e];
      const f3 p1 = mk3(x_in[ed.x]), q1 = mk3(x_in[ed.y]);
      const float s = cb.w, t = cc.w;
      const f3 fn = mk3(cc);
      const f3 c1 = (1 - s) * p1 + s * q1;
      const f3 c2 = (1 - t) * mk3(ca.y, ca.z, ca.w) + t * mk3(cb);
      const f3 d = c1 - c2;
      const float len = length(d);
      if (len < kEps) continue;
      const float lambda = dot(d, fn) - 1e-3f;
      if (lambda > 0) continue;
      const f3 corr = (code & 1u) ? (-(s)*lambda * fn) : (-(1 - s) * lambda * fn);
      delta = delta + corr;
      ++count;
    }
    const float fc = (float)count;
    if (fc > 0.0f) q = q + delta / fc * relaxation;
  }
  if (BINDINGS && p.w >= kEps) {
    for (uint32_t k = bind_ptr[i]; k < bind_ptr[i + 1]; ++k) {
      const float4 ba = bind_a[k];
      const int4 bb = bind_b[k];
      const f3 pob = ba.x * mk3(ox[bb.x]) + ba.y * mk3(ox[bb.y]) + ba.z * mk3(ox[bb.z]);
      const float C = length(q - pob) - ba.w;
      const f3 nn = normalize(q - pob);
      float s = p.w;
      s = C / s;
      if (C < 0.0f) continue;
      s *= __int_as_float(bb.w);
      q = q + (-s * p.w * nn);
    }
  }
  x_out[i] = mk4(q, p.w);
}

}  // namespace

void launch_predict(Context& c, const FrameConst& k) {
  k_predict<<<grid_for(c.nv), kBlock, 0, c.stream>>>(c.x.p, c.x0.p, c.v.p, c.nv, k.dt, k.gx, k.gy,
                                                     k.gz);
}

void launch_finalize_predict(Context& c, const FrameConst& k, bool predict_next, bool normals) {
  const unsigned g = grid_for(c.nv);
  if (predict_next)
    k_finalize<true, false><<<g, kBlock, 0, c.stream>>>(c.x.p, c.x0.p, c.v.p, c.nv, k.dt, k.damping,
                                                        k.gx, k.gy, k.gz, c.tri.p, c.vf_ptr.p,
                                                        c.vf_list.p, c.n.p);
  else if (normals)
    k_finalize<false, true><<<g, kBlock, 0, c.stream>>>(c.x.p, c.x0.p, c.v.p, c.nv, k.dt, k.damping,
                                                        k.gx, k.gy, k.gz, c.tri.p, c.vf_ptr.p,
                                                        c.vf_list.p, c.n.p);
  else
    k_finalize<false, false><<<g, kBlock, 0, c.stream>>>(c.x.p, c.x0.p, c.v.p, c.nv, k.dt,
                                                         k.damping, k.gx, k.gy, k.gz, c.tri.p,
                                                         c.vf_ptr.p, c.vf_list.p, c.n.p);
}

void launch_stretch(Context& c, const FrameConst& k, ColorRange r, bool reset_lambda) {
  const uint32_t n = r.end - r.begin;
  if (n == 0) return;
  if (reset_lambda)
    k_stretch<true><<<grid_for(n), kBlock, 0, c.stream>>>(c.s_con.p, c.s_lambda.p, c.x.p, r.begin,
                                                          r.end, k.dt);
  else
    k_stretch<false><<<grid_for(n), kBlock, 0, c.stream>>>(c.s_con.p, c.s_lambda.p, c.x.p, r.begin,
                                                           r.end, k.dt);
}

void launch_bend(Context& c, const FrameConst& k, ColorRange r) {
  const uint32_t n = r.end - r.begin;
  if (n == 0) return;
  k_bend<<<grid_for(n), kBlock, 0, c.stream>>>(c.b_idx.p, c.b_tc.p, c.x.p, r.begin, r.end, k.dt);
}

cudaError_t configure_tile_kernels(size_t max_smem_bytes) {
  const int bytes = (int)max_smem_bytes;
  cudaError_t e = cudaFuncSetAttribute(k_stretch_tiles<true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_stretch_tiles<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_bend_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  return e;
}

size_t tile_smem_bytes(const TiledSet& T, size_t record_bytes) {
  return sizeof(float4) * T.max_foot + record_bytes * T.max_cons;
}

void launch_stretch_tiles(Context& c, const FrameConst& k, ColorRange tiles, bool reset_lambda) {
  const uint32_t nt = tiles.end - tiles.begin;
  if (nt == 0) return;
  const TiledSet& T = c.s_tiles;
  const size_t smem = tile_smem_bytes(T, sizeof(int4) + sizeof(float));
  if (reset_lambda)
    k_stretch_tiles<true><<<nt, kBlock, smem, c.stream>>>(c.s_con.p, c.s_lambda.p, c.x.p, T.foot.p,
                                                          T.foot_ptr.p, T.lc_ptr.p, tiles.begin,
                                                          T.num_local, T.max_foot, T.max_cons,
                                                          k.dt);
  else
    k_stretch_tiles<false><<<nt, kBlock, smem, c.stream>>>(
        c.s_con.p, c.s_lambda.p, c.x.p, T.foot.p, T.foot_ptr.p, T.lc_ptr.p, tiles.begin,
        T.num_local, T.max_foot, T.max_cons, k.dt);
}

void launch_bend_tiles(Context& c, const FrameConst& k, ColorRange tiles) {
  const uint32_t nt = tiles.end - tiles.begin;
  if (nt == 0) return;
  const TiledSet& T = c.b_tiles;
  k_bend_tiles<<<nt, kBlock, tile_smem_bytes(T, sizeof(int4) + sizeof(float2)), c.stream>>>(
      c.b_idx.p, c.b_tc.p, c.x.p, T.foot.p, T.foot_ptr.p, T.lc_ptr.p, tiles.begin, T.num_local,
      T.max_foot, T.max_cons, k.dt);
}

// LRA phase: one per-target launch when every slot vertex is pinned (slot positions are then
// constant during the phase), else one launch per slot block in list order.
void launch_lra(Context& c, const FrameConst& k) {
  if (c.nl == 0) return;
  if (c.lra_by_target) {
    k_lra_by_target<<<grid_for(c.nv), kBlock, 0, c.stream>>>(c.lra_ptr.p, c.lra_src.p,
                                                             c.lra_rest.p, c.x.p, c.nv,
                                                             k.lra_stretch);
  } else {
    for (const ColorRange& r : c.lra_blocks)
      k_lra_block<<<grid_for(r.end - r.begin), kBlock, 0, c.stream>>>(
          c.lra_l_tgt.p, c.lra_l_src.p, c.lra_l_rest.p, c.x.p, r.begin, r.end, k.lra_stretch);
  }
}

void launch_vf_solve(Context& c) {
  k_vf_solve<<<grid_for(c.nv), kBlock, 0, c.stream>>>(c.x.p, c.rt_idx.p, c.rt_qc.p, c.vf_idx.p,
                                                      c.vf_qs.p, c.bvh.pred.p, c.nv);
}

void launch_ee_apply(Context& c, const FrameConst& k, bool contacts, bool bindings) {
  const unsigned g = grid_for(c.nv);
  auto args = [&](auto kern) {
    kern<<<g, kBlock, 0, c.stream>>>(c.x.p, c.x_alt.p, c.nv, c.ve_ptr.p, c.ve_list.p, c.edge.p,
                                     c.ee_a.p, c.ee_b.p, c.ee_c.p, k.relaxation, c.bind_ptr.p,
                                     c.bind_a.p, c.bind_b.p, c.ox.p);
  };
  if (contacts && bindings) args(k_ee_apply<true, true>);
  else if (contacts) args(k_ee_apply<true, false>);
  else if (bindings) args(k_ee_apply<false, true>);
}

}  // namespace xrt
