// project_dev.cuh — the constraint projections of the Swift substep, shared by the forward
// kernels (solver.cu) and the adjoint (diff.cu), which re-evaluates them from taped inputs.
//
//   stretch_project ... SolveStretch_Kernel (xrtailor/src/physics/dynamics/BasicSolverHelper.cu:80-132)
//   bend_project ...... SolveBend_Kernel (BasicSolverHelper.cu:8-72)
//   lra_project ....... SolveGeodesicLRA_Kernel (xrtailor/src/physics/dynamics/LongRangeAttachments.cu:5-26)
//   prim_normal ....... face normal of an obstacle primitive's predicted vertices
#pragma once
#include "common.cuh"
#include "context.h"

namespace xrt {

// One tile of a tile-local Gauss-Seidel launch (block = tile): its metadata and the footprint
// vertex ids of this thread (kFootPerThread per thread, NT threads).
struct TileFrame {
  int4 m;                          // first footprint entry, footprint size, first record, count
  uint32_t fi[kFootPerThread];     // footprint vertex ids of this thread
};

template <int NT>
__device__ __forceinline__ TileFrame tile_prologue(const uint32_t* __restrict__ foot,
                                                   const int4* __restrict__ meta,
                                                   const uint32_t* __restrict__ lofs, uint32_t t,
                                                   uint32_t num_local, uint32_t* so) {
  TileFrame f;
  f.m = __ldg(&meta[t]);
  for (uint32_t k = threadIdx.x; k <= num_local; k += NT)
    so[k] = __ldg(&lofs[(size_t)t * (num_local + 1) + k]);
#pragma unroll
  for (int r = 0; r < kFootPerThread; ++r) {
    const uint32_t k = threadIdx.x + (uint32_t)r * NT;
    f.fi[r] = k < (uint32_t)f.m.y ? __ldg(&foot[f.m.x + k]) : 0u;
  }
  return f;
}

// The gather also parks the ids in shared memory (slot k is written and later read by the same
// thread), so they need no registers through the local-color loop.
template <int NT>
__device__ __forceinline__ void tile_gather(const TileFrame& f, const float4* __restrict__ x,
                                            float4* sx, uint32_t* sf) {
#pragma unroll
  for (int r = 0; r < kFootPerThread; ++r) {
    const uint32_t k = threadIdx.x + (uint32_t)r * NT;
    if (k < (uint32_t)f.m.y) {
      sx[k] = x[f.fi[r]];
      sf[k] = f.fi[r];
    }
  }
}

template <int NT>
__device__ __forceinline__ void tile_scatter(uint32_t nfoot, float4* __restrict__ x,
                                             const float4* sx, const uint32_t* sf) {
#pragma unroll
  for (int r = 0; r < kFootPerThread; ++r) {
    const uint32_t k = threadIdx.x + (uint32_t)r * NT;
    if (k < nfoot) x[sf[k]] = sx[k];
  }
}

// XPBD distance constraint on two vertices, alpha_tilde = stretch_alpha(compliance, dt); returns
// true when it moved them (lam updated).
__device__ __forceinline__ bool stretch_project_alpha(float4& a, float4& b, float rest,
                                                      float alpha_tilde, float& lam) {
  const f3 diff = mk3(a) - mk3(b);
  const float distance = sqrtf(fdot(diff, diff));
  const float w1 = a.w, w2 = b.w;
  if (!(distance != rest && w1 + w2 > 0.0f)) return false;
  const f3 gradient = diff * (1.0f / (distance + kEps));
  const float constraint = distance - rest;
  const float dl = fmaf(-alpha_tilde, lam, -constraint) / (w1 + w2 + alpha_tilde);
  const f3 corr = dl * gradient;
  lam = lam + dl;
  a = mk4(fmad(corr, w1, mk3(a)), a.w);
  b = mk4(fmad(-corr, w2, mk3(b)), b.w);
  return true;
}

__device__ __forceinline__ bool stretch_project(float4& a, float4& b, float rest, float compliance,
                                                float dt, float& lam) {
  return stretch_project_alpha(a, b, rest, stretch_alpha(compliance, dt), lam);
}


// Dihedral bend projection of SolveBend_Kernel on four vertices, xpbd_bend =
// bend_alpha(compliance, dt).
__device__ __forceinline__ void bend_project_alpha(float4& a1, float4& a2, float4& a3, float4& a4,
                                                   float theta, float xpbd_bend) {
  const float w1 = a1.w, w2 = a2.w, w3 = a3.w, w4 = a4.w;
  const f3 p1 = mk3(a1);
  const f3 p2 = mk3(a2) - p1;
  const f3 p3 = mk3(a3) - p1;
  const f3 p4 = mk3(a4) - p1;
  const f3 c23 = fcross(p2, p3), c24 = fcross(p2, p4);
  const float l23 = sqrtf(fdot(c23, c23)), l24 = sqrtf(fdot(c24, c24));
  const f3 n1 = c23 * (1.0f / l23);  // normalize
  const f3 n2 = c24 * (1.0f / l24);
  const float d = tclamp(fdot(n1, n2), 0.0f, 1.0f);
  const float angle = acos_as(d);  // d in [0, 1] (or NaN, rejected below)
  if (angle < kEps || isnan(d)) return;
  const float r3 = 1.0f / (l23 + kEps);
  const float r4 = 1.0f / (l24 + kEps);
  // q3 = (p2 x n2 + (n1 x p2) d) / (|p2 x p3| + eps), q4 likewise, q2 = -(p3 x n2 + (n1 x p3) d)
  // / (|p2 x p3| + eps) - (p4 x n1 + (n2 x p4) d) / (|p2 x p4| + eps)
  const f3 q3 = fmad(fcross(n1, p2), d, fcross(p2, n2)) * r3;
  const f3 q4 = fmad(fcross(n2, p2), d, fcross(p2, n1)) * r4;
  const f3 q2 = -(fmad(fcross(n1, p3), d, fcross(p3, n2)) * r3) -
                fmad(fcross(n2, p4), d, fcross(p4, n1)) * r4;
  const f3 q1 = -q2 - q3 - q4;
  const float denom =
      xpbd_bend +
      fmaf(w4, fdot(q4, q4), fmaf(w3, fdot(q3, q3), fmaf(w2, fdot(q2, q2), w1 * fdot(q1, q1))));
  if (denom < kEps) return;
  const float lambda = sqrtf(fmaf(-d, d, 1.0f)) * (angle - theta) / denom;
  const float scaling = 1.0f;
  a1 = mk4(fmad(q1, scaling * w1 * lambda, mk3(a1)), w1);
  a2 = mk4(fmad(q2, scaling * w2 * lambda, mk3(a2)), w2);
  a3 = mk4(fmad(q3, scaling * w3 * lambda, mk3(a3)), w3);
  a4 = mk4(fmad(q4, scaling * w4 * lambda, mk3(a4)), w4);
}

__device__ __forceinline__ void bend_project(float4& a1, float4& a2, float4& a3, float4& a4,
                                             float theta, float compliance, float dt) {
  bend_project_alpha(a1, a2, a3, a4, theta, bend_alpha(compliance, dt));
}


// The same projection on a lane pair (lanes 2m, 2m+1 of a warp, `half` = lane & 1), for the
// shared-memory footprint of a tile: each lane evaluates one of the two independent halves of
// the expression (normal n1 and gradient q3 / normal n2, gradient q4 and the angle), the halves
// are exchanged by shuffles, and lane 0 writes vertices 1-2, lane 1 vertices 3-4.  Every value is
// produced by the same operations (fused ones included) as bend_project_alpha, so the result is
// identical.  All 32 lanes
// call it; `active` is false for lanes past the color's last element (they write nothing).
// With (nA, nB, rA) = (n1, n2, 1 / (|p2 x p3| + eps)) on lane 0 and (n2, n1, 1 / (|p2 x p4| +
// eps)) on lane 1, and pA = p3 / p4:
//   q3 (lane 0) and q4 (lane 1) are both (p2 x nB + (nA x p2) d) rA,
//   the two terms of q2 are -(pA x nB + (nA x pA) d) rA on lane 0 and +(...) rA on lane 1;
// (-X) r equals -(X r) bit for bit, so both lanes run one instruction stream.
__device__ __forceinline__ void bend_project_pair(float4* sx, int4 b, float theta, float xpbd_bend,
                                                  uint32_t half, bool active) {
  constexpr unsigned kAll = 0xffffffffu;
  const float4 a1 = sx[b.x], a2 = sx[b.y], a3 = sx[b.z], a4 = sx[b.w];
  const f3 p1 = mk3(a1);
  const f3 p2 = mk3(a2) - p1;
  const f3 p3 = mk3(a3) - p1;
  const f3 p4 = mk3(a4) - p1;
  const f3 pA = half ? p4 : p3;
  const f3 cA = fcross(p2, pA);
  const float lA = sqrtf(fdot(cA, cA));
  const f3 nA = cA * (1.0f / lA);  // normalize
  const float rA = 1.0f / (lA + kEps);
  const f3 nB = mk3(__shfl_xor_sync(kAll, nA.x, 1), __shfl_xor_sync(kAll, nA.y, 1),
                    __shfl_xor_sync(kAll, nA.z, 1));
  const f3 n1 = half ? nB : nA, n2 = half ? nA : nB;
  const float d = tclamp(fdot(n1, n2), 0.0f, 1.0f);
  const float angle = acos_as(d);
  const f3 qA = fmad(fcross(nA, p2), d, fcross(p2, nB)) * rA;  // q3 on lane 0, q4 on lane 1
  const f3 vA = fmad(fcross(nA, pA), d, fcross(pA, nB)) * rA;  // |terms| of q2
  const f3 qB = mk3(__shfl_xor_sync(kAll, qA.x, 1), __shfl_xor_sync(kAll, qA.y, 1),
                    __shfl_xor_sync(kAll, qA.z, 1));
  const f3 vB = mk3(__shfl_xor_sync(kAll, vA.x, 1), __shfl_xor_sync(kAll, vA.y, 1),
                    __shfl_xor_sync(kAll, vA.z, 1));
  const f3 q3 = half ? qB : qA, q4 = half ? qA : qB;
  const f3 v23 = half ? vB : vA, v24 = half ? vA : vB;
  const f3 q2 = -v23 - v24;
  const f3 q1 = -q2 - q3 - q4;
  const float w1 = a1.w, w2 = a2.w, w3 = a3.w, w4 = a4.w;
  const float denom =
      xpbd_bend +
      fmaf(w4, fdot(q4, q4), fmaf(w3, fdot(q3, q3), fmaf(w2, fdot(q2, q2), w1 * fdot(q1, q1))));
  if (!active || angle < kEps || isnan(d) || denom < kEps) return;
  const float lambda = sqrtf(fmaf(-d, d, 1.0f)) * (angle - theta) / denom;
  const float scaling = 1.0f;
  // lane 0 moves vertices 1 and 2, lane 1 vertices 3 and 4
  const float wa = half ? w3 : w1, wb = half ? w4 : w2;
  const f3 qa = half ? q3 : q1, qb = half ? q4 : q2;
  const float4 aa = half ? a3 : a1, ab = half ? a4 : a2;
  sx[half ? b.z : b.x] = mk4(fmad(qa, scaling * wa * lambda, mk3(aa)), wa);
  sx[half ? b.w : b.y] = mk4(fmad(qb, scaling * wb * lambda, mk3(ab)), wb);
}

// ---- FEM fabric (FEMHelper.cu) -------------------------------------------------------------
// The orthotropic elasticity tensor's non-zero entries (ComputeStrainCorrection's C, computed
// once on the host): c00 = Ex/d, c01 = Ex nu_yx/d, c10 = Ey nu_xy/d, c11 = Ey/d, c22 = Es with
// d = 1 - nu_xy nu_yx.
struct FemTensor {
  float c00, c01, c10, c11, c22;
};

// ComputeStrainCorrection + SolveStrain_Kernel (FEMHelper.cu:96-173, 175-207): inv holds the
// rest triangle's inverse material matrix in glm's column-major order (inv[0][0], inv[0][1],
// inv[1][0], inv[1][1]); the deformation gradient, Green strain, stress, first Piola stress and
// H = inv^T P area are the reference's products in its order.  Moves the vertices with w > eps;
// returns false when the gradient norm is too small.
__device__ __forceinline__ bool fem_strain_project(float4& a0, float4& a1, float4& a2, float area,
                                                   float4 inv, const FemTensor& C) {
  const f3 p13 = mk3(a0) - mk3(a2);
  const f3 p23 = mk3(a1) - mk3(a2);
  const float i00 = inv.x, i01 = inv.y, i10 = inv.z, i11 = inv.w;
  // F[c][r], c spatial, r material
  const float F00 = p13.x * i00 + p23.x * i10, F01 = p13.x * i01 + p23.x * i11;
  const float F10 = p13.y * i00 + p23.y * i10, F11 = p13.y * i01 + p23.y * i11;
  const float F20 = p13.z * i00 + p23.z * i10, F21 = p13.z * i01 + p23.z * i11;
  const float e00 = 0.5f * (F00 * F00 + F10 * F10 + F20 * F20 - 1.0f);
  const float e11 = 0.5f * (F01 * F01 + F11 * F11 + F21 * F21 - 1.0f);
  const float e01 = 0.5f * (F00 * F01 + F10 * F11 + F20 * F21);
  const float s00 = C.c00 * e00 + C.c01 * e11;
  const float s11 = C.c10 * e00 + C.c11 * e11;
  const float s01 = C.c22 * e01;
  // P = stress F: P[c][0] = s00 F[c][0] + s01 F[c][1], P[c][1] = s01 F[c][0] + s11 F[c][1]
  const float P00 = s00 * F00 + s01 * F01, P01 = s01 * F00 + s11 * F01;
  const float P10 = s00 * F10 + s01 * F11, P11 = s01 * F10 + s11 * F11;
  const float P20 = s00 * F20 + s01 * F21, P21 = s01 * F20 + s11 * F21;
  const float psi = 0.5f * (((e00 * s00 + e01 * s01) + e01 * s01) + e11 * s11);
  const float energy = area * psi;
  // H[c][0] = (i00 P[c][0] + i01 P[c][1]) area, H[c][1] = (i10 P[c][0] + i11 P[c][1]) area
  const f3 g0 = mk3((i00 * P00 + i01 * P01) * area, (i00 * P10 + i01 * P11) * area,
                    (i00 * P20 + i01 * P21) * area);
  const f3 g1 = mk3((i10 * P00 + i11 * P01) * area, (i10 * P10 + i11 * P11) * area,
                    (i10 * P20 + i11 * P21) * area);
  const f3 g2 = -g0 - g1;
  const float w0 = a0.w, w1 = a1.w, w2 = a2.w;
  float sum = w0 * dot(g0, g0);
  sum = sum + w1 * dot(g1, g1);
  sum = sum + w2 * dot(g2, g2);
  if (!(fabsf(sum) > kEps)) return false;
  const float s = energy / sum;
  if (w0 > kEps) a0 = mk4(mk3(a0) + (-(s * w0)) * g0, w0);
  if (w1 > kEps) a1 = mk4(mk3(a1) + (-(s * w1)) * g1, w1);
  if (w2 > kEps) a2 = mk4(mk3(a2) + (-(s * w2)) * g2, w2);
  return true;
}

// SolveIsometricBending_Kernel (FEMHelper.cu:325-388): energy 1/2 sum_k sum_j Q[j][k] x_k.x_j,
// derivatives d_j = sum_i Q[j][i] x_i, XPBD step with alpha = 1 / (stiffness dt^2) (passed in).
// Q is row-major (Q[4 j + k] = Q[j][k]).  Returns false (nothing moves, lam unchanged) when
// |energy| < eps.
__device__ __forceinline__ bool iso_bend_project(float4& a0, float4& a1, float4& a2, float4& a3,
                                                 const float* Q, float alpha, float& lam) {
  const f3 x[4] = {mk3(a0), mk3(a1), mk3(a2), mk3(a3)};
  float energy = 0.0f;
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int j = 0; j < 4; ++j) energy = energy + Q[4 * j + k] * dot(x[k], x[j]);
  energy = energy * 0.5f;
  if (fabsf(energy) < kEps) return false;
  f3 d[4] = {mk3(0, 0, 0), mk3(0, 0, 0), mk3(0, 0, 0), mk3(0, 0, 0)};
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) d[j] = d[j] + Q[4 * j + i] * x[i];
  const float w[4] = {a0.w, a1.w, a2.w, a3.w};
  const float coeff = (w[0] * dot(d[0], d[0]) + w[1] * dot(d[1], d[1])) +
                      (w[2] * dot(d[2], d[2]) + w[3] * dot(d[3], d[3]));
  const float dl = (-energy - alpha * lam) / (coeff + alpha);
  a0 = mk4(x[0] + (dl * w[0]) * d[0], w[0]);
  a1 = mk4(x[1] + (dl * w[1]) * d[1], w[1]);
  a2 = mk4(x[2] + (dl * w[2]) * d[2], w[2]);
  a3 = mk4(x[3] + (dl * w[3]) * d[3], w[3]);
  lam = lam + dl;
  return true;
}

__device__ __forceinline__ f3 lra_project(f3 xt, f3 xs, float w_t, float rest, float stretch) {
  const float target = rest * stretch;
  if (w_t < kEps && target > 0) return xt;
  const f3 diff = xt - xs;
  const float dist = length(diff);
  if (dist > target) xt = xt + (-diff + diff / dist * target);
  return xt;
}

__device__ __forceinline__ f3 prim_normal(const float4* __restrict__ pred, int f) {
  return face_normal(mk3(pred[3 * f]), mk3(pred[3 * f + 1]), mk3(pred[3 * f + 2]));
}

}  // namespace xrt
