// diff.cu — hand-written adjoint (reverse mode) of the Swift frame, with per-frame checkpoints.
//
// Differentiated: predict, XPBD stretch with its multipliers (BasicSolverHelper.cu:80-132), the
// dihedral bend (BasicSolverHelper.cu:8-72, through the shared arccos polynomial), geodesic LRA
// with pinned slots (LongRangeAttachments.cu:5-26), the VF-CCD / VF-DCD and EE-DCD obstacle
// responses (PBDCollision.cu:57-80, 163-212, 279-298; ApplyDeltas ClothSolverHelper.cu:139-148)
// with the contact set held as recorded in the forward pass, and finalize
// (ClothSolverHelper.cu:222-236).  Gradients: per-edge stretch compliance, per-bend compliance,
// per-vertex inverse mass (reported as mass), initial velocity and initial position.
//
// Checkpoint / replay: xrt_diff_begin records the state at the start of every following frame
// (cloth x, x0, v and the obstacle's x0, targets and normals).  The reverse pass restores each
// frame's checkpoint, newest first, and replays the frame once with taping kernels: the same
// colors in the same order as the forward, one launch per color (tiles of one tile color have
// disjoint footprints, so a tile color's local colors run as whole colors), which gives the
// forward's bits.  The tape of that one frame holds every projection's inputs, the inputs of the
// per-vertex LRA+VF and EE launches and every collision pass's contacts and obstacle
// primitives.  Memory is the checkpoints plus one frame of tape, whatever the rollout
// length.
//
// Reverse order per substep: finalize, then iterations last to first (EE, LRA+VF, bend colors in
// reverse, stretch colors in reverse), then predict.  Within a color the constraints are
// independent, so each backward launch updates the adjoints of its vertices without atomics; the
// inverse-mass adjoint rides in the w lane of the position adjoint.
#include <algorithm>
#include <map>
#include <mutex>
#include <utility>

#include "common.cuh"
#include "context.h"
#include "lbvh_dev.cuh"
#include "project_dev.cuh"

namespace xrt {
namespace {

// ---- taping forward ------------------------------------------------------------------------

template <bool RESET>
__global__ void k_stretch_tape(const uint32_t* __restrict__ order, uint32_t begin, uint32_t end,
                               const int2* __restrict__ gidx, const int4* __restrict__ con,
                               float* __restrict__ lambda, float4* __restrict__ x,
                               float4* __restrict__ tx, float* __restrict__ tl, float dt) {
  pdl_release();
  pdl_wait();
  const uint32_t k = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= end) return;
  const uint32_t j = order[k];
  const int2 g = gidx[j];
  const int4 c = con[j];
  float lam = RESET ? 0.0f : lambda[j];
  float4 a = x[g.x], b = x[g.y];
  tx[2 * (size_t)j] = a;
  tx[2 * (size_t)j + 1] = b;
  tl[j] = lam;
  if (stretch_project(a, b, __int_as_float(c.z), __int_as_float(c.w), dt, lam)) {
    x[g.x] = a;
    x[g.y] = b;
    lambda[j] = lam;
  } else if (RESET) {
    lambda[j] = 0.0f;
  }
}

__global__ void k_bend_tape(const uint32_t* __restrict__ order, uint32_t begin, uint32_t end,
                            const int4* __restrict__ gidx, const float2* __restrict__ tc,
                            float4* __restrict__ x, float4* __restrict__ tx, float dt) {
  pdl_release();
  pdl_wait();
  const uint32_t k = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= end) return;
  const uint32_t j = order[k];
  const int4 b = gidx[j];
  const float2 th = tc[j];
  float4 a1 = x[b.x], a2 = x[b.y], a3 = x[b.z], a4 = x[b.w];
  float4* t = tx + 4 * (size_t)j;
  t[0] = a1;
  t[1] = a2;
  t[2] = a3;
  t[3] = a4;
  bend_project(a1, a2, a3, a4, th.x, th.y, dt);
  x[b.x] = a1;
  x[b.y] = a2;
  x[b.z] = a3;
  x[b.w] = a4;
}

// ---- adjoints of the projections -----------------------------------------------------------
// Notation: for c = a x b with adjoint cb, the adjoints are a += b x cb, b += cb x a.

__device__ __forceinline__ void cross_bwd(f3 a, f3 b, f3 cb, f3& ab, f3& bb) {
  ab = ab + cross(b, cb);
  bb = bb + cross(cb, a);
}

// The reverse's own arithmetic is not replayed, so it need not match the forward's IEEE-rounded
// divisions and square roots bit for bit: reciprocals come from the hardware approximation
// (__fdividef, rsqrtf; a few ulp), which shortens each VJP's dependency chain.  Every value that
// decides whether a projection ran (distance, normals, clamped cosine, angle) is recomputed
// exactly as the forward computes it.
__device__ __forceinline__ float frcp(float x) { return __fdividef(1.0f, x); }

// XPBD distance (stretch_project): inputs (a, b, lambda), outputs (a', b', lambda').  ga, gb hold
// the outputs' adjoints on entry (xyz; w accumulates the inverse-mass adjoint) and the inputs'
// on exit; lbo is lambda'-bar.  Returns false for an inactive projection (the identity: nothing
// changes, lambda-bar = lbo); else sets lam_in_bar and adds the compliance adjoint to cbar.
__device__ __forceinline__ bool stretch_vjp(float4 A, float4 B, float lam, float rest, float comp,
                                            float dt, float lbo, float4& ga, float4& gb,
                                            float& lam_in_bar, float& cbar) {
  const f3 d = mk3(A) - mk3(B);
  const float dist = sqrtf(fdot(d, d));  // as the forward: it decides whether the projection ran
  const float wa = A.w, wb = B.w;
  if (!(dist != rest && wa + wb > 0.0f)) return false;
  const float re = frcp(dist + kEps);
  const f3 n = d * re;
  const float idt2 = frcp(dt * dt);
  const float at = comp * idt2;
  const float C = dist - rest;
  const float rD = frcp(wa + wb + at);
  const float dl = (-C - at * lam) * rD;
  const f3 corr = dl * n;
  // x_a' = x_a + w_a corr, x_b' = x_b - w_b corr, lambda' = lambda + dl
  const f3 corr_bar = wa * mk3(ga) - wb * mk3(gb);
  float wa_bar = dot(corr, mk3(ga));
  float wb_bar = -dot(corr, mk3(gb));
  const float dl_bar = dot(corr_bar, n) + lbo;
  const f3 n_bar = dl * corr_bar;
  const float N_bar = dl_bar * rD;       // dl = N / D
  const float D_bar = -dl_bar * dl * rD;
  const float C_bar = -N_bar;            // N = -C - at lambda
  const float at_bar = -N_bar * lam + D_bar;
  lam_in_bar = lbo - N_bar * at;
  wa_bar += D_bar;
  wb_bar += D_bar;
  const float dist_bar = C_bar - dot(n_bar, n) * re;  // n = d / (dist + eps)
  const f3 d_bar = n_bar * re + (dist > 0.0f ? (dist_bar * frcp(dist)) * d : mk3(0, 0, 0));
  ga = mk4(mk3(ga) + d_bar, ga.w + wa_bar);
  gb = mk4(mk3(gb) - d_bar, gb.w + wb_bar);
  cbar += at_bar * idt2;
  return true;
}

// Per color: G holds x-bar and the inverse-mass bar; lam_bar holds lambda'-bar on entry,
// lambda-bar on exit (0 when RESET: the iteration started from lambda = 0).
template <bool RESET>
__global__ void k_stretch_bwd(const uint32_t* __restrict__ order, uint32_t begin, uint32_t end,
                              const int2* __restrict__ gidx, const int4* __restrict__ con,
                              const float4* __restrict__ tx, const float* __restrict__ tl,
                              float4* __restrict__ G, float* __restrict__ lam_bar,
                              float* __restrict__ comp_bar, float dt) {
  pdl_release();
  pdl_wait();
  const uint32_t k = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= end) return;
  const uint32_t j = order[k];
  const int2 g = gidx[j];
  const int4 c = con[j];
  const float lbo = lam_bar[j];
  float4 ga = G[g.x], gb = G[g.y];
  float lin = lbo, cb = 0.0f;
  if (stretch_vjp(tx[2 * (size_t)j], tx[2 * (size_t)j + 1], tl[j], __int_as_float(c.z),
                  __int_as_float(c.w), dt, lbo, ga, gb, lin, cb)) {
    G[g.x] = ga;
    G[g.y] = gb;
    comp_bar[j] += cb;
  }
  lam_bar[j] = RESET ? 0.0f : lin;
}

// d/dx of acos_as (the polynomial of common.cuh): sqrt(1-x) P'(x) - P(x) / (2 sqrt(1-x)).
__device__ __forceinline__ float acos_as_deriv(float x) {
  const float c[8] = {-0.0012624911f, 0.0066700901f, -0.0170881256f, 0.0308918810f,
                      -0.0501743046f, 0.0889789874f, -0.2145988016f, 1.5707963050f};
  float p = c[0], dp = 0.0f;
#pragma unroll
  for (int i = 1; i < 8; ++i) {
    dp = dp * x + p;
    p = p * x + c[i];
  }
  const float rs = rsqrtf(1.0f - x);  // x < 1 wherever the projection ran
  return (1.0f - x) * rs * dp - 0.5f * p * rs;
}

// Dihedral bend: inputs x1..x4 (w in .w), outputs x_i' = x_i + w_i lambda q_i.
// G1..G4 hold the outputs' adjoints on entry and the inputs' on exit; returns false for an
// inactive projection (the identity), else adds the compliance adjoint to cbar.
__device__ __forceinline__ bool bend_vjp(float4 A1, float4 A2, float4 A3, float4 A4, float theta,
                                         float comp, float dt, float4& G1, float4& G2, float4& G3,
                                         float4& G4, float& cbar) {
  const float w1 = A1.w, w2 = A2.w, w3 = A3.w, w4 = A4.w;
  const f3 p1 = mk3(A1);
  const f3 p2 = mk3(A2) - p1, p3 = mk3(A3) - p1, p4 = mk3(A4) - p1;
  const f3 c23 = fcross(p2, p3), c24 = fcross(p2, p4);  // the forward's fused forms, exactly
  const float d23 = fdot(c23, c23), d24 = fdot(c24, c24);
  const float i23 = 1.0f / sqrtf(d23), i24 = 1.0f / sqrtf(d24);  // normalize's, exactly
  const f3 n1 = c23 * i23, n2 = c24 * i24;
  const float draw = fdot(n1, n2);
  const float d = tclamp(draw, 0.0f, 1.0f);
  const float angle = acos_as(d);
  if (angle < kEps || isnan(d)) return false;  // not projected: identity
  const float L23 = d23 * i23, L24 = d24 * i24;  // |c23|, |c24|
  const float r23 = frcp(L23 + kEps), r24 = frcp(L24 + kEps);
  const f3 B3 = cross(n1, p2), B4 = cross(n2, p2), B23 = cross(n1, p3), B24 = cross(n2, p4);
  const f3 A3v = cross(p2, n2) + B3 * d;
  const f3 A4v = cross(p2, n1) + B4 * d;
  const f3 A23 = cross(p3, n2) + B23 * d;
  const f3 A24 = cross(p4, n1) + B24 * d;
  const f3 q3 = A3v * r23, q4 = A4v * r24;
  const f3 q2 = -(A23 * r23) - A24 * r24;
  const f3 q1 = -q2 - q3 - q4;
  const float idt2 = frcp(dt * dt);
  const float at = comp * idt2;
  const float denom = at + (w1 * dot(q1, q1) + w2 * dot(q2, q2) + w3 * dot(q3, q3) +
                            w4 * dot(q4, q4));
  if (denom < kEps) return false;
  const float om = 1.0f - d * d;  // > 0: d < 1 wherever the angle passed
  const float rs = rsqrtf(om);
  const float s = om * rs;
  const float rden = frcp(denom);
  const float lam = s * (angle - theta) * rden;
  const f3 g1 = mk3(G1), g2 = mk3(G2), g3 = mk3(G3), g4 = mk3(G4);
  // c_i = w_i lam q_i
  const float lam_bar = w1 * dot(g1, q1) + w2 * dot(g2, q2) + w3 * dot(g3, q3) + w4 * dot(g4, q4);
  f3 q1b = (w1 * lam) * g1, q2b = (w2 * lam) * g2, q3b = (w3 * lam) * g3, q4b = (w4 * lam) * g4;
  float w1b = lam * dot(g1, q1), w2b = lam * dot(g2, q2), w3b = lam * dot(g3, q3),
        w4b = lam * dot(g4, q4);
  // lam = s (angle - theta) / denom
  const float s_bar = lam_bar * (angle - theta) * rden;
  const float angle_bar = lam_bar * s * rden;
  const float denom_bar = -lam_bar * lam * rden;
  // denom = at + sum w_i |q_i|^2
  q1b = q1b + (2.0f * denom_bar * w1) * q1;
  q2b = q2b + (2.0f * denom_bar * w2) * q2;
  q3b = q3b + (2.0f * denom_bar * w3) * q3;
  q4b = q4b + (2.0f * denom_bar * w4) * q4;
  w1b += denom_bar * dot(q1, q1);
  w2b += denom_bar * dot(q2, q2);
  w3b += denom_bar * dot(q3, q3);
  w4b += denom_bar * dot(q4, q4);
  cbar += denom_bar * idt2;
  // q1 = -q2 - q3 - q4
  q2b = q2b - q1b;
  q3b = q3b - q1b;
  q4b = q4b - q1b;
  // q3 = A3v / e23, q4 = A4v / e24, q2 = -A23 / e23 - A24 / e24  (e = |c| + eps)
  const f3 A3b = q3b * r23, A4b = q4b * r24, A23b = -(q2b * r23), A24b = -(q2b * r24);
  const float e23b = (-dot(q3b, q3) + dot(q2b, A23) * r23) * r23;
  const float e24b = (-dot(q4b, q4) + dot(q2b, A24) * r24) * r24;
  f3 p2b = mk3(0, 0, 0), p3b = mk3(0, 0, 0), p4b = mk3(0, 0, 0);
  f3 n1b = mk3(0, 0, 0), n2b = mk3(0, 0, 0);
  float db = 0.0f;
  // A3v = p2 x n2 + (n1 x p2) d
  cross_bwd(p2, n2, A3b, p2b, n2b);
  cross_bwd(n1, p2, A3b * d, n1b, p2b);
  db += dot(A3b, B3);
  // A4v = p2 x n1 + (n2 x p2) d
  cross_bwd(p2, n1, A4b, p2b, n1b);
  cross_bwd(n2, p2, A4b * d, n2b, p2b);
  db += dot(A4b, B4);
  // A23 = p3 x n2 + (n1 x p3) d
  cross_bwd(p3, n2, A23b, p3b, n2b);
  cross_bwd(n1, p3, A23b * d, n1b, p3b);
  db += dot(A23b, B23);
  // A24 = p4 x n1 + (n2 x p4) d
  cross_bwd(p4, n1, A24b, p4b, n1b);
  cross_bwd(n2, p4, A24b * d, n2b, p4b);
  db += dot(A24b, B24);
  // s = sqrt(1 - d^2); angle = acos_as(d)
  db += s_bar * (-d * rs) + angle_bar * acos_as_deriv(d);
  // d = clamp(n1 . n2, 0, 1)
  if (draw > 0.0f && draw < 1.0f) {
    n1b = n1b + db * n2;
    n2b = n2b + db * n1;
  }
  // n = c / |c|, e = |c| + eps
  const f3 c23b = (n1b - dot(n1, n1b) * n1) * i23 + e23b * n1;
  const f3 c24b = (n2b - dot(n2, n2b) * n2) * i24 + e24b * n2;
  cross_bwd(p2, p3, c23b, p2b, p3b);
  cross_bwd(p2, p4, c24b, p2b, p4b);
  const f3 p1b = -(p2b + p3b + p4b);
  G1 = mk4(g1 + p1b, G1.w + w1b);
  G2 = mk4(g2 + p2b, G2.w + w2b);
  G3 = mk4(g3 + p3b, G3.w + w3b);
  G4 = mk4(g4 + p4b, G4.w + w4b);
  return true;
}

__global__ void k_bend_bwd(const uint32_t* __restrict__ order, uint32_t begin, uint32_t end,
                           const int4* __restrict__ gidx, const float2* __restrict__ tc,
                           const float4* __restrict__ tx, float4* __restrict__ G,
                           float* __restrict__ bcomp_bar, float dt) {
  pdl_release();
  pdl_wait();
  const uint32_t k = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= end) return;
  const uint32_t j = order[k];
  const int4 b = gidx[j];
  const float2 th = tc[j];
  const float4* t = tx + 4 * (size_t)j;
  float4 G1 = G[b.x], G2 = G[b.y], G3 = G[b.z], G4 = G[b.w];
  float cb = 0.0f;
  if (bend_vjp(t[0], t[1], t[2], t[3], th.x, th.y, dt, G1, G2, G3, G4, cb)) {
    G[b.x] = G1;
    G[b.y] = G2;
    G[b.z] = G3;
    G[b.w] = G4;
    bcomp_bar[j] += cb;
  }
}

// ---- tiled replay and reverse ---------------------------------------------------------------
// With the tile-local schedule the replay runs the forward's own tile launches (solver.cu
// k_stretch_tiles / k_bend_tiles instantiated with TAPE: the forward's code, hence its bits),
// which tape each projection's inputs by execution slot (a local color's slots are contiguous,
// so the tape writes coalesce).  The reverse of a tile color launch is one block per tile, tile
// colors last to first: the block stages the footprint's adjoint in shared memory and walks the
// tile's local colors backwards, reading the taped inputs.  Tiles of one tile color have
// disjoint footprints, so the write-back of the adjoint needs no atomics.  Shared memory of the
// reverse: adjoint (16 B) and id (4 B) per footprint vertex; record (16 B) + multiplier adjoint
// (stretch, 4 B) or rest angle and compliance (bend, 8 B) per constraint; num_local + 1
// offsets.

// STAGE: the tile's slice of the tape (contiguous slots c0 .. c0 + nc) is loaded into shared
// memory up front, all loads in flight at once, instead of one dependent global load per local
// color step; for tiles whose slice does not fit, the reverse reads the tape in place.
template <bool RESET, int NT, bool STAGE>
__global__ void __launch_bounds__(NT) k_stretch_tiles_bwd(
    const int4* __restrict__ con, const uint32_t* __restrict__ foot,
    const int4* __restrict__ meta, const uint32_t* __restrict__ lofs, uint32_t tile_begin,
    uint32_t num_local, uint32_t max_foot, uint32_t max_cons, float dt,
    const float4* __restrict__ tx, const float* __restrict__ tl, float4* __restrict__ G,
    float* __restrict__ lam_bar, float* __restrict__ comp_bar) {
  extern __shared__ float4 smem[];
  float4* sg = smem;
  float4* stx = sg + max_foot;                               // STAGE: 2 x max_cons
  int4* sc = reinterpret_cast<int4*>(stx + (STAGE ? 2 * max_cons : 0));
  float* slb = reinterpret_cast<float*>(sc + max_cons);
  float* stl = slb + max_cons;                               // STAGE: max_cons
  uint32_t* so = reinterpret_cast<uint32_t*>(stl + (STAGE ? max_cons : 0));
  uint32_t* sf = so + num_local + 1;
  const TileFrame f = tile_prologue<NT>(foot, meta, lofs, tile_begin + blockIdx.x, num_local, so);
  const uint32_t c0 = (uint32_t)f.m.z, nc = (uint32_t)f.m.w;
  for (uint32_t j = threadIdx.x; j < nc; j += NT) sc[j] = __ldg(&con[c0 + j]);  // setup data
  pdl_wait();  // the tape and the adjoints are written by earlier launches of the reverse
  if (STAGE) {
    const float4* src = tx + 2 * (size_t)c0;
    for (uint32_t k = threadIdx.x; k < 2 * nc; k += NT) stx[k] = src[k];
  }
  for (uint32_t j = threadIdx.x; j < nc; j += NT) {
    slb[j] = lam_bar[c0 + j];
    if (STAGE) stl[j] = tl[c0 + j];
  }
  tile_gather<NT>(f, G, sg, sf);
  __syncthreads();
  const float4* ax = STAGE ? stx : tx + 2 * (size_t)c0;
  const float* al = STAGE ? stl : tl + c0;
  for (int l = (int)num_local - 1; l >= 0; --l) {
    const uint32_t ce = so[l + 1];
    for (uint32_t j = so[l] + threadIdx.x; j < ce; j += NT) {
      const int4 c = sc[j];
      float4 ga = sg[c.x], gb = sg[c.y];
      float lin = slb[j], cb = 0.0f;
      if (stretch_vjp(ax[2 * j], ax[2 * j + 1], al[j], __int_as_float(c.z), __int_as_float(c.w),
                      dt, slb[j], ga, gb, lin, cb)) {
        sg[c.x] = ga;
        sg[c.y] = gb;
        comp_bar[c0 + j] += cb;
      }
      slb[j] = RESET ? 0.0f : lin;
    }
    __syncthreads();
  }
  pdl_release();
  tile_scatter<NT>((uint32_t)f.m.y, G, sg, sf);
  for (uint32_t j = threadIdx.x; j < nc; j += NT) lam_bar[c0 + j] = slb[j];
}

template <int NT, bool STAGE>
__global__ void __launch_bounds__(NT) k_bend_tiles_bwd(
    const int4* __restrict__ idx, const float2* __restrict__ tc,
    const uint32_t* __restrict__ foot, const int4* __restrict__ meta,
    const uint32_t* __restrict__ lofs, uint32_t tile_begin, uint32_t num_local,
    uint32_t max_foot, uint32_t max_cons, float dt, const float4* __restrict__ tx,
    float4* __restrict__ G, float* __restrict__ bcomp_bar) {
  extern __shared__ float4 smem[];
  float4* sg = smem;
  float4* stx = sg + max_foot;                               // STAGE: 4 x max_cons
  int4* sc = reinterpret_cast<int4*>(stx + (STAGE ? 4 * max_cons : 0));
  float2* st = reinterpret_cast<float2*>(sc + max_cons);
  uint32_t* so = reinterpret_cast<uint32_t*>(st + max_cons);
  uint32_t* sf = so + num_local + 1;
  const TileFrame f = tile_prologue<NT>(foot, meta, lofs, tile_begin + blockIdx.x, num_local, so);
  const uint32_t c0 = (uint32_t)f.m.z, nc = (uint32_t)f.m.w;
  for (uint32_t j = threadIdx.x; j < nc; j += NT) {  // setup data
    sc[j] = __ldg(&idx[c0 + j]);
    st[j] = __ldg(&tc[c0 + j]);
  }
  pdl_wait();  // the tape and the adjoints are written by earlier launches of the reverse
  if (STAGE) {
    const float4* src = tx + 4 * (size_t)c0;
    for (uint32_t k = threadIdx.x; k < 4 * nc; k += NT) stx[k] = src[k];
  }
  tile_gather<NT>(f, G, sg, sf);
  __syncthreads();
  const float4* ax = STAGE ? stx : tx + 4 * (size_t)c0;
  for (int l = (int)num_local - 1; l >= 0; --l) {
    const uint32_t ce = so[l + 1];
    for (uint32_t j = so[l] + threadIdx.x; j < ce; j += NT) {
      const int4 b = sc[j];
      const float2 th = st[j];
      const float4* s = ax + 4 * (size_t)j;
      float4 G1 = sg[b.x], G2 = sg[b.y], G3 = sg[b.z], G4 = sg[b.w];
      float cb = 0.0f;
      if (bend_vjp(s[0], s[1], s[2], s[3], th.x, th.y, dt, G1, G2, G3, G4, cb)) {
        sg[b.x] = G1;
        sg[b.y] = G2;
        sg[b.z] = G3;
        sg[b.w] = G4;
        bcomp_bar[c0 + j] += cb;
      }
    }
    __syncthreads();
  }
  pdl_release();
  tile_scatter<NT>((uint32_t)f.m.y, G, sg, sf);
}

// LRA (all slots pinned) + VF-CCD + VF-DCD, per vertex, Jacobi (Gin -> Gout).  The slot sources'
// share of the LRA Jacobian goes to Gs by atomics (sources are the few pinned slot vertices).
constexpr int kMaxLraSlots = 8;

__global__ void k_stage_bwd(const float4* __restrict__ X, const float4* __restrict__ Gin,
                            float4* __restrict__ Gout, float4* __restrict__ Gs, uint32_t nv,
                            bool lra, const uint32_t* __restrict__ lra_ptr,
                            const uint32_t* __restrict__ lra_src,
                            const float* __restrict__ lra_rest, float stretch, bool contacts,
                            const int* __restrict__ rt_idx, const float4* __restrict__ rt_qc,
                            const int* __restrict__ vf_idx, const float4* __restrict__ vf_qs,
                            const float4* __restrict__ pred, uint32_t* err) {
  pdl_release();
  pdl_wait();
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nv) return;
  const float4 p = X[t];
  const float4 gin = Gin[t];
  f3 q = mk3(p);
  // forward, keeping what the reverse needs
  f3 diffs[kMaxLraSlots];
  float ratio[kMaxLraSlots];
  uint32_t src[kMaxLraSlots];
  int nslots = 0;
  if (lra) {
    const uint32_t b = lra_ptr[t], e = lra_ptr[t + 1];
    if (e - b > (uint32_t)kMaxLraSlots) {
      raise_error(err, kErrIndex);
    } else if (b != e) {
      f3 xt = q;
      for (uint32_t k = b; k < e; ++k, ++nslots) {
        const f3 s = mk3(X[lra_src[k]]);
        const float target = lra_rest[k] * stretch;
        src[nslots] = lra_src[k];
        ratio[nslots] = -1.0f;  // inactive
        if (p.w < kEps && target > 0) continue;
        const f3 df = xt - s;
        const float dist = length(df);
        if (dist > target) {
          ratio[nslots] = target / dist;
          diffs[nslots] = df / dist;
        }
        xt = lra_project(xt, s, p.w, lra_rest[k], stretch);
      }
      q = xt;
    }
  }
  bool rt_on = false, vf_on = false;
  f3 nc = mk3(0, 0, 0), ns = mk3(0, 0, 0);
  if (contacts) {
    const int rc = rt_idx[t], vc = vf_idx[t];
    if (rc != -1) {
      nc = prim_normal(pred, rc);
      const float lambda = dot(nc, q - mk3(rt_qc[t]));
      if (lambda < 0) {
        q = q + (-lambda * nc);
        rt_on = true;
      }
    }
    if (vc != -1) {
      ns = prim_normal(pred, vc);
      const float lambda = dot(ns, q - mk3(vf_qs[t])) - 1e-3f;
      if (lambda < 0) vf_on = true;
    }
  }
  // reverse
  f3 g = mk3(gin);
  if (vf_on) g = g - dot(ns, g) * ns;   // x' = x - ((x - qs).n - m) n
  if (rt_on) g = g - dot(nc, g) * nc;
  for (int k = nslots - 1; k >= 0; --k) {
    if (ratio[k] < 0.0f) continue;
    // x' = s + (x - s) target / |x - s|:  dx'/dx = r (I - n n^T), dx'/ds = I - r (I - n n^T)
    const f3 n = diffs[k];
    const f3 gx = ratio[k] * (g - dot(n, g) * n);
    const f3 gs = g - gx;
    atomicAdd(&Gs[src[k]].x, gs.x);
    atomicAdd(&Gs[src[k]].y, gs.y);
    atomicAdd(&Gs[src[k]].z, gs.z);
    g = gx;
  }
  Gout[t] = mk4(g, gin.w);
}

__global__ void k_add_sources(float4* __restrict__ G, float4* __restrict__ Gs, uint32_t nv) {
  pdl_release();
  pdl_wait();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const float4 s = Gs[i];
  if (s.x == 0.0f && s.y == 0.0f && s.z == 0.0f) return;
  const float4 g = G[i];
  G[i] = make_float4(g.x + s.x, g.y + s.y, g.z + s.z, g.w);
  Gs[i] = make_float4(0, 0, 0, 0);
}

// EE contact of edge e as seen by the forward (k_ee): active, and its record.
struct EeTerm {
  bool on;
  float s;
  f3 fn;
};
__device__ __forceinline__ EeTerm ee_term(uint32_t e, const float4* __restrict__ X,
                                          const uint2* __restrict__ edge,
                                          const float4* __restrict__ ee_a,
                                          const float4* __restrict__ ee_b,
                                          const float4* __restrict__ ee_c) {
  EeTerm r{false, 0.0f, mk3(0, 0, 0)};
  const float4 ca = ee_a[e];
  if (ca.x > 1e6f) return r;
  const float4 cb = ee_b[e], cc = ee_c[e];
  const uint2 ed = edge[e];
  const f3 p1 = mk3(X[ed.x]), q1 = mk3(X[ed.y]);
  const float s = cb.w, t = cc.w;
  const f3 fn = mk3(cc);
  const f3 c1 = (1 - s) * p1 + s * q1;
  const f3 c2 = (1 - t) * mk3(ca.y, ca.z, ca.w) + t * mk3(cb);
  const f3 d = c1 - c2;
  if (length(d) < kEps) return r;
  if (dot(d, fn) - 1e-3f > 0) return r;
  r.on = true;
  r.s = s;
  r.fn = fn;
  return r;
}

// out_i = x_i + relax / cnt_i * sum_{e active at i} -sigma_ie lambda_e fn_e, with
// lambda_e = ((1-s) x_e.x + s x_e.y - c2) . fn - m; sigma / omega = 1-s at e.x, s at e.y.
__global__ void k_ee_bwd(const float4* __restrict__ X, const float4* __restrict__ Gin,
                         float4* __restrict__ Gout, uint32_t nv,
                         const uint32_t* __restrict__ ve_ptr, const uint32_t* __restrict__ ve_list,
                         const uint2* __restrict__ edge, const float4* __restrict__ ee_a,
                         const float4* __restrict__ ee_b, const float4* __restrict__ ee_c,
                         const float* __restrict__ cnt, float relaxation) {
  pdl_release();
  pdl_wait();
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nv) return;
  const float4 gj = Gin[j];
  f3 g = mk3(gj);
  for (uint32_t k = ve_ptr[j]; k < ve_ptr[j + 1]; ++k) {
    const uint32_t code = ve_list[k];
    const uint32_t e = code >> 1;
    const EeTerm term = ee_term(e, X, edge, ee_a, ee_b, ee_c);
    if (!term.on) continue;
    const uint2 ed = edge[e];
    float tot = 0.0f;
    const float cx = cnt[ed.x], cy = cnt[ed.y];
    if (cx > 0.0f) tot += relaxation / cx * (1.0f - term.s) * dot(term.fn, mk3(Gin[ed.x]));
    if (cy > 0.0f) tot += relaxation / cy * term.s * dot(term.fn, mk3(Gin[ed.y]));
    const float omega = (code & 1u) ? term.s : 1.0f - term.s;
    g = g - (omega * tot) * term.fn;
  }
  Gout[j] = mk4(g, gj.w);
}

// finalize: v' = (x_end - x0) / dt * kd, x0' = x_end.  G: x0'-bar -> x_end-bar, H: x0-bar part.
__global__ void k_finalize_bwd(float4* __restrict__ G, float4* __restrict__ Gv,
                               float4* __restrict__ H, uint32_t nv, float dt, float kd) {
  pdl_release();
  pdl_wait();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const float4 g = G[i];
  const f3 a = mk3(Gv[i]) * (kd / dt);
  G[i] = mk4(mk3(g) + a, g.w);
  H[i] = mk4(-a, 0.0f);
  Gv[i] = make_float4(0, 0, 0, 0);
}

// predict: x_p = x0 + v_p dt, v_p = v + g dt.  G: x_p-bar -> x0-bar, Gv: v-bar.
__global__ void k_predict_bwd(float4* __restrict__ G, float4* __restrict__ Gv,
                              const float4* __restrict__ H, uint32_t nv, float dt) {
  pdl_release();
  pdl_wait();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const float4 g = G[i];
  G[i] = mk4(mk3(H[i]) + mk3(g), g.w);
  Gv[i] = mk4(mk3(g) * dt, 0.0f);
}

}  // namespace

// ---- host side ---------------------------------------------------------------------------------

namespace {

template <typename T>
cudaError_t put(DBuf<T>& d, const std::vector<T>& h, cudaStream_t s) {
  cudaError_t e = d.reserve(std::max<size_t>(h.size(), 1));
  if (e == cudaSuccess && !h.empty())
    e = cudaMemcpyAsync(d.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s);
  return e;
}

// Execution slots of one constraint kind grouped by color, colors in forward order.
void color_groups(const Context& c, int kind, std::vector<uint32_t>& order,
                  std::vector<ColorRange>& colors) {
  order.clear();
  colors.clear();
  const TiledSet& T = kind == 0 ? c.s_tiles : c.b_tiles;
  const uint32_t n = kind == 0 ? c.ne : c.nb;
  if (T.on) {
    const uint32_t L = T.num_local;
    const std::vector<int4>& meta = c.h_tile_meta[kind];
    const std::vector<uint32_t>& lofs = c.h_tile_lofs[kind];
    for (const ColorRange& tcr : T.tile_colors)
      for (uint32_t l = 0; l < L; ++l) {
        const uint32_t b = (uint32_t)order.size();
        for (uint32_t t = tcr.begin; t < tcr.end; ++t) {
          const uint32_t c0 = (uint32_t)meta[t].z;
          const uint32_t* lo = &lofs[(size_t)t * (L + 1)];
          for (uint32_t j = c0 + lo[l]; j < c0 + lo[l + 1]; ++j) order.push_back(j);
        }
        if (order.size() > b) colors.push_back(ColorRange{b, (uint32_t)order.size()});
      }
  } else {
    for (uint32_t j = 0; j < n; ++j) order.push_back(j);
    for (const ColorRange& r : (kind == 0 ? c.s_ranges : c.b_ranges))
      if (r.end > r.begin) colors.push_back(r);
  }
}

// Shared memory per constraint of the tiled reverse: record + multiplier adjoint (stretch),
// record + rest angle and compliance (bend); plus, when the tape slice is staged, the taped
// inputs (two vertices + multiplier, four vertices).
constexpr size_t kStretchBwdRecord = sizeof(int4) + sizeof(float);
constexpr size_t kBendBwdRecord = sizeof(int4) + sizeof(float2);
constexpr size_t kStretchStaged = 2 * sizeof(float4) + sizeof(float);
constexpr size_t kBendStaged = 4 * sizeof(float4);

size_t tiles_bwd_smem(const TiledSet& T, size_t record) {
  return (sizeof(float4) + sizeof(uint32_t)) * T.max_foot + record * T.max_cons +
         sizeof(uint32_t) * (T.num_local + 1);
}
size_t stretch_bwd_smem(const TiledSet& T, bool stage) {
  return tiles_bwd_smem(T, kStretchBwdRecord + (stage ? kStretchStaged : 0));
}
size_t bend_bwd_smem(const TiledSet& T, bool stage) {
  return tiles_bwd_smem(T, kBendBwdRecord + (stage ? kBendStaged : 0));
}
size_t stretch_bwd_smem(const Context& c) { return stretch_bwd_smem(c.s_tiles, c.diff.s_stage); }
size_t bend_bwd_smem(const Context& c) { return bend_bwd_smem(c.b_tiles, c.diff.b_stage); }

using StretchBwdKernel = void (*)(const int4*, const uint32_t*, const int4*, const uint32_t*,
                                  uint32_t, uint32_t, uint32_t, uint32_t, float, const float4*,
                                  const float*, float4*, float*, float*);
using BendBwdKernel = void (*)(const int4*, const float2*, const uint32_t*, const int4*,
                               const uint32_t*, uint32_t, uint32_t, uint32_t, uint32_t, float,
                               const float4*, float4*, float*);

template <int NT>
StretchBwdKernel stretch_bwd_nt(bool reset, bool stage) {
  return reset ? (stage ? k_stretch_tiles_bwd<true, NT, true> : k_stretch_tiles_bwd<true, NT, false>)
               : (stage ? k_stretch_tiles_bwd<false, NT, true>
                        : k_stretch_tiles_bwd<false, NT, false>);
}
StretchBwdKernel stretch_bwd_kernel(uint32_t block, bool reset, bool stage) {
  return block == 128 ? stretch_bwd_nt<128>(reset, stage)
         : block == 256 ? stretch_bwd_nt<256>(reset, stage)
                        : stretch_bwd_nt<512>(reset, stage);
}
StretchBwdKernel stretch_bwd_kernel(const Context& c, bool reset) {
  return stretch_bwd_kernel(c.diff.s_block, reset, c.diff.s_stage);
}
template <int NT>
BendBwdKernel bend_bwd_nt(bool stage) {
  return stage ? k_bend_tiles_bwd<NT, true> : k_bend_tiles_bwd<NT, false>;
}
BendBwdKernel bend_bwd_kernel(uint32_t block, bool stage) {
  return block == 128 ? bend_bwd_nt<128>(stage)
         : block == 256 ? bend_bwd_nt<256>(stage)
                        : bend_bwd_nt<512>(stage);
}
BendBwdKernel bend_bwd_kernel(const Context& c) {
  return bend_bwd_kernel(c.diff.b_block, c.diff.b_stage);
}

// Launch shape of a tiled reverse: 128-thread blocks where the footprints fit (a local color of
// a tile rarely has more elements, and four blocks per SM hold more tiles at once), else the
// forward's; the tape slice is staged when the staged blocks still hold the largest tile color
// in one wave (or lose no resident blocks), read in place otherwise.
template <typename K>
cudaError_t choose_reverse_shape(const Context& c, const TiledSet& T, K (*kernel)(uint32_t, bool),
                                 size_t smem_plain, size_t smem_staged, int smem_max,
                                 uint32_t& block, bool& stage) {
  block = T.max_foot <= kFootPerThread * 128u ? 128u : T.block;
  uint32_t widest = 0;
  for (const ColorRange& r : T.tile_colors) widest = std::max(widest, r.end - r.begin);
  int occ_plain = 0, occ_staged = 0;
  cudaError_t e = raise_smem((const void*)kernel(block, false), smem_plain);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_plain, kernel(block, false),
                                                      (int)block, smem_plain);
  if (e != cudaSuccess) return e;
  stage = false;
  if (smem_staged <= (size_t)smem_max) {
    e = raise_smem((const void*)kernel(block, true), smem_staged);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_staged, kernel(block, true),
                                                        (int)block, smem_staged);
    if (e != cudaSuccess) return e;
    stage = occ_staged > 0 && ((uint64_t)occ_staged * (uint64_t)c.num_sms >= widest ||
                               occ_staged >= occ_plain);
  }
  return cudaSuccess;
}

cudaError_t configure_tiled_adjoint(Context& c, int smem_max) {
  DiffState& D = c.diff;
  cudaError_t e = cudaSuccess;
  auto set = [&](const void* k, size_t b) {
    if (e == cudaSuccess) e = raise_smem(k, b);
  };
  if (D.s_tiled) {
    const TiledSet& T = c.s_tiles;
    if (e == cudaSuccess)
      e = choose_reverse_shape(
          c, T, +[](uint32_t b, bool s) { return stretch_bwd_kernel(b, false, s); },
          stretch_bwd_smem(T, false), stretch_bwd_smem(T, true), smem_max, D.s_block, D.s_stage);
    set((const void*)stretch_bwd_kernel(c, true), stretch_bwd_smem(c));
  }
  if (D.b_tiled) {
    const TiledSet& T = c.b_tiles;
    if (e == cudaSuccess)
      e = choose_reverse_shape(
          c, T, +[](uint32_t b, bool s) { return bend_bwd_kernel(b, s); },
          bend_bwd_smem(T, false), bend_bwd_smem(T, true), smem_max, D.b_block, D.b_stage);
  }
  return e;
}

// Reverse of one tiled stretch / bend phase (all tile colors, last to first).
void stretch_tiles_bwd(Context& c, float dt, bool reset, size_t ti) {
  DiffState& D = c.diff;
  const TiledSet& T = c.s_tiles;
  const size_t smem = stretch_bwd_smem(c);
  const StretchBwdKernel kern = stretch_bwd_kernel(c, reset);
  const float4* tx = D.t_sx.p + 2 * ti * c.ne;
  const float* tl = D.t_sl.p + ti * c.ne;
  for (int k = (int)T.tile_colors.size() - 1; k >= 0; --k) {
    const ColorRange r = T.tile_colors[k];
    if (r.end > r.begin)
      launch_k(c.pdl, kern, r.end - r.begin, D.s_block, smem, c.stream, c.s_con.p, T.foot.p,
               T.meta.p, T.lofs.p, r.begin, T.num_local, T.max_foot, T.max_cons, dt, tx, tl,
               D.G.p, D.lam_bar.p, D.comp_bar.p);
  }
}

void bend_tiles_bwd(Context& c, float dt, size_t ti) {
  DiffState& D = c.diff;
  const TiledSet& T = c.b_tiles;
  const size_t smem = bend_bwd_smem(c);
  const BendBwdKernel kern = bend_bwd_kernel(c);
  const float4* tx = D.t_bx.p + 4 * ti * c.nb;
  for (int k = (int)T.tile_colors.size() - 1; k >= 0; --k) {
    const ColorRange r = T.tile_colors[k];
    if (r.end > r.begin)
      launch_k(c.pdl, kern, r.end - r.begin, D.b_block, smem, c.stream, c.b_idx.p, c.b_tc.p,
               T.foot.p, T.meta.p, T.lofs.p, r.begin, T.num_local, T.max_foot, T.max_cons, dt,
               tx, D.G.p, D.bcomp_bar.p);
  }
}

cudaError_t copy_d(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, s) : cudaSuccess;
}

// One frame, as record_frame issues it, with the projections' and per-vertex launches' inputs
// taped by the launches themselves and each collision pass's contacts generated into their tape
// slots (the obstacle primitives are copied).
void record_frame_diff(Context& c) {
  DiffState& D = c.diff;
  const xrt_swift_params& p = c.params;
  const FrameConst k = frame_const(c);
  const uint32_t V = c.nv, E = c.ne, B = c.nb;
  Timed timed(c, kAdjReplay, 1, V);  // the frame's launches as one group
  float4* const x_start = c.x.p;
  int swaps = 0;
  auto swap_x = [&]() {
    std::swap(c.x.p, c.x_alt.p);
    ++swaps;
  };
  const bool obstacle_updated = p.update_obstacle_animation && c.onf > 0;
  if (obstacle_updated) {
    launch_prims_obstacle(c, 0.0f);
    c.bvh.construct(0.0f, c.stream, c.err.p);
  }
  const bool has_obstacle = c.onf > 0;
  const bool lra_fused = p.geodesic_lra && c.nl && c.lra_by_target;
  const int frequency = (p.num_substeps * p.num_iterations) / p.num_collision_passes;
  const unsigned blk = kBlock;
  int cnt = 0;
  int* const vf_idx = c.vf_idx.p;  // the contact buffers, redirected to tape slots per pass
  int* const rt_idx = c.rt_idx.p;
  float4* const vf_qs = c.vf_qs.p;
  float4* const rt_qc = c.rt_qc.p;
  float4* const ee_a = c.ee_a.p;
  float4* const ee_b = c.ee_b.p;
  float4* const ee_c = c.ee_c.p;
  D.it_pass.assign((size_t)D.S * D.I, 0);
  for (uint32_t s = 0; s < D.S; ++s) {
    if (s == 0) launch_predict(c, k);
    for (uint32_t it = 0; it < D.I; ++it) {
      const uint32_t cur = s * D.I + it;
      if ((int)cur % frequency == 0) {
        if (obstacle_updated) launch_obstacle_pass(c, cnt, p.num_collision_passes);
        if (has_obstacle) {
          // the pass's contacts are generated straight into their tape slots, which the stage
          // and EE launches up to the next pass then read (the context's buffers are restored
          // at the end of the frame)
          const size_t pv = (size_t)cnt * V, pe = (size_t)cnt * E;
          c.vf_idx.p = D.t_vf_idx.p + pv;
          c.rt_idx.p = D.t_rt_idx.p + pv;
          c.vf_qs.p = D.t_vf_qs.p + pv;
          c.rt_qc.p = D.t_rt_qc.p + pv;
          c.ee_a.p = D.t_ee_a.p + pe;
          c.ee_b.p = D.t_ee_b.p + pe;
          c.ee_c.p = D.t_ee_c.p + pe;
          launch_generate_contacts(c);
          copy_d(D.t_pred.p + (size_t)cnt * 3 * c.onf, c.bvh.pred.p, sizeof(float4) * 3 * c.onf,
                 c.stream);
        }
        cnt++;
      }
      D.it_pass[cur] = cnt - 1;
      const size_t ti = (size_t)cur;
      // tiled: the forward's tile launches, taping each projection's inputs by execution slot
      if (D.s_tiled)
        for (const ColorRange& r : c.s_tiles.tile_colors)
          launch_stretch_tiles(c, k, r, it == 0, D.t_sx.p + 2 * ti * E, D.t_sl.p + ti * E);
      else for (const ColorRange& r : D.s_colors) {
        const unsigned g = grid_for(r.end - r.begin);
        launch_k(c.pdl, it == 0 ? k_stretch_tape<true> : k_stretch_tape<false>, g, blk, 0,
                 c.stream, D.s_order.p, r.begin, r.end, D.s_gidx.p, c.s_con.p, c.s_lambda.p,
                 c.x.p, D.t_sx.p + 2 * ti * E, D.t_sl.p + ti * E, k.dt);
      }
      if (p.solve_bending && D.b_tiled)
        for (const ColorRange& r : c.b_tiles.tile_colors)
          launch_bend_tiles(c, k, r, D.t_bx.p + 4 * ti * B);
      else if (p.solve_bending)
        for (const ColorRange& r : D.b_colors)
          launch_k(c.pdl, k_bend_tape, grid_for(r.end - r.begin), blk, 0, c.stream, D.b_order.p,
                   r.begin, r.end, D.b_gidx.p, c.b_tc.p, c.x.p, D.t_bx.p + 4 * ti * B, k.dt);
      if (lra_fused || has_obstacle) {  // the launches tape their input positions
        launch_stage(c, k, lra_fused, has_obstacle, D.t_stage.p + ti * V);
        swap_x();
      }
      if (has_obstacle) {
        launch_ee(c, k, has_obstacle, false, D.t_ee.p + ti * V, D.cnt.p + ti * V);
        swap_x();
      }
    }
    const bool last = s + 1 == D.S;
    launch_finalize_predict(c, k, !last, last);
  }
  if (c.onv > 0) launch_obstacle_commit(c);
  c.vf_idx.p = vf_idx;
  c.rt_idx.p = rt_idx;
  c.vf_qs.p = vf_qs;
  c.rt_qc.p = rt_qc;
  c.ee_a.p = ee_a;
  c.ee_b.p = ee_b;
  c.ee_c.p = ee_c;
  if (swaps & 1) {
    cudaMemcpyAsync(x_start, c.x.p, sizeof(float4) * c.nv, cudaMemcpyDeviceToDevice, c.stream);
    std::swap(c.x.p, c.x_alt.p);
  }
}

// Reverse pass through the frame just replayed; G / Gv hold the adjoint of the frame-end state
// on entry and of the frame-start state on exit.
void backward_frame(Context& c) {
  DiffState& D = c.diff;
  const xrt_swift_params& p = c.params;
  const FrameConst k = frame_const(c);
  const uint32_t V = c.nv, E = c.ne, B = c.nb;
  const bool has_obstacle = c.onf > 0;
  const bool lra_fused = p.geodesic_lra && c.nl && c.lra_by_target;
  const float kd = 1 - k.damping * k.dt;
  const unsigned gv = grid_for(V), blk = kBlock;
  const uint32_t n_vertex_launches = (has_obstacle ? 1 : 0) + (lra_fused || has_obstacle ? 1 : 0) +
                                     (lra_fused ? 1 : 0);
  const uint32_t n_bend_launches =
      D.b_tiled ? (uint32_t)c.b_tiles.tile_colors.size() : (uint32_t)D.b_colors.size();
  const uint32_t n_stretch_launches =
      D.s_tiled ? (uint32_t)c.s_tiles.tile_colors.size() : (uint32_t)D.s_colors.size();
  for (int s = (int)D.S - 1; s >= 0; --s) {
    {
      Timed t(c, kAdjVertex, 1, V);
      launch_k(c.pdl, k_finalize_bwd, gv, blk, 0, c.stream, D.G.p, D.Gv.p, D.H.p, V, k.dt, kd);
      cudaMemsetAsync(D.lam_bar.p, 0, sizeof(float) * std::max(E, 1u), c.stream);
    }
    for (int it = (int)D.I - 1; it >= 0; --it) {
      const size_t ti = (size_t)s * D.I + it;
      const int pass = D.it_pass[ti];
      const size_t pv = (size_t)pass * V, pe = (size_t)pass * E;
      {
        Timed tv(c, kAdjVertex, n_vertex_launches, V);
        if (has_obstacle) {
          const float4* X = D.t_ee.p + ti * V;
          launch_k(c.pdl, k_ee_bwd, gv, blk, 0, c.stream, X, D.G.p, D.G2.p, V, c.ve_ptr.p,
                   c.ve_list.p, c.edge.p, D.t_ee_a.p + pe, D.t_ee_b.p + pe, D.t_ee_c.p + pe,
                   D.cnt.p + ti * V, k.relaxation);
          std::swap(D.G.p, D.G2.p);
        }
        if (lra_fused || has_obstacle) {
          launch_k(c.pdl, k_stage_bwd, gv, blk, 0, c.stream, D.t_stage.p + ti * V, D.G.p, D.G2.p,
                   D.Gs.p, V, lra_fused, c.lra_ptr.p, c.lra_src.p, c.lra_rest.p, k.lra_stretch,
                   has_obstacle, D.t_rt_idx.p + pv, D.t_rt_qc.p + pv, D.t_vf_idx.p + pv,
                   D.t_vf_qs.p + pv, D.t_pred.p + (size_t)pass * 3 * c.onf, c.err.p);
          if (lra_fused) launch_k(c.pdl, k_add_sources, gv, blk, 0, c.stream, D.G2.p, D.Gs.p, V);
          std::swap(D.G.p, D.G2.p);
        }
      }
      if (p.solve_bending) {
        Timed tb(c, kAdjBend, n_bend_launches, B);
        if (D.b_tiled) bend_tiles_bwd(c, k.dt, ti);
        else
          for (int ci = (int)D.b_colors.size() - 1; ci >= 0; --ci) {
            const ColorRange r = D.b_colors[ci];
            launch_k(c.pdl, k_bend_bwd, grid_for(r.end - r.begin), blk, 0, c.stream, D.b_order.p,
                     r.begin, r.end, D.b_gidx.p, c.b_tc.p, D.t_bx.p + 4 * ti * B, D.G.p,
                     D.bcomp_bar.p, k.dt);
          }
      }
      Timed ts(c, kAdjStretch, n_stretch_launches, E);
      if (D.s_tiled) stretch_tiles_bwd(c, k.dt, it == 0, ti);
      else for (int ci = (int)D.s_colors.size() - 1; ci >= 0; --ci) {
        const ColorRange r = D.s_colors[ci];
        const unsigned g = grid_for(r.end - r.begin);
        launch_k(c.pdl, it == 0 ? k_stretch_bwd<true> : k_stretch_bwd<false>, g, blk, 0,
                 c.stream, D.s_order.p, r.begin, r.end, D.s_gidx.p, c.s_con.p,
                 D.t_sx.p + 2 * ti * E, D.t_sl.p + ti * E, D.G.p, D.lam_bar.p, D.comp_bar.p,
                 k.dt);
      }
    }
    Timed t(c, kAdjVertex, 1, V);
    launch_k(c.pdl, k_predict_bwd, gv, blk, 0, c.stream, D.G.p, D.Gv.p, D.H.p, V, k.dt);
  }
}

void destroy_frame_graphs(DiffState& D) {
  for (DiffState::FrameGraph& g : D.graph) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = DiffState::FrameGraph{};
  }
}

// Replay + reverse of the frame whose checkpoint is loaded, as a graph: captured on first use
// for the current G / G2 assignment (capture only records, so the host-side buffer swaps are
// undone and re-applied after each launch).
cudaError_t run_frame_graph(Context& c) {
  DiffState& D = c.diff;
  DiffState::FrameGraph* g = nullptr;
  for (DiffState::FrameGraph& fg : D.graph)
    if (fg.exec && fg.g_in == D.G.p) g = &fg;
  if (!g) {
    g = D.graph[0].exec ? &D.graph[1] : &D.graph[0];
    if (g->exec) cudaGraphExecDestroy(g->exec);
    *g = DiffState::FrameGraph{};
    float4* const g_in = D.G.p;
    float4* const g2_in = D.G2.p;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    record_frame_diff(c);
    backward_frame(c);
    e = cudaStreamEndCapture(c.stream, &graph);
    if (e != cudaSuccess) return e;
    e = cudaGraphInstantiate(&g->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      g->exec = nullptr;
      return e;
    }
    g->g_in = g_in;
    g->g_out = D.G.p;
    g->g2_out = D.G2.p;
    D.G.p = g_in;
    D.G2.p = g2_in;
  }
  cudaError_t e = cudaGraphLaunch(g->exec, c.stream);
  D.G.p = g->g_out;
  D.G2.p = g->g2_out;
  return e;
}

void save_state(Context& c, DiffState::Checkpoint& ck) {
  const uint32_t V = c.nv, O = c.onv;
  ck.x.reserve(V);
  ck.x0.reserve(V);
  ck.v.reserve(V);
  copy_d(ck.x.p, c.x.p, sizeof(float4) * V, c.stream);
  copy_d(ck.x0.p, c.x0.p, sizeof(float4) * V, c.stream);
  copy_d(ck.v.p, c.v.p, sizeof(float4) * V, c.stream);
  if (O) {
    ck.ox0.reserve(O);
    ck.ox.reserve(O);
    ck.on.reserve(O);
    copy_d(ck.ox0.p, c.ox0.p, sizeof(float4) * O, c.stream);
    copy_d(ck.ox.p, c.ox.p, sizeof(float4) * O, c.stream);
    copy_d(ck.on.p, c.on.p, sizeof(float4) * O, c.stream);
  }
  ck.frame_index = c.frame_index;
}

void load_state(Context& c, const DiffState::Checkpoint& ck) {
  const uint32_t V = c.nv, O = c.onv;
  copy_d(c.x.p, ck.x.p, sizeof(float4) * V, c.stream);
  copy_d(c.x_alt.p, ck.x.p, sizeof(float4) * V, c.stream);
  copy_d(c.x0.p, ck.x0.p, sizeof(float4) * V, c.stream);
  copy_d(c.v.p, ck.v.p, sizeof(float4) * V, c.stream);
  if (O) {
    copy_d(c.ox0.p, ck.ox0.p, sizeof(float4) * O, c.stream);
    copy_d(c.ox.p, ck.ox.p, sizeof(float4) * O, c.stream);
    copy_d(c.on.p, ck.on.p, sizeof(float4) * O, c.stream);
  }
  c.frame_index = ck.frame_index;
}

}  // namespace

xrt_status diff_prepare(Context& c) {
  const xrt_swift_params& p = c.params;
  if (p.enable_self_collision || p.pbd_repulsion || p.impact_zone || p.imminent_repulsion ||
      c.nbind > 0 || c.fem.on) {
    c.set_error("the adjoint covers frames of the Swift fabric without particle "
                "self-collision, Quality repulsion, impact zones or bindings");
    return XRT_ERR_INVALID_ARGUMENT;
  }
  if (p.geodesic_lra && c.nl && !c.lra_by_target) {
    c.set_error("the adjoint needs every LRA slot vertex pinned");
    return XRT_ERR_INVALID_ARGUMENT;
  }
  DiffState& D = c.diff;
  cudaStream_t s = c.stream;
  std::vector<uint32_t> order;
  color_groups(c, 0, order, D.s_colors);
  XRT_CUDA(&c, put(D.s_order, order, s));
  color_groups(c, 1, order, D.b_colors);
  XRT_CUDA(&c, put(D.b_order, order, s));
  std::vector<int2> g2(c.ne);
  for (uint32_t j = 0; j < c.ne; ++j) {
    const uint32_t o = c.s_perm[j];
    g2[j] = make_int2((int)c.h_edges[2 * o], (int)c.h_edges[2 * o + 1]);
  }
  XRT_CUDA(&c, put(D.s_gidx, g2, s));
  std::vector<int4> g4(c.nb);
  for (uint32_t j = 0; j < c.nb; ++j) {
    const uint32_t o = c.b_perm[j];
    g4[j] = make_int4((int)c.h_bends[4 * o], (int)c.h_bends[4 * o + 1], (int)c.h_bends[4 * o + 2],
                      (int)c.h_bends[4 * o + 3]);
  }
  XRT_CUDA(&c, put(D.b_gidx, g4, s));
  D.S = (uint32_t)p.num_substeps;
  D.I = (uint32_t)p.num_iterations;
  D.P = (uint32_t)p.num_collision_passes;
  const size_t V = c.nv, E = std::max(c.ne, 1u), Bn = std::max(c.nb, 1u), SI = (size_t)D.S * D.I;
  const size_t P = c.onf ? D.P : 1, F = std::max(c.onf, 1u);
  // tiled replay / reverse where the schedule is tiled and the reverse's shared memory fits
  int dev = 0, smem_max = 0;
  XRT_CUDA(&c, cudaGetDevice(&dev));
  XRT_CUDA(&c, cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  D.s_tiled = c.s_tiles.on && c.ne > 0 &&
              tiles_bwd_smem(c.s_tiles, kStretchBwdRecord) <= (size_t)smem_max;
  D.b_tiled = c.b_tiles.on && c.nb > 0 && p.solve_bending &&
              tiles_bwd_smem(c.b_tiles, kBendBwdRecord) <= (size_t)smem_max;
  if (D.s_tiled || D.b_tiled) XRT_CUDA(&c, configure_tiled_adjoint(c, smem_max));
  XRT_CUDA(&c, D.t_sx.reserve(2 * SI * E));
  XRT_CUDA(&c, D.t_sl.reserve(SI * E));
  XRT_CUDA(&c, D.t_bx.reserve(4 * SI * Bn));
  XRT_CUDA(&c, D.t_stage.reserve(SI * V));
  XRT_CUDA(&c, D.t_ee.reserve(c.onf ? SI * V : 1));
  XRT_CUDA(&c, D.t_vf_idx.reserve(P * V));
  XRT_CUDA(&c, D.t_rt_idx.reserve(P * V));
  XRT_CUDA(&c, D.t_vf_qs.reserve(P * V));
  XRT_CUDA(&c, D.t_rt_qc.reserve(P * V));
  XRT_CUDA(&c, D.t_ee_a.reserve(P * E));
  XRT_CUDA(&c, D.t_ee_b.reserve(P * E));
  XRT_CUDA(&c, D.t_ee_c.reserve(P * E));
  XRT_CUDA(&c, D.t_pred.reserve(P * 3 * F));
  for (DBuf<float4>* b : {&D.G, &D.G2, &D.Gv, &D.H, &D.Gs}) XRT_CUDA(&c, b->reserve(V));
  XRT_CUDA(&c, D.cnt.reserve(c.onf ? SI * V : 1));
  XRT_CUDA(&c, D.lam_bar.reserve(E));
  XRT_CUDA(&c, D.comp_bar.reserve(E));
  XRT_CUDA(&c, D.bcomp_bar.reserve(Bn));
  XRT_CUDA(&c, cudaMemsetAsync(D.Gs.p, 0, sizeof(float4) * V, s));
  D.active = true;
  D.frames = 0;
  return XRT_OK;
}

void diff_checkpoint(Context& c) {
  DiffState& D = c.diff;
  const uint32_t k = D.frames / D.interval;
  if (D.frames % D.interval == 0) {
    if (D.ck.size() <= k) D.ck.emplace_back();
    save_state(c, D.ck[k]);
  }
  if (D.targets.size() <= D.frames) D.targets.emplace_back();
  if (c.onv) {
    D.targets[D.frames].reserve(c.onv);
    copy_d(D.targets[D.frames].p, c.ox.p, sizeof(float4) * c.onv, c.stream);
  }
  D.frames++;
}

xrt_status diff_backward(Context& c, const float* dLdx, const float* dLdv, float* d_compliance,
                         float* d_bend_compliance, float* d_mass, float* d_velocity,
                         float* d_position) {
  DiffState& D = c.diff;
  if (!D.active) {
    c.set_error("call xrt_diff_begin and step frames before xrt_backward");
    return XRT_ERR_STATE;
  }
  if (!dLdx) return XRT_ERR_INVALID_ARGUMENT;
  cudaStream_t s = c.stream;
  const uint32_t V = c.nv;
  // the current state, restored at the end
  DiffState::Checkpoint now;
  save_state(c, now);
  std::vector<float4> g(V), gv(V, make_float4(0, 0, 0, 0));
  for (uint32_t i = 0; i < V; ++i) {
    g[i] = make_float4(dLdx[3 * i], dLdx[3 * i + 1], dLdx[3 * i + 2], 0.0f);
    if (dLdv) gv[i] = make_float4(dLdv[3 * i], dLdv[3 * i + 1], dLdv[3 * i + 2], 0.0f);
  }
  XRT_CUDA(&c, cudaMemcpyAsync(D.G.p, g.data(), sizeof(float4) * V, cudaMemcpyHostToDevice, s));
  XRT_CUDA(&c, cudaMemcpyAsync(D.Gv.p, gv.data(), sizeof(float4) * V, cudaMemcpyHostToDevice, s));
  XRT_CUDA(&c, cudaMemsetAsync(D.comp_bar.p, 0, sizeof(float) * std::max(c.ne, 1u), s));
  XRT_CUDA(&c, cudaMemsetAsync(D.bcomp_bar.p, 0, sizeof(float) * std::max(c.nb, 1u), s));
  const uint32_t m = D.interval;
  if (m > 1 && D.seg.size() < m) D.seg.resize(m);
  for (int f = (int)D.frames - 1; f >= 0; --f) {
    const uint32_t k = (uint32_t)f / m, first = k * m;
    if (m > 1 && ((uint32_t)f == D.frames - 1 || (uint32_t)f % m == m - 1)) {
      // a new segment (newest first): recompute its frames from its checkpoint, keeping the
      // start state of each
      load_state(c, D.ck[k]);
      for (uint32_t j = first; j <= (uint32_t)f; ++j) {
        if (c.onv) copy_d(c.ox.p, D.targets[j].p, sizeof(float4) * c.onv, c.stream);
        save_state(c, D.seg[j - first]);
        if (j == (uint32_t)f) break;  // the segment's last frame is replayed with taping below
        const int prof = c.profiling;
        c.profiling = 0;  // the recomputation is not part of the reverse pass's profile
        const xrt_status st = frame_core(c, false);
        c.profiling = prof;
        if (st != XRT_OK) {
          destroy_frame_graphs(D);
          load_state(c, now);
          return st;
        }
        c.frame_index++;
      }
    }
    load_state(c, m > 1 ? D.seg[(uint32_t)f - first] : D.ck[f]);
    if (c.graph_enabled && !c.profiling) {
      const cudaError_t e = run_frame_graph(c);
      if (e != cudaSuccess) {
        destroy_frame_graphs(D);
        load_state(c, now);
        c.set_error(std::string("reverse frame graph: ") + cudaGetErrorString(e));
        return XRT_ERR_CUDA;
      }
    } else {
      record_frame_diff(c);
      backward_frame(c);
      collect_profile(c);  // when profiling: the frame's replay and reverse phases
    }
  }
  destroy_frame_graphs(D);
  load_state(c, now);
  XRT_CUDA(&c, cudaGetLastError());
  // outputs
  XRT_CUDA(&c, cudaMemcpyAsync(g.data(), D.G.p, sizeof(float4) * V, cudaMemcpyDeviceToHost, s));
  XRT_CUDA(&c, cudaMemcpyAsync(gv.data(), D.Gv.p, sizeof(float4) * V, cudaMemcpyDeviceToHost, s));
  std::vector<float> cb(std::max(c.ne, 1u)), bb(std::max(c.nb, 1u));
  XRT_CUDA(&c, cudaMemcpyAsync(cb.data(), D.comp_bar.p, sizeof(float) * cb.size(),
                               cudaMemcpyDeviceToHost, s));
  XRT_CUDA(&c, cudaMemcpyAsync(bb.data(), D.bcomp_bar.p, sizeof(float) * bb.size(),
                               cudaMemcpyDeviceToHost, s));
  XRT_CUDA(&c, cudaStreamSynchronize(s));
  uint32_t flag = 0;
  XRT_CUDA(&c, cudaMemcpy(&flag, c.err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  if (flag) {
    c.set_error("device error flag raised during the reverse pass");
    return XRT_ERR_DEVICE_FLAG;
  }
  for (uint32_t i = 0; i < V; ++i) {
    if (d_position) {
      d_position[3 * i] = g[i].x;
      d_position[3 * i + 1] = g[i].y;
      d_position[3 * i + 2] = g[i].z;
    }
    if (d_velocity) {
      d_velocity[3 * i] = gv[i].x;
      d_velocity[3 * i + 1] = gv[i].y;
      d_velocity[3 * i + 2] = gv[i].z;
    }
    if (d_mass) {  // m = 1 / w: dL/dm = -w^2 dL/dw (pinned vertices: 0)
      const float w = c.h_w[i];
      d_mass[i] = w > 0.0f ? -w * w * g[i].w : 0.0f;
    }
  }
  if (d_compliance)
    for (uint32_t j = 0; j < c.ne; ++j) d_compliance[c.s_perm[j]] = cb[j];
  if (d_bend_compliance)
    for (uint32_t j = 0; j < c.nb; ++j) d_bend_compliance[c.b_perm[j]] = bb[j];
  return XRT_OK;
}

void diff_release(Context& c) {
  DiffState& D = c.diff;
  destroy_frame_graphs(D);
  for (auto& ck : D.ck)
    for (DBuf<float4>* b : {&ck.x, &ck.x0, &ck.v, &ck.ox0, &ck.ox, &ck.on}) b->release();
  D.ck.clear();
  for (auto& t : D.targets) t.release();
  D.targets.clear();
  for (auto& ck : D.seg)
    for (DBuf<float4>* b : {&ck.x, &ck.x0, &ck.v, &ck.ox0, &ck.ox, &ck.on}) b->release();
  D.seg.clear();
  D.s_order.release(); D.b_order.release(); D.s_gidx.release(); D.b_gidx.release();
  for (DBuf<float4>* b : {&D.t_sx, &D.t_bx, &D.t_stage, &D.t_ee, &D.t_vf_qs, &D.t_rt_qc,
                          &D.t_ee_a, &D.t_ee_b, &D.t_ee_c, &D.t_pred, &D.G, &D.G2, &D.Gv, &D.H,
                          &D.Gs})
    b->release();
  D.t_sl.release(); D.t_vf_idx.release(); D.t_rt_idx.release();
  D.cnt.release(); D.lam_bar.release(); D.comp_bar.release(); D.bcomp_bar.release();
  D.active = false;
  D.frames = 0;
}

}  // namespace xrt
