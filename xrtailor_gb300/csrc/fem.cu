// fem.cu — the FEM fabric (include/xrt_fem.h): strain per cloth face and isometric bending per
// bend element, projected like the Swift fabric's stretch and bend constraints.
//
// SolveStrain_Kernel and SolveIsometricBending_Kernel (xrtailor/src/physics/dynamics/
// FEMHelper.cu:175-207, 325-388) apply one color per launch and add their corrections with
// atomics; within a color no two constraints share a vertex, so the corrections here are plain
// read-modify-writes.  With the tile-local schedule a tile's footprint stays in shared memory
// across its local colors (tile kernels as solver.cu's); otherwise one launch per color.  The
// projections themselves are project_dev.cuh's fem_strain_project / iso_bend_project.
#include <algorithm>
#include <cmath>

#include "../../include/xrt_fem.h"
#include "common.cuh"
#include "context.h"
#include "project_dev.cuh"

namespace xrt {
namespace {

__device__ __forceinline__ void load_q(const float* __restrict__ Q, size_t slot, float* q) {
  const float4* q4 = reinterpret_cast<const float4*>(Q + 16 * slot);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float4 t = __ldg(&q4[k]);
    q[4 * k] = t.x;
    q[4 * k + 1] = t.y;
    q[4 * k + 2] = t.z;
    q[4 * k + 3] = t.w;
  }
}

// ---- one launch per color ------------------------------------------------------------------

__global__ void k_fem_strain(const int4* __restrict__ idx, const float4* __restrict__ inv,
                             const float* __restrict__ area, float4* __restrict__ x,
                             uint32_t begin, uint32_t end, FemTensor C) {
  pdl_release();
  pdl_wait();
  const uint32_t j = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= end) return;
  const int4 f = __ldg(&idx[j]);
  float4 a0 = x[f.x], a1 = x[f.y], a2 = x[f.z];
  if (fem_strain_project(a0, a1, a2, __ldg(&area[j]), __ldg(&inv[j]), C)) {
    x[f.x] = a0;
    x[f.y] = a1;
    x[f.z] = a2;
  }
}

template <bool RESET>
__global__ void k_iso_bend(const int4* __restrict__ idx, const float* __restrict__ Q,
                           float* __restrict__ lambda, float4* __restrict__ x, uint32_t begin,
                           uint32_t end, float alpha) {
  pdl_release();
  pdl_wait();
  const uint32_t j = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= end) return;
  const int4 b = __ldg(&idx[j]);
  float q[16];
  load_q(Q, j, q);
  float lam = RESET ? 0.0f : lambda[j];
  float4 a0 = x[b.x], a1 = x[b.y], a2 = x[b.z], a3 = x[b.w];
  if (iso_bend_project(a0, a1, a2, a3, q, alpha, lam)) {
    x[b.x] = a0;
    x[b.y] = a1;
    x[b.z] = a2;
    x[b.w] = a3;
  }
  lambda[j] = lam;
}

// ---- tile-local schedule -------------------------------------------------------------------
// Shared memory: footprint positions (16 B) and ids (4 B) per footprint vertex; the record
// (16 B) and, for bending, the multiplier (4 B) per constraint; num_local + 1 offsets.  The
// material data (inverse rest matrix and area, Hessian) are read from global memory by slot.

template <int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) k_fem_strain_tiles(
    const int4* __restrict__ idx, const float4* __restrict__ inv, const float* __restrict__ area,
    float4* __restrict__ x, const uint32_t* __restrict__ foot, const int4* __restrict__ meta,
    const uint32_t* __restrict__ lofs, uint32_t tile_begin, uint32_t num_local,
    uint32_t max_foot, uint32_t max_cons, FemTensor C) {
  extern __shared__ float4 smem[];
  float4* sx = smem;
  int4* sc = reinterpret_cast<int4*>(sx + max_foot);
  uint32_t* so = reinterpret_cast<uint32_t*>(sc + max_cons);
  uint32_t* sf = so + num_local + 1;
  const TileFrame f = tile_prologue<NT>(foot, meta, lofs, tile_begin + blockIdx.x, num_local, so);
  const uint32_t c0 = (uint32_t)f.m.z, nc = (uint32_t)f.m.w;
  for (uint32_t j = threadIdx.x; j < nc; j += NT) sc[j] = __ldg(&idx[c0 + j]);
  pdl_wait();
  tile_gather<NT>(f, x, sx, sf);
  __syncthreads();
  for (uint32_t l = 0; l < num_local; ++l) {
    const uint32_t ce = so[l + 1];
    for (uint32_t j = so[l] + threadIdx.x; j < ce; j += NT) {
      const int4 e = sc[j];
      float4 a0 = sx[e.x], a1 = sx[e.y], a2 = sx[e.z];
      if (fem_strain_project(a0, a1, a2, __ldg(&area[c0 + j]), __ldg(&inv[c0 + j]), C)) {
        sx[e.x] = a0;
        sx[e.y] = a1;
        sx[e.z] = a2;
      }
    }
    __syncthreads();
  }
  pdl_release();
  tile_scatter<NT>((uint32_t)f.m.y, x, sx, sf);
}

template <bool RESET, int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) k_iso_bend_tiles(
    const int4* __restrict__ idx, const float* __restrict__ Q, float* __restrict__ lambda,
    float4* __restrict__ x, const uint32_t* __restrict__ foot, const int4* __restrict__ meta,
    const uint32_t* __restrict__ lofs, uint32_t tile_begin, uint32_t num_local,
    uint32_t max_foot, uint32_t max_cons, float alpha) {
  extern __shared__ float4 smem[];
  float4* sx = smem;
  int4* sc = reinterpret_cast<int4*>(sx + max_foot);
  float* sl = reinterpret_cast<float*>(sc + max_cons);
  uint32_t* so = reinterpret_cast<uint32_t*>(sl + max_cons);
  uint32_t* sf = so + num_local + 1;
  const TileFrame f = tile_prologue<NT>(foot, meta, lofs, tile_begin + blockIdx.x, num_local, so);
  const uint32_t c0 = (uint32_t)f.m.z, nc = (uint32_t)f.m.w;
  for (uint32_t j = threadIdx.x; j < nc; j += NT) sc[j] = __ldg(&idx[c0 + j]);
  pdl_wait();
  for (uint32_t j = threadIdx.x; j < nc; j += NT) sl[j] = RESET ? 0.0f : lambda[c0 + j];
  tile_gather<NT>(f, x, sx, sf);
  __syncthreads();
  for (uint32_t l = 0; l < num_local; ++l) {
    const uint32_t ce = so[l + 1];
    for (uint32_t j = so[l] + threadIdx.x; j < ce; j += NT) {
      const int4 b = sc[j];
      float q[16];
      load_q(Q, c0 + j, q);
      float lam = sl[j];
      float4 a0 = sx[b.x], a1 = sx[b.y], a2 = sx[b.z], a3 = sx[b.w];
      if (iso_bend_project(a0, a1, a2, a3, q, alpha, lam)) {
        sx[b.x] = a0;
        sx[b.y] = a1;
        sx[b.z] = a2;
        sx[b.w] = a3;
        sl[j] = lam;
      }
    }
    __syncthreads();
  }
  pdl_release();
  tile_scatter<NT>((uint32_t)f.m.y, x, sx, sf);
  for (uint32_t j = threadIdx.x; j < nc; j += NT) lambda[c0 + j] = sl[j];
}

FemTensor tensor(const FemState& F) { return FemTensor{F.c00, F.c01, F.c10, F.c11, F.c22}; }

size_t strain_smem(const TiledSet& T) { return tile_smem_bytes(T, sizeof(int4)); }
size_t bend_smem(const TiledSet& T) { return tile_smem_bytes(T, sizeof(int4) + sizeof(float)); }

}  // namespace

cudaError_t fem_upload(Context& c) {
  FemState& F = c.fem;
  const xrt_fem_material& m = F.m;
  const float d = 1.0f - m.xy_poisson_ratio * m.yx_poisson_ratio;
  F.c00 = m.xx_stiffness / d;
  F.c01 = m.xx_stiffness * m.yx_poisson_ratio / d;
  F.c11 = m.yy_stiffness / d;
  F.c10 = m.yy_stiffness * m.xy_poisson_ratio / d;
  F.c22 = m.xy_stiffness;
  std::vector<float> area, inv, q;
  setup::fem_strain_rest(c.h_x0, c.h_tri, area, inv);
  setup::iso_bend_hessian(c.h_x0, c.h_bends, q);
  // strain: slot order
  const FemKind& S = F.strain;
  const size_t nf = c.h_tri.size() / 3;
  std::vector<int4> sidx(nf);
  std::vector<float4> sinv(nf);
  std::vector<float> sarea(nf);
  for (size_t j = 0; j < nf; ++j) {
    const uint32_t o = S.perm[j];
    const uint32_t* v = S.tiles.on ? &S.local[3 * j] : &c.h_tri[3 * o];
    sidx[j] = make_int4((int)v[0], (int)v[1], (int)v[2], 0);
    sinv[j] = make_float4(inv[4 * o], inv[4 * o + 1], inv[4 * o + 2], inv[4 * o + 3]);
    sarea[j] = area[o];
  }
  // bending
  const FemKind& B = F.bend;
  const size_t nb = c.h_bends.size() / 4;
  std::vector<int4> bidx(nb);
  std::vector<float> bq(16 * std::max<size_t>(nb, 1));
  for (size_t j = 0; j < nb; ++j) {
    const uint32_t o = B.perm[j];
    const uint32_t* v = B.tiles.on ? &B.local[4 * j] : &c.h_bends[4 * o];
    bidx[j] = make_int4((int)v[0], (int)v[1], (int)v[2], (int)v[3]);
    std::copy(&q[16 * o], &q[16 * o] + 16, &bq[16 * j]);
  }
  auto put = [&](auto& buf, const auto& h) {
    cudaError_t e = buf.reserve(std::max<size_t>(h.size(), 1));
    if (e == cudaSuccess && !h.empty())
      e = cudaMemcpyAsync(buf.p, h.data(), sizeof(h[0]) * h.size(), cudaMemcpyHostToDevice,
                          c.stream);
    return e;
  };
  cudaError_t e = put(F.strain.idx, sidx);
  if (e == cudaSuccess) e = put(F.s_inv, sinv);
  if (e == cudaSuccess) e = put(F.s_area, sarea);
  if (e == cudaSuccess) e = put(F.bend.idx, bidx);
  if (e == cudaSuccess) e = put(F.b_q, bq);
  if (e == cudaSuccess) e = F.b_lambda.reserve(std::max<size_t>(nb, 1));
  if (e == cudaSuccess)
    e = cudaMemsetAsync(F.b_lambda.p, 0, sizeof(float) * std::max<size_t>(nb, 1), c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  return e;
}

cudaError_t fem_configure(Context& c) {
  cudaError_t e = cudaSuccess;
  for (FemKind* K : {&c.fem.strain, &c.fem.bend}) {
    TiledSet& T = K->tiles;
    if (!T.on) continue;
    T.block = T.max_foot <= kFootPerThread * 256u ? 256u : 512u;
    const bool strain = K == &c.fem.strain;
    const size_t smem = strain ? strain_smem(T) : bend_smem(T);
    const void* kerns[3] = {
        strain ? (T.block == 256 ? (const void*)k_fem_strain_tiles<256>
                                 : (const void*)k_fem_strain_tiles<512>)
               : (T.block == 256 ? (const void*)k_iso_bend_tiles<true, 256>
                                 : (const void*)k_iso_bend_tiles<true, 512>),
        strain ? nullptr
               : (T.block == 256 ? (const void*)k_iso_bend_tiles<false, 256>
                                 : (const void*)k_iso_bend_tiles<false, 512>),
        nullptr};
    for (const void* k : kerns)
      if (k && e == cudaSuccess) e = raise_smem(k, smem);
  }
  return e;
}

void launch_fem(Context& c, const FrameConst& k, bool reset_lambda, int phase_strain,
                int phase_bend) {
  FemState& F = c.fem;
  const FemTensor C = tensor(F);
  {
    const FemKind& S = F.strain;
    const TiledSet& T = S.tiles;
    if (T.on) {
      auto kern = T.block == 256 ? k_fem_strain_tiles<256> : k_fem_strain_tiles<512>;
      for (size_t tc = 0; tc < T.tile_colors.size(); ++tc) {
        const ColorRange r = T.tile_colors[tc];
        if (r.end == r.begin) continue;
        Timed t(c, phase_strain, 1, T.tile_color_cons[tc]);
        launch_k(c.pdl, kern, r.end - r.begin, T.block, strain_smem(T), c.stream, S.idx.p,
                 F.s_inv.p, F.s_area.p, c.x.p, T.foot.p, T.meta.p, T.lofs.p, r.begin,
                 T.num_local, T.max_foot, T.max_cons, C);
      }
    } else {
      for (const ColorRange& r : S.ranges) {
        if (r.end == r.begin) continue;
        Timed t(c, phase_strain, 1, r.end - r.begin);
        launch_k(c.pdl, k_fem_strain, grid_for(r.end - r.begin), kBlock, 0, c.stream, S.idx.p,
                 F.s_inv.p, F.s_area.p, c.x.p, r.begin, r.end, C);
      }
    }
  }
  if (!F.m.solve_bending || c.h_bends.empty()) return;
  const float alpha = 1.0f / (F.m.bending_stiffness * k.dt * k.dt);
  const FemKind& B = F.bend;
  const TiledSet& T = B.tiles;
  if (T.on) {
    auto kern = T.block == 256 ? (reset_lambda ? k_iso_bend_tiles<true, 256>
                                               : k_iso_bend_tiles<false, 256>)
                               : (reset_lambda ? k_iso_bend_tiles<true, 512>
                                               : k_iso_bend_tiles<false, 512>);
    for (size_t tc = 0; tc < T.tile_colors.size(); ++tc) {
      const ColorRange r = T.tile_colors[tc];
      if (r.end == r.begin) continue;
      Timed t(c, phase_bend, 1, T.tile_color_cons[tc]);
      launch_k(c.pdl, kern, r.end - r.begin, T.block, bend_smem(T), c.stream, B.idx.p, F.b_q.p,
               F.b_lambda.p, c.x.p, T.foot.p, T.meta.p, T.lofs.p, r.begin, T.num_local,
               T.max_foot, T.max_cons, alpha);
    }
  } else {
    auto kern = reset_lambda ? k_iso_bend<true> : k_iso_bend<false>;
    for (const ColorRange& r : B.ranges) {
      if (r.end == r.begin) continue;
      Timed t(c, phase_bend, 1, r.end - r.begin);
      launch_k(c.pdl, kern, grid_for(r.end - r.begin), kBlock, 0, c.stream, B.idx.p, F.b_q.p,
               F.b_lambda.p, c.x.p, r.begin, r.end, alpha);
    }
  }
}

void fem_release(Context& c) {
  FemState& F = c.fem;
  for (FemKind* K : {&F.strain, &F.bend}) {
    K->idx.release();
    K->tiles.foot.release();
    K->tiles.meta.release();
    K->tiles.lofs.release();
  }
  F.s_inv.release();
  F.s_area.release();
  F.b_q.release();
  F.b_lambda.release();
}

}  // namespace xrt

using xrt::Context;

extern "C" {

xrt_status xrt_default_fem_material(xrt_fem_material* out) {
  if (!out) return XRT_ERR_INVALID_ARGUMENT;
  *out = xrt_fem_material{};
  out->xx_stiffness = out->yy_stiffness = out->xy_stiffness = 1.0f;  // config/Base.hpp:47-57
  out->xy_poisson_ratio = out->yx_poisson_ratio = 0.3f;
  out->bending_stiffness = 1.0f;
  out->solve_bending = 1;
  return XRT_OK;
}

xrt_status xrt_set_fem_material(xrt_ctx* h, const xrt_fem_material* m) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (c.started) {
    c.set_error("xrt_set_fem_material after xrt_start");
    return XRT_ERR_STATE;
  }
  if (!m) {
    c.fem.on = false;
    return XRT_OK;
  }
  const float d = 1.0f - m->xy_poisson_ratio * m->yx_poisson_ratio;
  if (!(d != 0.0f) || !(m->bending_stiffness > 0.0f) || !std::isfinite(m->xx_stiffness) ||
      !std::isfinite(m->yy_stiffness) || !std::isfinite(m->xy_stiffness)) {
    c.set_error("FEM material: Poisson ratios with nu_xy nu_yx = 1, a non-positive bending "
                "stiffness or a non-finite modulus");
    return XRT_ERR_INVALID_CONFIG;
  }
  c.fem.m = *m;
  c.fem.on = true;
  return XRT_OK;
}

}  // extern "C"
