// hash.cu — Swift particle self-collision: uniform-grid hash, stable sort, cell ranges,
// neighbor cache and the Jacobi push-out with friction.
//
//   ComputeIntCoord/HashCoords ...... xrtailor/src/physics/broad_phase/spatial_hash/SpatialHashGPU.cu:9-25
//   FindCellStart_Kernel ............ SpatialHashGPU.cu:27-54
//   CacheNeighbors_Kernel ........... SpatialHashGPU.cu:56-99
//   HashObjects ..................... SpatialHashGPU.cu:128-160 (cub radix sort -> radix.cu)
//   CollideParticles_Kernel ......... xrtailor/src/physics/ClothSolverHelper.cu:171-219
//   ComputeFriction / ApplyDeltas ... ClothSolverHelper.cu:139-169
//
// The push-out reads positions from one buffer and writes the relaxed result to the other (the
// caller swaps them), which is the reference's deltas + ApplyDeltas pair in one launch.
#include "common.cuh"
#include "context.h"
#include "lbvh_dev.cuh"

namespace xrt {
namespace {

__device__ __forceinline__ int int_coord(float value, float spacing) {
  return (int)floorf(value / spacing);
}
__device__ __forceinline__ int hash_coords(int x, int y, int z, int table) {
  const int h = (int)(((uint32_t)x * 92837111u) ^ ((uint32_t)y * 689287499u) ^
                      ((uint32_t)z * 283923481u));
  return abs(h % table);
}

// Keys of instance s lie in [table_base, table_base + table_size): each instance hashes into its
// own table of 2 V_s cells (the reference's 2V for that cloth alone), laid end to end.
__global__ void k_hash(const float4* __restrict__ x, uint32_t nv, InstView I,
                       uint32_t* __restrict__ key, uint32_t* __restrict__ val) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const InstanceRec r = inst_rec(I, inst_index(I, i));
  const float4 p = x[i];
  key[i] = r.table_base + (uint32_t)hash_coords(int_coord(p.x, r.spacing), int_coord(p.y, r.spacing),
                                                int_coord(p.z, r.spacing), (int)r.table_size);
  val[i] = i;
}

__global__ void k_cell_bounds(const uint32_t* __restrict__ skey, uint32_t nv,
                              uint32_t* __restrict__ cell_start, uint32_t* __restrict__ cell_end) {
  const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= nv) return;
  const uint32_t h = skey[id];
  if (id == 0 || h != skey[id - 1]) {
    cell_start[h] = id;
    if (id > 0) cell_end[skey[id - 1]] = id;
  }
  if (id == nv - 1) cell_end[h] = id + 1;
}

__global__ void k_cache_neighbors(const uint32_t* __restrict__ sidx,
                                  const uint32_t* __restrict__ cell_start,
                                  const uint32_t* __restrict__ cell_end,
                                  const float4* __restrict__ x, const float4* __restrict__ x_init,
                                  uint32_t nv, InstView I, uint32_t maxnb,
                                  uint32_t* __restrict__ neighbors) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= nv) return;
  const uint32_t id = sidx[tid];
  const InstanceRec r = inst_rec(I, inst_index(I, id));
  const float spacing = r.spacing, spacing2 = r.spacing2, d2 = r.d2;
  const int table = (int)r.table_size;
  const f3 pos = mk3(x[id]);
  const f3 orig = mk3(x_init[id]);
  const int ix = int_coord(pos.x, spacing), iy = int_coord(pos.y, spacing),
            iz = int_coord(pos.z, spacing);
  uint64_t ni = id;
  const uint64_t limit = (uint64_t)nv * maxnb;
  for (int xx = ix - 1; xx <= ix + 1; ++xx)
    for (int yy = iy - 1; yy <= iy + 1; ++yy)
      for (int zz = iz - 1; zz <= iz + 1; ++zz) {
        const uint32_t h = r.table_base + (uint32_t)hash_coords(xx, yy, zz, table);
        const uint32_t start = cell_start[h];
        if (start == kNone) continue;
        const uint32_t end = min(cell_end[h], start + maxnb);
        for (uint32_t k = start; k < end; ++k) {
          const uint32_t nb = sidx[k];
          const f3 dp = pos - mk3(x[nb]);
          const f3 d0 = orig - mk3(x_init[nb]);
          if (nb != id && dot(dp, dp) < spacing2 && dot(d0, d0) > d2) {
            neighbors[ni] = nb;
            ni += nv;
            if (ni >= limit) return;
          }
        }
      }
  if (ni < limit) neighbors[ni] = kNone;
}

__device__ __forceinline__ f3 friction_of(float mu, f3 correction, f3 rel_vel) {
  f3 fr = mk3(0, 0, 0);
  const float cl = length(correction);
  if (mu > 0.0f && cl > 0.0f) {
    const f3 nrm = correction / cl;
    const f3 tan_vel = rel_vel - nrm * dot(rel_vel, nrm);
    const float tl = length(tan_vel);
    const float max_tl = cl * mu;
    fr = -tan_vel * tmin(max_tl / tl, 1.0f);
  }
  return fr;
}

__global__ void k_collide(const float4* __restrict__ x_in, float4* __restrict__ x_out,
                          const float4* __restrict__ x0, const uint32_t* __restrict__ neighbors,
                          uint32_t nv, uint32_t maxnb, InstView I, float mu, float relaxation) {
  pdl_release();
  pdl_wait();
  const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= nv) return;
  const float diameter = inst_rec(I, inst_index(I, id)).diameter;
  const float4 pi = x_in[id];
  const f3 pred_i = mk3(pi);
  const f3 vel_i = pred_i - mk3(x0[id]);
  const float w_i = pi.w;
  f3 pd = mk3(0, 0, 0);
  int cnt = 0;
  // Neighbor slots are read a batch at a time (ids, then positions, all loads of a batch in
  // flight); the list ends at the first id >= nv (reference: j > num_particles; j == nv never
  // occurs) and the batch is then processed in slot order.
  constexpr uint32_t kBatch = 8;
  bool done = false;
  for (uint32_t base = 0; base < maxnb && !done; base += kBatch) {
    uint32_t nb[kBatch];
#pragma unroll
    for (uint32_t r = 0; r < kBatch; ++r)
      nb[r] = base + r < maxnb ? neighbors[(uint64_t)(base + r) * nv + id] : nv;
    float4 pj[kBatch];
#pragma unroll
    for (uint32_t r = 0; r < kBatch; ++r) pj[r] = nb[r] < nv ? x_in[nb[r]] : make_float4(0, 0, 0, 0);
#pragma unroll
    for (uint32_t r = 0; r < kBatch; ++r) {
      if (done) break;
      const uint32_t j = nb[r];
      if (j >= nv) {
        done = true;
        break;
      }
      const float denom = w_i + pj[r].w;
      if (denom <= 0) continue;
      const f3 pred_j = mk3(pj[r]);
      const f3 diff = pred_i - pred_j;
      const float distance = length(diff);
      if (distance >= diameter) continue;
      const f3 gradient = diff / (distance + kEps);
      const float lambda = (distance - diameter) / denom;
      const f3 common = lambda * gradient;
      ++cnt;
      pd = pd - w_i * common;
      const f3 rel = vel_i - (pred_j - mk3(x0[j]));
      pd = pd + w_i * friction_of(mu, common, rel);
    }
  }
  f3 q = pred_i;
  const float count = (float)cnt;
  if (count > 0.0f) q = q + pd / count * relaxation;
  x_out[id] = mk4(q, w_i);
}

}  // namespace

void launch_hash(Context& c) {
  const uint32_t nv = c.nv;
  if (nv == 0) return;
  const uint32_t table = 2 * nv;  // the instances' tables end to end
  int bits = 0;
  while ((1u << bits) < table) ++bits;
  const InstView I = c.inst_view();
  k_hash<<<grid_for(nv), kBlock, 0, c.stream>>>(c.x.p, nv, I, c.hash_key.p, c.hash_val.p);
  uint32_t *skey = nullptr, *sidx = nullptr;
  c.hash_sorter.sort(c.hash_key.p, c.hash_val.p, nv, bits, c.stream, &skey, &sidx);
  cudaMemsetAsync(c.cell_start.p, 0xFF, sizeof(uint32_t) * table, c.stream);
  k_cell_bounds<<<grid_for(nv), kBlock, 0, c.stream>>>(skey, nv, c.cell_start.p, c.cell_end.p);
  k_cache_neighbors<<<grid_for(nv), kBlock, 0, c.stream>>>(
      sidx, c.cell_start.p, c.cell_end.p, c.x.p, c.x_init.p, nv, I,
      (uint32_t)c.params.max_neighbor_size, c.neighbors.p);
}

void launch_collide(Context& c, const FrameConst& k) {
  launch_k(c.pdl, k_collide, grid_for(c.nv, c.vertex_block), c.vertex_block, 0, c.stream,
           c.x.p, c.x_alt.p, c.x0.p,
           c.neighbors.p, c.nv, (uint32_t)c.params.max_neighbor_size, c.inst_view(), k.friction,
           k.relaxation);
}

}  // namespace xrt
