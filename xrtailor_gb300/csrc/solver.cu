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
#include <algorithm>
#include <map>
#include <mutex>

#include "common.cuh"
#include "context.h"
#include "project_dev.cuh"

namespace xrt {
namespace {

__global__ void k_predict(float4* __restrict__ x, const float4* __restrict__ x0,
                          float4* __restrict__ v, uint32_t nv, float dt, float gx, float gy,
                          float gz) {
  pdl_release();
  pdl_wait();
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
  pdl_release();
  pdl_wait();
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

template <bool RESET>
__global__ void k_stretch(const int4* __restrict__ con, float* __restrict__ lambda,
                          float4* __restrict__ x, uint32_t begin, uint32_t end, float dt) {
  pdl_release();
  pdl_wait();
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

// Tile-local Gauss-Seidel: block = one tile of the launched tile color (TileFrame and the
// prologue / gather / scatter helpers in project_dev.cuh).  The tile's footprint is staged in
// shared memory, its local colors run in order with a block barrier between them, and the
// footprint is written back.  Tiles of one tile color have disjoint footprints.
// Shared memory of a tile launch: footprint positions, the tile's records (its whole block, or
// two local colors' segments), two mbarriers, the multipliers (stretch), then the num_local + 1
// local-color offsets and the footprint ids.
// Prologue before pdl_wait (setup-time data only): the tile's metadata, offsets and footprint
// vertex ids (kFootPerThread per thread in registers, so the gather and the write-back each
// issue all their loads and stores at once), and the first bulk copies of the tile's records
// (TiledSet::rec: 16-bit footprint-local ids, then float2 values) into shared memory, completed
// on mbarriers while the predecessor grid drains and the footprint is gathered.  Every wait on a
// barrier is bounded; a copy that does not complete raises kErrBulkCopy and the block waits
// (bounded) for its copies in flight and leaves.  NT threads per block: 512 for footprints up to
// 4,096 vertices, 256 (twice the resident blocks per SM) up to 2,048.
// Stretch tiles: the record block holds one segment per local color, as for bend (16-bit ids,
// then float2 rest length and stretch_alpha(compliance, dt), each padded to 16 bytes).  STREAM (throughput regime):
// the segments stream in two colors ahead through two shared-memory buffers; otherwise the whole
// block comes in one bulk copy.  The multipliers of the tile's constraints stay in shared memory
// from the prologue to the write-back.
template <bool RESET, int NT, bool STREAM, bool TAPE>
__global__ void __launch_bounds__(NT, 1024 / NT) k_stretch_tiles(
    const uint4* __restrict__ rec, const uint32_t* __restrict__ rec_ofs,
    float* __restrict__ lambda, float4* __restrict__ x, const uint32_t* __restrict__ foot,
    const int4* __restrict__ meta, const uint32_t* __restrict__ lofs, uint32_t tile_begin,
    uint32_t num_local, uint32_t max_foot, uint32_t max_seg16, uint32_t buf16, uint32_t max_cons,
    uint32_t* err, float4* __restrict__ tape_x, float* __restrict__ tape_l) {
  if (num_local == 0) return;  // no constraint in the schedule
  extern __shared__ float4 smem[];
  float4* sx = smem;
  uint4* buf = reinterpret_cast<uint4*>(sx + max_foot);  // buf16 uint4 (see the launcher)
  uint64_t* bar = reinterpret_cast<uint64_t*>(buf + buf16);
  float* sl = reinterpret_cast<float*>(bar + 2);
  uint32_t* so = reinterpret_cast<uint32_t*>(sl + max_cons);
  uint32_t* sf = so + num_local + 1;
  const uint32_t t = tile_begin + blockIdx.x;
  const TileFrame f = tile_prologue<NT>(foot, meta, lofs, t, num_local, so);
  const uint32_t c0 = (uint32_t)f.m.z, nc = (uint32_t)f.m.w;
  const uint32_t* tl = lofs + (size_t)t * (num_local + 1);
  uint32_t src = 0;  // thread 0: the next segment's first uint4
  auto issue = [&](uint32_t l) {  // thread 0: the copy of color l's segment
    const uint32_t seg = color_seg16(__ldg(&tl[l + 1]) - __ldg(&tl[l]), 2);
    uint64_t* b = bar + (l & 1);
    if (seg)
      bulk_load_g2s(buf + (l & 1) * max_seg16, rec + src, 16u * seg, b);
    else
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
    src += seg;
  };
  if (threadIdx.x == 0) {
    src = __ldg(&rec_ofs[t]);
    mbar_init(bar, 1);
    mbar_init(bar + 1, 1);
    if (!STREAM) {  // the whole block at once
      const uint32_t all = __ldg(&rec_ofs[t + 1]) - src;
      if (all)
        bulk_load_g2s(buf, rec + src, 16u * all, bar);
      else
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
    } else {
      issue(0);
      if (num_local > 1) issue(1);
    }
  }
  pdl_wait();
#pragma unroll 4
  for (uint32_t j = threadIdx.x; j < nc; j += NT) sl[j] = RESET ? 0.0f : lambda[c0 + j];
  tile_gather<NT>(f, x, sx, sf);
  __syncthreads();  // offsets, footprint, multipliers and the barriers' initialisation
  auto failed = [&](bool ok, uint32_t l) {
    if (!__syncthreads_or(!ok)) return false;
    if (threadIdx.x == 0) {
      raise_error(err, kErrBulkCopy);
      if (!STREAM)
        mbar_wait_bounded(bar, 0, kBulkWaitLimit);
      else
        for (uint32_t k = l; k < l + 2 && k < num_local; ++k)
          mbar_wait_bounded(bar + (k & 1), (k >> 1) & 1u, kBulkWaitLimit);
    }
    __syncthreads();
    return true;
  };
  if (failed(mbar_wait_bounded(bar, 0, kBulkWaitLimit), 0)) return;
  uint32_t at = 0;  // whole block: the color's segment
  for (uint32_t l = 0; l < num_local; ++l) {
    const uint4* cur = STREAM ? buf + (l & 1) * max_seg16 : buf + at;
    const uint32_t cb = so[l], n = so[l + 1] - cb;
    const ushort2* sid = reinterpret_cast<const ushort2*>(cur);
    const float2* sval = reinterpret_cast<const float2*>(cur + (4 * n + 15) / 16);
    for (uint32_t j = threadIdx.x; j < n; j += NT) {
      const ushort2 ab = sid[j];
      const float2 rc = sval[j];
      float lam = sl[cb + j];
      float4 a = sx[ab.x], b = sx[ab.y];
      if (TAPE) {  // the adjoint's replay: the projection's inputs by execution slot
        const size_t slot = (size_t)f.m.z + cb + j;
        tape_x[2 * slot] = a;
        tape_x[2 * slot + 1] = b;
        tape_l[slot] = lam;
      }
      if (stretch_project_alpha(a, b, rc.x, rc.y, lam)) {
        sx[ab.x] = a;
        sx[ab.y] = b;
        sl[cb + j] = lam;
      }
    }
    if (!STREAM) {
      at += color_seg16(n, 2);
      __syncthreads();
      continue;
    }
    const bool ok = l + 1 >= num_local ||
                    mbar_wait_bounded(bar + ((l + 1) & 1), ((l + 1) >> 1) & 1u, kBulkWaitLimit);
    if (failed(ok, l + 1)) return;
    if (threadIdx.x == 0 && l + 2 < num_local) issue(l + 2);  // into the buffer color l read
  }
  pdl_release();  // late: the successor's blocks arrive as this one drains (measured faster)
  tile_scatter<NT>((uint32_t)f.m.y, x, sx, sf);
#pragma unroll 4
  for (uint32_t j = threadIdx.x; j < nc; j += NT) lambda[c0 + j] = sl[j];
}

__global__ void k_bend(const int4* __restrict__ idx, const float2* __restrict__ tc,
                       float4* __restrict__ x, uint32_t begin, uint32_t end, float dt) {
  pdl_release();
  pdl_wait();
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

// PAIR: two lanes per bend element (bend_project_pair), half the dependency chain per step, for
// launches whose tiles are all resident at once (latency-bound); otherwise one lane per element
// (fewer instructions in total, for launches with many waves of tiles).
// Records: the tile's record block (TiledSet::rec) holds one segment per local color (16-bit
// footprint-local ids, then float2 rest angle and bend_alpha(compliance, dt), each padded to 16
// bytes).
//   one lane (throughput regime): the segments stream in by local color, each bulk-copied into
//     one of two shared-memory buffers on its own mbarrier, two colors ahead of its use; a buffer
//     is refilled right after the barrier that closes the color that read it.  Only two colors'
//     records occupy shared memory, so more tiles fit on an SM.
//   lane pairs (latency regime, every tile of the launch resident): the whole block comes in one
//     bulk copy before the first color, so no color waits on a copy.
template <int NT, bool PAIR, bool TAPE>
__global__ void __launch_bounds__(NT, 1024 / NT) k_bend_tiles(
    const uint4* __restrict__ rec, const uint32_t* __restrict__ rec_ofs, float4* __restrict__ x,
    const uint32_t* __restrict__ foot, const int4* __restrict__ meta,
    const uint32_t* __restrict__ lofs, uint32_t tile_begin, uint32_t num_local,
    uint32_t max_foot, uint32_t max_seg16, uint32_t buf16, uint32_t* err,
    float4* __restrict__ tape_x) {
  if (num_local == 0) return;  // no constraint in the schedule
  extern __shared__ float4 smem[];
  float4* sx = smem;
  // buf16 uint4 of records: one lane, two buffers of max_seg16; lane pairs, the largest block
  uint4* buf = reinterpret_cast<uint4*>(sx + max_foot);
  uint64_t* bar = reinterpret_cast<uint64_t*>(buf + buf16);
  uint32_t* so = reinterpret_cast<uint32_t*>(bar + 2);
  uint32_t* sf = so + num_local + 1;
  const uint32_t t = tile_begin + blockIdx.x;
  const TileFrame f = tile_prologue<NT>(foot, meta, lofs, t, num_local, so);
  const uint32_t* tl = lofs + (size_t)t * (num_local + 1);
  uint32_t src = 0;  // thread 0: the next segment's first uint4
  auto issue = [&](uint32_t l) {  // thread 0: the copy of color l's segment
    const uint32_t seg = color_seg16(__ldg(&tl[l + 1]) - __ldg(&tl[l]), 4);
    uint64_t* b = bar + (l & 1);
    if (seg)
      bulk_load_g2s(buf + (l & 1) * max_seg16, rec + src, 16u * seg, b);
    else
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
    src += seg;
  };
  if (threadIdx.x == 0) {
    src = __ldg(&rec_ofs[t]);
    mbar_init(bar, 1);
    mbar_init(bar + 1, 1);
    if (PAIR) {  // the whole block at once (barrier 1 completes without a copy)
      const uint32_t all = __ldg(&rec_ofs[t + 1]) - src;
      if (all)
        bulk_load_g2s(buf, rec + src, 16u * all, bar);
      else
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
    } else {
      issue(0);
      if (num_local > 1) issue(1);
    }
  }
  pdl_wait();
  tile_gather<NT>(f, x, sx, sf);
  __syncthreads();  // offsets, footprint and the barriers' initialisation are visible
  // a wait that runs out raises the error; the block waits (bounded) for its copies in flight
  // and leaves, the same in every thread
  auto failed = [&](bool ok, uint32_t l) {
    if (!__syncthreads_or(!ok)) return false;
    if (threadIdx.x == 0) {
      raise_error(err, kErrBulkCopy);
      if (PAIR)  // the one copy of the whole block
        mbar_wait_bounded(bar, 0, kBulkWaitLimit);
      else
        for (uint32_t k = l; k < l + 2 && k < num_local; ++k)
          mbar_wait_bounded(bar + (k & 1), (k >> 1) & 1u, kBulkWaitLimit);
    }
    __syncthreads();
    return true;
  };
  if (failed(mbar_wait_bounded(bar, 0, kBulkWaitLimit), PAIR ? num_local : 0)) return;
  uint32_t at = 0;  // PAIR: the color's segment in the whole block
  for (uint32_t l = 0; l < num_local; ++l) {
    const uint4* cur = PAIR ? buf + at : buf + (l & 1) * max_seg16;
    const uint32_t c0 = so[l], n = so[l + 1] - c0;
    const ushort4* sid = reinterpret_cast<const ushort4*>(cur);
    const float2* st = reinterpret_cast<const float2*>(cur + (n + 1) / 2);
    if (PAIR) {
      // the loop trip count is warp-uniform so the pair exchanges run with full warps
      const uint32_t lane0 = threadIdx.x & ~31u, ce = 2 * n;
      for (uint32_t base = lane0; base < ce; base += NT) {
        const uint32_t s = base + (threadIdx.x & 31u);
        const bool active = s < ce;
        const uint32_t j = active ? s >> 1 : 0;
        const ushort4 q = sid[j];
        const int4 b = make_int4(q.x, q.y, q.z, q.w);
        const float2 th = st[j];
        if (TAPE && active) {  // the adjoint's replay: each lane tapes the two inputs it owns
          const uint32_t half = s & 1u;
          float4* t = tape_x + 4 * ((size_t)f.m.z + c0 + j) + 2 * half;
          t[0] = sx[half ? b.z : b.x];
          t[1] = sx[half ? b.w : b.y];
        }
        bend_project_pair(sx, b, th.x, th.y, s & 1u, active);
      }
    } else {
      for (uint32_t j = threadIdx.x; j < n; j += NT) {
        const ushort4 b = sid[j];
        const float2 th = st[j];
        float4 a1 = sx[b.x], a2 = sx[b.y], a3 = sx[b.z], a4 = sx[b.w];
        if (TAPE) {  // the adjoint's replay: the projection's inputs by execution slot
          float4* t = tape_x + 4 * ((size_t)f.m.z + c0 + j);
          t[0] = a1;
          t[1] = a2;
          t[2] = a3;
          t[3] = a4;
        }
        bend_project_alpha(a1, a2, a3, a4, th.x, th.y);
        sx[b.x] = a1;
        sx[b.y] = a2;
        sx[b.z] = a3;
        sx[b.w] = a4;
      }
    }
    if (PAIR) {
      at += color_seg16(n, 4);
      __syncthreads();
      continue;
    }
    // the next color's records, then the barrier that closes this color
    const bool ok = l + 1 >= num_local ||
                    mbar_wait_bounded(bar + ((l + 1) & 1), ((l + 1) >> 1) & 1u, kBulkWaitLimit);
    if (failed(ok, l + 1)) return;
    if (threadIdx.x == 0 && l + 2 < num_local) issue(l + 2);  // into the buffer color l read
  }
  pdl_release();
  tile_scatter<NT>((uint32_t)f.m.y, x, sx, sf);
}


// Free slot vertices: one launch per slot over that slot's constraint block (list order).
__global__ void k_lra_block(const uint32_t* __restrict__ tgt, const uint32_t* __restrict__ src,
                            const float* __restrict__ rest, float4* __restrict__ x, uint32_t begin,
                            uint32_t end, float stretch) {
  pdl_release();
  pdl_wait();
  const uint32_t k = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= end) return;
  const uint32_t t = tgt[k];
  const float4 p = x[t];
  const f3 xt = lra_project(mk3(p), mk3(x[src[k]]), p.w, rest[k], stretch);
  if (xt.x != p.x || xt.y != p.y || xt.z != p.z) x[t] = mk4(xt, p.w);
}


// Iteration tail, two Jacobi kernels (each reads x_in, writes x_out):
//   k_stage: LRA (SolveGeodesicLRA_Kernel, all slots pinned: slot positions are constant in the
//            phase) then SolveVFCCD_Kernel and SolveVFDCD_Kernel (PBDCollision.cu:279-298,
//            57-80) -- both update a vertex from its own data only;
//   k_ee:    SolveEEDCD_Kernel + ApplyDeltas_Kernel (PBDCollision.cu:163-212,
//            ClothSolverHelper.cu:139-148) and SolveBinding_Kernel (BindingConstraint.cu:56-92).
struct TailArgs {
  const float4* x_in;
  float4* x_out;
  uint32_t nv;
  const uint32_t *lra_ptr, *lra_src;  // per target vertex, slot order
  const float* lra_rest;
  float lra_stretch;
  const int *rt_idx, *vf_idx;
  const float4 *rt_qc, *vf_qs, *pred;
  const uint32_t *ve_ptr, *ve_list;
  const uint2* edge;
  const float4 *ee_a, *ee_b, *ee_c;
  const uint8_t* ee_vflag;  // per vertex: an incident edge holds a contact
  float relaxation;
  const uint32_t* bind_ptr;
  const float4* bind_a;
  const int4* bind_b;
  const float4* ox;
  float4* tape;     // TAPE (the adjoint's recorded replay): each vertex's input x_in
  float* tape_cnt;  // TAPE, k_ee: each vertex's EE contact count
};

// Position of vertex j after the LRA and VF phases.
template <bool LRA, bool CONTACTS>
__device__ __forceinline__ f3 tail_stage(const TailArgs& a, uint32_t j, const float4 p) {
  f3 q = mk3(p);
  if (LRA) {
    const uint32_t b = __ldg(&a.lra_ptr[j]), e = __ldg(&a.lra_ptr[j + 1]);
    if (b != e) {
      f3 xt = q;
      for (uint32_t k = b; k < e; ++k)
        xt = lra_project(xt, mk3(a.x_in[__ldg(&a.lra_src[k])]), p.w, __ldg(&a.lra_rest[k]),
                         a.lra_stretch);
      if (xt.x != p.x || xt.y != p.y || xt.z != p.z) q = xt;  // the phase writes only changes
    }
  }
  if (CONTACTS) {
    const int rc = a.rt_idx[j], vc = a.vf_idx[j];
    if (rc != -1) {
      const f3 nc = prim_normal(a.pred, rc);
      const float lambda = dot(nc, q - mk3(a.rt_qc[j]));
      if (lambda < 0) q = q + (-lambda * nc);
    }
    if (vc != -1) {
      const f3 ns = prim_normal(a.pred, vc);
      const float lambda = dot(ns, q - mk3(a.vf_qs[j])) - 1e-3f;
      if (lambda < 0) q = q + (-lambda * ns);
    }
  }
  return q;
}

// LRA + VF: x_out = tail_stage(x_in), per vertex.
template <bool LRA, bool CONTACTS, bool TAPE>
__global__ void k_stage(const TailArgs a) {
  pdl_release();
  pdl_wait();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nv) return;
  const float4 p = a.x_in[i];
  if (TAPE) a.tape[i] = p;
  a.x_out[i] = mk4(tail_stage<LRA, CONTACTS>(a, i, p), p.w);
}

// EE + ApplyDeltas + binding on the post-VF positions x_in.
template <bool CONTACTS, bool BINDINGS, bool TAPE>
__global__ void k_ee(const TailArgs a) {
  pdl_release();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nv = a.nv;
  // incident-edge list (setup-time) ahead of the wait
  constexpr int kBatch = 8;
  uint32_t kb = 0, ke = 0, code[kBatch];
  if (CONTACTS && i < nv) {
    kb = __ldg(&a.ve_ptr[i]);
    ke = __ldg(&a.ve_ptr[i + 1]);
#pragma unroll
    for (int r = 0; r < kBatch; ++r) code[r] = kb + r < ke ? __ldg(&a.ve_list[kb + r]) : 0u;
  }
  pdl_wait();
  if (i >= nv) return;
  const float4* __restrict__ x_in = a.x_in;
  const float4* __restrict__ ee_a = a.ee_a;
  const float4* __restrict__ ee_b = a.ee_b;
  const float4* __restrict__ ee_c = a.ee_c;
  const uint32_t* __restrict__ ve_list = a.ve_list;
  const float relaxation = a.relaxation;
  const float4 p = x_in[i];
  if (TAPE) a.tape[i] = p;
  f3 q = mk3(p);
  int count = 0;  // the EE contacts applied to this vertex
  // a vertex none of whose edges holds a contact skips the list (delta 0, count 0)
  if (CONTACTS && a.ee_vflag[i]) {
    f3 delta = mk3(0, 0, 0);
    // The contact-flag loads of a batch of incident edges are issued together; the edges are
    // then processed one by one in list order.
    for (uint32_t base = kb; base < ke; base += kBatch) {
      if (base != kb) {
#pragma unroll
        for (int r = 0; r < kBatch; ++r) code[r] = base + r < ke ? ve_list[base + r] : 0u;
      }
      float flag[kBatch];
#pragma unroll
      for (int r = 0; r < kBatch; ++r) flag[r] = base + r < ke ? ee_a[code[r] >> 1].x : 2e6f;
#pragma unroll
      for (int r = 0; r < kBatch; ++r) {
        if (flag[r] > 1e6f) continue;  // no contact on this edge (or past the list)
        const uint32_t e = code[r] >> 1;
        const float4 ca = ee_a[e];
        const float4 cb = ee_b[e], cc = ee_c[e];
        const uint2 ed = a.edge[e];
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
        const f3 corr = (code[r] & 1u) ? (-(s)*lambda * fn) : (-(1 - s) * lambda * fn);
        delta = delta + corr;
        ++count;
      }
    }
    const float fc = (float)count;
    if (fc > 0.0f) q = q + delta / fc * relaxation;
  }
  if (BINDINGS && p.w >= kEps) {
    for (uint32_t k = a.bind_ptr[i]; k < a.bind_ptr[i + 1]; ++k) {
      const float4 ba = a.bind_a[k];
      const int4 bb = a.bind_b[k];
      const float4* __restrict__ ox = a.ox;
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
  if (TAPE) a.tape_cnt[i] = (float)count;
  a.x_out[i] = mk4(q, p.w);
}

}  // namespace

void launch_predict(Context& c, const FrameConst& k) {
  launch_k(c.pdl, k_predict, grid_for(c.nv, c.vertex_block), c.vertex_block, 0, c.stream, c.x.p, c.x0.p, c.v.p, c.nv, k.dt,
           k.gx, k.gy, k.gz);
}

void launch_finalize_predict(Context& c, const FrameConst& k, bool predict_next, bool normals) {
  auto kern = predict_next ? k_finalize<true, false>
                           : (normals ? k_finalize<false, true> : k_finalize<false, false>);
  launch_k(c.pdl, kern, grid_for(c.nv, c.vertex_block), c.vertex_block, 0, c.stream, c.x.p, c.x0.p, c.v.p, c.nv, k.dt,
           k.damping, k.gx, k.gy, k.gz, c.tri.p, c.vf_ptr.p, c.vf_list.p, c.n.p);
}

void launch_stretch(Context& c, const FrameConst& k, ColorRange r, bool reset_lambda) {
  const uint32_t n = r.end - r.begin;
  if (n == 0) return;
  launch_k(c.pdl, reset_lambda ? k_stretch<true> : k_stretch<false>, grid_for(n), kBlock, 0,
           c.stream, c.s_con.p, c.s_lambda.p, c.x.p, r.begin, r.end, k.dt);
}

void launch_bend(Context& c, const FrameConst& k, ColorRange r) {
  const uint32_t n = r.end - r.begin;
  if (n == 0) return;
  launch_k(c.pdl, k_bend, grid_for(n), kBlock, 0, c.stream, c.b_idx.p, c.b_tc.p, c.x.p, r.begin,
           r.end, k.dt);
}

cudaError_t raise_smem(const void* kern, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> set;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = set[{dev, kern}];
  if (bytes <= cur) return cudaSuccess;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

// Every instantiation of the forward tile kernels, indexed by their template flags (reset, 512
// threads, streamed records, tape / 512 threads, lane pairs, tape).
using StretchTilesK = decltype(&k_stretch_tiles<false, 256, false, false>);
using BendTilesK = decltype(&k_bend_tiles<256, false, false>);
static const StretchTilesK kStretchTiles[16] = {
    k_stretch_tiles<false, 256, false, false>,
    k_stretch_tiles<false, 256, false, true>,
    k_stretch_tiles<false, 256, true, false>,
    k_stretch_tiles<false, 256, true, true>,
    k_stretch_tiles<false, 512, false, false>,
    k_stretch_tiles<false, 512, false, true>,
    k_stretch_tiles<false, 512, true, false>,
    k_stretch_tiles<false, 512, true, true>,
    k_stretch_tiles<true, 256, false, false>,
    k_stretch_tiles<true, 256, false, true>,
    k_stretch_tiles<true, 256, true, false>,
    k_stretch_tiles<true, 256, true, true>,
    k_stretch_tiles<true, 512, false, false>,
    k_stretch_tiles<true, 512, false, true>,
    k_stretch_tiles<true, 512, true, false>,
    k_stretch_tiles<true, 512, true, true>,
};
static const BendTilesK kBendTiles[8] = {
    k_bend_tiles<256, false, false>,
    k_bend_tiles<256, false, true>,
    k_bend_tiles<256, true, false>,
    k_bend_tiles<256, true, true>,
    k_bend_tiles<512, false, false>,
    k_bend_tiles<512, false, true>,
    k_bend_tiles<512, true, false>,
    k_bend_tiles<512, true, true>,
};
static StretchTilesK stretch_tiles_kernel(bool reset, bool b512, bool stream, bool tape) {
  return kStretchTiles[(reset ? 8 : 0) + (b512 ? 4 : 0) + (stream ? 2 : 0) + (tape ? 1 : 0)];
}
static BendTilesK bend_tiles_kernel(bool b512, bool pair, bool tape) {
  return kBendTiles[(b512 ? 4 : 0) + (pair ? 2 : 0) + (tape ? 1 : 0)];
}

// The limit is a property of the kernel function on the current device, shared by every
// context of the process, so it only ever grows: a context started later with smaller tiles
// must not lower it under one that is already running.
cudaError_t configure_tile_kernels(size_t max_smem_bytes) {
  static std::mutex mu;
  static std::map<int, int> configured;  // device -> bytes
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  int& cur = configured[dev];
  const int bytes = std::max(cur, (int)max_smem_bytes);
  if (bytes == cur) return cudaSuccess;
  for (const StretchTilesK kern : kStretchTiles) {
    e = cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
  }
  for (const BendTilesK kern : kBendTiles) {
    e = cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
  }
  cur = bytes;
  return cudaSuccess;
}

static_assert(512 * kFootPerThread >= (int)kTileMaxFootprint,
              "tile kernels hold every footprint vertex id in registers");

size_t tile_smem_bytes(const TiledSet& T, size_t record_bytes) {
  return sizeof(float4) * T.max_foot + record_bytes * T.max_cons +
         sizeof(uint32_t) * (T.num_local + 1) + sizeof(uint32_t) * T.max_foot;
}

// Shared memory of the forward tile kernels: footprint, records (`whole`: the tile's whole block;
// otherwise two colors' segments), two mbarriers, the stretch multipliers, offsets and footprint
// ids.
size_t tile_smem_fwd(const TiledSet& T, bool stretch, bool whole) {
  const size_t records = whole ? 16 * (size_t)T.max_tile16 + 16 : 32 * (size_t)T.max_seg16 + 16;
  return sizeof(float4) * T.max_foot + records + (stretch ? sizeof(float) * T.max_cons : 0) +
         sizeof(uint32_t) * (T.num_local + 1) + sizeof(uint32_t) * T.max_foot;
}

// Block size of a tile set: 256 threads when the footprint fits 256 x kFootPerThread and a local
// color's elements (two lanes each for bend) fill at most one pass, else 512; and how many of its
// bend blocks the GPU holds at once.
cudaError_t choose_tile_block(TiledSet& T, bool bend) {
  const uint32_t lanes = bend ? 2 * T.max_step : T.max_step;
  T.block = (T.max_foot <= 256u * kFootPerThread && lanes <= 256) ? 256 : 512;
  // streamed (throughput-regime) blocks: 256 threads whenever the footprint allows (a large color
  // takes a second pass, but twice the blocks fit on an SM)
  T.block1 = T.max_foot <= 256u * kFootPerThread ? 256 : T.block;
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const size_t smem = tile_smem_fwd(T, !bend, true);
  const void* kern = bend ? (const void*)bend_tiles_kernel(T.block != 256, true, false)
                          : (const void*)stretch_tiles_kernel(false, T.block != 256, false, false);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, (int)T.block, smem);
  if (e != cudaSuccess) return e;
  T.resident = (uint32_t)std::max(per_sm, 1) * (uint32_t)sms;
  return cudaSuccess;
}

// float4 {x, y, z, w} <-> packed xyz, for the host copies of the C ABI (one DMA of 12 B per
// element instead of 16 B and a host-side repacking loop).
static __global__ void k_pack_xyz(const float4* __restrict__ in, float* __restrict__ out,
                                  uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 v = in[i];
  out[3 * (size_t)i] = v.x;
  out[3 * (size_t)i + 1] = v.y;
  out[3 * (size_t)i + 2] = v.z;
}

static __global__ void k_unpack_xyz(const float* __restrict__ in, float4* __restrict__ out,
                                    uint32_t n, float w) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = make_float4(in[3 * (size_t)i], in[3 * (size_t)i + 1], in[3 * (size_t)i + 2], w);
}

void launch_pack_xyz(const float4* in, float* out, uint32_t n, cudaStream_t s) {
  if (n) k_pack_xyz<<<grid_for(n), kBlock, 0, s>>>(in, out, n);
}

void launch_unpack_xyz(const float* in, float4* out, uint32_t n, float w, cudaStream_t s) {
  if (n) k_unpack_xyz<<<grid_for(n), kBlock, 0, s>>>(in, out, n, w);
}

void launch_stretch_tiles(Context& c, const FrameConst& k, ColorRange tiles, bool reset_lambda,
                          float4* tape_x, float* tape_l) {
  const uint32_t nt = tiles.end - tiles.begin;
  if (nt == 0) return;
  const TiledSet& T = c.s_tiles;
  const bool stream = nt > T.resident;  // many waves of tiles: throughput regime
  const uint32_t block = stream ? T.block1 : T.block;
  const uint32_t buf16 = stream ? 2 * T.max_seg16 : T.max_tile16;  // as tile_smem_fwd sizes it
  const StretchTilesK kern = stretch_tiles_kernel(reset_lambda, block != 256, stream, tape_x);
  launch_k(c.pdl, kern, nt, block, tile_smem_fwd(T, true, !stream), c.stream, T.rec.p,
           T.rec_ofs.p, c.s_lambda.p, c.x.p, T.foot.p, T.meta.p, T.lofs.p, tiles.begin,
           T.num_local, T.max_foot, T.max_seg16, buf16, T.max_cons, c.err.p, tape_x, tape_l);
}

void launch_bend_tiles(Context& c, const FrameConst& k, ColorRange tiles, float4* tape_x) {
  const uint32_t nt = tiles.end - tiles.begin;
  if (nt == 0) return;
  const TiledSet& T = c.b_tiles;
  // two lanes per element when the launch's tiles are all resident (latency-bound: halve the
  // chain), or when every local color's lane pairs fit one pass of the block (the pairs then
  // use lanes that would idle at the color's barrier)
  const bool pair = nt <= T.resident || 2 * T.max_step <= T.block;
  const uint32_t block = pair ? T.block : T.block1;
  const BendTilesK kern = bend_tiles_kernel(block != 256, pair, tape_x);
  const uint32_t buf16 = pair ? T.max_tile16 : 2 * T.max_seg16;  // as tile_smem_fwd sizes it
  launch_k(c.pdl, kern, nt, block, tile_smem_fwd(T, false, pair), c.stream, T.rec.p, T.rec_ofs.p,
           c.x.p, T.foot.p, T.meta.p, T.lofs.p, tiles.begin, T.num_local, T.max_foot, T.max_seg16,
           buf16, c.err.p, tape_x);
}

// LRA phase with a free slot vertex: one launch per slot block in list order.  (With every slot
// vertex pinned, slot positions are constant during the phase and it runs per target inside
// k_tail.)
void launch_lra(Context& c, const FrameConst& k) {
  if (c.nl == 0) return;
  for (const ColorRange& r : c.lra_blocks)
    launch_k(c.pdl, k_lra_block, grid_for(r.end - r.begin), kBlock, 0, c.stream, c.lra_l_tgt.p,
             c.lra_l_src.p, c.lra_l_rest.p, c.x.p, r.begin, r.end, k.lra_stretch);
}

static TailArgs tail_args(Context& c, const FrameConst& k) {
  TailArgs a;
  a.x_in = c.x.p;
  a.x_out = c.x_alt.p;
  a.nv = c.nv;
  a.lra_ptr = c.lra_ptr.p;
  a.lra_src = c.lra_src.p;
  a.lra_rest = c.lra_rest.p;
  a.lra_stretch = k.lra_stretch;
  a.rt_idx = c.rt_idx.p;
  a.vf_idx = c.vf_idx.p;
  a.rt_qc = c.rt_qc.p;
  a.vf_qs = c.vf_qs.p;
  a.pred = c.bvh.pred.p;
  a.ve_ptr = c.ve_ptr.p;
  a.ve_list = c.ve_list.p;
  a.edge = c.edge.p;
  a.ee_a = c.ee_a.p;
  a.ee_b = c.ee_b.p;
  a.ee_c = c.ee_c.p;
  a.ee_vflag = c.ee_vflag.p;
  a.relaxation = k.relaxation;
  a.bind_ptr = c.bind_ptr.p;
  a.bind_a = c.bind_a.p;
  a.bind_b = c.bind_b.p;
  a.ox = c.ox.p;
  a.tape = nullptr;
  a.tape_cnt = nullptr;
  return a;
}

void launch_stage(Context& c, const FrameConst& k, bool lra, bool contacts, float4* tape) {
  if (!lra && !contacts) return;
  auto kern = tape ? (lra ? (contacts ? k_stage<true, true, true> : k_stage<true, false, true>)
                          : k_stage<false, true, true>)
                   : (lra ? (contacts ? k_stage<true, true, false> : k_stage<true, false, false>)
                          : k_stage<false, true, false>);
  TailArgs a = tail_args(c, k);
  a.tape = tape;
  launch_k(c.pdl, kern, grid_for(c.nv, c.vertex_block), c.vertex_block, 0, c.stream, a);
}

void launch_ee(Context& c, const FrameConst& k, bool contacts, bool bindings, float4* tape,
               float* tape_cnt) {
  if (!contacts && !bindings) return;
  auto kern = tape ? (contacts ? (bindings ? k_ee<true, true, true> : k_ee<true, false, true>)
                               : k_ee<false, true, true>)
                   : (contacts ? (bindings ? k_ee<true, true, false> : k_ee<true, false, false>)
                               : k_ee<false, true, false>);
  TailArgs a = tail_args(c, k);
  a.tape = tape;
  a.tape_cnt = tape_cnt;
  launch_k(c.pdl, kern, grid_for(c.nv, c.vertex_block), c.vertex_block, 0, c.stream, a);
}

}  // namespace xrt
