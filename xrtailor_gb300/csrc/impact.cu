// impact.cu — the impact-zone collision step of XRTailor's Quality mode on the GB300.
//
//   CollisionStep ........................ xrtailor/src/physics/impact_zone/Entry.cu:140-256
//   FindImpacts .......................... ImpactHelper.cu:207-232 (pairs, CheckImpacts, compaction)
//   independentImpacts ................... Entry.cu:25-63, ImpactHelper.cu:234-343
//   IsolateImpacts / AddImpacts / Flatten  ImpactZoneHelper.cu:31-120, 214-396; ImpactZone.cu:47-83
//   ParallelImpactZoneOptimizer .......... ParallelImpactZoneOptimizer.cu:13-528,
//                                          ParallelOptimizer.cu:45-880 (Solve)
//
// Device: the LBVHs over x0 -> x boxes, face pairs and the 15 CCD tests per pair (proximity.cu),
// the compaction of the impacts found, the impact store, and the zone solve.  The reference runs
// the augmented-Lagrangian solve of all zones as one sequence of grid-wide launches with a host
// round trip per line-search step; here one 256-thread block owns one zone and runs its whole
// solve (up to 100 iterations, each with its backtracking search) with block reductions only.
// A zone's arithmetic does not depend on the others, so this gives the reference's per-zone
// results; the one coupling, which zones skip the last position copy, is settled by
// k_zone_finalize.
//
// Host: the bookkeeping of the impact graph between the device stages (sort by time of impact,
// independence rounds, mesh-adjacency flood fill, zone merging), over the few hundred to few
// thousand impacts of a pass, as the reference's own host loop and single-thread kernels do.
//
// Sums over a zone follow the reference's blocked reduction (ReduceBaselineLocal/Global_Kernel,
// ParallelOptimizer.cu:335-428): 256-element blocks summed by the stride tree s[t] += s[t + d],
// d = 1, 2, ..., 128, then the block sums by the same tree.  With --fmad=false every value is the
// IEEE result of the reference's expression order.
#include <mutex>
#include <cooperative_groups.h>

#include <algorithm>
#include <iterator>
#include <numeric>

#include "common.cuh"
#include "context.h"

namespace cg = cooperative_groups;

namespace xrt {
namespace {

constexpr int kZT = 256;              // threads of a zone block = IZO_BLOCK_SIZE
constexpr int kZoneCluster = 8;       // blocks per zone of more than 256 nodes or impacts
constexpr int kZoneClusterWide = 16;  // blocks per zone of more than 2,048 (non-portable size)
constexpr int kWideGroups = 4;        // 256-thread groups per block of those clusters
constexpr int kMaxChunks = 256;       // 256 x 256 nodes / impacts per zone (the reduction's reach)
constexpr int kMaxOptIters = 100;     // MAX_ITERATIONS (ParallelOptimizer.cuh)
constexpr int kMaxLineSearch = 1024;  // the reference's search ends by s < 1e-12 within ~110 steps
constexpr int kMaxPasses = 100;       // MAX_COLLISION_ITERATION (ImpactHelper.cuh:41)
constexpr float kMu = 1e3f;           // mu_ (ParallelOptimizer.cu:533)
constexpr float kAlpha = 0.5f;        // ALPHA, Wolfe condition
constexpr float kEpsS = 1e-12f;       // EPSILON_S
constexpr float kEpsF = 1e-10f;       // EPSILON_F
constexpr float kStepCoeff = 1e-3f;   // STEP_LENGTH_COEFF_SCALAR

__device__ __forceinline__ float comp4(float4 v, int j) {
  return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}

// Two sums of one value per thread each, every thread getting both; the tree256 order, taken
// separately by every group of 256 threads of the block.  ws: 18 floats per group; callers
// alternate two ws buffers, so a call needs no barrier after its reads.
__device__ __forceinline__ void tree256_2(float& a, float& b, float* wsg) {
  const int lane = threadIdx.x & 31, warp = (threadIdx.x >> 5) & 7;
  float* ws = wsg + 18 * (threadIdx.x >> 8);
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const float oa = __shfl_down_sync(0xFFFFFFFFu, a, d);
    const float ob = __shfl_down_sync(0xFFFFFFFFu, b, d);
    if ((lane & (2 * d - 1)) == 0) {
      a += oa;
      b += ob;
    }
  }
  if (lane == 0) {
    ws[warp] = a;
    ws[9 + warp] = b;
  }
  __syncthreads();
  if (warp == 0) {
    float u = lane < 8 ? ws[lane] : 0.0f, w = lane < 8 ? ws[9 + lane] : 0.0f;
#pragma unroll
    for (int d = 1; d < 8; d <<= 1) {
      const float ou = __shfl_down_sync(0xFFFFFFFFu, u, d);
      const float ow = __shfl_down_sync(0xFFFFFFFFu, w, d);
      if ((lane & (2 * d - 1)) == 0) {
        u += ou;
        w += ow;
      }
    }
    if (lane == 0) {
      ws[8] = u;
      ws[17] = w;
    }
  }
  __syncthreads();
  a = ws[8];
  b = ws[17];
}

// Sum of one value per thread of a 256-thread block in the order of the reference's stride tree:
// pairs within a warp by shuffles, then the 8 warp sums by the same pattern.  Every thread gets
// the sum.  ws: 9 floats of shared memory.
__device__ float tree256(float v, float* ws) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const float o = __shfl_down_sync(0xFFFFFFFFu, v, d);
    if ((lane & (2 * d - 1)) == 0) v += o;
  }
  if (lane == 0) ws[warp] = v;
  __syncthreads();
  if (warp == 0) {
    float u = lane < 8 ? ws[lane] : 0.0f;
#pragma unroll
    for (int d = 1; d < 8; d <<= 1) {
      const float o = __shfl_down_sync(0xFFFFFFFFu, u, d);
      if ((lane & (2 * d - 1)) == 0) u += o;
    }
    if (lane == 0) ws[8] = u;
  }
  __syncthreads();
  const float r = ws[8];
  __syncthreads();
  return r;
}

struct ZoneArgs {
  const int4* zone;        // entry begin, entry end, node begin, node end
  const uint32_t* zimp;    // store id per entry
  const int32_t* zloc;     // 4 per entry
  const uint32_t* znode;   // unified node per node position
  const uint32_t* gptr;    // per node position: slots [gptr[k], gptr[k + 1])
  const uint32_t* gslot;   // 4 entry + j
  const float4* sw;
  const float4* sn;
  const uint4* snodes;
  const float4* cx;        // cloth x (w = inverse mass)
  const float4* ox;        // obstacle x
  const float4* cx1;       // Node::x1
  const float4* ox1;
  float4* X;
  float4* Xt;
  float4* grad;
  float* lambda;
  float* cc;
  int32_t* conv;
  const float* inv_avg;
  uint32_t V;
  float obstacle_mass;
  float thickness;
  uint32_t* err;
};

__device__ __forceinline__ f3 pos_of(const ZoneArgs& a, uint32_t v) {
  return v < a.V ? mk3(a.cx[v]) : mk3(a.ox[v - a.V]);
}
__device__ __forceinline__ f3 x1_of(const ZoneArgs& a, uint32_t v) {
  return v < a.V ? mk3(a.cx1[v]) : mk3(a.ox1[v - a.V]);
}
// CollisionObjective_Kernel: is_cloth ? 1 / inv_mass : obstacle_mass
__device__ __forceinline__ float mass_of(const ZoneArgs& a, uint32_t v) {
  return v < a.V ? 1.0f / a.cx[v].w : a.obstacle_mass;
}

// CollisionConstraint_Kernel: -thickness + sum_j w_j dot(n, x_j), x_j the optimizer's copy of an
// optimized node, else the node's position.
__device__ __forceinline__ float constraint_at(const ZoneArgs& a, int e, const float4* Xs) {
  const uint32_t id = a.zimp[e];
  const float4 w = a.sw[id];
  const f3 n = mk3(a.sn[id]);
  const uint4 nd = a.snodes[id];
  const uint32_t nds[4] = {nd.x, nd.y, nd.z, nd.w};
  float c = -a.thickness;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int k = a.zloc[4 * e + j];
    const f3 x = k > -1 ? mk3(__ldcg(&Xs[k])) : pos_of(a, nds[j]);
    c += comp4(w, j) * dot(n, x);
  }
  return c;
}

template <int C>
__device__ __forceinline__ void zone_sync(cg::cluster_group& cl) {
  if constexpr (C == 1) {
    __syncthreads();
  } else {
    cl.sync();
  }
}

// One zone per cluster of C blocks (C = 1 for zones of at most 256 nodes and impacts).  Block r
// of the cluster owns the 256-element chunks ch = r, r + C, ...: it computes their values and
// chunk sums and writes the sums into block 0's shared memory (distributed shared memory); after
// a cluster barrier every block reads the chunk sums from block 0 and sums them by the same
// tree, so every block of the cluster holds the same totals and takes the same branches.  The
// chunk sums alternate between two buffer sets: a set is written again only after a later
// barrier that every block reaches after its reads.  Zone arrays written by one block and read
// by others go through L2 (ld/st .cg) and are published by a barrier before they are read.
// A block has G groups of 256 threads; group g of block r owns chunks r G + g, (r + C) G + g, ...
template <int C, int G>
__global__ void __cluster_dims__(C, 1, 1) __launch_bounds__(kZT * G)
    k_zone_solve(ZoneArgs a, const int32_t* __restrict__ zid) {
  __shared__ float part[2 * 2 * kMaxChunks];  // [buffer set][quantity][chunk], read in block 0
  __shared__ float wsb[2 * 18 * G];
  cg::cluster_group cl = cg::this_cluster();
  const int tid = threadIdx.x;
  const int grp = tid >> 8, lt = tid & (kZT - 1);  // group, thread of the group
  const int rank = (int)cl.block_rank();
  const int zi = zid[blockIdx.x / C];
  float* lead = cl.map_shared_rank(part, 0);
  int set = 0, wsp = 0;
  auto buf = [&](int q) { return lead + (2 * set + q) * kMaxChunks; };
  auto tree2 = [&](float& x, float& y) {
    tree256_2(x, y, wsb + 18 * G * wsp);
    wsp ^= 1;
  };
  // the chunk sums of a quantity pair, then the totals of both (every group takes the same tree)
  auto totals = [&](int nch, float& x, float& y) {
    x = lt < nch ? buf(0)[lt] : 0.0f;
    y = lt < nch ? buf(1)[lt] : 0.0f;
    tree2(x, y);
    set ^= 1;
  };
  const int4 z = a.zone[zi];
  const int eb = z.x, ni = z.y - z.x, nb = z.z, nn = z.w - z.z;
  if (ni > kZT * kMaxChunks || nn > kZT * kMaxChunks) {
    if (tid == 0 && rank == 0) {
      raise_error(a.err, kErrZoneSize);
      a.conv[zi] = -1;  // positions stay
    }
    return;
  }
  const int nce = (ni + kZT - 1) / kZT, ncn = (nn + kZT - 1) / kZT;
  const int first = rank * G * kZT + tid, stride = C * G * kZT;  // this block's elements
  for (int k = first; k < nn; k += stride) {  // Initialize_Kernel
    const float4 p = mk4(pos_of(a, a.znode[nb + k]), 0.0f);
    __stcg(&a.X[nb + k], p);
    __stcg(&a.Xt[nb + k], p);
  }
  for (int e = first; e < ni; e += stride) __stcg(&a.lambda[eb + e], 0.0f);
  zone_sync<C>(cl);
  const float inv = *a.inv_avg;
  float s = kStepCoeff * (float)nn;  // InitStepLength_Kernel
  int conv_it = kMaxOptIters;
  float zero = 0.0f;
  for (int it = 0; it < kMaxOptIters; ++it) {
    // constraints at X: coefficients min(c + lambda / mu, 0), C2 and lambda2
    for (int cb = rank * G; cb < nce; cb += C * G) {
      const int ch = cb + grp, e = ch * kZT + lt;
      float c2 = 0.0f, l2 = 0.0f;
      if (e < ni) {
        const float lam = __ldcg(&a.lambda[eb + e]);
        const float q = tmin(constraint_at(a, eb + e, a.X) + lam / kMu, 0.0f);
        __stcg(&a.cc[eb + e], q);
        c2 = q * q;
        l2 = lam * lam;
      }
      tree2(c2, l2);
      if (lt == 0 && ch < nce) {
        buf(0)[ch] = c2;
        buf(1)[ch] = l2;
      }
    }
    zone_sync<C>(cl);
    float C2, L2;
    totals(nce, C2, L2);
    // gradient at X: inv * m * (x - x1) + sum of mu * coefficient * w_j * n (slot order); G2, O
    for (int cb = rank * G; cb < ncn; cb += C * G) {
      const int ch = cb + grp, k = ch * kZT + lt;
      float g2 = 0.0f, o = 0.0f;
      if (k < nn) {
        const int idx = nb + k;
        const uint32_t v = a.znode[idx];
        const f3 x = mk3(__ldcg(&a.X[idx])), x1 = x1_of(a, v);
        const float m = mass_of(a, v);
        f3 g = (inv * m) * (x - x1);
        f3 acc = mk3(0.0f, 0.0f, 0.0f);
        for (uint32_t q = a.gptr[idx]; q < a.gptr[idx + 1]; ++q) {
          const uint32_t slot = a.gslot[q];
          const int e = (int)(slot >> 2), j = (int)(slot & 3u);
          const uint32_t id = a.zimp[e];
          const f3 t = ((kMu * __ldcg(&a.cc[e])) * comp4(a.sw[id], j)) * mk3(a.sn[id]);
          acc = q == a.gptr[idx] ? t : acc + t;
        }
        g = g + acc;
        __stcg(&a.grad[idx], mk4(g, 0.0f));
        g2 = dot(g, g);
        const f3 d = x - x1;
        o = m * dot(d, d);
      }
      tree2(g2, o);
      if (lt == 0 && ch < ncn) {
        buf(0)[ch] = g2;
        buf(1)[ch] = o;
      }
    }
    zone_sync<C>(cl);
    float G2, O;
    totals(ncn, G2, O);
    const float f = (0.5f * inv) * O + (0.5f * kMu) * C2 - (0.5f * L2) / kMu;
    s = s / 0.7f;  // PreconditionStepLength_Kernel
    for (int ls = 0;; ++ls) {
      s = s * 0.7f;  // AdjustStepLength_Kernel
      for (int cb = rank * G; cb < ncn; cb += C * G) {  // NextX_Kernel + CollisionObjective_Kernel
        const int ch = cb + grp, k = ch * kZT + lt;
        float o = 0.0f;
        if (k < nn) {
          const int idx = nb + k;
          const uint32_t v = a.znode[idx];
          const f3 xt = mk3(__ldcg(&a.X[idx])) - s * mk3(__ldcg(&a.grad[idx]));
          __stcg(&a.Xt[idx], mk4(xt, 0.0f));
          const f3 d = xt - x1_of(a, v);
          o = mass_of(a, v) * dot(d, d);
        }
        tree2(o, zero);
        if (lt == 0 && ch < ncn) buf(0)[ch] = o;
      }
      zone_sync<C>(cl);  // also publishes Xt
      for (int cb = rank * G; cb < nce; cb += C * G) {
        const int ch = cb + grp, e = ch * kZT + lt;
        float c2 = 0.0f;
        if (e < ni) {
          const float q = tmin(constraint_at(a, eb + e, a.Xt) + __ldcg(&a.lambda[eb + e]) / kMu,
                               0.0f);
          c2 = q * q;
        }
        tree2(c2, zero);
        if (lt == 0 && ch < nce) buf(1)[ch] = c2;
      }
      zone_sync<C>(cl);
      // Ot over the nodes' chunks, C2t over the impacts' chunks
      float Ot = lt < ncn ? buf(0)[lt] : 0.0f, C2t = lt < nce ? buf(1)[lt] : 0.0f;
      tree2(Ot, C2t);
      set ^= 1;
      // BacktrackingLineSearchAdvanced_Kernel (ParallelImpactZoneOptimizer.cu:413-497)
      const float ft = (0.5f * inv) * Ot + (0.5f * kMu) * C2t - (0.5f * L2) / kMu;
      if (s < kEpsS || ft < f - (kAlpha * s) * G2 || tabs(f - ft) < kEpsF) break;
      if (ls + 1 >= kMaxLineSearch) {  // only a non-finite objective gets here
        if (tid == 0 && rank == 0) raise_error(a.err, kErrLineSearch);
        s = 0.0f;
        break;
      }
    }
    if (s < kEpsS) {  // UpdateConvergency_Kernel
      conv_it = it;
      break;
    }
    for (int k = first; k < nn; k += stride)  // current_X = next_X
      __stcg(&a.X[nb + k], __ldcg(&a.Xt[nb + k]));
    zone_sync<C>(cl);
    for (int e = first; e < ni; e += stride) {  // UpdateMultiplier_Kernel (own impacts only)
      const float c = constraint_at(a, eb + e, a.X);
      __stcg(&a.lambda[eb + e], tmin(__ldcg(&a.lambda[eb + e]) + kMu * c, 0.0f));
    }
  }
  if (tid == 0 && rank == 0) a.conv[zi] = conv_it;
}

// 16-block clusters need the non-portable cluster size opt-in; they are used once the device
// reports that it can hold one (else zones stay on 8-block clusters).
// Which 16-block clusters the current device holds: bit 0 with blocks of 256 threads, bit 1 with
// blocks of 1,024 (kWideGroups groups).  The opt-in is a per-device function attribute, so the
// answer is established and cached once per device, under a lock.
int wide_clusters() {
  constexpr int kMaxDevices = 256;
  static std::mutex lock;
  static int state[kMaxDevices];
  static bool known[kMaxDevices] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 0;
  std::lock_guard<std::mutex> guard(lock);
  if (!known[dev]) {
    int st = 0;
    auto fits = [](const void* k, int threads) {
      if (cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
        return false;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(kZoneClusterWide);
      cfg.blockDim = dim3(threads);
      int n = 0;
      return cudaOccupancyMaxActiveClusters(&n, k, &cfg) == cudaSuccess && n > 0;
    };
    if (fits((const void*)k_zone_solve<kZoneClusterWide, 1>, kZT)) st |= 1;
    if (fits((const void*)k_zone_solve<kZoneClusterWide, kWideGroups>, kWideGroups * kZT))
      st |= 2;
    (void)cudaGetLastError();  // a refused opt-in is not an error of the step
    state[dev] = st;
    known[dev] = true;
  }
  return state[dev];
}

// Finalize_Kernel.  The reference's iteration loop stops once every zone has converged, before
// the position copy of that iteration, so the zones converging last keep X; every other zone
// (and every zone if one never converged) took the copy X = Xt at its convergence iteration.
__global__ void __launch_bounds__(kZT) k_zone_finalize(const int4* __restrict__ zone,
                                                       const int32_t* __restrict__ conv,
                                                       uint32_t nzones, const uint32_t* znode,
                                                       const float4* __restrict__ X,
                                                       const float4* __restrict__ Xt, float4* cx,
                                                       float4* ox, uint32_t V) {
  __shared__ int km[kZT / 32];
  int k = -1;
  for (uint32_t q = threadIdx.x; q < nzones; q += kZT) k = max(k, conv[q]);
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) k = max(k, __shfl_xor_sync(0xFFFFFFFFu, k, d));
  if ((threadIdx.x & 31) == 0) km[threadIdx.x >> 5] = k;
  __syncthreads();
  int K = km[0];
  for (int w = 1; w < kZT / 32; ++w) K = max(K, km[w]);
  const int c = conv[blockIdx.x];
  if (c < 0) return;  // zone too large: not solved
  const bool keep = c == K && K < kMaxOptIters;
  const int4 z = zone[blockIdx.x];
  for (int i = z.z + (int)threadIdx.x; i < z.w; i += kZT) {
    const f3 p = mk3(keep ? X[i] : Xt[i]);
    const uint32_t v = znode[i];
    if (v < V) {
      cx[v] = mk4(p, cx[v].w);
    } else {
      ox[v - V] = mk4(p, ox[v - V].w);
    }
  }
}

// CollisionInv_Kernel + thrust::reduce / n_nodes: the mean inverse mass over every optimized node
// of the active zones.  One block; the sum is the blocked stride tree, repeated over the block
// sums until one value is left.
__global__ void __launch_bounds__(kZT) k_inv_avg(const uint32_t* __restrict__ znode, uint32_t n,
                                                 const float4* __restrict__ cx, uint32_t V,
                                                 float obstacle_mass, float* __restrict__ partial,
                                                 float* __restrict__ out) {
  __shared__ float ws[9];
  uint32_t m = n;
  for (uint32_t ch = 0; ch * kZT < m; ++ch) {
    const uint32_t i = ch * kZT + threadIdx.x;
    float v = 0.0f;
    if (i < m) {
      const uint32_t id = znode[i];
      v = id < V ? cx[id].w : 1.0f / obstacle_mass;
    }
    v = tree256(v, ws);
    if (threadIdx.x == 0) partial[ch] = v;
  }
  __syncthreads();
  m = (m + kZT - 1) / kZT;
  while (true) {
    const uint32_t nch = (m + kZT - 1) / kZT;
    for (uint32_t ch = 0; ch < nch; ++ch) {
      const uint32_t i = ch * kZT + threadIdx.x;
      float v = i < m ? partial[i] : 0.0f;
      v = tree256(v, ws);
      if (threadIdx.x == 0) partial[ch] = v;  // ch <= i: read before written
      __syncthreads();
    }
    if (nch <= 1) break;
    m = nch;
  }
  if (threadIdx.x == 0) *out = n ? partial[0] / (float)n : 0.0f;
}

// impacts (t >= 0) per pair: the IsNull filter of FindImpacts
__global__ void k_count_hits(const float* __restrict__ t, uint32_t np, uint32_t* __restrict__ hits) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  uint32_t c = 0;
  for (int k = 0; k < 15; ++k) c += !(t[15 * (size_t)p + k] < 0.0f);
  hits[p] = c;
}

// thrust::remove_if (stable): the impacts in (pair, test) order
__global__ void k_compact_hits(const float* __restrict__ t, const uint4* __restrict__ nodes,
                               uint32_t np, const uint32_t* __restrict__ incl,
                               float* __restrict__ out_t, uint4* __restrict__ out_nodes,
                               uint32_t* __restrict__ out_src) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  uint32_t o = p ? incl[p - 1] : 0u;
  for (int k = 0; k < 15; ++k) {
    const size_t i = 15 * (size_t)p + k;
    const float tt = t[i];
    if (tt < 0.0f) continue;
    out_t[o] = tt;
    out_nodes[o] = nodes[i];
    out_src[o] = (uint32_t)i;
    ++o;
  }
}

// Appends the independent impacts (compacted ids) to the step's impact store.
__global__ void k_store_gather(const uint32_t* __restrict__ pick, uint32_t n,
                               const uint32_t* __restrict__ src, const float4* __restrict__ w,
                               const float4* __restrict__ nrm, const uint4* __restrict__ nodes,
                               uint32_t base, float4* sw, float4* sn, uint4* snodes) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t c = pick[i], s = src[c];
  sw[base + i] = w[s];
  sn[base + i] = nrm[s];
  snodes[base + i] = nodes[c];
}

template <typename T>
cudaError_t put(DBuf<T>& d, const std::vector<T>& h, cudaStream_t s) {
  cudaError_t e = d.reserve(h.empty() ? 1 : h.size());
  if (e != cudaSuccess || h.empty()) return e;
  return cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

// Grows a buffer keeping its first `keep` elements (stream-ordered copy).
template <typename T>
cudaError_t grow_keep(DBuf<T>& d, size_t count, size_t keep, cudaStream_t s) {
  if (count <= d.n && d.p) return cudaSuccess;
  DBuf<T> nb;
  cudaError_t e = nb.reserve(std::max(count, 2 * d.n));
  if (e != cudaSuccess) return e;
  if (keep) e = cudaMemcpyAsync(nb.p, d.p, keep * sizeof(T), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    nb.release();
    return e;
  }
  d.release();
  d = nb;
  return cudaSuccess;
}

void csr_node_faces(const std::vector<uint32_t>& tri, uint32_t nv, std::vector<uint32_t>& ptr,
                    std::vector<uint32_t>& list) {
  ptr.assign(nv + 1, 0);
  for (uint32_t v : tri) ptr[v + 1]++;
  for (uint32_t i = 0; i < nv; ++i) ptr[i + 1] += ptr[i];
  list.assign(tri.size(), 0);
  std::vector<uint32_t> fill(ptr.begin(), ptr.end() - 1);
  for (uint32_t f = 0; f < tri.size() / 3; ++f)
    for (int k = 0; k < 3; ++k) list[fill[tri[3 * f + k]]++] = f;
}

// ---- host bookkeeping ----------------------------------------------------------------------------

struct Graph {
  const Context& c;
  const ImpactZoneState& z;
  int deform;
  bool is_free(uint32_t v) const { return v < c.nv && c.h_cfree[v] != 0; }
  // nodes the independence test and the flood fill treat as movable (deform == 1 || is_free)
  bool deformable(uint32_t v) const { return deform == 1 || is_free(v); }
  // nodes the optimizer moves: free cloth nodes; at deform 1 also obstacle nodes (pinned cloth
  // nodes keep their positions: their mass 1 / 0 would make the objective NaN)
  bool optimized(uint32_t v) const { return is_free(v) || (deform == 1 && v >= c.nv); }
};

// independentImpacts: `order` = compacted ids by time of impact; returns the ids of the impacts
// each of which is, in rounds, the earliest unremoved impact at every deformable node it has.
std::vector<uint32_t> independent_impacts(const Graph& g, const std::vector<uint32_t>& order,
                                          const std::vector<uint4>& nodes, uint32_t num_nodes) {
  const uint32_t n = (uint32_t)order.size();
  std::vector<uint8_t> removed(num_nodes, 0), selected(n, 0);
  std::vector<uint32_t> min_index(num_nodes, n);
  auto nd = [&](uint32_t r, int j) {
    const uint4 q = nodes[order[r]];
    return j == 0 ? q.x : (j == 1 ? q.y : (j == 2 ? q.z : q.w));
  };
  uint32_t num, new_num = n;
  do {
    num = new_num;
    std::vector<uint32_t> touched;
    for (uint32_t r = 0; r < n; ++r) {  // CollectRelativeImpacts + reduce_by_key(minimum)
      bool avail = true;
      for (int j = 0; j < 4; ++j)
        if (g.deformable(nd(r, j)) && removed[nd(r, j)]) avail = false;
      if (!avail) continue;
      for (int j = 0; j < 4; ++j) {
        const uint32_t v = nd(r, j);
        if (!g.deformable(v)) continue;
        if (min_index[v] == n) touched.push_back(v);
        min_index[v] = std::min(min_index[v], r);
      }
    }
    for (uint32_t r = 0; r < n; ++r) {  // CheckIndependentImpacts
      bool ok = true;
      for (int j = 0; j < 4; ++j) {
        const uint32_t v = nd(r, j);
        if (g.deformable(v) && (removed[v] || min_index[v] != r)) ok = false;
      }
      if (!ok) continue;
      selected[r] = 1;
      for (int j = 0; j < 4; ++j)
        if (g.deformable(nd(r, j))) removed[nd(r, j)] = 1;
    }
    for (uint32_t v : touched) min_index[v] = n;
    new_num = n - (uint32_t)std::count(selected.begin(), selected.end(), 1);
  } while (num > new_num);
  std::vector<uint32_t> out;
  for (uint32_t r = 0; r < n; ++r)
    if (selected[r]) out.push_back(order[r]);
  return out;
}

// IsolateImpacts: new impacts (store ids, in order) grouped by a flood fill from the first
// ungrouped impact over the faces around its nodes (a cloth node spreads only when free).  An
// impact none of whose nodes the fill reaches (all its nodes pinned) is dropped; the reference
// would stop after 100 zones with it unassigned.
std::vector<HostZone> isolate(const Graph& g, const std::vector<uint32_t>& ids) {
  const Context& c = g.c;
  const ImpactZoneState& z = g.z;
  const uint32_t NV = c.nv + c.onv;
  constexpr int kOutside = -2, kInside = -1;
  std::vector<int> color(NV, kOutside);
  auto node = [&](uint32_t id, int j) {
    const uint4 q = z.h_snodes[id];
    return j == 0 ? q.x : (j == 1 ? q.y : (j == 2 ? q.z : q.w));
  };
  for (uint32_t id : ids)
    for (int j = 0; j < 4; ++j) color[node(id, j)] = kInside;
  std::vector<int> icolor(ids.size(), -1);
  std::vector<HostZone> out;
  std::vector<uint32_t> stack;
  int ncolors = 0;
  while (true) {
    size_t first = 0;
    while (first < ids.size() && icolor[first] != -1) ++first;
    if (first == ids.size()) break;
    stack.clear();
    for (int j = 0; j < 4; ++j) stack.push_back(node(ids[first], j));
    while (!stack.empty()) {
      const uint32_t v = stack.back();
      stack.pop_back();
      const bool cloth = v < c.nv;
      if (cloth && !g.is_free(v)) continue;
      const std::vector<uint32_t>& ptr = cloth ? z.cvf_ptr : z.ovf_ptr;
      const std::vector<uint32_t>& list = cloth ? z.cvf_list : z.ovf_list;
      const std::vector<uint32_t>& tri = cloth ? c.h_tri : c.h_otri;
      const uint32_t lv = cloth ? v : v - c.nv, base = cloth ? 0u : c.nv;
      for (uint32_t q = ptr[lv]; q < ptr[lv + 1]; ++q) {
        const uint32_t f = list[q];
        for (int k = 0; k < 3; ++k) {
          const uint32_t u = base + tri[3 * f + k];
          if (color[u] == kInside) {
            color[u] = ncolors;
            stack.push_back(u);
          }
        }
      }
    }
    HostZone zone;
    for (size_t m = 0; m < ids.size(); ++m) {  // WriteBackNodeColor_Kernel
      if (icolor[m] != -1) continue;
      for (int j = 0; j < 4; ++j) {
        if (color[node(ids[m], j)] >= 0) {
          icolor[m] = ncolors;
          zone.impacts.push_back(ids[m]);
          break;
        }
      }
    }
    if (icolor[first] == -1) icolor[first] = -2;  // unreachable: dropped
    if (!zone.impacts.empty()) {
      for (uint32_t id : zone.impacts)
        for (int j = 0; j < 4; ++j) zone.nodes.push_back(node(id, j));
      std::sort(zone.nodes.begin(), zone.nodes.end());
      zone.nodes.erase(std::unique(zone.nodes.begin(), zone.nodes.end()), zone.nodes.end());
      out.push_back(std::move(zone));
    }
    ++ncolors;
  }
  return out;
}

bool intersects(const HostZone& a, const HostZone& b) {
  size_t i = 0, j = 0;
  while (i < a.nodes.size() && j < b.nodes.size()) {
    if (a.nodes[i] == b.nodes[j]) return true;
    if (a.nodes[i] < b.nodes[j]) ++i; else ++j;
  }
  return false;
}

void absorb(HostZone& a, HostZone& b) {  // ImpactZone::Merge
  a.impacts.insert(a.impacts.end(), b.impacts.begin(), b.impacts.end());
  std::vector<uint32_t> u;
  std::set_union(a.nodes.begin(), a.nodes.end(), b.nodes.begin(), b.nodes.end(),
                 std::back_inserter(u));
  a.nodes.swap(u);
  a.active = true;
  a.enabled = true;
  b.enabled = false;
}

// AddImpacts: the earlier zones turn passive; each absorbs, in order, the new zones it shares a
// node with; the remaining new zones are appended; then zones absorb later zones they share a node
// with, repeated until no two zones share a node.
void add_impacts(std::vector<HostZone>& zones, std::vector<HostZone>& fresh) {
  const size_t n0 = zones.size();
  for (HostZone& zz : zones) zz.active = false;
  for (size_t i = 0; i < n0; ++i)
    for (HostZone& f : fresh)
      if (f.enabled && intersects(zones[i], f)) absorb(zones[i], f);
  for (HostZone& f : fresh)
    if (f.enabled) zones.push_back(std::move(f));
  bool changed = true;
  while (changed) {
    changed = false;
    for (size_t i = 0; i < zones.size(); ++i) {
      if (!zones[i].enabled) continue;
      for (size_t j = i + 1; j < zones.size(); ++j) {
        if (zones[j].enabled && intersects(zones[i], zones[j])) {
          absorb(zones[i], zones[j]);
          changed = true;
        }
      }
    }
  }
  zones.erase(std::remove_if(zones.begin(), zones.end(), [](const HostZone& q) { return !q.enabled; }),
              zones.end());
}

xrt_status izone_prepare(Context& c) {
  ImpactZoneState& z = c.izone;
  if (z.ready) return XRT_OK;
  csr_node_faces(c.h_tri, c.nv, z.cvf_ptr, z.cvf_list);
  csr_node_faces(c.h_otri, c.onv, z.ovf_ptr, z.ovf_list);
  XRT_CUDA(&c, z.cbvh.reserve(c.nf));
  if (c.onf) XRT_CUDA(&c, z.obvh.reserve(c.onf));
  XRT_CUDA(&c, z.cx1.reserve(std::max(c.nv, 1u)));
  XRT_CUDA(&c, z.ox1.reserve(std::max(c.onv, 1u)));
  XRT_CUDA(&c, z.hit_total.reserve(1));
  XRT_CUDA(&c, z.inv_avg.reserve(1));
  z.ready = true;
  return XRT_OK;
}

// One pass of FindImpacts: pairs, CCD tests, compaction; the impacts' t and nodes on the host.
xrt_status find_impacts(Context& c, float thickness, std::vector<float>& t,
                        std::vector<uint4>& nodes) {
  ImpactZoneState& z = c.izone;
  const cudaStream_t s = c.stream;
  XRT_CUDA(&c, prox_face_pairs(c, z.cbvh, z.obvh, thickness));
  XRT_CUDA(&c, prox_check_impacts(c, thickness));
  const uint32_t np = c.prox.npairs;
  t.clear();
  nodes.clear();
  if (np == 0) return XRT_OK;
  XRT_CUDA(&c, z.hits.reserve(np));
  XRT_CUDA(&c, z.hit_incl.reserve(np));
  k_count_hits<<<grid_for(np), kBlock, 0, s>>>(c.prox.imp_t.p, np, z.hits.p);
  XRT_CUDA(&c, scan_inclusive(c.prox.scan, z.hits.p, z.hit_incl.p, np, z.hit_total.p, s));
  uint32_t total = 0;
  XRT_CUDA(&c, cudaMemcpyAsync(&total, z.hit_total.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  XRT_CUDA(&c, cudaStreamSynchronize(s));
  if (total == 0) return XRT_OK;
  XRT_CUDA(&c, z.new_t.reserve(total));
  XRT_CUDA(&c, z.new_nodes.reserve(total));
  XRT_CUDA(&c, z.new_src.reserve(total));
  k_compact_hits<<<grid_for(np), kBlock, 0, s>>>(c.prox.imp_t.p, c.prox.imp_nodes.p, np,
                                                 z.hit_incl.p, z.new_t.p, z.new_nodes.p,
                                                 z.new_src.p);
  t.resize(total);
  nodes.resize(total);
  XRT_CUDA(&c, cudaMemcpyAsync(t.data(), z.new_t.p, sizeof(float) * total, cudaMemcpyDeviceToHost, s));
  XRT_CUDA(&c, cudaMemcpyAsync(nodes.data(), z.new_nodes.p, sizeof(uint4) * total,
                               cudaMemcpyDeviceToHost, s));
  XRT_CUDA(&c, cudaStreamSynchronize(s));
  return XRT_OK;
}

// ParallelImpactZoneOptimizer over the active zones (list order), then Finalize.
xrt_status solve_zones(Context& c, const Graph& g, float obstacle_mass, float thickness,
                       uint32_t& nsolved, uint32_t* by_group) {
  ImpactZoneState& z = c.izone;
  const cudaStream_t s = c.stream;
  std::vector<int4> zone;
  std::vector<uint32_t> zimp, znode, gptr{0}, gslot;
  std::vector<int32_t> zloc;
  for (const HostZone& hz : z.zones) {
    if (!hz.active) continue;
    const int eb = (int)zimp.size(), nb = (int)znode.size();
    std::vector<uint32_t> opt;
    for (uint32_t v : hz.nodes)
      if (g.optimized(v)) opt.push_back(v);
    std::vector<std::vector<uint32_t>> slots(opt.size());
    for (size_t e = 0; e < hz.impacts.size(); ++e) {
      const uint32_t id = hz.impacts[e];
      const uint4 q = z.h_snodes[id];
      const uint32_t nd[4] = {q.x, q.y, q.z, q.w};
      const uint32_t ge = (uint32_t)zimp.size();
      zimp.push_back(id);
      for (int j = 0; j < 4; ++j) {
        auto it = std::lower_bound(opt.begin(), opt.end(), nd[j]);
        if (it != opt.end() && *it == nd[j]) {
          const size_t k = (size_t)(it - opt.begin());
          zloc.push_back(nb + (int)k);
          slots[k].push_back(4 * ge + (uint32_t)j);
        } else {
          zloc.push_back(-1);
        }
      }
    }
    for (size_t k = 0; k < opt.size(); ++k) {
      znode.push_back(opt[k]);
      gslot.insert(gslot.end(), slots[k].begin(), slots[k].end());
      gptr.push_back((uint32_t)gslot.size());
    }
    zone.push_back(make_int4(eb, (int)zimp.size(), nb, (int)znode.size()));
  }
  nsolved = (uint32_t)zone.size();
  if (zone.empty()) return XRT_OK;
  const uint32_t nz = (uint32_t)zone.size(), ne = (uint32_t)zimp.size(), nn = (uint32_t)znode.size();
  XRT_CUDA(&c, put(z.zone, zone, s));
  XRT_CUDA(&c, put(z.zimp, zimp, s));
  XRT_CUDA(&c, put(z.zloc, zloc, s));
  XRT_CUDA(&c, put(z.znode, znode, s));
  XRT_CUDA(&c, put(z.gptr, gptr, s));
  XRT_CUDA(&c, put(z.gslot, gslot, s));
  XRT_CUDA(&c, z.X.reserve(std::max(nn, 1u)));
  XRT_CUDA(&c, z.Xt.reserve(std::max(nn, 1u)));
  XRT_CUDA(&c, z.grad.reserve(std::max(nn, 1u)));
  XRT_CUDA(&c, z.lambda.reserve(ne));
  XRT_CUDA(&c, z.cc.reserve(ne));
  XRT_CUDA(&c, z.conv.reserve(nz));
  XRT_CUDA(&c, z.partial.reserve(grid_for(std::max(nn, 1u), kZT)));
  k_inv_avg<<<1, kZT, 0, s>>>(z.znode.p, nn, c.x.p, c.nv, obstacle_mass, z.partial.p, z.inv_avg.p);
  ZoneArgs a{z.zone.p, z.zimp.p, z.zloc.p, z.znode.p, z.gptr.p, z.gslot.p, z.sw.p, z.sn.p,
             z.snodes.p, c.x.p, c.ox.p, z.cx1.p, z.ox1.p, z.X.p, z.Xt.p, z.grad.p, z.lambda.p,
             z.cc.p, z.conv.p, z.inv_avg.p, c.nv, obstacle_mass, thickness, c.err.p};
  // zones by size: one block (<= 1 chunk), a cluster of 8 (<= 8 chunks), of 16 blocks
  // (<= 16 chunks), of 16 blocks of 4 groups (more)
  const int wg = wide_clusters();
  std::vector<int32_t> group[4];
  for (uint32_t q = 0; q < nz; ++q) {
    const int n = std::max(zone[q].y - zone[q].x, zone[q].w - zone[q].z);
    int g = n <= kZT ? 0 : (n <= kZoneCluster * kZT ? 1 : (n <= kZoneClusterWide * kZT ? 2 : 3));
    if (g == 3 && !(wg & 2)) g = 2;
    if (g == 2 && !(wg & 1)) g = 1;
    group[g].push_back((int32_t)q);
  }
  std::vector<int32_t> order;
  uint32_t off[5] = {0, 0, 0, 0, 0};
  for (int g = 0; g < 4; ++g) {
    order.insert(order.end(), group[g].begin(), group[g].end());
    off[g + 1] = (uint32_t)order.size();
  }
  XRT_CUDA(&c, put(z.zid, order, s));
  const uint32_t n0 = off[1], n1 = off[2] - off[1], n2 = off[3] - off[2], n3 = off[4] - off[3];
  by_group[0] += n2;
  by_group[1] += n3;
  if (n0) k_zone_solve<1, 1><<<n0, kZT, 0, s>>>(a, z.zid.p);
  if (n1) k_zone_solve<kZoneCluster, 1><<<n1 * kZoneCluster, kZT, 0, s>>>(a, z.zid.p + off[1]);
  if (n2)
    k_zone_solve<kZoneClusterWide, 1><<<n2 * kZoneClusterWide, kZT, 0, s>>>(a, z.zid.p + off[2]);
  if (n3)
    k_zone_solve<kZoneClusterWide, kWideGroups><<<n3 * kZoneClusterWide, kWideGroups * kZT, 0, s>>>(
        a, z.zid.p + off[3]);
  k_zone_finalize<<<nz, kZT, 0, s>>>(z.zone.p, z.conv.p, nz, z.znode.p, z.X.p, z.Xt.p, c.x.p,
                                     c.ox.p, c.nv);
  XRT_CUDA(&c, cudaGetLastError());
  return XRT_OK;
}

}  // namespace

xrt_status collision_step(Context& c, float obstacle_mass, float thickness, xrt_collision_stats* out) {
  xrt_collision_stats st{};
  if (out) *out = st;
  if (c.nf == 0) {
    if (out) out->success = 1;
    return XRT_OK;
  }
  xrt_status r = prox_prepare(c);
  if (r != XRT_OK) return r;
  if ((r = izone_prepare(c)) != XRT_OK) return r;
  ImpactZoneState& z = c.izone;
  const cudaStream_t s = c.stream;
  // SetupNode_Kernel / SetupObstacleNode_Kernel: x1 = x; obstacle v = (x - x0) / substep time
  XRT_CUDA(&c, cudaMemcpyAsync(z.cx1.p, c.x.p, sizeof(float4) * c.nv, cudaMemcpyDeviceToDevice, s));
  if (c.onv) {
    XRT_CUDA(&c, cudaMemcpyAsync(z.ox1.p, c.ox.p, sizeof(float4) * c.onv, cudaMemcpyDeviceToDevice, s));
    launch_node_velocity(c.ox.p, c.ox0.p, c.prox.ov.p, c.onv,
                         c.params.frame_time / (float)c.params.num_substeps, s);
  }
  // UpdateData(faces, 0, ccd = true) + Construct(0) of both meshes
  z.cbvh.n = c.nf;
  launch_prims_ccd(z.cbvh, c.x.p, c.x0.p, c.n.p, c.tri.p, c.nf, 0.0f, s);
  z.cbvh.construct(0.0f, s, c.err.p);
  if (c.onf) {
    z.obvh.n = c.onf;
    launch_prims_ccd(z.obvh, c.ox.p, c.ox0.p, c.on.p, c.otri.p, c.onf, 0.0f, s);
    z.obvh.construct(0.0f, s, c.err.p);
  }
  float mass = obstacle_mass;
  bool success = false;
  std::vector<float> t;
  std::vector<uint4> nodes;
  for (int deform = 0; deform < 2 && !success; ++deform) {
    const Graph g{c, z, deform};
    z.zones.clear();
    z.h_snodes.clear();
    z.nstore = 0;
    st.deform = deform;
    st.passes = 0;
    for (int pass = 0; pass < kMaxPasses; ++pass) {
      st.passes = pass + 1;
      if ((r = find_impacts(c, thickness, t, nodes)) != XRT_OK) return r;
      if (t.empty()) {
        success = true;
        break;
      }
      std::vector<uint32_t> order(t.size());
      std::iota(order.begin(), order.end(), 0u);
      std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return t[a] < t[b]; });
      const std::vector<uint32_t> pick = independent_impacts(g, order, nodes, c.nv + c.onv);
      const uint32_t base = z.nstore, np = (uint32_t)pick.size();
      XRT_CUDA(&c, grow_keep(z.sw, base + np, base, s));
      XRT_CUDA(&c, grow_keep(z.sn, base + np, base, s));
      XRT_CUDA(&c, grow_keep(z.snodes, base + np, base, s));
      XRT_CUDA(&c, put(z.pick, pick, s));
      k_store_gather<<<grid_for(np), kBlock, 0, s>>>(z.pick.p, np, z.new_src.p, c.prox.imp_w.p,
                                                     c.prox.imp_n.p, z.new_nodes.p, base, z.sw.p,
                                                     z.sn.p, z.snodes.p);
      std::vector<uint32_t> ids(np);
      for (uint32_t i = 0; i < np; ++i) {
        ids[i] = base + i;
        z.h_snodes.push_back(nodes[pick[i]]);
      }
      z.nstore = base + np;
      st.impacts += np;
      std::vector<HostZone> fresh = isolate(g, ids);
      add_impacts(z.zones, fresh);
      uint32_t nsolved = 0;
      if ((r = solve_zones(c, g, mass, thickness, nsolved, st.wide_solves)) != XRT_OK) return r;
      st.solves += nsolved;
      launch_update_ccd(z.cbvh, c.x.p, c.x0.p, c.tri.p, s, c.err.p);
      if (deform == 1) {
        if (c.onf) launch_update_ccd(z.obvh, c.ox.p, c.ox0.p, c.otri.p, s, c.err.p);
        mass *= 0.5f;
      }
    }
    st.zones = (uint32_t)z.zones.size();
  }
  st.success = success ? 1 : 0;
  XRT_CUDA(&c, cudaGetLastError());
  if (out) *out = st;
  return XRT_OK;
}

void izone_release(Context& c) {
  ImpactZoneState& z = c.izone;
  z.cbvh.release();
  z.obvh.release();
  DBuf<float4>* f4[] = {&z.cx1, &z.ox1, &z.sw, &z.sn, &z.X, &z.Xt, &z.grad};
  for (auto* b : f4) b->release();
  DBuf<uint32_t>* u[] = {&z.hits, &z.hit_incl, &z.hit_total, &z.new_src, &z.pick, &z.zimp,
                         &z.znode, &z.gptr, &z.gslot};
  for (auto* b : u) b->release();
  DBuf<float>* f[] = {&z.new_t, &z.lambda, &z.cc, &z.inv_avg, &z.partial};
  for (auto* b : f) b->release();
  z.new_nodes.release();
  z.snodes.release();
  z.zone.release();
  z.zloc.release();
  z.conv.release();
  z.zid.release();
  z.zones.clear();
  z.ready = false;
}

}  // namespace xrt

extern "C" xrt_status xrt_collision_step(xrt_ctx* h, float obstacle_mass, float thickness,
                                         xrt_collision_stats* out) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  xrt::Context& c = h->c;
  if (!c.started) {
    c.set_error("call xrt_start first");
    return XRT_ERR_STATE;
  }
  if (!(obstacle_mass > 0.0f) || !(thickness >= 0.0f)) {
    c.set_error("obstacle_mass must be > 0 and thickness >= 0");
    return XRT_ERR_INVALID_CONFIG;
  }
  cudaSetDevice(c.device);
  return xrt::collision_step(c, obstacle_mass, thickness, out);
}
