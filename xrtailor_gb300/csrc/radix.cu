// radix.cu — stable LSD radix sort of (uint32 key, uint32 value) pairs, 8-bit digits.
//
// Replaces the library sorts of the reference path: thrust::stable_sort_by_key of Morton codes
// (xrtailor/src/physics/broad_phase/lbvh/BVH.cu:666-668) and cub::DeviceRadixSort::SortPairs of
// particle hashes (xrtailor/src/physics/broad_phase/spatial_hash/SpatialHashGPU.cu:102-119).
// Both are stable, so equal keys keep their input order; the sort here is stable too, which is
// what makes the sorted primitive order and the neighbor lists bit-identical to the reference's.
//
// Per 8-bit pass: (1) one block per 2048-key tile counts its digits (digit-major histogram);
// (2) the histogram is scanned into global offsets (one block, or three phases when large);
// (3) each tile ranks its keys stably (warp match + per-warp digit counts in shared memory, items
// in tile order) and scatters.
#include "common.cuh"
#include "context.h"

namespace xrt {
namespace {

constexpr int kItems = 8;
constexpr int kThreads = 256;
constexpr int kTile = kItems * kThreads;
constexpr int kWarps = kThreads / 32;
constexpr int kRadix = 256;
static_assert(kTile == (int)RadixSort::kTileKeys && kRadix == (int)RadixSort::kDigits,
              "tile and digit counts are shared with the fixed layouts of other files");

__global__ void __launch_bounds__(kThreads) k_histogram(const uint32_t* __restrict__ keys,
                                                        uint32_t n, int shift, uint32_t num_tiles,
                                                        uint32_t* __restrict__ hist) {
  __shared__ uint32_t s_count[kRadix];
  s_count[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * kTile;
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    uint32_t i = base + r * kThreads + threadIdx.x;
    if (i < n) atomicAdd(&s_count[(keys[i] >> shift) & 0xFFu], 1u);
  }
  __syncthreads();
  hist[threadIdx.x * num_tiles + blockIdx.x] = s_count[threadIdx.x];
}

// Exclusive scan of the digit-major histogram in three phases: each block of 1024 threads scans
// kScanChunk consecutive entries (4 per thread, coalesced) and records its total; one block scans
// the totals; each block adds its offset.  Integer sums, so the result does not depend on the
// split.
constexpr int kScanChunk = 4096;
static_assert(kScanChunk == (int)RadixSort::kScanChunk, "scan chunk shared through context.h");

__device__ __forceinline__ uint32_t block_exclusive_scan_1024(uint32_t v, uint32_t* s_warp,
                                                             uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = s_warp[lane];
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, off);
      if (lane >= off) w += y;
    }
    s_warp[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  const uint32_t before = warp > 0 ? s_warp[warp - 1] : 0u;
  if (total) *total = s_warp[31];
  return before + x - v;
}

__global__ void __launch_bounds__(1024) k_scan_chunks(uint32_t* __restrict__ data, uint32_t count,
                                                      uint32_t* __restrict__ sums) {
  __shared__ uint32_t s_warp[32];
  const uint32_t base = blockIdx.x * kScanChunk + threadIdx.x * 4;
  uint32_t v[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) v[r] = base + r < count ? data[base + r] : 0u;
  const uint32_t mine = v[0] + v[1] + v[2] + v[3];
  uint32_t total = 0;
  uint32_t run = block_exclusive_scan_1024(mine, s_warp, &total);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    if (base + r < count) data[base + r] = run;
    run += v[r];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Exclusive scan of the chunk totals (one block; `n` small) in place.
__global__ void __launch_bounds__(1024) k_scan_sums(uint32_t* __restrict__ sums, uint32_t n) {
  __shared__ uint32_t s_warp[32];
  uint32_t carry = 0;
  for (uint32_t b = 0; b < n; b += 1024) {
    const uint32_t i = b + threadIdx.x;
    const uint32_t v = i < n ? sums[i] : 0u;
    uint32_t total = 0;
    const uint32_t ex = block_exclusive_scan_1024(v, s_warp, &total);
    if (i < n) sums[i] = carry + ex;
    carry += total;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(1024) k_scan_add(uint32_t* __restrict__ data, uint32_t count,
                                                   const uint32_t* __restrict__ sums) {
  const uint32_t off = sums[blockIdx.x];
  const uint32_t base = blockIdx.x * kScanChunk + threadIdx.x * 4;
#pragma unroll
  for (int r = 0; r < 4; ++r)
    if (base + r < count) data[base + r] += off;
}

// Exclusive scan of `count` entries by one block of 1024 threads (small histograms).
__global__ void __launch_bounds__(1024) k_scan(uint32_t* __restrict__ data, uint32_t count) {
  __shared__ uint32_t s_part[1024];
  const uint32_t per = (count + 1023) / 1024;
  const uint32_t begin = threadIdx.x * per;
  const uint32_t end = min(begin + per, count);
  uint32_t sum = 0;
  for (uint32_t i = begin; i < end; ++i) sum += data[i];
  s_part[threadIdx.x] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    uint32_t v = threadIdx.x >= (unsigned)off ? s_part[threadIdx.x - off] : 0u;
    __syncthreads();
    s_part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = s_part[threadIdx.x] - sum;
  for (uint32_t i = begin; i < end; ++i) {
    uint32_t v = data[i];
    data[i] = run;
    run += v;
  }
}

__global__ void __launch_bounds__(kThreads) k_scatter(const uint32_t* __restrict__ keys_in,
                                                      const uint32_t* __restrict__ vals_in,
                                                      uint32_t* __restrict__ keys_out,
                                                      uint32_t* __restrict__ vals_out, uint32_t n,
                                                      int shift, uint32_t num_tiles,
                                                      const uint32_t* __restrict__ offsets) {
  __shared__ uint32_t s_warp_cnt[kWarps][kRadix];
  __shared__ uint32_t s_warp_off[kWarps][kRadix];
  __shared__ uint32_t s_run[kRadix];
  __shared__ uint32_t s_base[kRadix];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int w = 0; w < kWarps; ++w) s_warp_cnt[w][threadIdx.x] = 0;
  s_run[threadIdx.x] = 0;
  s_base[threadIdx.x] = offsets[threadIdx.x * num_tiles + blockIdx.x];
  __syncthreads();
  const uint32_t base = blockIdx.x * kTile;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int r = 0; r < kItems; ++r) {
    const uint32_t i = base + r * kThreads + threadIdx.x;
    const bool valid = i < n;
    uint32_t key = 0, val = 0, digit = kRadix;  // kRadix marks "no item"
    if (valid) {
      key = keys_in[i];
      val = vals_in[i];
      digit = (key >> shift) & 0xFFu;
    }
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, digit);
    const uint32_t lane_rank = __popc(peers & lt_mask);
    if (valid && lane_rank == 0) s_warp_cnt[warp][digit] = __popc(peers);
    __syncthreads();
    {
      const int d = threadIdx.x;
      uint32_t run = s_run[d];
#pragma unroll
      for (int w = 0; w < kWarps; ++w) {
        uint32_t c = s_warp_cnt[w][d];
        s_warp_off[w][d] = run;
        run += c;
        s_warp_cnt[w][d] = 0;
      }
      s_run[d] = run;
    }
    __syncthreads();
    if (valid) {
      const uint32_t dst = s_base[digit] + s_warp_off[warp][digit] + lane_rank;
      keys_out[dst] = key;
      vals_out[dst] = val;
    }
    __syncthreads();
  }
}

}  // namespace

cudaError_t RadixSort::reserve(uint32_t n) {
  cudaError_t e = keys_tmp.reserve(n);
  if (e == cudaSuccess) e = vals_tmp.reserve(n);
  if (e == cudaSuccess) e = hist.reserve(hist_entries(n));
  if (e == cudaSuccess) e = sums.reserve(sums_entries(n));
  return e;
}

void RadixSort::sort(uint32_t* keys, uint32_t* vals, uint32_t n, int bits, cudaStream_t s,
                     uint32_t** out_keys, uint32_t** out_vals) {
  uint32_t* k_in = keys;
  uint32_t* v_in = vals;
  uint32_t* k_out = keys_tmp.p;
  uint32_t* v_out = vals_tmp.p;
  if (n > 0) {
    const uint32_t tiles = (n + kTile - 1) / kTile;
    for (int shift = 0; shift < bits; shift += 8) {
      k_histogram<<<tiles, kThreads, 0, s>>>(k_in, n, shift, tiles, hist.p);
      const uint32_t entries = kRadix * tiles;
      if (entries <= kSingleBlockScan) {
        k_scan<<<1, 1024, 0, s>>>(hist.p, entries);
      } else {
        const uint32_t chunks = (entries + kScanChunk - 1) / kScanChunk;
        k_scan_chunks<<<chunks, 1024, 0, s>>>(hist.p, entries, sums.p);
        k_scan_sums<<<1, 1024, 0, s>>>(sums.p, chunks);
        k_scan_add<<<chunks, 1024, 0, s>>>(hist.p, entries, sums.p);
      }
      k_scatter<<<tiles, kThreads, 0, s>>>(k_in, v_in, k_out, v_out, n, shift, tiles, hist.p);
      uint32_t* t = k_in;
      k_in = k_out;
      k_out = t;
      t = v_in;
      v_in = v_out;
      v_out = t;
    }
  }
  *out_keys = k_in;
  *out_vals = v_in;
}

}  // namespace xrt
