// noalloc.cu — LBVH build that allocates nothing: xrt_lbvh_build_noalloc.
//
// Who needs it: applications that embed the cloth step inside their own frame loop, such as a
// game engine or a DCC plugin host.  These hosts own the GPU memory budget and forbid plugins from
// allocating after start-up, because cudaMalloc / cudaFree can synchronise the device and stall
// the host's frame, and may fail halfway through a frame when memory is tight.  Such a caller
// provides its own input and output buffers; this entry point never asks the CUDA runtime for
// memory.  Its working memory is one fixed array in device global memory, declared below.
//
// Limits and sharing:
//   - at most kNoAllocMaxPrims (65,536) primitives per call; larger inputs are rejected with
//     XRT_ERR_FACE_CAPACITY before any work is queued;
//   - the scratch array is about 17 MiB per GPU.  It exists on every GPU that loads this
//     library, from the first use on that GPU until the process exits;
//   - every call on a GPU uses the same array, which keeps the last call's contents.  Each call
//     clears what it relies on being zero.  Calls whose device work overlaps in time (different
//     streams, or different host threads without ordering) race on the array and corrupt each
//     other's results; serialise them on one stream.
//   - The first call on each GPU looks up the device address of the array (cudaGetSymbolAddress),
//     with that GPU current.  Make that first call before any stream capture begins on the GPU.
#include <mutex>

#include "../../include/xrt.h"
#include "common.cuh"
#include "context.h"

namespace xrt {
namespace {

constexpr uint32_t kNoAllocMaxPrims = 65536;

constexpr size_t al(size_t x) { return (x + 255) & ~size_t(255); }

struct Layout {
  size_t v, pred, leaf_lo, leaf_hi, lo, hi, node, morton, index, keys_tmp, vals_tmp, hist, sums,
      key64, flags, iesc, eesc, root, dup, err, total;
};

constexpr Layout make_layout(size_t n) {
  Layout L{};
  size_t o = 0;
  L.v = o;        o += al(3 * n * 16);
  L.pred = o;     o += al(3 * n * 16);
  L.leaf_lo = o;  o += al(n * 16);
  L.leaf_hi = o;  o += al(n * 16);
  L.lo = o;       o += al(2 * n * 16);
  L.hi = o;       o += al(2 * n * 16);
  L.node = o;     o += al(2 * n * 16);
  L.morton = o;   o += al(n * 4);
  L.index = o;    o += al(n * 4);
  L.keys_tmp = o; o += al(n * 4);
  L.vals_tmp = o; o += al(n * 4);
  L.hist = o;     o += al(RadixSort::hist_entries(n) * 4);
  L.sums = o;     o += al(RadixSort::sums_entries(n) * 4);
  L.key64 = o;    o += al(n * 8);
  L.flags = o;    o += al(n * 4);
  L.iesc = o;     o += al(n * 4);
  L.eesc = o;     o += al(n * 4);
  L.root = o;     o += al(6 * 4);
  L.dup = o;      o += al(4);
  L.err = o;      o += al(4);
  L.total = o;
  return L;
}

constexpr Layout kLayout = make_layout(kNoAllocMaxPrims);

// The sort's histogram at the cap is scanned by one block, so the build stays within the layout
// whatever the radix sort's tile size; `sums` is carved out all the same, so a larger cap or a
// smaller scan chunk cannot send the multi-block scan through a null pointer.
static_assert(RadixSort::hist_entries(kNoAllocMaxPrims) <= RadixSort::kSingleBlockScan,
              "the no-allocation cap must keep the radix histogram in the single-block scan");
static_assert(kLayout.total < (size_t(64) << 20), "the fixed scratch array stays modest");

// The fixed working memory of xrt_lbvh_build_noalloc (see the header comment of this file).
static __device__ __align__(256) unsigned char g_lbvh_scratch[kLayout.total];

std::mutex g_scratch_mutex;
constexpr int kMaxDevices = 256;
unsigned char* g_scratch_addr[kMaxDevices] = {};

// Device address of g_lbvh_scratch on the current device; looked up once per device.
cudaError_t scratch_address(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_lbvh_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

__global__ void k_export_boxes(const float4* __restrict__ lo, const float4* __restrict__ hi,
                               uint32_t nn, float* __restrict__ out) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nn) return;
  const float4 a = lo[k], b = hi[k];
  float* r = out + 6 * (size_t)k;
  r[0] = a.x; r[1] = a.y; r[2] = a.z;
  r[3] = b.x; r[4] = b.y; r[5] = b.z;
}

template <typename T>
void point_at(DBuf<T>& d, unsigned char* base, size_t offset, size_t count) {
  d.p = reinterpret_cast<T*>(base + offset);  // non-owning: DBuf has no destructor
  d.n = count;
}

}  // namespace
}  // namespace xrt

extern "C" xrt_status xrt_lbvh_build_noalloc(const float* d_prims, const float* d_pred, uint32_t n,
                                             float scr, uint32_t* d_sorted_morton,
                                             uint32_t* d_sorted_objects, uint32_t* d_nodes,
                                             float* d_aabbs, int32_t* d_iesc, int32_t* d_eesc,
                                             void* stream) {
  using namespace xrt;
  if (!d_prims || !d_sorted_morton || !d_sorted_objects || !d_nodes || !d_aabbs || !d_eesc ||
      (n > 1 && !d_iesc))
    return XRT_ERR_INVALID_ARGUMENT;
  if (n == 0) return XRT_ERR_INVALID_ARGUMENT;
  if (n > kNoAllocMaxPrims) return XRT_ERR_FACE_CAPACITY;
  unsigned char* base = nullptr;
  if (scratch_address(&base) != cudaSuccess) return XRT_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t N = kNoAllocMaxPrims;
  Lbvh b;
  point_at(b.v, base, kLayout.v, 3 * N);
  point_at(b.pred, base, kLayout.pred, 3 * N);
  point_at(b.leaf_lo, base, kLayout.leaf_lo, N);
  point_at(b.leaf_hi, base, kLayout.leaf_hi, N);
  point_at(b.lo, base, kLayout.lo, 2 * N);
  point_at(b.hi, base, kLayout.hi, 2 * N);
  point_at(b.node, base, kLayout.node, 2 * N);
  point_at(b.morton, base, kLayout.morton, N);
  point_at(b.index, base, kLayout.index, N);
  point_at(b.sorter.keys_tmp, base, kLayout.keys_tmp, N);
  point_at(b.sorter.vals_tmp, base, kLayout.vals_tmp, N);
  point_at(b.sorter.hist, base, kLayout.hist, RadixSort::hist_entries(N));
  point_at(b.sorter.sums, base, kLayout.sums, RadixSort::sums_entries(N));
  point_at(b.key64, base, kLayout.key64, N);
  point_at(b.flags, base, kLayout.flags, N);
  point_at(b.iesc, base, kLayout.iesc, N);
  point_at(b.eesc, base, kLayout.eesc, N);
  point_at(b.root, base, kLayout.root, 6);
  point_at(b.dup, base, kLayout.dup, 1);
  uint32_t* err = reinterpret_cast<uint32_t*>(base + kLayout.err);
  b.n = n;
  // Zero what the build relies on: the error word here; the arrival counters and the root box
  // are reset inside construct() (cudaMemsetAsync / k_root_init).  Every other array is fully
  // overwritten before it is read.
  if (cudaMemsetAsync(err, 0, sizeof(uint32_t), s) != cudaSuccess) return XRT_ERR_CUDA;
  launch_float9_to_float4(d_prims, b.v.p, n, s);
  launch_float9_to_float4(d_pred ? d_pred : d_prims, b.pred.p, n, s);
  b.construct(scr, s, err);
  const size_t nn = 2 * (size_t)n - 1;
  cudaError_t e = cudaMemcpyAsync(d_sorted_morton, b.sorted_morton, 4 * (size_t)n,
                                  cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_sorted_objects, b.sorted_index, 4 * (size_t)n, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_nodes, b.node.p, 16 * nn, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && n > 1)
    e = cudaMemcpyAsync(d_iesc, b.iesc.p, 4 * ((size_t)n - 1), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_eesc, b.eesc.p, 4 * (size_t)n, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return XRT_ERR_CUDA;
  k_export_boxes<<<grid_for((uint32_t)nn), kBlock, 0, s>>>(b.lo.p, b.hi.p, (uint32_t)nn, d_aabbs);
  return cudaGetLastError() == cudaSuccess ? XRT_OK : XRT_ERR_CUDA;
}
