// common.cuh — device vector math and launch helpers of the GB300 cloth step.
//
// Vector operations keep glm's evaluation order (dot = (x*x' + y*y') + z*z', cross, length =
// sqrt(dot), normalize = v * (1/sqrt(dot))) and the library is compiled with --fmad=false and
// IEEE division / square root, so every float the kernels produce is reproducible on the host.
// That is what lets Morton codes, LBVH topology and candidate lists match the CPU restatement
// bit-for-bit (xrtailor/src/physics/broad_phase/lbvh/BVH.cu:22-46 feeds integer codes from float
// box centres; one ulp moves a code across a cell boundary).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

#define XRT_HD __host__ __device__ __forceinline__

namespace xrt {

struct f3 {
  float x, y, z;
};
XRT_HD f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
XRT_HD f3 mk3(float4 v) { return f3{v.x, v.y, v.z}; }
XRT_HD float4 mk4(f3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
XRT_HD f3 operator+(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
XRT_HD f3 operator-(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
XRT_HD f3 operator-(f3 a) { return f3{-a.x, -a.y, -a.z}; }
XRT_HD f3 operator*(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
XRT_HD f3 operator*(float s, f3 a) { return f3{s * a.x, s * a.y, s * a.z}; }
XRT_HD f3 operator/(f3 a, float s) { return f3{a.x / s, a.y / s, a.z / s}; }
XRT_HD float dot(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
XRT_HD f3 cross(f3 a, f3 b) {
  return f3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
XRT_HD float length(f3 v) { return sqrtf(dot(v, v)); }
XRT_HD f3 normalize(f3 v) { return v * (1.0f / sqrtf(dot(v, v))); }
XRT_HD float comp(f3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
template <typename T> XRT_HD T tmin(T a, T b) { return a < b ? a : b; }
template <typename T> XRT_HD T tmax(T a, T b) { return a > b ? a : b; }
template <typename T> XRT_HD T tclamp(T x, T a, T b) { return x < a ? a : (x > b ? b : x); }
template <typename T> XRT_HD T tabs(T x) { return x < T(0) ? -x : x; }

// Fused forms of the stretch and bend projections: every product-plus-term below is one fused
// multiply-add (fmaf, rounded once), in this expression tree on the device and in the CPU oracle
// (std::fma), so both sides still round identically while the projections issue about a fifth
// fewer floating-point instructions.
//   fdot(a,b)      = fma(a.z, b.z, fma(a.y, b.y, a.x*b.x))
//   fcross(a,b)    = (fma(a.y, b.z, -(b.y*a.z)), fma(a.z, b.x, -(b.z*a.x)), fma(a.x, b.y, -(b.x*a.y)))
//   fmad(a, s, b)  = a*s + b per component
XRT_HD float fdot(f3 a, f3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }
XRT_HD f3 fcross(f3 a, f3 b) {
  return f3{fmaf(a.y, b.z, -(b.y * a.z)), fmaf(a.z, b.x, -(b.z * a.x)),
            fmaf(a.x, b.y, -(b.x * a.y))};
}
XRT_HD f3 fmad(f3 a, float s, f3 b) {
  return f3{fmaf(a.x, s, b.x), fmaf(a.y, s, b.y), fmaf(a.z, s, b.z)};
}

// arccos on [0, 1] by Abramowitz & Stegun, Handbook of Mathematical Functions, formula 4.4.46:
// acos(x) = sqrt(1 - x) * (a0 + a1 x + ... + a7 x^7), |error| <= 2e-8, Horner steps fused.  The
// same expression is compiled for the device and for the CPU oracle, so bend projections agree
// bit for bit (the two platforms' acosf differ in the last place, and the bend solve amplifies
// that).
XRT_HD float acos_as(float x) {
  float p = -0.0012624911f;
  p = fmaf(p, x, 0.0066700901f);
  p = fmaf(p, x, -0.0170881256f);
  p = fmaf(p, x, 0.0308918810f);
  p = fmaf(p, x, -0.0501743046f);
  p = fmaf(p, x, 0.0889789874f);
  p = fmaf(p, x, -0.2145988016f);
  p = fmaf(p, x, 1.5707963050f);
  return sqrtf(1.0f - x) * p;
}

// MathFunctions::FaceNormal (src/math/MathFunctions.cu:14-20)
XRT_HD f3 face_normal(f3 a, f3 b, f3 c) { return normalize(cross(b - a, c - a)); }

constexpr float kEps = 1e-6f;             // EPSILON (core/Scalar.hpp:39)
constexpr float kScalarMax = 3.402823466e+38f;  // SCALAR_MAX = FLT_MAX (core/Scalar.cuh:10)
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kMaxCandidates = 256;  // LBVH_MAX_BUFFER_SIZE (core/Common.cuh:23)
constexpr int kBlock = 256;
constexpr int kFootPerThread = 8;   // footprint vertices per tile-block thread (x 512 <= 4096)

// Bits of the sticky device error word.
enum : uint32_t {
  kErrTraversal = 1u << 0,  // a traversal exceeded its visit bound
  kErrTreeWalk = 1u << 1,   // a bottom-up / escape walk exceeded its depth bound
  kErrIndex = 1u << 2,      // an index was out of range
  kErrZoneSize = 1u << 3,   // an impact zone exceeded 65,536 nodes or impacts
  kErrLineSearch = 1u << 4, // a zone's backtracking line search exceeded its step bound
  kErrBulkCopy = 1u << 5,   // a bulk copy into shared memory did not complete within its bound
};

__device__ __forceinline__ void raise_error(uint32_t* err, uint32_t bit) { atomicOr(err, bit); }

inline unsigned grid_for(uint32_t n, int block = kBlock) {
  return (unsigned)((n + (uint32_t)block - 1) / (uint32_t)block);
}

// Programmatic dependent launch.  A kernel launched with programmatic stream serialization may
// start while its predecessor on the stream still runs.  pdl_wait() returns once every
// prerequisite grid has completed and its writes are visible; everything before it may touch
// only data that no earlier kernel of the frame writes (setup-time records, index lists) and
// must not write global memory.  pdl_release() lets the successor grid start its own prologue.
// Both are no-ops for a kernel launched without the attribute.  Every kernel launched through
// launch_k with pdl set calls pdl_wait() in every block before its first dependent access, so
// grid completion stays ordered along the stream.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Bulk copy global -> shared memory completed on an mbarrier (cp.async.bulk with complete_tx,
// sm_90 and later).  Source and destination must be 16-byte aligned and the size a multiple of
// 16 bytes.  One thread initialises the barrier, announces the byte count and issues the copy;
// the block then waits on phase 0.
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
  // make the initialised barrier visible to the async proxy that completes it
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void bulk_load_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Waits for the barrier's phase `parity` to complete, polling at most `limit` times; returns
// false when the limit ran out (the caller reports it and leaves without using the data).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t k = 0; k < limit; ++k) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
constexpr uint32_t kBulkWaitLimit = 1u << 22;

template <typename... P, typename... A>
inline cudaError_t launch_k(bool pdl, void (*kern)(P...), unsigned grid, unsigned block,
                            size_t smem, cudaStream_t s, A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...);
}

}  // namespace xrt
