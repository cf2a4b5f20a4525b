// skin.cu — obstacle skinning on the device: the obstacle's targets for the coming frame from
// its joint transforms, so a moving body costs one upload of its joints per frame instead of its
// vertex positions.
//
// Linear blend skinning as SMPL's lbs kernel (xrtailor/src/runtime/rag_doll/smpl/cuda/body.cu:39-60):
// per vertex and output row i, over the vertex's influences (CSR) in order,
//   out_i += (w T[i][j]) v_j  for j = 0, 1, 2,   then   out_i += w T[i][3],
// T the joint's global transform (top 3 rows of the 4x4, row-major).  The same products and sums
// in the same order; the library's no-contraction flags make the result reproducible (the
// reference builds with fast math).
#include "common.cuh"
#include "context.h"

namespace xrt {
namespace {

__global__ void k_skin(const float4* __restrict__ rest, const uint32_t* __restrict__ outer,
                       const uint32_t* __restrict__ joint, const float* __restrict__ weight,
                       const float* __restrict__ T, float4* __restrict__ out, uint32_t n) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const float4 p = rest[v];
  float o0 = 0.0f, o1 = 0.0f, o2 = 0.0f;
  const uint32_t b = outer[v], e = outer[v + 1];
  for (uint32_t k = b; k < e; ++k) {
    const float w = weight[k];
    const float* t = T + 12 * (size_t)joint[k];
    o0 += (w * t[0]) * p.x;
    o0 += (w * t[1]) * p.y;
    o0 += (w * t[2]) * p.z;
    o0 += w * t[3];
    o1 += (w * t[4]) * p.x;
    o1 += (w * t[5]) * p.y;
    o1 += (w * t[6]) * p.z;
    o1 += w * t[7];
    o2 += (w * t[8]) * p.x;
    o2 += (w * t[9]) * p.y;
    o2 += (w * t[10]) * p.z;
    o2 += w * t[11];
  }
  out[v] = make_float4(o0, o1, o2, 0.0f);
}

}  // namespace

void launch_skin(Context& c) {
  if (!c.skin.on || c.onv == 0) return;
  k_skin<<<grid_for(c.onv), kBlock, 0, c.stream>>>(c.skin.rest.p, c.skin.outer.p,
                                                   c.skin.joint.p, c.skin.weight.p,
                                                   c.skin.transforms.p, c.ox.p, c.onv);
}

}  // namespace xrt
