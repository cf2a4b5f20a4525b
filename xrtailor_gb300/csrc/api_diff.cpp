// api_diff.cpp — C ABI of the adjoint (include/xrt_diff.h); the work is in diff.cu.
#include <cuda_runtime.h>

#include "../../include/xrt_diff.h"
#include "context.h"

using xrt::Context;

extern "C" {

xrt_status xrt_diff_begin(xrt_ctx* h) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (!c.started) {
    c.set_error("call xrt_start first");
    return XRT_ERR_STATE;
  }
  cudaSetDevice(c.device);
  if (c.diff.active) xrt::diff_release(c);
  xrt_status st = xrt::diff_prepare(c);
  c.diff.interval = 1;
  return st;
}

xrt_status xrt_diff_begin_interval(xrt_ctx* h, int32_t substeps) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  const int32_t S = c.params.num_substeps;
  if (substeps <= 0 || S <= 0 || substeps % S != 0) {
    c.set_error("the checkpoint interval must be a positive multiple of num_substeps");
    return XRT_ERR_INVALID_ARGUMENT;
  }
  const xrt_status st = xrt_diff_begin(h);
  if (st == XRT_OK) c.diff.interval = (uint32_t)(substeps / S);
  return st;
}

xrt_status xrt_backward(xrt_ctx* h, const float* dL_dx, const float* dL_dv,
                        const xrt_grads* out) {
  if (!h || !dL_dx) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  cudaSetDevice(c.device);
  const xrt_grads none{};
  const xrt_grads& o = out ? *out : none;
  return xrt::diff_backward(c, dL_dx, dL_dv, o.stretch_compliance, o.bend_compliance, o.mass,
                            o.velocity, o.position);
}

xrt_status xrt_diff_end(xrt_ctx* h) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  cudaSetDevice(c.device);
  cudaStreamSynchronize(c.stream);
  xrt::diff_release(c);
  return XRT_OK;
}

}  // extern "C"
