// cache.cu — frame cache and OBJ-sequence export (include/xrt_cache.h).
//
// The reference caches a frame by copying positions and normals to the host synchronously at
// the end of each frame (ClothSolverUniversal::SaveCache, universal/ClothSolver.cpp:107-144) and
// writes the sequence at the end (ObjSequenceExporter::ExportObjSequence,
// runtime/export/ObjSequenceExporter.cpp:155-250).  Here the end of each frame packs the cached
// arrays (float4 -> 3 floats) into one of a few device staging slots on the context's stream,
// and a copy stream, ordered after that packing by an event, moves the slot into a pinned host
// store.  The next frames run while the copies drain; a slot is reused only after its previous
// copy completed.
#include <cuda_runtime.h>

#include <cstdio>
#include <string>
#include <vector>

#include "../../include/xrt_cache.h"
#include "common.cuh"
#include "context.h"

namespace xrt {
namespace {

__global__ void k_pack3(const float4* __restrict__ src, uint32_t n, float* __restrict__ dst) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = src[i];
  dst[3 * i] = p.x;
  dst[3 * i + 1] = p.y;
  dst[3 * i + 2] = p.z;
}

// The cached arrays of one frame, in store order, with their element counts.
struct Part {
  const float4* src;
  uint32_t n;
};
std::vector<Part> parts(const Context& c) {
  std::vector<Part> out;
  const uint32_t f = c.cache.flags;
  if (f & XRT_CACHE_CLOTH) out.push_back({c.x0.p, c.nv});
  if ((f & XRT_CACHE_CLOTH) && (f & XRT_CACHE_NORMALS)) out.push_back({c.n.p, c.nv});
  if (f & XRT_CACHE_OBSTACLE) out.push_back({c.ox0.p, c.onv});
  if ((f & XRT_CACHE_OBSTACLE) && (f & XRT_CACHE_NORMALS)) out.push_back({c.on.p, c.onv});
  return out;
}

}  // namespace

void cache_release(Context& c) {
  CacheState& K = c.cache;
  if (K.copy) cudaStreamSynchronize(K.copy);
  if (K.host) cudaFreeHost(K.host);
  K.host = nullptr;
  for (int s = 0; s < CacheState::kSlots; ++s) {
    K.stage[s].release();
    if (K.staged[s]) cudaEventDestroy(K.staged[s]);
    if (K.copied[s]) cudaEventDestroy(K.copied[s]);
    K.staged[s] = K.copied[s] = nullptr;
    K.used[s] = false;
  }
  if (K.copy) cudaStreamDestroy(K.copy);
  K.copy = nullptr;
  K.on = false;
  K.count = K.capacity = K.per_frame = 0;
}

cudaError_t cache_frame(Context& c) {
  CacheState& K = c.cache;
  if (!K.on || K.count >= K.capacity) return cudaSuccess;
  const int s = (int)(K.count % CacheState::kSlots);
  cudaError_t e = cudaSuccess;
  if (K.used[s]) e = cudaStreamWaitEvent(c.stream, K.copied[s], 0);
  float* dst = K.stage[s].p;
  for (const Part& p : parts(c)) {
    if (e != cudaSuccess) return e;
    if (p.n) k_pack3<<<grid_for(p.n), kBlock, 0, c.stream>>>(p.src, p.n, dst);
    dst += 3 * (size_t)p.n;
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventRecord(K.staged[s], c.stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(K.copy, K.staged[s], 0);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(K.host + (size_t)K.count * K.per_frame, K.stage[s].p,
                        sizeof(float) * K.per_frame, cudaMemcpyDeviceToHost, K.copy);
  if (e == cudaSuccess) e = cudaEventRecord(K.copied[s], K.copy);
  K.used[s] = true;
  K.count++;
  return e;
}

}  // namespace xrt

using xrt::CacheState;
using xrt::Context;

namespace {

xrt_status cache_check(Context& c) {
  if (!c.cache.on) {
    c.set_error("call xrt_cache_begin first");
    return XRT_ERR_STATE;
  }
  return XRT_OK;
}

}  // namespace

extern "C" {

xrt_status xrt_cache_begin(xrt_ctx* h, uint32_t capacity_frames, int32_t flags) {
  if (!h || capacity_frames == 0) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  if (!c.started) {
    c.set_error("call xrt_start first");
    return XRT_ERR_STATE;
  }
  if (!(flags & (XRT_CACHE_CLOTH | XRT_CACHE_OBSTACLE)) ||
      (flags & ~(XRT_CACHE_CLOTH | XRT_CACHE_OBSTACLE | XRT_CACHE_NORMALS))) {
    c.set_error("cache flags: cloth and / or obstacle, optionally normals");
    return XRT_ERR_INVALID_ARGUMENT;
  }
  cudaSetDevice(c.device);
  XRT_CUDA(&c, cudaStreamSynchronize(c.stream));
  xrt::cache_release(c);
  CacheState& K = c.cache;
  K.flags = (uint32_t)flags;
  const size_t nrm = (flags & XRT_CACHE_NORMALS) ? 2 : 1;
  K.per_frame = (uint32_t)(3 * nrm *
                           (((flags & XRT_CACHE_CLOTH) ? c.nv : 0) +
                            ((flags & XRT_CACHE_OBSTACLE) ? c.onv : 0)));
  const size_t bytes = sizeof(float) * (size_t)K.per_frame * capacity_frames;
  cudaError_t e = cudaHostAlloc((void**)&K.host, bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    K.host = nullptr;
    c.set_error("frame cache: pinned host allocation of " + std::to_string(bytes) +
                " bytes failed");
    return XRT_ERR_CUDA;
  }
  for (int s = 0; s < CacheState::kSlots; ++s) {
    XRT_CUDA(&c, K.stage[s].reserve(std::max<size_t>(K.per_frame, 1)));
    XRT_CUDA(&c, cudaEventCreateWithFlags(&K.staged[s], cudaEventDisableTiming));
    XRT_CUDA(&c, cudaEventCreateWithFlags(&K.copied[s], cudaEventDisableTiming));
  }
  XRT_CUDA(&c, cudaStreamCreateWithFlags(&K.copy, cudaStreamNonBlocking));
  K.capacity = capacity_frames;
  K.count = 0;
  K.on = true;
  return XRT_OK;
}

xrt_status xrt_cache_count(xrt_ctx* h, uint32_t* out_frames) {
  if (!h || !out_frames) return XRT_ERR_INVALID_ARGUMENT;
  *out_frames = h->c.cache.on ? h->c.cache.count : 0;
  return XRT_OK;
}

xrt_status xrt_cache_read(xrt_ctx* h, uint32_t frame, float* cloth_positions,
                          float* cloth_normals, float* obstacle_positions,
                          float* obstacle_normals) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  xrt_status st = cache_check(c);
  if (st != XRT_OK) return st;
  CacheState& K = c.cache;
  if (frame >= K.count) {
    c.set_error("frame not cached");
    return XRT_ERR_INVALID_ARGUMENT;
  }
  cudaSetDevice(c.device);
  XRT_CUDA(&c, cudaStreamSynchronize(K.copy));
  const float* src = K.host + (size_t)frame * K.per_frame;
  auto take = [&](bool present, uint32_t n, float* out) {
    if (!present) return;
    if (out) std::copy(src, src + 3 * (size_t)n, out);
    src += 3 * (size_t)n;
  };
  const bool cl = K.flags & XRT_CACHE_CLOTH, ob = K.flags & XRT_CACHE_OBSTACLE,
             nr = K.flags & XRT_CACHE_NORMALS;
  take(cl, c.nv, cloth_positions);
  take(cl && nr, c.nv, cloth_normals);
  take(ob, c.onv, obstacle_positions);
  take(ob && nr, c.onv, obstacle_normals);
  return XRT_OK;
}

xrt_status xrt_cache_export_obj(xrt_ctx* h, const char* directory, int32_t which) {
  if (!h || !directory) return XRT_ERR_INVALID_ARGUMENT;
  Context& c = h->c;
  xrt_status st = cache_check(c);
  if (st != XRT_OK) return st;
  CacheState& K = c.cache;
  const bool obstacle = which == XRT_CACHE_OBSTACLE;
  if ((which != XRT_CACHE_CLOTH && !obstacle) || !(K.flags & (uint32_t)which)) {
    c.set_error("export: `which` must be a cached mesh (XRT_CACHE_CLOTH or XRT_CACHE_OBSTACLE)");
    return XRT_ERR_INVALID_ARGUMENT;
  }
  cudaSetDevice(c.device);
  XRT_CUDA(&c, cudaStreamSynchronize(K.copy));
  const bool nr = K.flags & XRT_CACHE_NORMALS;
  const uint32_t n = obstacle ? c.onv : c.nv;
  const std::vector<uint32_t>& tri = obstacle ? c.h_otri : c.h_tri;
  // offset of the mesh's positions within a cached frame
  size_t off = 0;
  if (obstacle && (K.flags & XRT_CACHE_CLOTH)) off = 3 * (size_t)c.nv * (nr ? 2 : 1);
  std::string line;
  char buf[160];
  for (uint32_t f = 0; f < K.count; ++f) {
    std::snprintf(buf, sizeof(buf), "%s/%06u.obj", directory, f);
    FILE* fp = std::fopen(buf, "w");
    if (!fp) {
      c.set_error(std::string("cannot write ") + buf);
      return XRT_ERR_INVALID_ARGUMENT;
    }
    const float* p = K.host + (size_t)f * K.per_frame + off;
    std::fputs("# Generated by XRTailor\no mesh\n", fp);
    for (uint32_t i = 0; i < n; ++i)
      std::fprintf(fp, "v %.6f %.6f %.6f\n", p[3 * i], p[3 * i + 1], p[3 * i + 2]);
    if (nr) {
      const float* q = p + 3 * (size_t)n;
      for (uint32_t i = 0; i < n; ++i)
        std::fprintf(fp, "vn %.6f %.6f %.6f\n", q[3 * i], q[3 * i + 1], q[3 * i + 2]);
    }
    std::fputs("s 1\n", fp);
    for (size_t t = 0; t + 2 < tri.size(); t += 3)
      std::fprintf(fp, "f %u %u %u\n", tri[t] + 1, tri[t + 1] + 1, tri[t + 2] + 1);
    if (std::fclose(fp) != 0) {
      c.set_error(std::string("cannot write ") + buf);
      return XRT_ERR_INVALID_ARGUMENT;
    }
  }
  return XRT_OK;
}

xrt_status xrt_cache_end(xrt_ctx* h) {
  if (!h) return XRT_ERR_INVALID_ARGUMENT;
  cudaSetDevice(h->c.device);
  xrt::cache_release(h->c);
  return XRT_OK;
}

}  // extern "C"
