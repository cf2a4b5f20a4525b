/* xrt_cache.h — frame cache and OBJ-sequence export.
 *
 * Replaces ClothSolverUniversal::SaveCache (src/pipeline/impl/universal/ClothSolver.cpp:107-144),
 * which copies each frame's positions and normals to the host synchronously at the end of the
 * frame, and ObjSequenceExporter::ExportObjSequence
 * (src/runtime/export/ObjSequenceExporter.cpp:155-250).  After xrt_cache_begin each
 * xrt_step_frame ends by packing the cached arrays on the device and copying them, on a copy
 * stream that overlaps the following frames, into a pinned host store of capacity_frames frames;
 * frames past the capacity are not recorded (the reference stops at num_frames).
 */
#ifndef XRT_CACHE_H
#define XRT_CACHE_H

#include "xrt.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  XRT_CACHE_CLOTH = 1,     /* cloth positions (record_cloth) */
  XRT_CACHE_OBSTACLE = 2,  /* obstacle positions (record_obstacle) */
  XRT_CACHE_NORMALS = 4    /* and the normals of the cached meshes */
};

/* Starts recording the following frames (replaces any earlier recording).  After xrt_start.
 * Pinned host memory: capacity_frames x (3 floats per cached vertex, x2 with normals). */
xrt_status xrt_cache_begin(xrt_ctx* ctx, uint32_t capacity_frames, int32_t flags);
/* Frames recorded so far (their copies may still be in flight). */
xrt_status xrt_cache_count(xrt_ctx* ctx, uint32_t* out_frames);
/* Cached frame `frame` (0 = the first frame after xrt_cache_begin): 3 floats per vertex into each
 * non-NULL output whose array was cached.  Waits for the copies in flight. */
xrt_status xrt_cache_read(xrt_ctx* ctx, uint32_t frame, float* cloth_positions,
                          float* cloth_normals, float* obstacle_positions,
                          float* obstacle_normals);
/* Writes the cached frames of one mesh (which = XRT_CACHE_CLOTH or XRT_CACHE_OBSTACLE) as
 * directory/000000.obj, 000001.obj, ... in the reference's format: "o mesh", "v x y z" lines
 * (6 decimals), "vn" lines when normals were cached, "s 1", "f a b c" (1-based).  The
 * directory must exist. */
xrt_status xrt_cache_export_obj(xrt_ctx* ctx, const char* directory, int32_t which);
/* Stops recording and frees the store. */
xrt_status xrt_cache_end(xrt_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif
