/* xrt_diff.h — hand-written adjoint of the Swift frame (reverse mode).
 *
 * No reference counterpart: XRTailor has no differentiable path.  The adjoint differentiates the
 * frame of xrt_step_frame (ClothSolverBase::SimulateSwift, ClothSolverBase.cpp:171-261):
 * predict, XPBD stretch with its multipliers, dihedral bend, geodesic LRA (pinned slots), the
 * obstacle VF / EE responses with the contact set held as recorded in the forward pass, and
 * finalize.  Frames with particle self-collision, Quality repulsion or bindings are rejected.
 *
 * Usage:  xrt_diff_begin(ctx) (or xrt_diff_begin_interval);  then any number of xrt_step_frame
 * calls (obstacle targets as usual);  then xrt_backward(ctx, dL/dx of the final positions, ...).
 * The state at every k-th substep boundary (k a multiple of the frame's substeps; k = one frame
 * by default) is checkpointed (cloth and obstacle state, 48 B per cloth vertex), and every
 * frame's obstacle targets are kept (16 B per obstacle vertex).  The reverse pass walks the
 * checkpoint segments newest first: it recomputes a segment's frames from its checkpoint, then
 * replays each of them, newest first, with taping kernels and walks the tape back.  Memory is
 * the checkpoints, one segment of frame states and one frame of tape; a longer interval trades
 * checkpoint memory for one more forward frame per recorded frame.  The recomputation is the
 * forward itself, so the gradients do not depend on the interval.  The context's state after
 * xrt_backward is the state before it.  The arithmetic is fp32, like the forward.
 */
#ifndef XRT_DIFF_H
#define XRT_DIFF_H

#include "xrt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Gradient outputs; any pointer may be NULL.  Orders are those of xrt_get_edges,
 * xrt_get_bends and the vertex numbering. */
typedef struct xrt_grads {
  float* stretch_compliance; /* num_edges */
  float* bend_compliance;    /* num_bends */
  float* mass;               /* num_vertices: dL/dm, m = 1 / inverse mass (0 for pinned) */
  float* velocity;           /* 3 x num_vertices: dL / d initial velocity */
  float* position;           /* 3 x num_vertices: dL / d initial position */
} xrt_grads;

/* Starts recording: the following frames are checkpointed for xrt_backward, every frame. */
xrt_status xrt_diff_begin(xrt_ctx* ctx);
/* The same with a checkpoint every `substeps` substeps: a positive multiple of num_substeps
 * (XRT_ERR_INVALID_ARGUMENT otherwise). */
xrt_status xrt_diff_begin_interval(xrt_ctx* ctx, int32_t substeps);
/* Reverse pass over the frames recorded since xrt_diff_begin.  dL_dx: 3 x num_vertices
 * (gradient of the loss with respect to the final positions); dL_dv: the same for the final
 * velocities, or NULL. */
xrt_status xrt_backward(xrt_ctx* ctx, const float* dL_dx, const float* dL_dv,
                        const xrt_grads* out);
/* Stops recording and frees the checkpoints and the tape. */
xrt_status xrt_diff_end(xrt_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif
