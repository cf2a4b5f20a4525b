/*
 * xrt_contact.h — cloth self-contact operators of XRTailor's Quality mode on a started xrt_ctx.
 *
 * These replace the reference's cloth-LBVH face-pair broad phase, PBD proximity repulsion and
 * CCD impact test (used by ClothSolverBase::SimulateQuality, ClothSolverBase.cpp:263-362).
 * Nodes, faces and edges are numbered cloth first, then obstacle (the reference's Node*, Face*,
 * Edge* pointers).  All entry points run on the context's stream and return xrt_status.
 */
#ifndef XRT_CONTACT_H_
#define XRT_CONTACT_H_

#include "xrt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* cloth_bvh_->UpdateData(faces, 0, false) + Construct() (ClothSolverBase.cpp:277-278):
 * LBVH over the cloth triangles at x0. */
xrt_status xrt_cloth_bvh_build(xrt_ctx* ctx);
/* obstacle_bvh_->Update(faces, true) (ClothSolverBase.cpp:293, BVH.cu:820-852): primitives take
 * the obstacle's current positions; leaves grow by the x / x0 bounds of their triangle. */
xrt_status xrt_obstacle_bvh_update_ccd(xrt_ctx* ctx);
/* PBDRepulsionSolver::UpdatePairs (PBDRepulsion.cu:22-32): cloth BVH Update(ccd), then the face
 * pairs cloth x obstacle followed by cloth x cloth whose boxes overlap after dilating the query
 * by `thickness` (Traverse, BVH.cu:1315-1340).  Synchronises to size the list. */
xrt_status xrt_proximity_update_pairs(xrt_ctx* ctx, float thickness, uint32_t* out_num_pairs);
/* PBDRepulsionSolver::SolveNoProximity (PBDRepulsion.cu:517-531): vertex-face and edge-edge
 * proximity constraints of every pair (EvaluateRep_Kernel), averaged impulses applied to the
 * cloth's predicted positions x with `relaxation` (ApplyPBDImpulse_Kernel). */
xrt_status xrt_proximity_solve(xrt_ctx* ctx, float thickness, float relaxation);
/* ImminentRepulsion::UpdateProximity + Generate (ImminentRepulsion.cu:21-102): face pairs cloth x
 * cloth then cloth x obstacle (thickness 1e-6) on the cloth LBVH as built and the obstacle LBVH
 * as it stands, then the edge-edge and vertex-face quadratures at x0.  Synchronises. */
xrt_status xrt_imminent_generate(xrt_ctx* ctx, uint32_t* out_num_quads);
/* the quadratures in Generate's order (edge-edge of every pair, then vertex-face): 4 unified
 * nodes and 4 weights each; either pointer may be NULL */
xrt_status xrt_export_quads(xrt_ctx* ctx, uint32_t* nodes, float* bary);
/* ImminentRepulsion::Solve (ImminentRepulsion.cu:153-169): cloth velocities (x - x0) / dt, the
 * quadratures' impulses (float atomics), ApplyImminentImpulse with `relaxation` */
xrt_status xrt_imminent_solve(xrt_ctx* ctx, float thickness, float relaxation, float dt);
/* CheckImpacts (ImpactHelper.cu:116-177) over the current pairs: 15 tests per pair (3 + 3
 * vertex-face, 9 edge-edge), coplanarity cubic over t in [0, 1] from x0 to x. */
xrt_status xrt_impacts_check(xrt_ctx* ctx, float thickness, uint32_t* out_num_impacts);

/* exports (synchronising): pairs 2 x uint32 per pair; impacts: t (-1 = none), w 4, n 3,
 * nodes 4 (unified), is_vf 1 per impact; any pointer may be NULL */
xrt_status xrt_export_pairs(xrt_ctx* ctx, uint32_t* pairs);
xrt_status xrt_export_impacts(xrt_ctx* ctx, float* t, float* w, float* n, uint32_t* nodes,
                              int32_t* is_vf);
xrt_status xrt_export_cloth_bvh(xrt_ctx* ctx, uint32_t* sorted_morton, uint32_t* sorted_objects,
                                uint32_t* nodes, float* aabbs, int32_t* i_esc, int32_t* e_esc);
/* cloth predicted positions x (3 floats per vertex); setting keeps the inverse masses */
xrt_status xrt_get_predicted(xrt_ctx* ctx, float* out);
xrt_status xrt_set_predicted(xrt_ctx* ctx, const float* positions);

#ifdef __cplusplus
}
#endif
#endif /* XRT_CONTACT_H_ */
