/*
 * xrt_impact.h — the impact-zone collision step of XRTailor's Quality mode on a started xrt_ctx.
 *
 * Replaces ImpactZoneOptimization::CollisionStep (xrtailor/src/physics/impact_zone/Entry.cu:140-256),
 * called once per substep by ClothSolverBase::SimulateQuality (ClothSolverBase.cpp:329-336) after
 * the constraint iterations.  Merged contexts only (the reference's one cloth mesh and one
 * obstacle mesh).
 *
 * What a call does, on the cloth's x0 -> x and the obstacle's x0 -> x:
 *   - builds two LBVHs over the x0 -> x boxes of the cloth and the obstacle faces;
 *   - for deform = 0, then (if impacts remain after 100 passes) deform = 1, passes of
 *       FindImpacts (ImpactHelper.cu:207-232): face pairs cloth x obstacle and cloth x cloth,
 *         15 CCD tests per pair;
 *       independentImpacts (Entry.cu:25-63): impacts by time of impact, greedily independent;
 *       AddImpacts / FlattenImpactZones (ImpactZoneHelper.cu:325-396): new impacts grouped by
 *         mesh adjacency, merged with the earlier zones they share a node with;
 *       the augmented-Lagrangian zone solve (ParallelOptimizer.cu:513-880,
 *         ParallelImpactZoneOptimizer.cu) of every zone that gained impacts, one device block
 *         per zone, each zone with its own backtracking line search;
 *       refit of the cloth LBVH (and of the obstacle's, halving the obstacle mass, at deform 1);
 *     until a pass finds no impact.
 * Deform 0 moves free cloth vertices only; deform 1 also moves obstacle vertices (weighted by
 * `obstacle_mass`, IMPACT_ZONE.OBSTACLE_MASS, default 1e3).  `thickness` is
 * IMPACT_ZONE.THICKNESS (default 1e-4).
 */
#ifndef XRT_IMPACT_H_
#define XRT_IMPACT_H_

#include "xrt.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct xrt_collision_stats {
  int32_t success;        /* 1: the last pass found no impact */
  int32_t deform;         /* the deform level of the last pass (0 or 1) */
  int32_t passes;         /* passes of the last deform level */
  uint32_t impacts;       /* independent impacts solved, over both levels */
  uint32_t zones;         /* zones at the end of the last level */
  uint32_t solves;        /* zone solves launched (sum of active zones over the passes) */
  uint32_t wide_solves[2]; /* of those, zones too large for an 8-block cluster: solved by
                              16-block clusters of 256-thread blocks ([0]) or of 1,024-thread
                              blocks ([1]); a launch-shape record, not part of the algorithm */
} xrt_collision_stats;

/* One CollisionStep on the context's current state.  `out` may be NULL.  Synchronises (impact
 * counts are read back after each pass, as in the reference). */
xrt_status xrt_collision_step(xrt_ctx* ctx, float obstacle_mass, float thickness,
                              xrt_collision_stats* out);

#ifdef __cplusplus
}
#endif
#endif /* XRT_IMPACT_H_ */
