/* xrt_fem.h — the FEM fabric: orthotropic StVK strain per cloth face and isometric bending per
 * bend element (FEMFabricSettings, xrtailor/include/xrtailor/config/Base.hpp:47-57;
 * src/physics/dynamics/FEMHelper.cu), projected by the same colored / tile-local Gauss-Seidel
 * engine as the Swift fabric.
 *
 * With a FEM material set, each iteration of the frame projects the strain constraints (all
 * colors) and then the isometric bending constraints (when solve_bending) in place of the XPBD
 * stretch and dihedral bend constraints; everything else in the frame is unchanged.  The
 * reference runs this fabric inside SimulateQuality (src/pipeline/base/ClothSolverBase.cpp:
 * 263-345: strain colors, bending colors, LRA, bindings per iteration) together with its
 * repulsions and its impact-zone collision step, which xrt_swift_params switches on
 * (imminent_repulsion, pbd_repulsion, impact_zone; include/xrt_impact.h).
 *
 * Strain (ComputeStrainCorrection, FEMHelper.cu:96-173): Green strain from the deformation
 * gradient against the rest triangle's inverse 2x2 material matrix, orthotropic stress
 * C = [Ex, Ex nu_yx, 0; Ey nu_xy, Ey, 0; 0, 0, Es] / (1 - nu_xy nu_yx) (shear unscaled),
 * energy-based PBD step s = E / sum_i w_i |grad_i|^2.  Isometric bending (FEMHelper.cu:196-388):
 * energy 1/2 sum Q_jk x_j.x_k with the cotangent Hessian Q of the rest hinge, XPBD with
 * alpha = 1 / (stiffness dt^2) and a multiplier reset at iteration 0.
 */
#ifndef XRT_FEM_H
#define XRT_FEM_H

#include "xrt.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct xrt_fem_material {
  float xx_stiffness;       /* QUALITY.FABRIC.XX_STIFFNESS (1): Young's modulus along x */
  float yy_stiffness;       /* YY_STIFFNESS (1) */
  float xy_stiffness;       /* XY_STIFFNESS (1): shear modulus */
  float xy_poisson_ratio;   /* XY_POISSON_RATIO (0.3) */
  float yx_poisson_ratio;   /* YX_POISSON_RATIO (0.3) */
  float bending_stiffness;  /* BENDING_STIFFNESS (1) */
  int32_t solve_bending;    /* SOLVE_BENDING (1) */
  int32_t reserved[3];
} xrt_fem_material;

xrt_status xrt_default_fem_material(xrt_fem_material* out);
/* Selects the FEM fabric for the context (before xrt_start); NULL selects the Swift fabric (XPBD
 * stretch + dihedral bend, the default).  The strain rest state (area, inverse material matrix)
 * and the bending Hessians come from the cloths' initial world positions. */
xrt_status xrt_set_fem_material(xrt_ctx* ctx, const xrt_fem_material* material);

#ifdef __cplusplus
}
#endif

#endif
