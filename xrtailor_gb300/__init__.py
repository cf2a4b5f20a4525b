"""GB300-native per-substep cloth step of XRTailor's Swift mode.

The product is libxrt.so (C ABI in include/xrt.h, CUDA kernels for sm_103a under csrc/); this
package is its Python mirror of the reference's solver / configuration interface.
"""
from ._lib import XrtError, load  # noqa: F401
from .solver import (BasicFabricSettings, ClothSolver, Lbvh, Mesh, ParticleCollisionSettings,  # noqa: F401
                     SolverSettings, SwiftModeCollisionSettings, SwiftModeSettings, apply_swift,
                     parse_swift)

__all__ = ["ClothSolver", "Lbvh", "Mesh", "SwiftModeSettings", "parse_swift", "apply_swift",
           "XrtError", "load"]
