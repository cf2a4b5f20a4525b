"""The oracle's FEM fabric (restating FEMHelper.cu) on its own: a sheet at rest stays at rest,
and a hanging sheet stays bounded.  CPU only."""
import numpy as np

from oracle.oracle import OracleSolver
from xrtailor_gb300 import ClothSolver, scenes


def _solver(cloth, obstacle=None, **kw):
    base = dict(num_substeps=4, num_iterations=5, num_collision_passes=4,
                enable_self_collision=0)
    base.update(kw)
    o = OracleSolver(scenes._params(**base))
    o.set_fem_material(ClothSolver.fem_material())
    o.add_cloth(cloth)
    if obstacle is not None:
        o.add_obstacle(obstacle)
    o.start()
    return o


def test_flat_sheet_at_rest_stays_at_rest():
    # flat rest state: zero Green strain, and the isometric bending energy of a flat hinge is 0
    cloth = scenes.grid_cloth(12, 0.5, origin=(0.0, 1.0, 0.0), jitter=0.0)
    o = _solver(cloth, gravity=(0.0, 0.0, 0.0))
    x0 = o.host_positions().copy()
    o.step(5)
    assert np.abs(o.host_positions() - x0).max() < 1e-6


def test_hanging_sheet_stays_bounded():
    cloth = scenes.grid_cloth(16, 0.6, origin=(0.0, 1.0, 0.0), jitter=1e-3)
    cloth.fixed_indices = scenes.two_corner_pins(16)
    o = _solver(cloth)
    o.step(20)
    x = o.host_positions()
    assert np.isfinite(x).all()
    # the sheet hangs from its pinned edge corners: it falls, but the strain keeps its extent
    edges, rest = o.edges()
    ln = np.linalg.norm(x[edges[:, 0]] - x[edges[:, 1]], axis=1)
    assert x[:, 1].max() <= 1.0 + 2e-3 and np.median(ln / rest) < 1.1   # jitter is 1e-3
