"""The FEM fabric (include/xrt_fem.h) on the GPU against the oracle's restatement of
FEMHelper.cu: strain and isometric bending frames bit for bit, tile-local and per-color
schedules, with obstacle contact and LRA."""
import numpy as np
import pytest

from tests.helpers import bits, make_pair, small_scene
from xrtailor_gb300 import ClothSolver, XrtError, scenes

pytestmark = pytest.mark.gpu


def _params(**kw):
    base = dict(num_substeps=4, num_iterations=5, num_collision_passes=4)
    base.update(kw)
    return scenes._params(**base)


@pytest.mark.parametrize("tile", [None, 0, 64])
def test_fem_frames_match_oracle(xrt, tile):
    cloth, obs = small_scene(20, attached=[0, 19])
    fem = ClothSolver.fem_material(xx_stiffness=2.0, yy_stiffness=1.5, xy_stiffness=0.7,
                                   bending_stiffness=5.0)
    g, o = make_pair(_params(), [cloth], [obs], fem=fem, tile_vertices=tile)
    for f in range(6):
        g.step()
        o.step()
        np.testing.assert_array_equal(bits(g.host_positions()), bits(o.host_positions()),
                                      err_msg=f"frame {f}")


def test_fem_without_bending_matches_oracle(xrt):
    cloth, obs = small_scene(16)
    fem = ClothSolver.fem_material(solve_bending=0)
    g, o = make_pair(_params(), [cloth], [obs], fem=fem)
    for _ in range(4):
        g.step()
        o.step()
    np.testing.assert_array_equal(bits(g.host_positions()), bits(o.host_positions()))


def test_fem_colorings_are_independent_sets(xrt):
    cloth, obs = small_scene(24)
    g = ClothSolver(_params())
    g.set_fem_material(ClothSolver.fem_material())
    g.add_cloth(cloth)
    g.add_obstacle(obs)
    g.start()
    for kind, idx in ((2, cloth.triangles), (3, g.bends()[0])):
        col = g.coloring(kind)
        assert len(col) == len(idx)
        seen = set()
        for c, verts in zip(col.tolist(), np.asarray(idx).tolist()):
            for v in verts:
                assert (c, v) not in seen, (kind, c, v)
                seen.add((c, v))


def test_fem_material_errors(xrt):
    cloth, obs = small_scene(8)
    s = ClothSolver(_params(enable_self_collision=0))
    with pytest.raises(XrtError):     # nu_xy nu_yx = 1: the tensor is singular
        s.set_fem_material(ClothSolver.fem_material(xy_poisson_ratio=1.0, yx_poisson_ratio=1.0))
    with pytest.raises(XrtError):
        s.set_fem_material(ClothSolver.fem_material(bending_stiffness=0.0))
    s.set_fem_material(ClothSolver.fem_material())
    s.add_cloth(cloth)
    s.start()
    with pytest.raises(XrtError):     # after start
        s.set_fem_material(ClothSolver.fem_material())
    with pytest.raises(XrtError):     # the adjoint covers the Swift fabric only
        s.diff_begin()
    s.step()
    assert np.isfinite(s.host_positions()).all()
